"""GPU FD1D-BS control variate (kwg_fd1d_bs_price: FD(asset) + BS(European copy) -
FD(European copy)) against the reference's golden output and the oracle.
Tolerance: REL_TOL = 1e-10 relative (FP64), like the plain FD1D path."""
import math

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10
# FD(asset) + BS - FD(copy) of a deep out-of-the-money option is a cancellation
# residue of O(1e-3 .. 1) terms (the oracle can give exactly 0, the GPU 1e-14):
# prices below this floor are compared absolutely, to REL_TOL * PRICE_FLOOR = 1e-13
PRICE_FLOOR = 1e-3


def rel_err(got, want):
    return float(np.max(np.abs(got - want) / np.maximum(np.abs(want), PRICE_FLOOR)))


def bs_price(ctx, opts, **kw):
    import kwg

    rc, p, st = ctx.fd1d_bs_price(opts, kwg.params(**kw))
    assert rc == kwg.KWG_OK, ctx.last_error()
    return p, st


@pytest.mark.parametrize("solver", [1, 2], ids=["thomas", "pcr"])
def test_pricer_test_table(ctx, solver):
    """test/kwPricer_test.cpp:87-107 (FD1D-BS, 12 options incl. European ones) at the
    reference defaults, against the reference's own output."""
    g = golden("pricer_test.npz")
    p, st = bs_price(ctx, g["opts"], solver=solver)
    assert (st == 0).all()
    assert rel_err(p, g["ref_fd1d_bs"]) <= REL_TOL
    assert np.max(np.abs(p - g["want"])) <= 1.3e-3


def test_128_options_vs_oracle(ctx):
    import kwor

    g = golden("synthetic.npz")
    kw = dict(t_dim=512, x_dim=512, scale=5.0, density=0.25)
    p, st = bs_price(ctx, g["small_opts"], **kw)
    rc, msg, want, _ = kwor.fd1d_price(g["small_opts"], bs=True, **kw)
    assert rc == 0, msg
    assert (st == 0).all()
    assert rel_err(p, want) <= REL_TOL


def test_portfolio_qdfp_vs_oracle(ctx):
    """6000 American puts (dedup to 600 PDEs; with the European copies 1200)."""
    import kwor

    g = golden("portfolio_qdfp.npz")
    p, st = bs_price(ctx, g["opts"])
    rc, msg, want, _ = kwor.fd1d_price(g["opts"], bs=True, nthreads=16)
    assert rc == 0, msg
    assert (st == 0).all()
    assert rel_err(p, want) <= REL_TOL
    assert np.max(np.abs(p - g["quantlib"])) <= 0.005


def test_european_assets_get_black_scholes(ctx):
    """For a European asset FD(asset) and FD(copy) are the same PDE, so the control
    variate returns the Black-Scholes price up to rounding."""
    import kwor
    import portfolio

    o = portfolio.american_portfolio(256, seed=8)
    o["e"] = 0
    p, st = bs_price(ctx, o, t_dim=256, x_dim=256, scale=5.0, density=math.inf)
    assert (st == 0).all()
    bs = kwor.bs_price(o)
    assert np.max(np.abs(p - bs)) <= 1e-12 * np.max(np.abs(bs))


def test_fp32_close_to_fp64(ctx):
    import kwg
    import portfolio

    o = portfolio.american_portfolio(2048, seed=9)
    kw = dict(t_dim=1024, x_dim=1024, scale=5.0, density=math.inf)
    p64, _ = bs_price(ctx, o, **kw)
    p32, st = bs_price(ctx, o, precision=kwg.FP32, **kw)
    assert (st == 0).all()
    assert np.max(np.abs(p32 - p64)) <= 1e-5


def test_strict_out_of_grid(ctx):
    """Strict mode fails the whole call like the reference; non-strict gives NaN and a
    per-option status."""
    import kwg

    g = golden("edge.npz")
    bad = g["bad_opts"]
    rc, p, st = ctx.fd1d_bs_price(bad, kwg.params(strict=1))
    rc2, p2, st2 = ctx.fd1d_price(bad, kwg.params(strict=1))
    assert rc == rc2
    rc, p, st = ctx.fd1d_bs_price(bad, kwg.params(strict=0))
    rc2, p2, st2 = ctx.fd1d_price(bad, kwg.params(strict=0))
    assert rc == kwg.KWG_OK
    assert np.array_equal(st, st2)
    assert np.array_equal(np.isnan(p), np.isnan(p2))


def test_pricer_factory(ctx):
    import kwg

    g = golden("pricer_test.npz")
    cfg = kwg.Config()
    cfg.set("PRICER", "FD1D-BS")
    err, pricer = kwg.PricerFactory.create(cfg)
    assert err == "" and isinstance(pricer, kwg.Fd1dBsGpuPricer)
    prices = [0.0] * len(g["opts"])
    assert pricer.price(g["opts"], prices) == ""
    assert rel_err(np.array(prices), g["ref_fd1d_bs"]) <= REL_TOL


@pytest.mark.parametrize("density", [0.25, math.inf])
def test_twin_tiles_streaming_solver(ctx, density):
    """The streaming FP64 solver runs each American PDE beside its European copy
    (lanes 2k, 2k+1 of the first tiles) on one shared coefficient and payoff record.
    A mix of American and European puts and calls with duplicates: 2 x 16 x 21 twin
    pairs fill 21 twin tiles with leftovers in ordinary tiles, against the oracle."""
    import kwor
    import portfolio

    o = portfolio.american_portfolio(700, seed=41)
    o["w"][::2] = -o["w"][::2]
    o["e"][5::7] = 0
    o = np.concatenate([o, o[:60]])  # duplicates share their PDEs
    kw = dict(t_dim=257, x_dim=384, scale=5.0, density=density)
    p, st = bs_price(ctx, o, solver=1, **kw)
    rc, msg, want, _ = kwor.fd1d_price(o, bs=True, **kw)
    assert rc == 0, msg
    assert (st == 0).all()
    assert rel_err(p, want) <= REL_TOL


def test_twin_tiles_qdfp_portfolio(ctx):
    """6000 American puts at the reference defaults through the streaming solver:
    600 twin pairs, 37 twin tiles."""
    import kwor

    g = golden("portfolio_qdfp.npz")
    p, st = bs_price(ctx, g["opts"], solver=1)
    rc, msg, want, _ = kwor.fd1d_price(g["opts"], bs=True, nthreads=16)
    assert rc == 0, msg
    assert (st == 0).all() and rel_err(p, want) <= REL_TOL


def test_twin_tiles_repeat_bit_for_bit(ctx):
    """Twin tiles under full load on the sinh grid (32768 options, 65536 PDEs, 1024
    nodes, 48 levels): eight calls give the same bits."""
    import portfolio

    o = portfolio.american_portfolio(32768, seed=43)
    kw = dict(t_dim=48, x_dim=1024, scale=5.0, density=0.25, solver=1)
    first, st = bs_price(ctx, o, **kw)
    assert (st == 0).all()
    for _ in range(8):
        again, st2 = bs_price(ctx, o, **kw)
        assert (st2 == 0).all() and np.array_equal(again, first)
