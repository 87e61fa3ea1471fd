"""GPU FP32 stepping path (float-float state, FP32 increments, on-chip partitioned
solve) against the FP64 oracle.  Tolerance: ABS_TOL = 1e-5 absolute on every price."""
import math

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

ABS_TOL = 1e-5


def price32(ctx, opts, **kw):
    import kwg

    rc, p, st = ctx.fd1d_price(opts, kwg.params(precision=kwg.FP32, **kw))
    assert rc == kwg.KWG_OK, ctx.last_error()
    return p, st


def oracle(opts, **kw):
    import kwor

    rc, msg, p, st = kwor.fd1d_price(opts, **kw)
    assert rc == 0, msg
    return p


def test_128_options_512_grid(ctx):
    g = golden("synthetic.npz")
    p, st = price32(ctx, g["small_opts"], t_dim=512, x_dim=512, scale=5.0, density=0.25)
    assert (st == 0).all()
    assert np.max(np.abs(p - g["small_ref"])) <= ABS_TOL


def test_1024_grid_sample_uniform(ctx):
    g = golden("synthetic.npz")
    p, st = price32(ctx, g["batch1024_opts"], t_dim=1024, x_dim=1024, scale=5.0, density=math.inf)
    assert (st == 0).all()
    assert np.max(np.abs(p - g["batch1024_ref"])) <= ABS_TOL


def test_2048_grid_sample(ctx):
    g = golden("synthetic.npz")
    p, st = price32(ctx, g["fine2048_opts"], t_dim=2048, x_dim=2048, scale=5.0, density=0.25)
    assert (st == 0).all()
    assert np.max(np.abs(p - g["fine2048_ref"])) <= ABS_TOL


def test_portfolio_qdfp(ctx):
    """Reference defaults (scale 50, density 0.25, 512x512) on the 6000-put fixture."""
    g = golden("portfolio_qdfp.npz")
    p, st = price32(ctx, g["opts"], t_dim=512, x_dim=512)
    assert (st == 0).all()
    assert np.max(np.abs(p - g["ref_fd1d"])) <= ABS_TOL
    assert np.max(np.abs(p - g["quantlib"])) <= 0.005


@pytest.mark.parametrize("warps", [0, 8])
@pytest.mark.parametrize("name,kw", [("default", {}), ("x3_t2", dict(x_dim=3, t_dim=2)),
                                     ("x7_t5", dict(x_dim=7, t_dim=5)),
                                     ("x64_t33", dict(x_dim=64, t_dim=33, scale=5.0))])
def test_edge_grids(ctx, name, kw, warps):
    """Tiny and non-power-of-two grids (padded with decoupled rows), Europeans,
    calls, duplicates; with the default launch and with eight warps per PDE asked
    for (reduced to what the grid allows: at least 2 nodes per lane)."""
    g = golden("edge.npz")
    p, st = price32(ctx, g["opts"], option_warps=warps, **kw)
    assert (st == 0).all()
    want = g[f"ref_{name}"]
    # a 3-node grid over +-50 sigma sqrt(T) prices some options in the tens of
    # thousands; there FP32 increments resolve the price to ~1e-7 relative
    assert (np.abs(p - want) <= np.maximum(ABS_TOL, 2e-7 * np.abs(want))).all()


@pytest.mark.parametrize("warps", [0, 8])
@pytest.mark.parametrize("x_dim,t_dim", [(100, 50), (300, 120), (1000, 700), (1500, 1200), (1000, 64), (1500, 40)])
def test_non_power_of_two_grids(ctx, x_dim, t_dim, warps):
    """Grids padded to 32*2^k nodes with decoupled identity rows.  The last two have
    few, long time steps: lambda = theta dt sigma^2 / (2 dx^2) reaches ~1e3 near the
    strike on the sinh grid, where the separator system nearly cancels -- its
    coefficients are built in FP64 for exactly this case."""
    import portfolio

    o = portfolio.american_portfolio(40, seed=21)
    p, st = price32(ctx, o, t_dim=t_dim, x_dim=x_dim, scale=5.0, density=0.25, option_warps=warps)
    want = oracle(o, t_dim=t_dim, x_dim=x_dim, scale=5.0, density=0.25)
    assert (st == 0).all() and np.max(np.abs(p - want)) <= ABS_TOL


def test_theta_and_status(ctx):
    import kwg

    o = golden("synthetic.npz")["small_opts"][:24]
    p, _ = price32(ctx, o, t_dim=200, x_dim=256, scale=5.0, density=0.25, theta=1.0)
    want = oracle(o, t_dim=200, x_dim=256, scale=5.0, density=0.25, theta=1.0)
    assert np.max(np.abs(p - want)) <= ABS_TOL
    bad = golden("edge.npz")["bad_opts"]
    p, st = price32(ctx, bad)
    assert st[3] == kwg.STATUS_OUT_OF_GRID and np.isnan(p[3]) and (st[np.arange(8) != 3] == 0).all()
    rc, _, _ = ctx.fd1d_price(bad, kwg.params(precision=kwg.FP32, x_dim=4096))
    assert rc == kwg.KWG_ERR_INVALID and "2048" in ctx.last_error()


def test_32768x1024_full_size_vs_fp64(ctx):
    """All 32768 options at 1024x1024: FP32 within 1e-5 of the GPU FP64 path."""
    import kwg
    import portfolio

    o = portfolio.american_portfolio(32768, seed=42)
    rc, p64, _ = ctx.fd1d_price(o, kwg.params(t_dim=1024, x_dim=1024, scale=5.0, density=math.inf))
    assert rc == 0
    p32, st = price32(ctx, o, t_dim=1024, x_dim=1024, scale=5.0, density=math.inf)
    assert (st == 0).all()
    err = np.abs(p32 - p64)
    assert err.max() <= ABS_TOL, (err.max(), int(err.argmax()))


@pytest.mark.parametrize("theta", [0.5, 0.75])
@pytest.mark.parametrize("x_dim", [128, 256, 512, 1024])
def test_uniform_full_lane_grids(ctx, x_dim, theta):
    """Uniform grids of 32 x 2^k nodes run the packed-pair step (nodes P-k and P+k of
    a lane in one float2, P = nodes per lane / 2): 4, 8, 16 and 32 nodes per lane, a
    mix of American and European puts and calls, against the oracle."""
    import portfolio

    o = portfolio.american_portfolio(96, seed=31)
    o["e"][1::3] = 0
    o["w"][::2] = -o["w"][::2]
    p, st = price32(ctx, o, t_dim=300, x_dim=x_dim, scale=5.0, density=math.inf, theta=theta)
    want = oracle(o, t_dim=300, x_dim=x_dim, scale=5.0, density=math.inf, theta=theta)
    assert (st == 0).all() and np.max(np.abs(p - want)) <= ABS_TOL
