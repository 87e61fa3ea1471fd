"""Uneven batches (per-option shapes): every option on its own grid, one device pass.
The oracle -- like the reference, one grid shape per call -- is run per (x_dim,
t_dim) group.  FP64 within REL_TOL = 1e-10 relative, FP32 within ABS_TOL = 1e-5."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10
ABS_TOL = 1e-5
SCALE = 5.0


def oracle_uneven(opts, xd, td, density=math.inf):
    import kwor

    out = np.full(len(opts), np.nan)
    st = np.zeros(len(opts), np.int32)
    keys = np.stack([xd, td], 1)
    for x, t in {tuple(k) for k in keys.tolist()}:
        idx = np.flatnonzero((xd == x) & (td == t))
        rc, msg, p, s = kwor.fd1d_price(opts[idx], t_dim=int(t), x_dim=int(x), scale=SCALE, density=density)
        out[idx] = p
        st[idx] = s
    return out, st


def sample(n, seed=42):
    import portfolio

    o, xd, td = portfolio.uneven_portfolio(131072, seed=seed)
    # a spread of shapes: evenly spaced options of the full 131072-option uneven stream
    idx = np.linspace(0, 131071, n).astype(int)
    return o[idx], xd[idx], td[idx]


def test_uneven_big_stages_match_small_stages(ctx):
    """One 4-warp block per SM (the tuned shape of uneven batches) runs the streaming
    solver's big stages; a full-residency launch runs the small ones.  Tiles of every
    node count from 128 to 2048, each lane with its own step count: the same bits."""
    import kwg

    o, xd, td = sample(4096, seed=3)
    td = np.minimum(td, 160)
    rc, small, st = ctx.fd1d_price_uneven(o, xd, td, kwg.params(scale=SCALE, density=math.inf, solver=1,
                                                                  block_warps=1, sm_blocks=0))
    assert rc == 0, ctx.last_error()
    rc, big, st2 = ctx.fd1d_price_uneven(o, xd, td, kwg.params(scale=SCALE, density=math.inf, solver=1,
                                                                 block_warps=4, sm_blocks=1))
    assert rc == 0, ctx.last_error()
    assert np.array_equal(st, st2) and (st == 0).sum() > 0.8 * len(o)
    ok = st == 0
    assert np.array_equal(big[ok], small[ok])


@pytest.mark.parametrize("solver", [1, 2], ids=["thomas", "pcr"])
def test_uneven_fp64_matches_oracle_per_shape(ctx, solver):
    import kwg

    o, xd, td = sample(160)
    if solver == 2:  # the FP64 PCR kernel stops at 1024 nodes
        keep = xd <= 1024
        o, xd, td = o[keep], xd[keep], td[keep]
    rc, p, st = ctx.fd1d_price_uneven(o, xd, td, kwg.params(scale=SCALE, density=math.inf, solver=solver))
    assert rc == 0, ctx.last_error()
    want, wst = oracle_uneven(o, xd, td)
    assert np.array_equal(st == kwg.STATUS_OUT_OF_GRID, wst == 1)  # out-of-grid flagged, not fatal
    ok = st == 0
    assert ok.sum() > 0.8 * len(o)
    rel = np.abs(p[ok] - want[ok]) / np.maximum(np.abs(want[ok]), 1e-12)
    assert rel.max() <= REL_TOL


def test_uneven_fp32_matches_oracle(ctx):
    import kwg

    o, xd, td = sample(120, seed=7)
    rc, p, st = ctx.fd1d_price_uneven(o, xd, td, kwg.params(scale=SCALE, density=math.inf, precision=kwg.FP32))
    assert rc == 0, ctx.last_error()
    want, wst = oracle_uneven(o, xd, td)
    ok = (st == 0) & (wst == 0)
    assert np.array_equal(st != 0, wst != 0)
    assert np.max(np.abs(p[ok] - want[ok])) <= ABS_TOL


def test_uneven_uniform_shapes_match_uniform_call(ctx):
    """All options on one shape: the uneven path equals the uniform one bit for bit."""
    import kwg
    import portfolio

    o = portfolio.american_portfolio(100, seed=3)
    prm = kwg.params(t_dim=130, x_dim=256, scale=SCALE, density=math.inf, solver=1)
    rc, a, _ = ctx.fd1d_price(o, prm)
    assert rc == 0
    rc, b, _ = ctx.fd1d_price_uneven(o, np.full(100, 256), np.full(100, 130), prm)
    assert rc == 0 and np.array_equal(a, b)


def test_uneven_graph_replay_and_duplicates(ctx):
    """A second call with the same layout replays the captured graph with new inputs;
    options repeated with different grids are different PDEs."""
    import kwg

    o, xd, td = sample(64, seed=11)
    prm = kwg.params(scale=SCALE, density=math.inf)
    rc, p1, s1 = ctx.fd1d_price_uneven(o, xd, td, prm)
    o2 = o.copy()
    o2["s"] *= 1.01  # same PDEs (dedup key has no spot), new interpolation points
    rc, p2, s2 = ctx.fd1d_price_uneven(o2, xd, td, prm)
    assert rc == 0
    want, wst = oracle_uneven(o2, xd, td)
    ok = (s2 == 0) & (wst == 0)
    assert np.max(np.abs(p2[ok] - want[ok]) / np.abs(want[ok])) <= REL_TOL
    # same option twice, two grids
    oo = np.concatenate([o[:4], o[:4]])
    xx = np.concatenate([np.full(4, 128), np.full(4, 256)]).astype(np.int32)
    tt = np.full(8, 100, np.int32)
    rc, p3, s3 = ctx.fd1d_price_uneven(oo, xx, tt, prm)
    want3, _ = oracle_uneven(oo, xx, tt)
    ok = s3 == 0
    assert np.max(np.abs(p3[ok] - want3[ok]) / np.abs(want3[ok])) <= REL_TOL
    assert not np.array_equal(p3[:4], p3[4:])


def test_uneven_replays_repeat_bit_for_bit(ctx):
    """The streaming solver's big stages under load (one 4-warp block per SM, 16384
    options of every node count, t_dim up to 128): eight graph replays give the same
    bits.  Ring refills that overtook the lanes' reads of a slot showed as whole tiles
    off on some runs."""
    import kwg

    o, xd, td = sample(16384, seed=21)
    td = np.minimum(td, 128)
    prm = kwg.params(scale=SCALE, density=math.inf, solver=1, block_warps=4, sm_blocks=1)
    rc, first, st = ctx.fd1d_price_uneven(o, xd, td, prm)
    assert rc == 0 and (st == 0).sum() > 0.8 * len(o)
    for _ in range(8):
        rc, again, st2 = ctx.fd1d_price_uneven(o, xd, td, prm)
        assert rc == 0 and np.array_equal(st2, st)
        assert np.array_equal(again[st == 0], first[st == 0])


def test_uneven_rejects_bad_shapes(ctx):
    import kwg

    o, xd, td = sample(8)
    xd = xd.copy()
    xd[3] = 2
    rc, _, _ = ctx.fd1d_price_uneven(o, xd, td, kwg.params())
    assert rc == kwg.KWG_ERR_INVALID and "option 3" in ctx.last_error()


def test_uneven_131072_full_size(ctx):
    """All 131072 options: statuses match the grid bounds, a sample matches the oracle."""
    import kwg
    import portfolio

    o, xd, td = portfolio.uneven_portfolio(131072)
    rc, p, st = ctx.fd1d_price_uneven(o, xd, td, kwg.params(scale=SCALE, density=math.inf))
    assert rc == 0, ctx.last_error()
    out = np.abs(np.log(o["s"] / o["k"])) >= 5 * o["z"] * np.sqrt(o["t"]) * (1 - 1e-9)
    inside = np.abs(np.log(o["s"] / o["k"])) < 5 * o["z"] * np.sqrt(o["t"]) * (1 - 1e-6)
    assert (st[inside] == 0).all() and np.isfinite(p[inside]).all()
    assert (st[~inside & out] == kwg.STATUS_OUT_OF_GRID).all()
    idx = np.arange(0, 131072, 4099)
    want, wst = oracle_uneven(o[idx], xd[idx], td[idx])
    ok = (wst == 0) & (st[idx] == 0)
    assert np.max(np.abs(p[idx][ok] - want[ok]) / np.abs(want[ok])) <= REL_TOL
