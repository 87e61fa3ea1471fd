"""Launch-shape knobs and the autotuner: options per block of the streaming FP64
solver (1, 2, 4 warps of 32 options) and its resident blocks per SM, threads per
option of the FP32 solver (1, 2, 4 or 8 warps), Thomas vs PCR.  Every shape must price identically (FP64 streaming: bit for
bit, lanes do not depend on their neighbours) or within the FP32 bar."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def price(ctx, o, **kw):
    import kwg

    rc, p, st = ctx.fd1d_price(o, kwg.params(**kw))
    assert rc == kwg.KWG_OK, ctx.last_error()
    assert (st == 0).all()
    return p


@pytest.mark.parametrize("bw,sm", [(2, 0), (4, 0), (4, 1), (1, 3)])
def test_block_warps_are_bit_identical(ctx, bw, sm):
    """Block size and residency only change which warp takes which tile from the
    persistent queue; every lane's arithmetic is the same."""
    import portfolio

    o = portfolio.american_portfolio(3000, seed=17)  # 94 tiles: blocks with fewer warps than tiles at the tail
    kw = dict(t_dim=96, x_dim=320, scale=5.0, density=0.25, solver=1)
    assert np.array_equal(price(ctx, o, block_warps=bw, sm_blocks=sm, **kw), price(ctx, o, block_warps=1, **kw))


@pytest.mark.parametrize("warps", [2, 4, 8])
@pytest.mark.parametrize("x_dim", [128, 256, 512, 1000, 1024, 2048])
def test_fp32_multi_warp_options(ctx, x_dim, warps):
    """Two, four or eight warps per option (64, 128 or 256 lanes, 6 to 8 reduction
    levels through shared memory; fewer warps where a lane would get under 2 nodes)
    against the FP64 oracle, on uniform grids (shared factor tables) and the padded
    1000-node grid."""
    import kwg
    import kwor
    import portfolio

    o = portfolio.american_portfolio(96, seed=x_dim)
    dens = 0.25 if x_dim == 1000 else math.inf
    kw = dict(t_dim=128, x_dim=x_dim, scale=5.0, density=dens)
    p2 = price(ctx, o, precision=kwg.FP32, option_warps=warps, **kw)
    rc, msg, want, _ = kwor.fd1d_price(o, **kw)
    assert rc == 0, msg
    assert np.max(np.abs(p2 - want)) <= 1e-5


def test_autotune_records_and_applies_the_choice(ctx):
    import kwg
    import portfolio

    prm = kwg.params(t_dim=64, x_dim=256, scale=5.0, density=math.inf)
    t = ctx.autotune_ex(prm, 4096)
    d = t.as_dict()
    timed = [v for v in d["thomas_ms_by_block_warps"].values() if v >= 0] + [d["thomas_ms_one_4warp_block_per_sm"]]
    timed += [d["pcr_ms"]] if d["pcr_ms"] >= 0 else []
    assert len(timed) >= 4 and all(v > 0 for v in timed)
    best = min(timed)
    if d["solver"] == "pcr":
        chosen = d["pcr_ms"]
    elif d["sm_blocks"] == 1:
        chosen = d["thomas_ms_one_4warp_block_per_sm"]
    else:
        chosen = d["thomas_ms_by_block_warps"][d["block_warps"]]
    assert chosen == best
    o = portfolio.american_portfolio(4096, seed=2)
    auto = price(ctx, o, t_dim=64, x_dim=256, scale=5.0, density=math.inf)
    explicit = price(ctx, o, t_dim=64, x_dim=256, scale=5.0, density=math.inf, solver=t.solver,
                     block_warps=t.block_warps, sm_blocks=t.sm_blocks)
    assert np.array_equal(auto, explicit)
    # FP32: threads per option
    t32 = ctx.autotune_ex(kwg.params(t_dim=64, x_dim=512, scale=5.0, density=math.inf, precision=kwg.FP32), 2048)
    assert t32.option_warps in (1, 2, 4, 8) and min(t32.fp32_ms) > 0 and t32.fp32_8w_ms > 0


def test_autotune_uneven(ctx):
    import kwg
    import portfolio

    o, xd, td = portfolio.uneven_portfolio(3000, seed=9)
    xd = np.minimum(xd, 1024)
    td = np.minimum(td, 200)
    prm = kwg.params(scale=5.0, density=math.inf)
    t = ctx.autotune_uneven(o, xd, td, prm)
    assert t.solver in (kwg.SOLVER_THOMAS, kwg.SOLVER_PCR) and t.block_warps in (1, 2, 4)
    rc, auto, st = ctx.fd1d_price_uneven(o, xd, td, prm)
    assert rc == 0
    rc, explicit, st2 = ctx.fd1d_price_uneven(o, xd, td, kwg.params(scale=5.0, density=math.inf, solver=t.solver,
                                                                    block_warps=t.block_warps,
                                                                    sm_blocks=t.sm_blocks))
    assert rc == 0 and np.array_equal(st, st2)
    ok = st == 0
    assert np.array_equal(auto[ok], explicit[ok])
