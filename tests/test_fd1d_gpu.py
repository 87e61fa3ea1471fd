"""GPU parity of the FP64 FD1D path against the oracle and the reference's golden
vectors, through the C ABI, for both FP64 solvers (thread-per-option Thomas and
warp-per-option PCR).  Tolerance: the FP64 path must match the reference to
REL_TOL = 1e-10 relative on every option."""
import math

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10
# prices below this are compared absolutely (a reference price can be exactly 0)
PRICE_FLOOR = 1e-12


def rel_err(got, want):
    return float(np.max(np.abs(got - want) / np.maximum(np.abs(want), PRICE_FLOOR)))


def gpu_price(ctx, opts, **kw):
    import kwg

    rc, p, st = ctx.fd1d_price(opts, kwg.params(**kw))
    assert rc == kwg.KWG_OK, ctx.last_error()
    return p, st


SOLVERS = pytest.mark.parametrize("solver", [1, 2], ids=["thomas", "pcr"])


@SOLVERS
def test_pricer_test_table(ctx, solver):
    """test/kwPricer_test.cpp:63-84 at the reference defaults (512x512, scale 50, d 0.25)."""
    g = golden("pricer_test.npz")
    p, st = gpu_price(ctx, g["opts"], solver=solver)
    assert (st == 0).all()
    assert rel_err(p, g["ref_fd1d"]) <= REL_TOL
    assert np.max(np.abs(p - g["want"])) <= 1.3e-3


@SOLVERS
@pytest.mark.parametrize("name", ["qdfp", "fd1d"])
def test_portfolio_fixtures(ctx, name, solver):
    """test/kwPortfolio_test.cpp:41-56: 6000 puts, 600 distinct PDEs (dedup path)."""
    g = golden(f"portfolio_{name}.npz")
    p, st = gpu_price(ctx, g["opts"], t_dim=512, x_dim=512, solver=solver)
    assert (st == 0).all()
    assert rel_err(p, g["ref_fd1d"]) <= REL_TOL
    if name == "qdfp":
        assert np.max(np.abs(p - g["quantlib"])) <= 0.005


@SOLVERS
def test_128_options_512_grid(ctx, solver):
    g = golden("synthetic.npz")
    p, st = gpu_price(ctx, g["small_opts"], t_dim=512, x_dim=512, scale=5.0, density=0.25, solver=solver)
    assert (st == 0).all() and rel_err(p, g["small_ref"]) <= REL_TOL


@SOLVERS
def test_1024_grid_sample_sinh_and_uniform(ctx, solver):
    """1024x1024: the reference at density 1e6, the GPU both at 1e6 and exactly uniform."""
    g = golden("synthetic.npz")
    p, _ = gpu_price(ctx, g["batch1024_opts"], t_dim=1024, x_dim=1024, scale=5.0, density=1e6, solver=solver)
    assert rel_err(p, g["batch1024_ref"]) <= REL_TOL
    u, _ = gpu_price(ctx, g["batch1024_opts"], t_dim=1024, x_dim=1024, scale=5.0, density=math.inf, solver=solver)
    assert rel_err(u, g["batch1024_ref"]) <= REL_TOL


def test_2048_grid_sample(ctx):
    g = golden("synthetic.npz")
    p, _ = gpu_price(ctx, g["fine2048_opts"], t_dim=2048, x_dim=2048, scale=5.0, density=0.25)
    assert rel_err(p, g["fine2048_ref"]) <= REL_TOL


@SOLVERS
@pytest.mark.parametrize("name,kw", [("default", {}), ("x3_t2", dict(x_dim=3, t_dim=2)),
                                     ("x7_t5", dict(x_dim=7, t_dim=5)),
                                     ("x64_t33", dict(x_dim=64, t_dim=33, scale=5.0))])
def test_edge_grids_european_calls_duplicates(ctx, name, kw, solver):
    g = golden("edge.npz")
    p, st = gpu_price(ctx, g["opts"], solver=solver, **kw)
    assert (st == 0).all() and rel_err(p, g[f"ref_{name}"]) <= REL_TOL


def test_out_of_grid_status_and_strict(ctx):
    import kwg

    g = golden("edge.npz")
    p, st = gpu_price(ctx, g["bad_opts"])
    assert st[3] == kwg.STATUS_OUT_OF_GRID and np.isnan(p[3])
    ok = np.arange(8) != 3
    assert (st[ok] == 0).all() and rel_err(p[ok], g["ref_default"][ok]) <= REL_TOL
    rc, _, _ = ctx.fd1d_price(g["bad_opts"], kwg.params(strict=1))
    assert rc == kwg.KWG_ERR_OUT_OF_GRID and "not in grid range" in ctx.last_error()


def test_device_call_refuses_strict_mode(ctx):
    """The asynchronous device call cannot fail the call on a bad option without
    waiting for the results, so it refuses strict = 1 before any launch; its caller
    reads the per-option status instead."""
    import torch

    import kwg

    g = golden("edge.npz")
    o = g["bad_opts"]
    d_o = torch.from_numpy(o.view(np.uint8).copy()).cuda()
    d_p = torch.full((len(o),), float("nan"), dtype=torch.float64, device="cuda")
    d_s = torch.full((len(o),), -1, dtype=torch.int32, device="cuda")
    rc = ctx.fd1d_price_device(d_o.data_ptr(), len(o), kwg.params(strict=1), d_p.data_ptr(), d_s.data_ptr())
    assert rc == kwg.KWG_ERR_INVALID and "strict" in ctx.last_error()
    torch.cuda.synchronize()
    assert torch.isnan(d_p).all()
    rc = ctx.fd1d_price_device(d_o.data_ptr(), len(o), kwg.params(), d_p.data_ptr(), d_s.data_ptr())
    assert rc == kwg.KWG_OK, ctx.last_error()
    torch.cuda.synchronize()
    st = d_s.cpu().numpy()
    assert st[3] == kwg.STATUS_OUT_OF_GRID and (st[np.arange(8) != 3] == 0).all()


@SOLVERS
@pytest.mark.parametrize("theta", [0.6, 0.75, 1.0])
def test_theta_other_than_half(ctx, theta, solver):
    """theta is hard-coded to 0.5 in the reference; other values follow the oracle."""
    import kwor

    o = golden("synthetic.npz")["small_opts"][:40]
    p, _ = gpu_price(ctx, o, t_dim=200, x_dim=160, scale=5.0, density=0.25, theta=theta, solver=solver)
    rc, msg, want, _ = kwor.fd1d_price(o, t_dim=200, x_dim=160, scale=5.0, density=0.25, theta=theta)
    assert rc == 0, msg
    assert rel_err(p, want) <= REL_TOL


@SOLVERS
@pytest.mark.parametrize("n", [1, 31, 33, 100])
def test_ragged_batches(ctx, n, solver):
    """PDE counts that are not a multiple of the 32-lane tile; x_dim not a power of 2."""
    import kwor
    import portfolio

    o = portfolio.american_portfolio(n, seed=99)
    p, st = gpu_price(ctx, o, t_dim=64, x_dim=96, scale=5.0, density=0.25, solver=solver)
    rc, msg, want, _ = kwor.fd1d_price(o, t_dim=64, x_dim=96, scale=5.0, density=0.25)
    assert (st == 0).all() and rel_err(p, want) <= REL_TOL


def test_empty_batch_and_invalid_params(ctx):
    import kwg

    rc, p, st = ctx.fd1d_price(np.zeros(0, kwg.OPTION_DTYPE), kwg.params())
    assert rc == kwg.KWG_OK and len(p) == 0
    o = golden("edge.npz")["opts"]
    for bad in (dict(x_dim=2), dict(t_dim=1), dict(theta=0.0), dict(theta=1.5), dict(scale=-1.0),
                dict(density=0.0), dict(solver=2, x_dim=2048)):
        rc, _, _ = ctx.fd1d_price(o, kwg.params(**bad))
        assert rc == kwg.KWG_ERR_INVALID, bad
        assert ctx.last_error().startswith("kwg:")


@SOLVERS
def test_bad_option_fields(ctx, solver):
    import kwg

    o = golden("edge.npz")["opts"].copy()
    o[1]["t"] = 0.0
    o[5]["z"] = -0.2
    o[7]["s"] = 0.0
    p, st = gpu_price(ctx, o, solver=solver)
    assert st[1] == kwg.STATUS_BAD_INPUT and st[5] == kwg.STATUS_BAD_INPUT and st[7] == kwg.STATUS_BAD_INPUT
    assert np.isnan(p[[1, 5, 7]]).all()
    assert (st[[0, 2, 3, 4, 6]] == 0).all()


@pytest.mark.parametrize("api", ["host", "uneven"])
def test_nan_key_never_merges(ctx, api):
    """Dedup compares keys by value: an option whose vol is NaN matches nothing, so it
    keeps its own PDE and reports bad input, while its otherwise identical twin (and
    a -0.0 / +0.0 rate pair, equal by value) price normally."""
    import kwg
    import portfolio

    o = portfolio.american_portfolio(8, seed=21)
    o[1] = o[0]
    o[1]["z"] = np.nan
    o[2] = o[0]
    o[3] = o[0]
    o[2]["r"] = 0.0
    o[3]["r"] = -0.0
    prm = kwg.params(t_dim=64, x_dim=128, scale=5.0)
    if api == "host":
        rc, p, st = ctx.fd1d_price(o, prm)
    else:
        xd = np.full(len(o), 128, np.int32)
        td = np.full(len(o), 64, np.int32)
        rc, p, st = ctx.fd1d_price_uneven(o, xd, td, prm)
    assert rc == kwg.KWG_OK
    assert st[1] == kwg.STATUS_BAD_INPUT and np.isnan(p[1])
    keep = np.arange(len(o)) != 1
    assert (st[keep] == 0).all() and np.isfinite(p[keep]).all()
    assert p[2] == p[3]


def test_contexts_on_threads_price_concurrently(built):
    """One context per thread (the reference's pricers are not re-entrant either):
    four threads price different portfolios at once, with both solvers, FP32 and an
    uneven batch among them; every result equals the same call made alone."""
    import threading

    import kwg
    import portfolio

    jobs = [
        ("price", portfolio.american_portfolio(3000, seed=31), kwg.params(t_dim=96, x_dim=256, scale=5.0, solver=1)),
        ("price", portfolio.american_portfolio(500, seed=32), kwg.params(t_dim=64, x_dim=512, scale=5.0, solver=2)),
        ("price", portfolio.american_portfolio(2000, seed=33),
         kwg.params(t_dim=80, x_dim=1024, scale=5.0, precision=kwg.FP32)),
        ("uneven",) + portfolio.uneven_portfolio(1500, seed=34) + (kwg.params(scale=5.0, density=math.inf),),
    ]

    def run(c, job):
        if job[0] == "price":
            rc, p, st = c.fd1d_price(job[1], job[2])
        else:
            _, o, xd, td, prm = job
            rc, p, st = c.fd1d_price_uneven(o, np.minimum(xd, 512), np.minimum(td, 160), prm)
        assert rc == kwg.KWG_OK, c.last_error()
        return p, st

    ctxs = [kwg.Context(0) for _ in jobs]
    try:
        alone = [run(c, j) for c, j in zip(ctxs, jobs)]
        out = [None] * len(jobs)
        errors = []

        def worker(i):
            try:
                for _ in range(3):
                    out[i] = run(ctxs[i], jobs[i])
            except BaseException as e:  # noqa: BLE001 - reported below
                errors.append(e)

        threads = [threading.Thread(target=worker, args=(i,)) for i in range(len(jobs))]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        assert not errors, errors
        for (pa, sa), (pb, sb) in zip(alone, out):
            assert np.array_equal(sa, sb)
            ok = sa == 0
            assert np.array_equal(pa[ok], pb[ok])
    finally:
        for c in ctxs:
            c.close()


def test_device_api_matches_host_api(ctx):
    import torch

    import kwg
    import portfolio

    o = portfolio.american_portfolio(300, seed=5)
    prm = kwg.params(t_dim=128, x_dim=256, scale=5.0, density=0.25)
    want, _ = gpu_price(ctx, o, t_dim=128, x_dim=256, scale=5.0, density=0.25)
    d_o = torch.from_numpy(o.view(np.uint8).copy()).cuda()
    d_p = torch.empty(len(o), dtype=torch.float64, device="cuda")
    d_s = torch.empty(len(o), dtype=torch.int32, device="cuda")
    rc = ctx.fd1d_price_device(d_o.data_ptr(), len(o), prm, d_p.data_ptr(), d_s.data_ptr(),
                               torch.cuda.current_stream().cuda_stream)
    assert rc == 0, ctx.last_error()
    torch.cuda.synchronize()
    assert np.array_equal(d_p.cpu().numpy(), want)
    assert (d_s.cpu().numpy() == 0).all()


@pytest.mark.parametrize("precision,solver", [(0, 1), (0, 2), (1, 0)], ids=["fp64-thomas", "fp64-pcr", "fp32"])
def test_device_dedup_matches_host_dedup(ctx, precision, solver):
    """Device-side dedup (hash table on the key of src/Pricer/kwFd1d.cpp:28-65) on the
    QuantLib portfolio (6000 puts, 600 distinct keys) plus the edge fixture's
    duplicates, European options and calls: identical prices and statuses to the
    host path, which dedups like the reference."""
    import torch

    import kwg

    o = np.concatenate([golden("portfolio_qdfp.npz")["opts"], golden("edge.npz")["opts"]])
    o = np.ascontiguousarray(o, dtype=kwg.OPTION_DTYPE)
    prm = kwg.params(t_dim=256, x_dim=256, scale=50.0, density=0.25, precision=precision, solver=solver)
    rc, want, want_st = ctx.fd1d_price(o, prm)
    assert rc == 0, ctx.last_error()
    prm.device_dedup = 1
    d_o = torch.from_numpy(o.view(np.uint8).copy()).cuda()
    d_p = torch.empty(len(o), dtype=torch.float64, device="cuda")
    d_s = torch.empty(len(o), dtype=torch.int32, device="cuda")
    rc = ctx.fd1d_price_device(d_o.data_ptr(), len(o), prm, d_p.data_ptr(), d_s.data_ptr(),
                               torch.cuda.current_stream().cuda_stream)
    assert rc == 0, ctx.last_error()
    torch.cuda.synchronize()
    got = d_p.cpu().numpy()
    assert np.array_equal(d_s.cpu().numpy(), want_st)
    ok = want_st == 0
    assert np.array_equal(got[ok], want[ok])
    assert np.isnan(got[~ok]).all()


@pytest.mark.parametrize("x_dim,short", [(256, 250), (1024, 1000)])
def test_pcr_shared_tables_are_exact(ctx, x_dim, short):
    """On a uniform grid whose PDEs fill every lane (x_dim = 32 M) the FP64 PCR solver
    keeps one copy of the interior factors and spikes per PDE.  The rows are built
    from the exact spacing, so the copy is bit-identical to every lane's own: prices
    equal bit for bit those of the per-lane tables, which an uneven batch forces when
    its bucket also holds one shorter grid."""
    import kwg
    import portfolio

    o = portfolio.american_portfolio(200, seed=12)
    rc, shared, st = ctx.fd1d_price(o, kwg.params(t_dim=64, x_dim=x_dim, scale=5.0, density=math.inf, solver=2))
    assert rc == 0, ctx.last_error()
    oo = np.concatenate([o, portfolio.american_portfolio(1, seed=99)])
    xd = np.array([x_dim] * len(o) + [short], np.int32)
    td = np.full(len(oo), 64, np.int32)
    rc, per_lane, st2 = ctx.fd1d_price_uneven(oo, xd, td, kwg.params(scale=5.0, density=math.inf, solver=2))
    assert rc == 0, ctx.last_error()
    assert np.array_equal(st, st2[: len(o)])
    ok = st == 0
    assert ok.sum() > 150
    assert np.array_equal(shared[ok], per_lane[: len(o)][ok])


def test_million_option_batch(ctx):
    """Maximum-size batch through both entry points: 2^20 options (a quarter of
    them repeated keys), 64 x 64 grid.  Every option prices, the host call and the
    device call with on-device dedup agree bit for bit, and a sample matches the
    oracle."""
    import sys

    import torch

    import kwg
    import portfolio
    from conftest import ROOT

    sys.path.insert(0, f"{ROOT}/oracle")
    import kwor

    n = 1 << 20
    o = portfolio.american_portfolio(3 * n // 4, seed=45)
    rng = np.random.default_rng(5)
    o = np.concatenate([o, o[rng.integers(0, len(o), n - len(o))]])
    o = np.ascontiguousarray(o[rng.permutation(n)], dtype=kwg.OPTION_DTYPE)
    kw = dict(t_dim=64, x_dim=64, scale=5.0, density=0.25)
    rc, p, st = ctx.fd1d_price(o, kwg.params(**kw))
    assert rc == 0, ctx.last_error()
    assert (st == 0).all() and np.isfinite(p).all()
    prm = kwg.params(**kw)
    prm.device_dedup = 1
    d_o = torch.from_numpy(o.view(np.uint8).copy()).cuda()
    d_p = torch.empty(n, dtype=torch.float64, device="cuda")
    d_s = torch.empty(n, dtype=torch.int32, device="cuda")
    rc = ctx.fd1d_price_device(d_o.data_ptr(), n, prm, d_p.data_ptr(), d_s.data_ptr(),
                               torch.cuda.current_stream().cuda_stream)
    assert rc == 0, ctx.last_error()
    torch.cuda.synchronize()
    assert np.array_equal(d_s.cpu().numpy(), st)
    assert np.array_equal(d_p.cpu().numpy(), p)
    idx = rng.choice(n, 48, replace=False)
    rc, msg, want, _ = kwor.fd1d_price(o[idx], **kw)
    assert rc == 0, msg
    assert rel_err(p[idx], want) <= REL_TOL
    del d_o, d_p, d_s


def test_pricer_mirror(built):
    """kw::PricerFactory / kw::Pricer usage exactly like test/kwPricer_test.cpp:63-84."""
    import kwg

    g = golden("pricer_test.npz")
    assets = [kwg.Option(*[float(x) for x in tuple(r)[:6]], int(r["e"]), int(r["w"])) for r in g["opts"]]
    config = kwg.Config()
    config.set("PRICER", "FD1D")
    err, pricer = kwg.PricerFactory.create(config)
    assert err == ""
    prices = []
    assert pricer.price(assets, prices) == ""
    for want, got in zip(g["want"], prices):
        assert abs(want - got) <= 1.3e-3
    bad = golden("edge.npz")["bad_opts"]
    err = pricer.price(bad, prices)
    assert err.startswith("Fd1dGpu_Pricer::price:") and "not in grid range" in err


def test_32768x1024_full_size_properties(ctx):
    """All 32768 options at 1024x1024: finite, American >= intrinsic up to the
    interpolation error of the payoff, deterministic, and a sample equal to the oracle.
    The projection floors every node but the last at the payoff; between nodes the
    price is a chord, which for a put ((1 - e^x)+, concave where positive) lies below
    the payoff by at most K dx^2/8, as it does in the reference."""
    import kwor
    import portfolio

    o = portfolio.american_portfolio(32768, seed=42)
    p, st = gpu_price(ctx, o, t_dim=1024, x_dim=1024, scale=5.0, density=math.inf)
    assert (st == 0).all() and np.isfinite(p).all()
    intrinsic = np.where(o["w"] < 0, np.maximum(o["k"] - o["s"], 0), np.maximum(o["s"] - o["k"], 0))
    dx = 2 * 5.0 * o["z"] * np.sqrt(o["t"]) / (1024 - 1)
    assert (p >= intrinsic - 1.01 * o["k"] * dx * dx / 8 - 1e-9).all()
    p2, _ = gpu_price(ctx, o, t_dim=1024, x_dim=1024, scale=5.0, density=math.inf)
    assert np.array_equal(p, p2)
    idx = np.arange(0, 32768, 1024)
    rc, msg, want, _ = kwor.fd1d_price(o[idx], t_dim=1024, x_dim=1024, scale=5.0, density=math.inf)
    assert rc == 0 and rel_err(p[idx], want) <= REL_TOL


def test_streaming_solver_repeats_bit_for_bit(ctx):
    """The streaming FP64 solver under full load gives the same bits on every run:
    32768 options at 1024 nodes x 64 levels (one tile per warp, every SM full), 24
    device-call runs with one-warp blocks and the host call, against a sample of the
    oracle.  Its ring slots are refilled by the bulk-copy engine while the warp runs;
    a refill that overtook the lanes' reads of the slot showed as whole tiles off by
    up to 1e-1 on about one run in four."""
    import torch

    import kwg
    import kwor
    import portfolio

    n = 32768
    o = portfolio.american_portfolio(n, seed=42)
    grid = dict(t_dim=64, x_dim=1024, scale=5.0, density=math.inf)
    prm = kwg.params(solver=kwg.SOLVER_THOMAS, block_warps=1, **grid)
    d_o = torch.from_numpy(o.view(np.uint8).copy()).cuda()
    d_p = torch.empty(n, dtype=torch.float64, device="cuda")
    d_s = torch.empty(n, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    runs = []
    for _ in range(24):
        assert ctx.fd1d_price_device(d_o.data_ptr(), n, prm, d_p.data_ptr(), d_s.data_ptr(), stream) == 0, \
            ctx.last_error()
        torch.cuda.synchronize()
        assert (d_s.cpu().numpy() == 0).all()
        runs.append(d_p.cpu().numpy().copy())
    host, st = gpu_price(ctx, o, solver=kwg.SOLVER_THOMAS, block_warps=1, **grid)
    assert (st == 0).all()
    for r in runs:
        assert np.array_equal(r, host), int((r != host).sum())
    idx = np.arange(7, n, 512)
    rc, msg, want, _ = kwor.fd1d_price(o[idx], **grid)
    assert rc == 0 and rel_err(host[idx], want) <= REL_TOL


@pytest.mark.parametrize("grid", [dict(x_dim=1024, t_dim=64, density=math.inf),
                                  dict(x_dim=512, t_dim=48, density=0.25),
                                  dict(x_dim=2048, t_dim=16, density=math.inf),
                                  dict(x_dim=13, t_dim=9, density=math.inf)],
                         ids=["uniform1024", "sinh512", "uniform2048", "uniform13"])
def test_stage_geometries_agree_bit_for_bit(ctx, grid):
    """The streaming solver's big stages (16-node coefficient stages, 32-node middle
    stages, taken when the launch caps the residency: 4-warp blocks one per SM, 2-warp
    blocks two per SM, 1-warp blocks four per SM) give the same bits as the small
    stages of a full-residency launch, for FD1D and for FD1D-BS twin tiles.  On the
    13-node grid every big-stage sweep is a single tail stage."""
    import kwg
    import portfolio

    o = portfolio.american_portfolio(2048, seed=77)
    o["e"][::5] = 0  # some European options: mixed classes, and twin tiles for FD1D-BS
    common = dict(scale=5.0, solver=kwg.SOLVER_THOMAS, **grid)
    want, st = gpu_price(ctx, o, block_warps=1, sm_blocks=0, **common)
    assert (st == 0).all()
    for bw, sb in ((4, 1), (2, 2), (1, 4)):
        got, st = gpu_price(ctx, o, block_warps=bw, sm_blocks=sb, **common)
        assert (st == 0).all() and np.array_equal(got, want), (bw, sb, int((got != want).sum()))
    rc, bs_small, st = ctx.fd1d_bs_price(o, kwg.params(block_warps=1, sm_blocks=0, **common))
    assert rc == 0 and (st == 0).all()
    rc, bs_big, st = ctx.fd1d_bs_price(o, kwg.params(block_warps=4, sm_blocks=1, **common))
    assert rc == 0 and (st == 0).all() and np.array_equal(bs_big, bs_small)


def test_solvers_agree_and_autotune(ctx):
    """Both FP64 solvers give the same prices to 1e-10; the autotuner times both and
    AUTO then matches them too."""
    import kwg
    import portfolio

    o = portfolio.american_portfolio(777, seed=17)
    kw = dict(t_dim=300, x_dim=256, scale=5.0, density=0.25)
    a, _ = gpu_price(ctx, o, solver=kwg.SOLVER_THOMAS, **kw)
    b, _ = gpu_price(ctx, o, solver=kwg.SOLVER_PCR, **kw)
    assert rel_err(b, a) <= REL_TOL
    t_ms, p_ms = ctx.autotune(kwg.params(**kw), len(o))
    assert t_ms > 0 and p_ms > 0
    c, _ = gpu_price(ctx, o, **kw)
    assert rel_err(c, a) <= REL_TOL
    t_ms, p_ms = ctx.autotune(kwg.params(t_dim=64, x_dim=2048, scale=5.0), 64)
    assert t_ms > 0 and p_ms < 0  # PCR-FP64 stops at x_dim 1024


def test_large_grid_beyond_the_on_chip_limits(ctx):
    """The streaming FP64 solver has no grid-size cap: 4096 nodes x 300 time levels
    (twice the largest on-chip grid) against the oracle, puts and calls, sinh grid."""
    import kwor
    import portfolio

    o = portfolio.american_portfolio(12, seed=4096)
    kw = dict(t_dim=300, x_dim=4096, scale=5.0, density=0.25)
    p, st = gpu_price(ctx, o, solver=1, **kw)
    rc, msg, want, _ = kwor.fd1d_price(o, **kw)
    assert rc == 0, msg
    assert (st == 0).all() and rel_err(p, want) <= REL_TOL


@pytest.mark.parametrize("entry", ["host", "bs", "device", "device_dedup", "uneven"])
def test_single_option(ctx, entry):
    """n = 1 through every entry point (one partly filled tile / warp)."""
    import torch

    import kwg
    import kwor
    import portfolio

    o = portfolio.american_portfolio(1, seed=1)
    prm = kwg.params(t_dim=64, x_dim=96, scale=5.0, density=0.25)
    rc, msg, want, _ = kwor.fd1d_price(o, bs=(entry == "bs"), t_dim=64, x_dim=96, scale=5.0, density=0.25)
    assert rc == 0, msg
    if entry == "host":
        rc, p, st = ctx.fd1d_price(o, prm)
    elif entry == "bs":
        rc, p, st = ctx.fd1d_bs_price(o, prm)
    elif entry == "uneven":
        rc, p, st = ctx.fd1d_price_uneven(o, [96], [64], prm)
    else:
        prm.device_dedup = 1 if entry == "device_dedup" else 0
        d_o = torch.from_numpy(o.view(np.uint8).copy()).cuda()
        d_p = torch.empty(1, dtype=torch.float64, device="cuda")
        d_s = torch.empty(1, dtype=torch.int32, device="cuda")
        rc = ctx.fd1d_price_device(d_o.data_ptr(), 1, prm, d_p.data_ptr(), d_s.data_ptr(),
                                   torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        p, st = d_p.cpu().numpy(), d_s.cpu().numpy()
    assert rc == 0 and st[0] == 0
    assert rel_err(p, want) <= REL_TOL


def extreme_sweep():
    """1296 options over the corners of the parameter space: spot 50/100/200 against
    strike 100, vol 2 %..150 %, maturity 0.01..5 years, r and q 0..20 %, American and
    European puts and calls.  A third of them fall outside the grid."""
    import itertools

    import kwg

    rows = [(t, 100.0, z, r, q, s, e, w)
            for s, z, t, r, q, e, w in itertools.product((50.0, 100.0, 200.0), (0.02, 0.1, 0.6, 1.5),
                                                         (0.01, 0.5, 5.0), (0.0, 0.05, 0.2), (0.0, 0.03, 0.2),
                                                         (0, 1), (-1, 1))]
    return np.array(rows, dtype=kwg.OPTION_DTYPE)


@pytest.mark.parametrize("grid", [dict(x_dim=256, t_dim=128, scale=5.0, density=math.inf),
                                  dict(x_dim=256, t_dim=128, scale=5.0, density=0.25),
                                  dict(x_dim=1024, t_dim=64, scale=5.0, density=math.inf),
                                  dict(x_dim=300, t_dim=50, scale=50.0, density=0.25)],
                         ids=["uniform256", "sinh256", "uniform1024x64", "sinh300_scale50"])
def test_extreme_parameters_match_the_oracle(ctx, grid):
    """FD1D and FD1D-BS on the extreme sweep, both FP64 solvers: the out-of-grid
    options flagged as the oracle flags them, every other price within REL_TOL of the
    oracle (prices below 1e-6 K within 1e-13 K absolute: they reach 1e-29).  The FP32
    path reports every price it cannot represent with a status, never as a NaN with
    status OK (at scale 50 a call's grid reaches e^168 K, beyond FP32's range).  The
    pivots freeze only at an exact fixed point: with the earlier 2^-50 tolerance the
    drift-dominated options (vol 2 %, |r - q| = 0.2, T = 5) missed REL_TOL at 1024 x 64."""
    import kwg
    import kwor

    o = extreme_sweep()
    rc, msg, want, wst = kwor.fd1d_price(o, **grid)
    ok = wst == 0
    assert 0.5 * len(o) < ok.sum() < len(o)
    v = o[ok]
    rc, msg, want_bs, _ = kwor.fd1d_price(v, bs=True, **grid)  # the reference fails a batch with an out-of-grid option
    assert rc == 0, msg

    def check(got, ref):
        k = v["k"]
        big = np.abs(ref) >= 1e-6 * k
        assert rel_err(got[big], ref[big]) <= REL_TOL
        assert np.max(np.abs(got[~big] - ref[~big]) / k[~big], initial=0.0) <= 1e-13

    for solver in (kwg.SOLVER_THOMAS, kwg.SOLVER_PCR):
        prm = kwg.params(solver=solver, **grid)
        p, st = gpu_price(ctx, o, solver=solver, **grid)
        assert np.array_equal(st == kwg.STATUS_OUT_OF_GRID, wst == 1) and (st[ok] == 0).all()
        check(p[ok], want[ok])
        rc, p_bs, st_bs = ctx.fd1d_bs_price(v, prm)
        assert rc == 0 and (st_bs == 0).all()
        check(p_bs, want_bs)
    p32, st32 = gpu_price(ctx, o, precision=kwg.FP32, **grid)
    assert np.isfinite(p32[st32 == 0]).all()
    assert np.isnan(p32[st32 != 0]).all()
    assert np.array_equal(st32 == kwg.STATUS_OUT_OF_GRID, wst == 1)
