"""Multi-rank (one process per GPU) host logic on CPU: two gloo ranks shard the option
stream with no data-path collective, and only the timing is reduced across ranks.
The prices are the oracle's, so these run without a GPU."""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

from conftest import ROOT

N_PER_RANK = 24
GRID = dict(t_dim=48, x_dim=64, scale=5.0, density=0.25)
# the QdFp portfolio's reference grid width (scale 50) keeps every spot inside the grid
GRID_Q = dict(t_dim=48, x_dim=64, scale=50.0, density=0.25)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    import sys

    for sub in ("kwinto-cuda_gb300", "oracle"):
        sys.path.insert(0, os.path.join(ROOT, sub))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import kwor
    import shard

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        opts = shard.portfolio_shard(N_PER_RANK, rank)
        rc, msg, prices, status = kwor.fd1d_price(opts, nthreads=1, **GRID)
        slowest = shard.max_over_ranks(1.5 + rank)
        gathered = [None] * world
        dist.all_gather_object(gathered, (opts.tobytes(), prices.tobytes(), int(rc)))
        if rank == 0:
            out.put((slowest, gathered))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_the_stream():
    import kwor
    import portfolio

    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    slowest, gathered = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # the timing reduction is the max over ranks
    assert slowest == 1.5 + (world - 1)
    # the shards are the consecutive windows of the single-process stream ...
    whole = portfolio.american_portfolio(world * N_PER_RANK, seed=42)
    import kwg

    got = np.concatenate([np.frombuffer(g[0], dtype=kwg.OPTION_DTYPE) for g in gathered])
    assert all(np.array_equal(got[f], whole[f]) for f in kwg.OPTION_DTYPE.names)
    # ... and each rank's prices equal the single-process prices of its window
    rc, msg, want, _ = kwor.fd1d_price(whole, nthreads=1, **GRID)
    assert rc == 0 and all(g[2] == 0 for g in gathered)
    prices = np.concatenate([np.frombuffer(g[1], dtype=np.float64) for g in gathered])
    assert np.array_equal(prices, want)


def test_max_over_ranks_without_a_process_group():
    import shard

    assert shard.max_over_ranks(3.25) == 3.25


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_partition_by_work_is_contiguous_and_balanced(world):
    import portfolio
    import shard

    _, xd, td = portfolio.uneven_portfolio(4096, seed=5)
    chunks = shard.partition_by_work(xd, td, world)
    assert len(chunks) == world and chunks[0][0] == 0 and chunks[-1][1] == len(xd)
    assert all(chunks[r][1] == chunks[r + 1][0] for r in range(world - 1))
    work = xd.astype(np.int64) * (td.astype(np.int64) - 1)
    per = [int(work[b:e].sum()) for b, e in chunks]
    # every chunk is within one PDE's work of the even share
    assert max(per) - work.sum() / world <= work.max()


def test_partition_by_work_edge_cases():
    import shard

    assert shard.partition_by_work([], [], 2) == [(0, 0), (0, 0)]
    one = shard.partition_by_work([64], [10], 3)
    assert sum(e - b for b, e in one) == 1 and one[0][0] == 0 and one[-1][1] == 1
    with pytest.raises(ValueError):
        shard.partition_by_work([1, 2], [3], 2)


def _strong_rank_main(rank: int, world: int, port: int, out):
    import sys

    for sub in ("kwinto-cuda_gb300", "oracle"):
        sys.path.insert(0, os.path.join(ROOT, sub))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import kwor
    import shard
    from conftest import golden

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        opts = golden("portfolio_qdfp.npz")["opts"]  # 6000 options, 600 PDEs
        idx = shard.strong_shard(opts, rank, world, x_dim=GRID_Q["x_dim"], t_dim=GRID_Q["t_dim"])
        rc, msg, prices, status = kwor.fd1d_price(opts[idx], nthreads=1, **GRID_Q)
        whole, st = shard.gather_prices(len(opts), idx, prices, status)
        sizes = [None] * world
        dist.all_gather_object(sizes, len(idx))
        if rank == 0:
            out.put((whole.tobytes(), st.tobytes(), sizes, int(rc)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_split_one_portfolio():
    """Strong scaling: one portfolio, deduplicated by every rank alike, its PDEs cut in
    two by work; each rank prices its options and the prices are gathered.  The
    result equals the single-process prices bit for bit."""
    import kwor
    import shard
    from conftest import golden

    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_strong_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    whole, st, sizes, rc = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    opts = golden("portfolio_qdfp.npz")["opts"]
    rc1, msg, want, _ = kwor.fd1d_price(opts, nthreads=1, **GRID_Q)
    assert rc == 0 and rc1 == 0
    assert sum(sizes) == len(opts) and min(sizes) > 0
    assert np.array_equal(np.frombuffer(whole, np.float64), want)
    assert (np.frombuffer(st, np.int32) == 0).all()


def test_strong_shards_cover_every_option_once_and_split_no_pde(built):
    import kwg
    import portfolio
    import shard

    o, xd, td = portfolio.uneven_portfolio(2048, seed=9)
    o = np.concatenate([o, o[:300]]).astype(kwg.OPTION_DTYPE)  # duplicates share PDEs
    xd, td = np.concatenate([xd, xd[:300]]), np.concatenate([td, td[:300]])
    a2p, _ = kwg.dedup(o, xd, td)
    for world in (1, 2, 3, 4):
        parts = [shard.strong_shard(o, r, world, x_dims=xd, t_dims=td) for r in range(world)]
        allidx = np.sort(np.concatenate(parts))
        assert np.array_equal(allidx, np.arange(len(o)))
        pdes = [set(a2p[p].tolist()) for p in parts]
        assert all(not (pdes[i] & pdes[j]) for i in range(world) for j in range(i + 1, world))


def test_bench_gpus_flag_launches_the_ranks():
    """bench.py --gpus 2 without a launcher starts two ranks itself (torch.distributed.run
    on 127.0.0.1); the reference arm's line then reports n_gpus 2.  CPU only: the
    reference arm runs on the host cores on rank 0."""
    import json
    import subprocess
    import sys

    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                          "--steps", "1", "--warmup", "0", "--ref-options", "4", "--t-dim", "16"],
                         capture_output=True, text=True, timeout=300, env={k: v for k, v in os.environ.items()
                                                                          if k not in ("WORLD_SIZE", "RANK")})
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [json.loads(l) for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    assert lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2
