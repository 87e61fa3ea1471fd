"""Multi-GPU sharding of FD1D batches: one process per GPU, no collective on the data path.

Options are independent -- every PDE is solved on its own (src/Math/kwFd1d.cpp:45-55)
and dedup only merges identical keys -- so a portfolio splits across GPUs into
contiguous chunks, each priced by its own rank.  Two uses:
  * weak scaling (bench.py): rank r prices its own window of the seeded option
    stream, options r*n .. r*n+n-1;
  * strong scaling: one portfolio partitioned after dedup into contiguous chunks
    balanced by x_dim * (t_dim - 1) node-steps (partition_by_work).
The only cross-rank traffic is the timing reduction (max over ranks) and, for
strong scaling, gathering 8-byte prices back to the caller (strong_shard,
gather_prices).
"""
from __future__ import annotations

import numpy as np


def window(n_per_rank: int, rank: int) -> tuple[int, int]:
    """First option index and count of `rank`'s window of the option stream."""
    return rank * n_per_rank, n_per_rank


def portfolio_shard(n_per_rank: int, rank: int, seed: int = 42) -> np.ndarray:
    """Rank's window of the American-option stream (weak scaling)."""
    import portfolio

    start, n = window(n_per_rank, rank)
    return portfolio.american_portfolio(n, seed=seed, start=start)


def partition_by_work(x_dims, t_dims, world: int) -> list[tuple[int, int]]:
    """Contiguous [begin, end) chunks of a PDE list, one per rank, balanced by
    node-steps x_dim * (t_dim - 1): chunk r ends at the first PDE whose running total
    reaches (r + 1) / world of the whole.  Empty chunks only when PDEs < ranks."""
    x = np.asarray(x_dims, np.int64)
    t = np.asarray(t_dims, np.int64)
    if x.shape != t.shape or world < 1:
        raise ValueError("partition_by_work: x_dims and t_dims must match and world >= 1")
    work = np.cumsum(x * np.maximum(t - 1, 0))
    total = int(work[-1]) if len(work) else 0
    bounds = [0]
    for r in range(1, world):
        target = total * r / world
        bounds.append(max(bounds[-1], int(np.searchsorted(work, target, side="left")) + 1))
    bounds.append(len(x))
    bounds = [min(b, len(x)) for b in bounds]
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def strong_shard(opts, rank: int, world: int, x_dim: int = 0, t_dim: int = 0, x_dims=None, t_dims=None):
    """Indices of the options `rank` prices when one portfolio is split over `world`
    ranks (strong scaling).  Every rank runs the same host dedup (kwg_fd1d_dedup, the
    reference's key, src/Pricer/kwFd1d.cpp:28-65, plus the grid shape for uneven
    batches), so all agree on the PDE list without exchanging it; the PDEs are cut
    into contiguous chunks balanced by node-steps (partition_by_work) and a rank
    takes every option whose PDE lies in its chunk, so no PDE is solved twice.  The
    grid is x_dim x t_dim for every option, or x_dims[i] x t_dims[i] per option."""
    import kwg

    a2p, p2a = kwg.dedup(opts, x_dims, t_dims)
    if len(p2a) == 0:
        return np.zeros(0, np.int64)
    if x_dims is not None and t_dims is not None:
        xs, ts = np.asarray(x_dims)[p2a], np.asarray(t_dims)[p2a]
    else:
        xs, ts = np.full(len(p2a), x_dim), np.full(len(p2a), t_dim)
    begin, end = partition_by_work(xs, ts, world)[rank]
    return np.nonzero((a2p >= begin) & (a2p < end))[0]


def gather_prices(n: int, idx, prices, status=None):
    """All ranks' (indices, prices[, status]) assembled into arrays of the whole
    portfolio on every rank: the only data that crosses ranks, 8 bytes (+4) per
    option, after the solve.  Without a process group the rank's own arrays are
    scattered into place."""
    import torch.distributed as dist

    mine = (np.asarray(idx, np.int64).tobytes(), np.asarray(prices, np.float64).tobytes(),
            None if status is None else np.asarray(status, np.int32).tobytes())
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        parts = [None] * dist.get_world_size()
        dist.all_gather_object(parts, mine)
    else:
        parts = [mine]
    out = np.full(n, np.nan)
    st = np.zeros(n, np.int32) if status is not None else None
    for ib, pb, sb in parts:
        ii = np.frombuffer(ib, np.int64)
        out[ii] = np.frombuffer(pb, np.float64)
        if st is not None and sb is not None:
            st[ii] = np.frombuffer(sb, np.int32)
    return out if st is None else (out, st)


def max_over_ranks(value: float) -> float:
    """Max of a per-rank value over all ranks (the slowest rank's time); the value
    itself when torch.distributed is not initialised.  The reduction runs on the
    process group's own device (CPU tensors for gloo, the current GPU for NCCL)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
