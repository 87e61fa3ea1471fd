"""Multi-GPU sharding of FD1D batches: one process per GPU, no collective on the data path.

Options are independent -- every PDE is solved on its own (src/Math/kwFd1d.cpp:45-55)
and dedup only merges identical keys -- so a portfolio splits across GPUs into
contiguous chunks, each priced by its own rank.  Two uses:
  * weak scaling (bench.py): rank r prices its own window of the seeded option
    stream, options r*n .. r*n+n-1;
  * strong scaling: one portfolio partitioned after dedup into contiguous chunks
    balanced by x_dim * (t_dim - 1) node-steps (partition_by_work).
The only cross-rank traffic is the timing reduction (max over ranks) and, for
strong scaling, gathering 8-byte prices back to the caller.
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
