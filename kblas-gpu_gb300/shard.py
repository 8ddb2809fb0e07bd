"""Splitting a batch of independent systems across ranks (one process per GPU).

The systems of a batch share nothing, so N ranks each take one contiguous
range of the batch and run the same single-GPU call on it; there is no
exchange between ranks on the data path, only a host-side reduction of the
step times. The reference's testers split batches into contiguous per-GPU
ranges of equal count (testing/batch_triangular/test_Xpotrf_batch.cpp:108,
123-131); here the ranges are balanced by the work of each system instead,
which matters for variable-size batches (n from 8 to 256 spans a 32,768x
range of factorization cost).
"""
from __future__ import annotations

import numpy as np


def system_cost(ns, nrhs: int = 1) -> np.ndarray:
    """Relative cost of one POSV of order n: factorization n^3/3, solves
    2 nrhs n^2, and the n^2 / 2 elements read (each weighted as a few flops)."""
    n = np.asarray(ns, dtype=np.float64)
    return n ** 3 / 3.0 + 2.0 * nrhs * n ** 2 + 4.0 * n ** 2


def shard_range(ns, rank: int, world: int, nrhs: int = 1) -> tuple[int, int]:
    """[lo, hi) of the contiguous range of systems owned by `rank`: the batch
    is cut where the running cost crosses k/world of the total, so every
    system belongs to exactly one rank and the ranges follow rank order."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of size {world}")
    count = len(ns)
    if world == 1 or count == 0:
        return (0, count) if rank == 0 else (count, count)
    cum = np.cumsum(system_cost(ns, nrhs))
    total = cum[-1]

    def cut(k: int) -> int:
        if k <= 0:
            return 0
        if k >= world:
            return count
        # first index whose running cost reaches k/world of the total
        return int(np.searchsorted(cum, total * k / world, side="left")) + 1

    lo, hi = cut(rank), cut(rank + 1)
    return min(lo, count), min(max(hi, lo), count)


def max_over_ranks(value: float) -> float:
    """Largest `value` over the ranks of the default process group (the step
    time of a multi-rank run is that of its slowest rank); the value itself
    when no group is initialised."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float) -> float:
    """Sum of `value` over the ranks (e.g. the systems every rank processed)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
