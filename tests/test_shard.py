"""Host-side logic of multi-rank runs, on the CPU: the work-balanced contiguous
split of a batch across ranks, and the max / sum reductions of a multi-rank
step, run as two gloo ranks (127.0.0.1)."""
import importlib
import os
import socket

import numpy as np
import pytest


def shard(kb):
    return importlib.import_module("kblas_gpu_gb300.shard")


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_ranges_partition_the_batch(kb, wl, world):
    sh = shard(kb)
    ns = wl.vbatch_sizes(100_000 * world, 8, 256, seed=0)
    ranges = [sh.shard_range(ns, r, world) for r in range(world)]
    assert ranges[0][0] == 0 and ranges[-1][1] == len(ns)
    for (lo0, hi0), (lo1, _) in zip(ranges, ranges[1:]):
        assert hi0 == lo1 and lo0 <= hi0
    cost = sh.system_cost(ns)
    per = np.array([cost[lo:hi].sum() for lo, hi in ranges])
    # balanced to within one system of the largest order
    assert per.max() - per.min() <= 2 * sh.system_cost([256])[0]
    counts = np.array([hi - lo for lo, hi in ranges])
    assert (np.abs(counts - 100_000) < 2_000).all()  # weak scaling: ~fixed work per rank


def test_ranges_edge_cases(kb):
    sh = shard(kb)
    assert sh.shard_range([], 0, 2) == (0, 0)
    assert sh.shard_range([], 1, 2) == (0, 0)
    assert sh.shard_range([64], 0, 1) == (0, 1)
    r = [sh.shard_range([64], k, 4) for k in range(4)]
    assert sum(hi - lo for lo, hi in r) == 1
    with pytest.raises(ValueError):
        sh.shard_range([8, 8], 2, 2)
    # equal orders split into equal counts
    r = [sh.shard_range([32] * 1000, k, 4) for k in range(4)]
    assert [hi - lo for lo, hi in r] == [250] * 4


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "tests"))
    sys.path.insert(0, root)
    from conftest import load_pkg, load_workloads
    load_pkg()
    wl = load_workloads()
    sh = importlib.import_module("kblas_gpu_gb300.shard")
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        ns = wl.vbatch_sizes(1000 * world, 8, 256, seed=0)
        lo, hi = sh.shard_range(ns, rank, world)
        step_ms = 10.0 + rank  # the slowest rank sets the step time
        out.put((rank, lo, hi, sh.max_over_ranks(step_ms), sh.sum_over_ranks(hi - lo)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_step_time_and_count(kb):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1] == 0 and res[0][2] == res[1][1] and res[1][2] == 2000
    assert all(r[3] == 11.0 for r in res)        # max over ranks
    assert all(r[4] == 2000 for r in res)        # every system counted once
