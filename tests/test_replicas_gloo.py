"""The multi-process (replicas) path of bench.py on the CPU: two gloo ranks, each with its own
step time, agree on the slowest one and report the whole-job throughput of both replicas."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(100.0 + 25.0 * rank, world)
        out[rank] = (ms, bench.aggregate_rows_per_s(1000, ms, world))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_step():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = 29500 + os.getpid() % 1000
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0] == res[1] == (125.0, 2 * 1000 / 0.125)


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(42.0, 1) == 42.0
    assert bench.aggregate_rows_per_s(500, 250.0, 1) == 2000.0
