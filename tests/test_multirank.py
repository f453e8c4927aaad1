"""The multi-rank path of bench.py (one process per GPU, each on its own
trails) with two gloo ranks on the CPU: the slowest rank's time and the sum of
the units make the whole-job rate."""
import os
import sys

import pytest

from conftest import ROOT


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    seconds, units = [(2.0, 100), (3.5, 250)][rank]
    t, u = bench.combine_ranks(dist, "cpu", seconds, units)
    dist.barrier()
    q.put((rank, t, u))
    dist.destroy_process_group()


def test_two_ranks_combine_time_and_units():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 3.5, 350.0), (1, 3.5, 350.0)]


def test_one_process_needs_no_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.combine_ranks(None, "cpu", 1.5, 7) == (1.5, 7.0)
