"""Multi-rank path of bench.py on CPU: two gloo ranks with different timed
regions agree on the slowest one, and the whole-job value counts the frames
of every rank against it (replicas, weak scaling)."""
import os
import socket
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = [12.5, 30.0][rank]
        slowest = bench.max_over_ranks(ms, world, device="cpu")
        out[rank] = (slowest, bench.job_value(240, world, slowest))
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time():
    world = 2
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1]
    slowest, value = res[0]
    assert slowest == 30.0
    assert value == pytest.approx(480 / 0.030)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(7.0, 1) == 7.0
    assert bench.job_value(240, 1, 1000.0) == pytest.approx(240.0)
