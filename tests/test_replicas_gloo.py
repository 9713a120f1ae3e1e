"""Multi-rank path of bench.py on CPU: two gloo ranks with different timed
regions agree on the slowest one, and the whole-job value counts the frames
of every rank against it (weak scaling); the ranks' shares of the frame cycle
and of a job list cover them exactly once."""
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


def _shard_rank(rank, world, port, per_rank, jobs, out):
    sys.path.insert(0, ROOT)
    from atomorph_gb300 import shard
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        frames = shard.frame_indices(rank, world, per_rank)
        mine = torch.tensor(frames, dtype=torch.int64)
        gathered = [torch.zeros_like(mine) for _ in range(world)]
        dist.all_gather(gathered, mine)
        js = shard.job_indices(rank, world, jobs)
        n = torch.tensor([len(js)], dtype=torch.int64)
        counts = [torch.zeros_like(n) for _ in range(world)]
        dist.all_gather(counts, n)
        jt = torch.full((jobs,), -1, dtype=torch.int64)
        jt[:len(js)] = torch.tensor(js, dtype=torch.int64)
        jall = [torch.zeros_like(jt) for _ in range(world)]
        dist.all_gather(jall, jt)
        out[rank] = ([g.tolist() for g in gathered], [int(c) for c in counts],
                     [[v for v in g.tolist() if v >= 0] for g in jall])
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_ranks_cover_the_frame_cycle_and_the_jobs_exactly_once(world):
    per_rank, jobs = 240, 32
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_shard_rank, args=(world, _free_port(), per_rank, jobs, out), nprocs=world, join=True)
        res = dict(out)
    frames, counts, job_lists = res[0]
    allf = sorted(f for fr in frames for f in fr)
    assert allf == list(range(per_rank * world))           # every frame of the cycle once
    assert all(len(fr) == per_rank for fr in frames)        # the same work on every rank
    allj = sorted(j for jl in job_lists for j in jl)
    assert allj == list(range(jobs)) and sum(counts) == jobs
    assert max(counts) - min(counts) <= 1
