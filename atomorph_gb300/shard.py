"""Partition of the morph path's independent units across ranks (one process
per GPU).  Output frames and morph jobs are independent (a frame reads the
chains, a job its own key frames and chains), so ranks split them with no
exchange on the data path; only the timing takes a collective (max over
ranks)."""
from __future__ import annotations


def frame_indices(rank: int, world: int, per_rank: int) -> list[int]:
    """Indices, in a cycle of per_rank * world frames, of the frames rank
    renders: every world-th frame from its rank on, per_rank of them, so the
    ranks together cover the cycle exactly once and each rank's frames span
    the whole morph (every key-frame pair, similar work per rank)."""
    if not 0 <= rank < world or per_rank < 0:
        raise ValueError(f"rank {rank} of {world}, {per_rank} frames per rank")
    return [rank + world * i for i in range(per_rank)]


def job_indices(rank: int, world: int, jobs: int) -> list[int]:
    """Jobs 0..jobs-1 dealt round-robin: rank gets every world-th job."""
    if not 0 <= rank < world or jobs < 0:
        raise ValueError(f"rank {rank} of {world}, {jobs} jobs")
    return list(range(rank, jobs, world))
