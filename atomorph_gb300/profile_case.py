"""Every kernel of the morph path, a few launches each, on one seeded
workload: the program per-kernel profiler captures are taken on.

    python -m atomorph_gb300.profile_case [--workload shapes1024] [--frames 3]

After the pipeline (components, blob matching, chain construction) it runs
4 plain sweeps, 4 guided sweeps, 2 recorded sweeps, one training epoch
and 4 gated (learned) sweeps, the allocation-free cost, `--frames` atom
frames, 2 fluid frames with 2 solver steps each on a (0.5 W + 20)^2 grid,
and one batched refinement of 4 small jobs.  Settings match bench.py's
(SPLINE motion, PERLIN fading, HSP delimiter)."""
from __future__ import annotations

import argparse
import ctypes as C

from atomorph_gb300 import capi, synth

SETTINGS = dict(seed=5, blob_delimiter=1, motion=4, fading=6, density=1)


def run(workload: str, frames: int) -> dict:
    import torch

    keys = synth.workload(workload)
    m = capi.Morph()
    m.load(keys, **SETTINGS)
    if m.run_until(capi.STATE_ATOM_MORPHING) != capi.STATE_ATOM_MORPHING:
        raise RuntimeError("pipeline stopped early")
    m.refine(4, capi.PROPOSAL_RANDOM)
    m.tune(guided_switch=0)
    m.refine(4, capi.PROPOSAL_LOCAL)
    m.tune(learned_adaptive=0)
    m.record_swaps(1 << 22)  # recording sweeps run the learned form's gate with every region kept
    m.refine(2, capi.PROPOSAL_LEARNED)
    f, y = m.recorded_swaps(1 << 22)
    m.record_swaps(0)
    if not len(y):
        raise RuntimeError("no recorded samples")
    m.train_proposal(f, y, epochs=1, lr=2e-3)
    m.refine(4, capi.PROPOSAL_LEARNED)
    v = C.c_uint64()
    rc = m.lib.am_get_cost_noalloc(m.h, C.byref(v))
    if rc:
        raise RuntimeError(f"am_get_cost_noalloc: {rc}")
    out = torch.empty((m.height, m.width, 4), dtype=torch.uint8, device="cuda")
    for i in range(frames):
        m.render_device(m.get_time(i * 7 + 1, 240), out.data_ptr())
    m.set(fluid=2, fluid_sparseness=0.5)
    for i in range(2):
        m.render_device(m.get_time(i, 240), out.data_ptr())
    m.set(fluid=0)
    torch.cuda.synchronize()
    jobs = []
    for j in range(4):
        a = capi.Morph()
        a.load(synth.workload("batch", j), seed=j + 1, blob_delimiter=0, motion=capi.SPLINE)
        if a.run_until(capi.STATE_ATOM_MORPHING) != capi.STATE_ATOM_MORPHING:
            raise RuntimeError(f"batch job {j}: pipeline stopped early")
        jobs.append(a)
    b = capi.Batch(jobs)
    b.refine(4)
    b.close()
    for a in jobs:
        a.close()
    res = {"workload": workload, "atoms": m.atoms, "cost": int(v.value), "samples": int(len(y))}
    m.close()
    return res


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="shapes1024")
    ap.add_argument("--frames", type=int, default=3)
    args = ap.parse_args()
    print(run(args.workload, args.frames))


if __name__ == "__main__":
    main()
