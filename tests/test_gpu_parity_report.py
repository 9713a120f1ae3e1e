"""Render parity per configuration, as a histogram of the per-channel
difference to the oracle's render of the same chains (0 / 1 / more LSB), on
each configuration's workload and settings: C1 (64², linear, RGB and HSP
delimiters, 16 frames), C2 (256², spline with the 2-px motion perturbation),
C3 (two batch jobs of 128² and 256², spline, through the batched render),
C4's evaluation canvas (512², spline).  The bar is at most 1 LSB; the
histograms are printed (`-s`) for the record.  C5's frames are checked by
tests/test_gpu_scale.py."""
import os

import numpy as np
import pytest

from atomorph_gb300 import synth
from oracle import oracle as orc
from test_gpu_render_options import _bbox

pytestmark = pytest.mark.gpu


def _state(m, frames, delimiter, seed, motion, oracle, noise=0.0):
    w, pts, order = m.export_chains()
    colors, present = orc.stored_frames(frames, delimiter, oracle)
    K = len(frames)
    return dict(K=K, width=m.width, height=m.height, bbox=_bbox(frames), seed=seed, motion=motion, fading=6,
                delimiter=delimiter, density=1, colors=colors, present=present, widths=w, pts=pts,
                blob_order=order, frame_keys=np.arange(K, dtype=np.uint64), motion_noise=noise)


def _hist(got, ref):
    d = np.abs(got.astype(np.int32) - ref.astype(np.int32))
    return np.array([(d == 0).sum(), (d == 1).sum(), (d > 1).sum()], np.int64)


CASES = [
    ("C1 64² linear RGB", "ellipses64", 0, 0, 3, 200, 0.0, 16),
    ("C1 64² linear HSP", "ellipses64", 0, 1, 3, 200, 0.0, 16),
    ("C2 256² spline + 2-px perturbation", "shapes256", 0, 1, 4, 200, 2.0, 8),
    ("C4 evaluation 512² spline", "shapes512", 0, 1, 4, 100, 0.0, 4),
]


@pytest.mark.parametrize("name,wl,job,delim,motion,sweeps,noise,nf", CASES)
def test_render_lsb_histogram(capi, oracle, name, wl, job, delim, motion, sweeps, noise, nf):
    frames = synth.workload(wl, job)
    m = capi.Morph()
    m.load(frames, seed=5, blob_delimiter=delim, motion=motion, fading=capi.PERLIN)
    if noise:
        m.set(motion_noise=noise)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    m.refine(sweeps, capi.PROPOSAL_RANDOM)
    st = _state(m, frames, delim, 5, motion, oracle, noise)
    ts = [(i + 0.5) / nf for i in range(nf)]
    ref = oracle.render_many(st, ts, threads=max(1, os.cpu_count() or 1))
    h = np.zeros(3, np.int64)
    for i, t in enumerate(ts):
        h += _hist(m.render(t), ref[i])
    n = int(h.sum())
    print(f"{name}: {nf} frames, {n} channel values: 0 LSB {h[0]} ({h[0] / n:.6f}), 1 LSB {h[1]}, >1 LSB {h[2]}")
    assert h[2] == 0
    m.close()


def test_render_lsb_histogram_batched_jobs(capi, oracle):
    jobs = [10, 0]  # 128² (4 key frames) and 256² (3 key frames)
    ms, sts = [], []
    for j in jobs:
        frames = synth.workload("batch", j)
        m = capi.Morph()
        m.load(frames, seed=j + 1, blob_delimiter=0, motion=capi.SPLINE, fading=capi.PERLIN)
        assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
        m.refine(50, capi.PROPOSAL_RANDOM)
        ms.append(m)
        sts.append(_state(m, frames, 0, j + 1, capi.SPLINE, oracle))
    ts = [(i + 0.5) / 8 for i in range(8)]
    b = capi.Batch(ms)
    got = b.render(ts)
    for j, m, st, g in zip(jobs, ms, sts, got):
        ref = oracle.render_many(st, ts, threads=max(1, os.cpu_count() or 1))
        h = sum(_hist(g[i], ref[i]) for i in range(len(ts)))
        n = int(h.sum())
        print(f"C3 batch job {j} ({m.width}², batched): 8 frames, {n} channel values: 0 LSB {h[0]} "
              f"({h[0] / n:.6f}), 1 LSB {h[1]}, >1 LSB {h[2]}")
        assert h[2] == 0
    b.close()
    for m in ms:
        m.close()
