"""Parity at the benchmarked workload: shapes1024 (8 seeded 1024x1024 key
frames, about 1M atoms per key frame, SPLINE motion with the 2-px Perlin
motion perturbation, PERLIN fading, HSP delimiter), the configuration
bench.py measures.  Integer results exact (blob and pixel counts per key
frame, chain widths, original points, the cost before and after
refinement); atom positions equal to the oracle's bit for bit; one frame
inside every key-frame pair within 1 LSB of the oracle's render."""
import os

import numpy as np
import pytest

from atomorph_gb300 import synth
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

SETTINGS = dict(seed=5, blob_delimiter=1, motion=4, fading=6, density=1)
NOISE = 2.0


@pytest.fixture(scope="module")
def scale(capi):
    frames = synth.workload("shapes1024")
    m = capi.Morph()
    m.load(frames, **SETTINGS)
    m.set(motion_noise=NOISE)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    yield frames, m
    m.close()


def oracle_state(O, m, frames):
    w, pts, order = m.export_chains()
    colors, present = orc.stored_frames(frames, SETTINGS["blob_delimiter"], O)
    xs, ys = [], []
    for f in frames:
        y, x = np.nonzero(f[..., 3])
        xs += [int(x.min()), int(x.max())]
        ys += [int(y.min()), int(y.max())]
    return dict(K=len(frames), width=m.width, height=m.height, bbox=np.array([min(xs), min(ys), max(xs), max(ys)]),
                seed=SETTINGS["seed"], motion=SETTINGS["motion"], fading=SETTINGS["fading"],
                delimiter=SETTINGS["blob_delimiter"], density=SETTINGS["density"], colors=colors, present=present,
                widths=w, pts=pts, blob_order=order, frame_keys=np.arange(len(frames), dtype=np.uint64),
                motion_noise=NOISE)


def test_counts_widths_and_points_at_scale(scale, oracle):
    frames, m = scale
    K = len(frames)
    assert K == 8 and m.width == 1024 and m.height == 1024
    comps = []
    for k, img in enumerate(frames):
        labels, stats = oracle.components(img)
        comps.append(len(stats))
        assert m.blob_count(k) == len(stats), k
        assert m.pixel_count(k) == synth.opaque_count(img), k
    w, pts, order = m.export_chains()
    assert m.chains == max(comps)
    P = pts.reshape(K, -1)
    off = 0
    for c, wc in enumerate(w):
        wc = int(wc)
        orig = (((P[:, off:off + wc] >> 48) & 3) == 3).sum(axis=1)
        assert wc == int(orig.max()) * SETTINGS["density"], c
        off += wc
    for k, img in enumerate(frames):
        o = P[k][((P[k] >> 48) & 3) == 3]
        ys, xs = np.nonzero(img[..., 3])
        assert len(o) == len(xs)
        key = np.sort((o & 0xFFFF) + ((o >> 16) & 0xFFFF) * 65536)
        assert np.array_equal(key, np.sort(xs.astype(np.uint64) + ys.astype(np.uint64) * 65536))
    for k in range(K):
        assert sorted(order[k].tolist()) == list(range(m.chains))
    assert m.cost() == oracle.energy(pts, w, K)[1]


def test_refined_cost_exact_at_scale(scale, oracle):
    frames, m = scale
    before = m.cost()
    gains = m.refine(40)
    after = m.cost()
    assert after == before - int(gains.sum()) and after < before
    w, pts, order = m.export_chains()
    assert oracle.energy(pts, w, len(frames))[1] == after


def test_positions_and_frames_in_every_pair_at_scale(scale, oracle):
    frames, m = scale
    K = len(frames)
    st = oracle_state(oracle, m, frames)
    ts = [(k + 0.37) / K for k in range(K)]
    for t in ts[::3]:
        assert np.array_equal(m.positions(t), oracle.positions(st, t)), t
    ref = oracle.render_many(st, ts, threads=max(1, os.cpu_count() or 1))
    for i, t in enumerate(ts):
        got = m.render(t).astype(np.int32)
        d = np.abs(got - ref[i].astype(np.int32))
        print(f"t={t:.4f}: max {int(d.max())} LSB, {int((d > 0).sum())} channel values differ")
        assert int(d.max()) <= 1, (t, int(d.max()))
