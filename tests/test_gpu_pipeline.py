"""End-to-end pipeline on the GPU through the C ABI: key frames in, blobs,
matching, chains, refinement, readout.  Integer results (blob counts, atom
counts, surface points) must be exact."""
import time

import numpy as np
import pytest

from atomorph_gb300 import synth
from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["ellipses64", "spline48"])
def test_blob_and_atom_counts_match_reference(capi, oracle, case):
    g = golden(case)
    frames = list(g["frames"])
    K = len(frames)
    m = capi.Morph()
    m.load(frames, seed=int(g["seed"]), blob_delimiter=int(g["delimiter"]), motion=int(g["motion"]),
           fading=int(g["fading"]), density=int(g["density"]))
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    for k in range(K):
        assert m.blob_count(k) == g["blob_counts"][k]
        assert m.pixel_count(k) == g["pixel_counts"][k]
    w, pts, order = m.export_chains()
    assert m.chains == len(g["widths"])
    # Chain widths are max blob size of the group times density: their sum
    # depends on the matching, but every chain must cover its largest blob.
    P = pts.reshape(K, -1)
    dens = int(g["density"])
    off = 0
    for c, wc in enumerate(w):
        wc = int(wc)
        assert wc % dens == 0
        sizes = [int((((P[k, off:off + wc] >> 48) & 3) == 3).sum()) for k in range(K)]
        assert wc == max(sizes) * dens
        off += wc
    # Original points (HAS_PIXEL|HAS_FLUID) are exactly the key frames' pixels.
    for k, img in enumerate(frames):
        orig = P[k][((P[k] >> 48) & 3) == 3]
        xy = set(zip((orig & 0xFFFF).tolist(), ((orig >> 16) & 0xFFFF).tolist()))
        ys, xs = np.nonzero(img[..., 3])
        assert len(orig) == len(xs)
        assert xy == set(zip(xs.tolist(), ys.tolist()))
        assert (((orig >> 32) & 0xFFFF) == 0).all()  # fractions zero
    # blob order is a permutation of the groups per frame
    for k in range(K):
        assert sorted(order[k].tolist()) == list(range(m.chains))
    assert m.cost() == oracle.energy(pts, w, K)[1]


def test_components_match_oracle_at_scale(capi, oracle):
    frames = synth.workload("shapes256")
    m = capi.Morph()
    m.load(frames)
    m.run_until(capi.STATE_BLOB_MATCHING)
    for k, img in enumerate(frames):
        labels, stats = oracle.components(img)
        assert m.blob_count(k) == len(stats)


def test_worker_thread_runs_and_suspends(capi):
    frames = synth.workload("shapes256")
    m = capi.Morph()
    m.load(frames, sweeps=4)
    assert m.synchronize() == capi.AM_OK
    m.compute()
    deadline = time.time() + 30
    while time.time() < deadline:
        time.sleep(0.05)
        m.suspend()
        assert m.synchronize() == capi.AM_OK
        if m.state == capi.STATE_ATOM_MORPHING and m.energy > 0:
            break
        m.compute()
    assert m.state == capi.STATE_ATOM_MORPHING
    e1 = m.energy
    m.compute()
    time.sleep(0.2)
    assert m.synchronize() == capi.AM_ERR_BUSY
    m.suspend()
    assert m.synchronize() == capi.AM_OK
    assert m.energy <= e1
    assert m.energy == m.cost()
    m.next_state()
    assert m.synchronize() == capi.AM_OK
    m.iterate(1)
    m.wait()
    m.synchronize()
    assert m.state == capi.STATE_DONE
