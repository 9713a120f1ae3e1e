"""Blob matching on the GPU (k_blob_match) against the reference's
(tests/golden/matching.npz): the GPU's groups, scored by the blob-map energy
(thread.cpp:1087-1107) with exact blob means, end within MATCH_EPS of the
reference's grouping scored the same way; every frame's blob order is a
permutation of the groups and every pixel's blob belongs to one group."""
import numpy as np
import pytest

from oracle import oracle as orc
from test_matching_pin import MATCH_EPS, cases, reference_energy_exact_means

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["ellipses64", "spline48", "features", "many96"])
def test_gpu_matching_energy_within_eps_of_reference(capi, oracle, case):
    z = cases()
    frames = list(z[f"{case}_frames"])
    delim = int(z[f"{case}_delimiter"])
    m = capi.Morph()
    m.load(frames, seed=int(z[f"{case}_seed"]), blob_delimiter=delim, motion=capi.LINEAR, fading=capi.PERLIN)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    w, pts, order = m.export_chains()
    G = m.chains
    glab = []
    for k in range(len(frames)):
        assert sorted(order[k].tolist()) == list(range(G))
        lab = m.blob_labels(k)
        glab.append(np.where(lab >= 0, order[k][np.maximum(lab, 0)], -1))
        assert np.array_equal(lab >= 0, frames[k][..., 3] > 0)
    colors, _ = orc.stored_frames(frames, delim, oracle)
    e = oracle.blob_energy(orc.group_desc(colors, np.stack(glab), G), orc.bbox_diag2(frames))
    ref = reference_energy_exact_means(oracle, z, case)
    print(f"{case}: GPU matching {e:.6f}, reference {ref:.6f} ({e / ref:.4f}x)")
    assert e <= (1 + MATCH_EPS) * ref
    m.close()
