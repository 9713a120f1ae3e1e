"""Blob matching (thread::match, thread.cpp:598-738) pinned to the reference
(tests/golden/matching.npz, made by the unmodified reference driven with a
valid bounding box): the oracle's blob-map energy (get_energy(blob***),
thread.cpp:1087-1107, with blob_distance, thread.cpp:1151-1174) equals the
reference's own best energy on the reference's descriptors, and the oracle's
matcher ends within MATCH_EPS of the reference's energy.  Both matchers are
random local searches (the reference's draws come from its worker's engine),
so the assignment itself is not expected to be identical."""
import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as orc

MATCH_EPS = 0.05  # the matched energy may exceed the reference's by at most 5%


def cases():
    with np.load(f"{GOLDEN}/matching.npz") as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="module")
def z():
    return cases()


@pytest.mark.parametrize("case", ["ellipses64", "spline48", "features", "many96"])
def test_energy_function_equals_reference(oracle, z, case):
    frames = list(z[f"{case}_frames"])
    e = float(z[f"{case}_energy"])
    got = oracle.blob_energy(z[f"{case}_desc"], orc.bbox_diag2(frames))
    assert abs(got - e) <= 1e-9 * max(e, 1.0), (got, e)


def reference_energy_exact_means(oracle, z, case):
    """The reference's grouping scored with exact blob means (the GPU and the
    oracle build blobs with exact means, the reference with running means)."""
    frames = list(z[f"{case}_frames"])
    colors, _ = orc.stored_frames(frames, int(z[f"{case}_delimiter"]), oracle)
    glab = z[f"{case}_group_labels"].astype(np.int32)
    return oracle.blob_energy(orc.group_desc(colors, glab, z[f"{case}_desc"].shape[0]), orc.bbox_diag2(frames))


@pytest.mark.parametrize("case", ["ellipses64", "spline48", "features", "many96"])
def test_oracle_matcher_within_eps_of_reference(oracle, z, case):
    frames = list(z[f"{case}_frames"])
    delim = int(z[f"{case}_delimiter"])
    colors, _ = orc.stored_frames(frames, delim, oracle)
    st = orc.pipeline(oracle, frames, delimiter=delim, density=1, seed=1, motion=3, fading=6)
    glab = []
    for k, img in enumerate(frames):
        lab, _ = oracle.components(img, colors[k].view(np.uint8).reshape(img.shape))
        order = st["blob_order"][k]
        glab.append(np.where(lab >= 0, order[np.maximum(lab, 0)], -1))
    e = oracle.blob_energy(orc.group_desc(colors, np.stack(glab), st["blob_order"].shape[1]),
                           orc.bbox_diag2(frames))
    ref = reference_energy_exact_means(oracle, z, case)
    print(f"{case}: oracle matcher {e:.6f}, reference {ref:.6f} ({e / ref:.4f}x)")
    assert e <= (1 + MATCH_EPS) * ref
