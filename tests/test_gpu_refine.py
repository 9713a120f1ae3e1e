"""Atom refinement on the GPU: exact invariants and convergence against the
oracle (the reference's own random-swap refinement restated bit-exactly)."""
import numpy as np
import pytest

from atomorph_gb300 import synth
from conftest import golden, morph_from_golden

pytestmark = pytest.mark.gpu


def _columns_are_permutations(pts0, pts, widths, K):
    """Each chain's points at each key frame are the same multiset (swaps only
    move points between columns of one frame)."""
    N = int(widths.sum())
    a = pts0.reshape(K, N)
    b = pts.reshape(K, N)
    off = 0
    for w in widths:
        w = int(w)
        for k in range(K):
            if not np.array_equal(np.sort(a[k, off:off + w]), np.sort(b[k, off:off + w])):
                return False
        off += w
    return True


@pytest.mark.parametrize("case", ["ellipses64", "spline48"])
def test_cost_is_exact_and_tracked(capi, oracle, case):
    g = golden(case)
    m = morph_from_golden(capi, g, "pts0")
    K = int(g["K"])
    assert m.cost() == int(g["energy0"])
    gains = m.refine(30)
    c1 = m.cost()
    assert c1 == int(g["energy0"]) - int(gains.sum())
    w, pts, order = m.export_chains()
    assert np.array_equal(w, g["widths"])
    assert oracle.energy(pts, w, K)[1] == c1
    assert _columns_are_permutations(g["pts0"], pts, w, K)
    assert np.array_equal(order, g["blob_order"])


def test_random_refinement_reaches_reference_converged_cost(capi, oracle):
    """Plain GPU refinement ends within 0.5% of the reference's converged
    cost on the same chains (ellipses64; the reference is run by its
    restatement for 2000 sweeps)."""
    g = golden("ellipses64")
    K = int(g["K"])
    ref_conv = oracle.energy(oracle.sweeps(g["pts0"], g["widths"], K, 2000, 5), g["widths"], K)[1]
    m = morph_from_golden(capi, g, "pts0")
    m.refine(2000)
    assert m.cost() <= 1.005 * ref_conv, (m.cost(), ref_conv)


def test_refinement_never_increases_cost(capi):
    g = golden("spline48")
    m = morph_from_golden(capi, g, "pts0")
    gains = m.refine(200)
    assert (gains >= 0).all()
    assert gains[:5].sum() > 0


def test_refine_requires_chains(capi):
    m = capi.Morph()
    m.load(synth.workload("ellipses64"))
    with pytest.raises(capi.AmError):
        m.refine(1)


def test_local_proposal_invariants_and_speed(capi, oracle):
    """Guided (spatially local) proposals keep every invariant of the plain
    refinement and get within 0.5% of the plain method's 2000-sweep cost in
    fewer sweeps (plain sweeps first, guided ones once plain stalls)."""
    frames = synth.workload("shapes256")
    m = capi.Morph()
    m.load(frames, seed=3, blob_delimiter=0, motion=capi.LINEAR, fading=capi.LINEAR)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    w, pts0, order = m.export_chains()
    K = len(frames)
    c0 = m.cost()
    g = m.refine(2000, capi.PROPOSAL_RANDOM)
    c_plain = m.cost()
    assert c_plain == c0 - int(g.sum())
    m.import_chains(w, pts0, order)
    total, sweeps = 0, 0
    while sweeps < 2000:
        gl = m.refine(10, capi.PROPOSAL_LOCAL)
        total += int(gl.sum())
        sweeps += 10
        if c0 - total <= 1.005 * c_plain:
            break
    c_local = m.cost()
    assert c_local == c0 - total
    _, pts, _ = m.export_chains()
    assert _columns_are_permutations(pts0, pts, w, K)
    assert oracle.energy(pts, w, K)[1] == c_local
    assert c_local <= 1.005 * c_plain, (c_local, c_plain)
    assert sweeps < 2000
    # switching back to random sweeps after guided ones stays consistent
    g2 = m.refine(5, capi.PROPOSAL_RANDOM)
    assert m.cost() == c_local - int(g2.sum())
    gl2 = m.refine(5, capi.PROPOSAL_LOCAL)
    assert m.cost() == c_local - int(g2.sum()) - int(gl2.sum())
