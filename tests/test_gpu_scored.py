"""The learned pair proposal (AM_PROPOSAL_SCORED): plain sweeps log their own
proposals' outcomes (pair features, accept / reject of the exact criterion,
thread.cpp:1014-1022); the network trained on them on the tensor cores
ranks random partners; every swap it leads to is checked exactly, so the
points stay a permutation per key frame and the cost is tracked exactly.
What the trained network gains over the same sweeps with an untrained one
is measured at an equal sweep budget."""
import numpy as np
import pytest

from atomorph_gb300 import synth
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _handle(capi, oracle, job=0):
    frames = synth.workload("shapes256", job)
    st = orc.pipeline(oracle, frames, delimiter=1, density=1, seed=5, motion=4, fading=6)
    m = capi.Morph()
    m.load(frames, seed=5, blob_delimiter=1, motion=4, fading=6, density=1)
    m.import_chains(st["widths"], st["pts"], st["blob_order"])
    return m, st


def test_outcome_log_of_plain_sweeps(capi, oracle):
    m, st = _handle(capi, oracle)
    K = st["K"]
    pairs = int(sum(int(w) // 2 for w in st["widths"] if int(w) > 1))
    m.record_outcomes(10 * pairs * K, every=1)
    m.refine(1, capi.PROPOSAL_RANDOM)
    f, y = m.recorded_swaps(10 * pairs * K)
    # one sweep proposes every pair of every chain once in every key frame
    assert len(y) == pairs * K
    assert set(np.unique(y).tolist()) <= {0.0, 1.0} and 0.0 < y.mean() < 1.0
    assert np.isfinite(f).all()
    assert (np.abs(f[:, 2:6]) <= 1.0 + 1e-6).all() and (f[:, 6:8] >= 0).all()
    assert set(np.unique(f[:, 8]).tolist()) <= {0.0, 1.0}
    assert np.allclose(f[:, 9], np.hypot(f[:, 0], f[:, 1]), rtol=1e-5, atol=1e-6)
    # 1 in 8 sampled
    m.record_outcomes(10 * pairs * K, every=8)
    m.refine(1, capi.PROPOSAL_RANDOM)
    n8 = m.recorded_count()
    assert 0.08 * pairs * K < n8 < 0.17 * pairs * K
    m.close()


def test_scored_sweeps_exact_and_trained_beats_untrained(capi, oracle):
    m, st = _handle(capi, oracle)
    K = st["K"]
    # training data: outcomes of 30 plain sweeps from the same start
    m.record_outcomes(4_000_000, every=1)
    m.refine(30, capi.PROPOSAL_RANDOM)
    n = m.recorded_count()
    assert n > 1_000_000
    loss = m.train_recorded(epochs=2, lr=2e-3)
    assert np.isfinite(loss) and loss < 0.25  # the Brier score of always predicting 1/2
    trained = m.proposal_weights()
    m.close()

    def run(weights, proposal, sweeps=40):
        h, _ = _handle(capi, oracle)
        if weights is not None:
            h.proposal_weights(weights)
        before = np.sort(h.export_chains()[1].reshape(K, -1), axis=1)
        c0 = h.cost()
        g = h.refine(sweeps, proposal)
        c = h.cost()
        assert c == c0 - int(g.sum())
        w, pts, order = h.export_chains()
        assert oracle.energy(pts, w, K)[1] == c
        assert np.array_equal(np.sort(pts.reshape(K, -1), axis=1), before)  # a permutation per key frame
        h.close()
        return c0, c

    fresh = capi.Morph()
    untrained = fresh.proposal_weights()  # the He-initialised network
    fresh.close()
    c0, c_trained = run(trained, capi.PROPOSAL_SCORED)
    _, c_untrained = run(untrained, capi.PROPOSAL_SCORED)
    _, c_plain = run(None, capi.PROPOSAL_RANDOM)
    print(f"40 sweeps from {c0}: scored trained {c_trained}, untrained {c_untrained}, plain {c_plain}")
    assert c_trained < c_untrained
    assert c_trained < c_plain


def test_scored_without_a_trained_network_runs_plain_sweeps(capi, oracle):
    a, _ = _handle(capi, oracle)
    b, _ = _handle(capi, oracle)
    ga = a.refine(5, capi.PROPOSAL_SCORED)
    gb = b.refine(5, capi.PROPOSAL_RANDOM)
    assert np.array_equal(ga, gb) and a.cost() == b.cost()
    a.close()
    b.close()
