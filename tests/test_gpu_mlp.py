"""The learned swap proposal: tensor-core forward/backward against the numpy
restatement, training, and what the trained network gains.

The network gates the guided candidate scan: it scores every 32-slot region
(a compact patch of a key frame) from cheap features of its slots, and only
the best-scored fraction of the regions runs the scan.  Trained on the gains
the full scan found per region, it should pick the patches where improving
swaps are left."""
import numpy as np
import pytest

import mlp_ref
from atomorph_gb300 import synth

pytestmark = pytest.mark.gpu


def _rand_params(seed):
    r = np.random.default_rng(seed)
    m = np.zeros(4929, np.float32)
    m[0:640] = r.normal(0, 0.45, 640)
    m[640:704] = r.normal(0, 0.1, 64)
    m[704:4800] = r.normal(0, 0.18, 4096)
    m[4800:4864] = r.normal(0, 0.1, 64)
    m[4864:4928] = r.normal(0, 0.2, 64)
    m[4928] = 0.05
    return m


def test_forward_matches_numpy(capi):
    m = capi.Morph()
    w = _rand_params(1)
    m.proposal_weights(w)
    X = np.random.default_rng(2).normal(0, 1.5, (1000, 10)).astype(np.float32)
    got = m.proposal_forward(X)
    ref, _ = mlp_ref.forward(w, X)
    np.testing.assert_allclose(got, ref, rtol=2e-3, atol=2e-3)


def test_gradients_match_numpy(capi):
    """Gradient check of the tensor-core backward pass (BF16 operands, FP32
    accumulation) against the float64 restatement; tolerance 1% of each
    block's largest gradient."""
    m = capi.Morph()
    w = _rand_params(3)
    m.proposal_weights(w)
    r = np.random.default_rng(4)
    X = r.normal(0, 1.2, (777, 10)).astype(np.float32)
    t = r.normal(0, 1.0, 777).astype(np.float32)
    g, loss = m.proposal_grad(X, t)
    gr, lr_ = mlp_ref.grad(w, X, t)
    assert loss == pytest.approx(lr_, rel=1e-3)
    for name, (a, b) in {"W1": (0, 640), "b1": (640, 704), "W2": (704, 4800), "b2": (4800, 4864),
                         "w3": (4864, 4928), "b3": (4928, 4929)}.items():
        scale = max(np.abs(gr[a:b]).max(), 1e-6)
        err = np.abs(g[a:b] - gr[a:b]).max() / scale
        assert err < 1e-2, (name, err)


def test_training_fits_a_known_function(capi):
    m = capi.Morph()
    r = np.random.default_rng(5)
    X = r.normal(0, 1, (60000, 10)).astype(np.float32)
    t = (np.tanh(X[:, 0] - 0.5 * X[:, 1]) + 0.3 * X[:, 6] * (X[:, 7] > 0)).astype(np.float32)
    l0 = float(np.mean((m.proposal_forward(X) - t) ** 2))
    loss = m.train_proposal(X, t, epochs=8, lr=3e-3)
    l1 = float(np.mean((m.proposal_forward(X) - t) ** 2))
    assert loss < 0.5 * l0 and l1 < 0.5 * l0, (l0, loss, l1)


def _chains(capi, frames, **kw):
    m = capi.Morph()
    m.load(frames, **kw)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    return m


def test_learned_gate_keep_all_equals_guided(capi):
    """With every column kept, the gated path runs exactly the guided sweeps:
    same proposals, same claims, same applied swaps, bit for bit.  Two
    handles with the same frames, seed and chains (sweep counters at 0)."""
    frames = synth.workload("shapes256")
    kw = dict(seed=3, blob_delimiter=0, motion=capi.LINEAR, fading=capi.LINEAR)
    a = _chains(capi, frames, **kw)
    b = capi.Morph()
    b.load(frames, **kw)
    b.import_chains(*a.export_chains())
    c0 = a.cost()
    assert b.cost() == c0
    a.tune(guided_switch=0)
    b.tune(guided_switch=0, learned_keep=1.0)
    b.proposal_weights(_rand_params(9))
    g_local = a.refine(12, capi.PROPOSAL_LOCAL)
    g_learned = b.refine(12, capi.PROPOSAL_LEARNED)
    assert np.array_equal(g_local, g_learned)
    assert np.array_equal(a.export_chains()[1], b.export_chains()[1])
    assert b.cost() == c0 - int(g_learned.sum())


def test_learned_proposal_end_to_end(capi, oracle):
    """Record the full scan's outcomes, train on the GPU, refine with the
    gate: exact invariants hold, and at the same scan budget (a quarter of the
    columns) the trained gate gains more than an untrained one."""
    frames = synth.workload("shapes256")
    m = _chains(capi, frames, seed=3, blob_delimiter=0, motion=capi.LINEAR, fading=capi.LINEAR)
    m.tune(guided_switch=0)  # guided from the first sweep: every sweep records
    w, pts0, order = m.export_chains()
    K = len(frames)
    c0 = m.cost()
    m.record_swaps(1 << 20)
    gains = m.refine(20, capi.PROPOSAL_LEARNED)
    feats, targets = m.recorded_swaps(1 << 20)
    assert len(targets) > 20000  # one sample per 32-slot region and phase
    assert np.isfinite(feats).all() and np.isfinite(targets).all() and (targets >= 0).all()
    assert m.cost() == c0 - int(gains.sum())
    untrained = m.proposal_weights()
    perm = np.random.default_rng(0).permutation(len(targets))
    loss = m.train_proposal(feats[perm], targets[perm], epochs=6, lr=2e-3)
    assert np.isfinite(loss)
    trained = m.proposal_weights()
    m.proposal_weights(untrained)
    pred_u = m.proposal_forward(feats[:20000])
    m.proposal_weights(trained)
    pred_t = m.proposal_forward(feats[:20000])
    mse_u = float(np.mean((pred_u - targets[:20000]) ** 2))
    mse_t = float(np.mean((pred_t - targets[:20000]) ** 2))
    print("gate regression mse untrained %.4f trained %.4f" % (mse_u, mse_t))
    assert mse_t < 0.5 * mse_u
    sweeps = 20
    results = {}
    for name, wts in (("untrained", untrained), ("trained", trained)):
        # a fresh twin per arm: same frames, seed, chains and sweep counter,
        # so both arms draw the same random candidates
        t = capi.Morph()
        t.load(frames, seed=3, blob_delimiter=0, motion=capi.LINEAR, fading=capi.LINEAR)
        t.import_chains(w, pts0, order)
        t.tune(guided_switch=0, learned_keep=0.25, learned_adaptive=0)
        t.proposal_weights(wts)
        g = t.refine(sweeps, capi.PROPOSAL_LEARNED)
        results[name] = t.cost()
        assert results[name] == c0 - int(g.sum())
        _, pts, _ = t.export_chains()
        assert oracle.energy(pts, w, K)[1] == results[name]
        t.close()
    print("cost after %d gated sweeps (keep 1/4):" % sweeps, results, "start", c0)
    assert results["trained"] < results["untrained"], results


def test_train_recorded_trains_on_device_samples(capi):
    """am_train_recorded trains on the sample log where the recording sweeps
    left it: the regression error on the recorded samples falls as with
    am_train_proposal on the same samples copied through the host, and
    without a recording it reports AM_ERR_STATE."""
    import ctypes as C
    frames = synth.workload("shapes256")
    m = _chains(capi, frames, seed=3, blob_delimiter=0, motion=capi.LINEAR, fading=capi.LINEAR)
    loss = C.c_float()
    assert m.lib.am_train_recorded(m.h, 2, 2e-3, C.byref(loss)) == capi.AM_ERR_STATE
    m.tune(guided_switch=0)
    m.record_swaps(1 << 20)
    m.refine(20, capi.PROPOSAL_LEARNED)
    feats, targets = m.recorded_swaps(1 << 20)
    untrained = m.proposal_weights()
    pred_u = m.proposal_forward(feats[:20000])
    l_dev = m.train_recorded(epochs=6, lr=2e-3)
    assert np.isfinite(l_dev)
    pred_t = m.proposal_forward(feats[:20000])
    mse_u = float(np.mean((pred_u - targets[:20000]) ** 2))
    mse_t = float(np.mean((pred_t - targets[:20000]) ** 2))
    assert mse_t < 0.5 * mse_u
    # the same samples through the host, from the same starting weights
    h = _chains(capi, frames, seed=3, blob_delimiter=0, motion=capi.LINEAR, fading=capi.LINEAR)
    h.proposal_weights(untrained)
    l_host = h.train_proposal(feats, targets, epochs=6, lr=2e-3)
    assert abs(l_host - l_dev) <= 0.05 * max(l_host, l_dev) + 1e-3
