"""Batched refinement (am_batch_*): many jobs of uneven size in one persistent
launch give exactly what refining each job on its own gives, for plain and
for guided sweeps; the autotuners (launch shape, plain/guided schedule) leave
the chains untouched, and jobs continue identically afterwards."""
import numpy as np
import pytest

from atomorph_gb300 import synth

pytestmark = pytest.mark.gpu

JOBS = 6


def _job(capi, j):
    frames = synth.workload("batch", j)
    m = capi.Morph()
    m.load(frames, seed=j + 1, blob_delimiter=0, motion=capi.SPLINE)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    return m


@pytest.fixture(scope="module")
def pairs(capi):
    """Two identical handles per job: one refined alone, one in the batch
    (the twin gets the same key frames and seed, then the first's chains)."""
    out = []
    for j in range(JOBS):
        a = _job(capi, j)
        b = capi.Morph()
        b.load(synth.workload("batch", j), seed=j + 1, blob_delimiter=0, motion=capi.SPLINE)
        b.import_chains(*a.export_chains())
        assert b.cost() == a.cost()
        out.append((a, b))
    return out


def test_batch_equals_jobs_refined_one_by_one(capi, oracle, pairs):
    sizes = [a.atoms for a, _ in pairs]
    frames = [a.export_chains()[2].shape[0] for a, _ in pairs]
    print("batch jobs: atoms", sizes, "key frames", frames)
    assert max(sizes) > 4 * min(sizes)  # uneven sizes
    batch = capi.Batch([b for _, b in pairs])
    S = 30
    g_batch = batch.refine(S)
    for j, (a, b) in enumerate(pairs):
        g = a.refine(S, capi.PROPOSAL_RANDOM)
        assert np.array_equal(g, g_batch[j]), j
        wa, pa, oa = a.export_chains()
        wb, pb, ob = b.export_chains()
        assert np.array_equal(pa, pb) and np.array_equal(wa, wb), j
        assert a.cost() == b.cost()
        assert oracle.energy(pb, wb, ob.shape[0])[1] == b.cost()
    batch.close()


def test_autotuner_keeps_chains_and_results(capi, pairs):
    batch = capi.Batch([b for _, b in pairs])
    before = [b.export_chains()[1].copy() for _, b in pairs]
    costs = [b.cost() for _, b in pairs]
    t = batch.tune(2)
    print("tuned:", t)
    assert t["threads"] in (128, 256, 512) and t["chunk"] in (1024, 4096, 16384)
    for (a, b), p0, c0 in zip(pairs, before, costs):
        assert np.array_equal(b.export_chains()[1], p0) and b.cost() == c0
    g_batch = batch.refine(10)
    for j, (a, b) in enumerate(pairs):
        assert np.array_equal(a.refine(10, capi.PROPOSAL_RANDOM), g_batch[j])
        assert np.array_equal(a.export_chains()[1], b.export_chains()[1])
    # every launch shape and schedule gives the same result
    for shape in ((128, 1, 1024, 1), (512, 2, 16384, 0)):
        batch.set_tuning(*shape)
        g_batch = batch.refine(3)
        for j, (a, b) in enumerate(pairs):
            assert np.array_equal(a.refine(3, capi.PROPOSAL_RANDOM), g_batch[j]), (shape, j)
    # jobs continue identically on their own after batch calls
    for a, b in pairs:
        assert np.array_equal(a.refine(5, capi.PROPOSAL_RANDOM), b.refine(5, capi.PROPOSAL_RANDOM))
    batch.close()


def test_batched_guided_equals_jobs_refined_one_by_one(capi, oracle, pairs):
    """Guided sweeps of every job in one persistent launch (am_batch_refine_guided)
    equal each job's own guided sweeps bit for bit, and the jobs continue
    identically afterwards."""
    for a, b in pairs:
        a.tune(guided_switch=0)
        b.tune(guided_switch=0)
    batch = capi.Batch([b for _, b in pairs])
    for S in (12, 7):
        g_batch = batch.refine_guided(S)
        for j, (a, b) in enumerate(pairs):
            g = a.refine(S, capi.PROPOSAL_LOCAL)
            assert np.array_equal(g, g_batch[j]), (S, j)
            assert np.array_equal(a.export_chains()[1], b.export_chains()[1]), (S, j)
            assert a.cost() == b.cost()
    for a, b in pairs:
        w, pb, ob = b.export_chains()
        assert oracle.energy(pb, w, ob.shape[0])[1] == b.cost()
        assert np.array_equal(a.refine(4, capi.PROPOSAL_LOCAL), b.refine(4, capi.PROPOSAL_LOCAL))
    batch.close()


def test_schedule_tuner_and_tuned_schedule(capi, pairs):
    """The schedule autotuner picks a plain/guided split for a sweep budget
    and leaves the chains as they were; the tuned schedule equals the same
    split run job by job."""
    batch = capi.Batch([b for _, b in pairs])
    # one plain sweep on both sides: the guided indices are rebuilt from the
    # points at the next guided call, as after the tuner's trials
    g1 = batch.refine(1)
    for j, (a, b) in enumerate(pairs):
        assert np.array_equal(a.refine(1, capi.PROPOSAL_RANDOM), g1[j])
    before = [b.export_chains()[1].copy() for _, b in pairs]
    costs = [b.cost() for _, b in pairs]
    S = 64
    np_ = batch.tune_schedule(S)
    print("plain sweeps before the guided ones:", np_, "of", S)
    assert np_ in (0, S // 8, S // 4, S // 2)
    for (a, b), p0, c0 in zip(pairs, before, costs):
        assert np.array_equal(b.export_chains()[1], p0) and b.cost() == c0
    g_batch = batch.refine_schedule(S)
    for j, (a, b) in enumerate(pairs):
        g = np.concatenate([a.refine(np_, capi.PROPOSAL_RANDOM) if np_ else np.zeros(0, np.uint64),
                            a.refine(S - np_, capi.PROPOSAL_LOCAL)])
        assert np.array_equal(g, g_batch[j]), j
        assert np.array_equal(a.export_chains()[1], b.export_chains()[1]), j
    batch.close()


def test_batch_rejects_jobs_without_chains(capi):
    m = capi.Morph()
    with pytest.raises(capi.AmError):
        capi.Batch([m])
