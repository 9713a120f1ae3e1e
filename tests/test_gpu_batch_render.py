"""Batched frames (am_batch_render): the atom frames of many jobs of uneven
size, canvas and render settings rendered by one binning, one resolve and one
tile-plan launch per time equal each job's own am_render at that time, byte
for byte, into pageable host, pinned host and device memory; more than 32
jobs take several launches; a fluid job in the batch renders through its own
path; jobs render on their own identically before and after batch calls."""
import numpy as np
import pytest

from atomorph_gb300 import synth

pytestmark = pytest.mark.gpu

TS = [0.0, 0.06, 0.31, 0.5, 0.74, 0.999]


def _job(capi, j, **settings):
    m = capi.Morph()
    m.load(synth.workload("batch", j), seed=j + 1, blob_delimiter=0, **settings)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    return m


@pytest.fixture(scope="module")
def jobs(capi):
    out = [
        _job(capi, 0, motion=capi.SPLINE),
        _job(capi, 1, motion=capi.LINEAR),
        _job(capi, 2, motion=capi.SPLINE),
        _job(capi, 3, motion=capi.SPLINE, fading=capi.COSINE),
        _job(capi, 4, motion=capi.SPLINE),
        _job(capi, 5, motion=capi.SPLINE),
    ]
    out[0].set(motion_noise=2.0)
    out[2].set(feather=3)
    out[3].set(keep_background=1)
    out[4].set(show_blobs=1)  # AM_AVERAGE
    for m in out:
        m.refine(20, capi.PROPOSAL_RANDOM)
    yield out
    for m in out:
        m.close()


def _own(jobs, ts):
    return [np.stack([m.render(t) for t in ts]) for m in jobs]


def test_batched_frames_equal_each_jobs_own(capi, jobs):
    sizes = sorted({(m.width, m.height) for m in jobs})
    print("jobs: atoms", [m.atoms for m in jobs], "canvases", sizes)
    assert len(sizes) > 1
    batch = capi.Batch(jobs)
    want = _own(jobs, TS)
    got = batch.render(TS)
    for j, (g, w) in enumerate(zip(got, want)):
        assert g.shape == w.shape
        for i, t in enumerate(TS):
            assert np.array_equal(g[i], w[i]), (j, t)
        assert w[:, :, :, 3].any(), j
    # the jobs' own frames after the batch: unchanged, and again batched
    assert all(np.array_equal(a, b) for a, b in zip(_own(jobs, TS[::-1]), [w[::-1] for w in want]))
    again = batch.render(TS[::-1])
    assert all(np.array_equal(a, b[::-1]) for a, b in zip(again, want))
    batch.close()


def test_batched_frames_into_device_and_pinned_memory(capi, jobs):
    torch = pytest.importorskip("torch")
    batch = capi.Batch(jobs)
    want = _own(jobs, TS)
    dev = [torch.zeros((len(TS), m.height, m.width, 4), dtype=torch.uint8, device="cuda") for m in jobs]
    batch.render_device(TS, [d.data_ptr() for d in dev])
    for j, d in enumerate(dev):
        assert np.array_equal(d.cpu().numpy(), want[j]), j
    pinned = [torch.zeros((len(TS), m.height, m.width, 4), dtype=torch.uint8).pin_memory() for m in jobs]
    import ctypes as C
    ts = np.asarray(TS, np.float64)
    arr = (C.c_void_p * len(jobs))(*[p.data_ptr() for p in pinned])
    rc = batch.lib.am_batch_render(batch.h, ts.ctypes.data_as(C.POINTER(C.c_double)), len(TS), arr, 0)
    assert rc == capi.AM_OK
    for j, p in enumerate(pinned):
        assert np.array_equal(p.numpy(), want[j]), j
    batch.close()


def test_more_than_32_jobs_and_a_fluid_job(capi):
    rng = np.random.default_rng(5)
    ms = []
    for j in range(35):
        frames = [synth.ellipses_frame(48, 3, 4.0, 10.0, rng) for _ in range(2 + j % 3)]
        m = capi.Morph()
        m.load(frames, seed=j + 3)
        assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
        ms.append(m)
    ts = [0.1, 0.55, 0.9]
    want = _own(ms[1:], ts)
    ms[0].set(fluid=2)
    batch = capi.Batch(ms)
    got = batch.render(ts)
    for j in range(1, len(ms)):
        assert np.array_equal(got[j], want[j - 1]), j
    assert got[0][..., 3].any()  # the fluid job's particles
    batch.close()
    for m in ms:
        m.close()


def test_batch_rejects_a_job_twice(capi, jobs):
    import ctypes as C
    lib = jobs[0].lib
    arr = (C.c_void_p * 2)(jobs[0].h, jobs[0].h)
    h = C.c_void_p()
    assert lib.am_batch_create(C.byref(h), arr, 2) == capi.AM_ERR_ARG and not h.value


def test_batch_workload_frames_repeatably_equal(capi):
    """The benchmark's batch workload (32 jobs of 2k-200k atoms, 3-8 key
    frames, 16 frames each at t = i/16: large jumps, so tile regions planned
    from the previous frame overflow often): job-by-job device frames and
    batched frames agree over repeated rounds."""
    torch = pytest.importorskip("torch")
    solo, twin = [], []
    for j in range(32):
        frames = synth.workload("batch", j)
        a = capi.Morph()
        a.load(frames, seed=j + 1, blob_delimiter=0, motion=capi.SPLINE)
        assert a.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
        a.refine(20, capi.PROPOSAL_RANDOM)
        b = capi.Morph()
        b.load(frames, seed=j + 1, blob_delimiter=0, motion=capi.SPLINE)
        b.import_chains(*a.export_chains())
        solo.append(a)
        twin.append(b)
    ts = [i / 16 for i in range(16)]
    ds = [torch.empty((16, a.height, a.width, 4), dtype=torch.uint8, device="cuda") for a in solo]
    dt = [torch.empty_like(d) for d in ds]
    batch = capi.Batch(twin)
    for rep in range(5):
        for a, d in zip(solo, ds):
            for i, t in enumerate(ts):
                a.render_device(t, d.data_ptr() + i * a.width * a.height * 4)
        torch.cuda.synchronize()
        batch.render_device(ts, [d.data_ptr() for d in dt])
        for j in range(32):
            assert torch.equal(ds[j], dt[j]), (rep, j)
    batch.close()
    for m in solo + twin:
        m.close()
