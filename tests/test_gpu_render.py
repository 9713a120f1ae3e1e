"""Frame render parity: the CUDA renderer against frames the reference itself
rendered (tests/golden) and against the oracle on larger seeded cases, from
identical atom positions.  Tolerance: at most 1 LSB per channel (the CUDA
path rounds exact rational weighted means where the reference rounds a
double sum; they can differ only at exact .5 ties, and FP32 colour fades can
move a value across a rounding boundary by one)."""
import numpy as np
import pytest

from atomorph_gb300 import synth
from conftest import golden, golden_state, morph_from_golden

pytestmark = pytest.mark.gpu


def _lsb(a, b):
    d = np.abs(a.astype(np.int32) - b.astype(np.int32))
    return int(d.max()), int((d > 0).sum())


@pytest.mark.parametrize("case", ["ellipses64", "spline48"])
def test_render_matches_reference_frames(capi, case):
    g = golden(case)
    m = morph_from_golden(capi, g)
    for t, ref in zip(g["ts"], g["renders"]):
        got = m.render(float(t))
        worst, ndiff = _lsb(got, ref)
        assert worst <= 1, f"t={t}: {ndiff} channels differ, worst {worst}"
        # COSINE fading at local time 0.5 puts every fading atom exactly on a
        # rounding tie (the ramp is cos(pi/2): +6e-17 in FP64, -4e-8 in FP32),
        # so odd colour sums may round the other way there; elsewhere the
        # frames agree except for rare ties.
        tie_frame = int(g["fading"]) == 5 and abs(float(t) * int(g["K"]) % 1 - 0.5) < 1e-9
        assert ndiff <= (ref.size // 20 if tie_frame else max(4, ref.size // 500)), f"t={t}: {ndiff} differ"


@pytest.mark.parametrize("motion,fading,delimiter,density", [
    (3, 6, 1, 1),   # LINEAR, PERLIN, HSP
    (4, 5, 0, 1),   # SPLINE, COSINE, RGB
    (4, 6, 1, 2),   # SPLINE, PERLIN, density 2
    (2, 3, 0, 1),   # NONE, LINEAR
])
def test_render_matches_oracle_on_gpu_built_chains(capi, oracle, motion, fading, delimiter, density):
    frames = synth.workload("shapes256")
    m = capi.Morph()
    m.load(frames, seed=11, blob_delimiter=delimiter, motion=motion, fading=fading, density=density)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    m.refine(20)
    w, pts, order = m.export_chains()
    from oracle.oracle import stored_frames
    colors, present = stored_frames(frames, delimiter, oracle)
    st = dict(K=len(frames), width=m.width, height=m.height, bbox=_bbox(frames), seed=11, motion=motion,
              fading=fading, delimiter=delimiter, density=density, colors=colors, present=present, widths=w,
              pts=pts, blob_order=order, frame_keys=np.arange(len(frames), dtype=np.uint64))
    for t in (0.0, 0.13, 0.5, 0.77, 0.96):
        ref = oracle.render(st, t)
        got = m.render(t)
        worst, ndiff = _lsb(got, ref)
        assert worst <= 1, f"t={t}: worst {worst}, {ndiff} channels differ"
        assert ndiff <= ref.size // 200


def _bbox(frames):
    xs, ys = [], []
    for f in frames:
        y, x = np.nonzero(f[..., 3])
        xs += [x.min(), x.max()]
        ys += [y.min(), y.max()]
    return np.array([min(xs), min(ys), max(xs), max(ys)], np.uint32)


def test_render_before_chains_shows_key_frame(capi):
    frames = synth.workload("ellipses64")
    m = capi.Morph()
    m.load(frames, blob_delimiter=0)
    m.run_until(capi.STATE_BLOB_MATCHING)
    got = m.render(0.0)
    exp = np.where(frames[0][..., 3:4] > 0, frames[0], 0)
    assert np.array_equal(got, exp)


def test_render_device_output_matches_host(capi):
    torch = pytest.importorskip("torch")
    g = golden("ellipses64")
    m = morph_from_golden(capi, g)
    buf = torch.zeros((m.height, m.width, 4), dtype=torch.uint8, device="cuda")
    for t in (0.2, 0.6):
        m.render_device(t, buf.data_ptr())
        assert m.lib.am_device_sync(m.h) == capi.AM_OK  # device frames are left in flight
        assert np.array_equal(buf.cpu().numpy(), m.render(t))


@pytest.mark.parametrize("pipeline", [1, 0])
def test_back_to_back_device_frames_match_host(capi, pipeline):
    """Device frames are left in flight, and (render_pipeline 1, the default)
    a frame's binning runs beside the previous frame's resolve over two
    record slots: 43 frames issued without a sync (crossing every key-frame
    pair, repeating times, in a scrambled order) must equal the same frames
    rendered one at a time."""
    torch = pytest.importorskip("torch")
    g = golden("spline48")
    m = morph_from_golden(capi, g)
    m.tune(render_pipeline=pipeline)
    ts = [((i * 7) % 40) / 40.0 for i in range(40)] + [0.5, 0.5, 0.0]
    want = [m.render(t) for t in ts]
    buf = torch.zeros((len(ts), m.height, m.width, 4), dtype=torch.uint8, device="cuda")
    for _ in range(2):
        for i, t in enumerate(ts):
            m.render_device(t, buf[i].data_ptr())
        assert m.lib.am_device_sync(m.h) == capi.AM_OK
        got = buf.cpu().numpy()
        for i, t in enumerate(ts):
            assert np.array_equal(got[i], want[i]), (i, t)


def test_interleaved_host_and_device_frames(capi):
    """Host frames (waited for) and device frames (left in flight) share the
    pipelined record slots: alternating them, with device frames still in
    flight when a host frame is rendered, changes no frame."""
    torch = pytest.importorskip("torch")
    g = golden("spline48")
    m = morph_from_golden(capi, g)
    ts = [((i * 11) % 24) / 24.0 for i in range(24)]
    want = {t: m.render(t) for t in ts}
    buf = torch.zeros((len(ts), m.height, m.width, 4), dtype=torch.uint8, device="cuda")
    host = {}
    for i, t in enumerate(ts):
        m.render_device(t, buf[i].data_ptr())
        if i % 3 == 2:
            u = ts[(i * 5) % len(ts)]
            host[(i, u)] = m.render(u)
    assert m.lib.am_device_sync(m.h) == capi.AM_OK
    got = buf.cpu().numpy()
    for i, t in enumerate(ts):
        assert np.array_equal(got[i], want[t]), (i, t)
    for (i, u), frame in host.items():
        assert np.array_equal(frame, want[u]), (i, u)


def test_device_frames_across_render_paths_match_host(capi):
    """Frames in flight while the resolution switches between the fused,
    pipelined binning (at most 2048 tiles) and the separate-kernel path
    (1600 x 1500: 2350 tiles) and back."""
    torch = pytest.importorskip("torch")
    g = golden("spline48")
    m = morph_from_golden(capi, g)
    small = (m.width, m.height)
    ts = [0.1, 0.6, 0.35, 0.85]
    plan = [small, (1600, 1500), small, (1600, 1500)]
    want, bufs = [], []
    for res in plan:
        m.set(resolution=res)
        want.append([m.render(t) for t in ts])
    for res in plan:
        m.set(resolution=res)
        b = torch.zeros((len(ts), res[1], res[0], 4), dtype=torch.uint8, device="cuda")
        for i, t in enumerate(ts):
            m.render_device(t, b[i].data_ptr())
        bufs.append(b)
    assert m.lib.am_device_sync(m.h) == capi.AM_OK
    for k, b in enumerate(bufs):
        got = b.cpu().numpy()
        for i, t in enumerate(ts):
            assert np.array_equal(got[i], want[k][i]), (plan[k], t)


def test_render_many_matches_single_frames(capi):
    """am_render_many_host into a pinned buffer covering all frames (stored by
    the GPU directly, pipelined) and into pageable memory (copied frame by
    frame), and am_render_many into device memory: every frame equals the
    single am_render frame."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    g = golden("spline48")
    m = morph_from_golden(capi, g)
    ts = np.array([((i * 7) % 30) / 30.0 for i in range(30)], np.float64)
    want = np.stack([m.render(float(t)) for t in ts])
    tp = ts.ctypes.data_as(C.POINTER(C.c_double))
    pinned = torch.full((len(ts), m.height, m.width, 4), 0x5A, dtype=torch.uint8).pin_memory()
    assert m.lib.am_render_many_host(m.h, tp, len(ts), pinned.data_ptr()) == capi.AM_OK
    assert np.array_equal(pinned.numpy(), want)
    pageable = np.zeros_like(want)
    assert m.lib.am_render_many_host(m.h, tp, len(ts), pageable.ctypes.data) == capi.AM_OK
    assert np.array_equal(pageable, want)
    # am_render_many: the same frames into device memory, left in flight
    dev = torch.zeros((len(ts), m.height, m.width, 4), dtype=torch.uint8, device="cuda")
    assert m.lib.am_render_many(m.h, tp, len(ts), dev.data_ptr()) == capi.AM_OK
    assert m.lib.am_device_sync(m.h) == capi.AM_OK
    assert np.array_equal(dev.cpu().numpy(), want)


def test_render_into_pinned_host_memory_matches_pageable(capi):
    """Pinned host buffers are mapped into the GPU's address space and the
    resolve kernel stores the frame there directly; the frame must equal the
    one copied into pageable memory, also at an offset inside a larger
    pinned allocation and with the buffer dirty beforehand."""
    torch = pytest.importorskip("torch")
    g = golden("spline48")
    m = morph_from_golden(capi, g)
    fb = m.height * m.width * 4
    pinned = torch.full((3 * fb,), 0xAB, dtype=torch.uint8).pin_memory()
    for t in (0.1, 0.45, 0.8):
        want = m.render(t)
        for off in (0, fb, 2 * fb):
            assert m.lib.am_render(m.h, t, pinned.data_ptr() + off, 0) == capi.AM_OK
            got = pinned[off:off + fb].numpy().reshape(m.height, m.width, 4)
            assert np.array_equal(got, want), (t, off)


@pytest.mark.parametrize("resolution", [(1600, 1500), (300, 200), (302, 199)])
def test_render_other_resolutions_match_oracle(capi, oracle, resolution):
    """Outputs above 2048 tiles of 32x32 px take the separate splat / scan /
    scatter kernels instead of the fused binning; an output smaller than the
    key frames drops the atoms outside it.  Same parity bar."""
    frames = synth.workload("shapes256")
    m = capi.Morph()
    m.load(frames, seed=3, blob_delimiter=1, motion=4, fading=6)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    m.refine(20)
    m.set(resolution=resolution)
    assert (m.width, m.height) == resolution
    w, pts, order = m.export_chains()
    from oracle.oracle import stored_frames
    colors, present = stored_frames(frames, 1, oracle)
    st = dict(K=len(frames), width=m.width, height=m.height, bbox=_bbox(frames), seed=3, motion=4, fading=6,
              delimiter=1, density=1, colors=colors, present=present, widths=w, pts=pts, blob_order=order,
              frame_keys=np.arange(len(frames), dtype=np.uint64))
    for t in (0.1, 0.45, 0.8):
        ref = oracle.render(st, t)
        got = m.render(t)
        worst, ndiff = _lsb(got, ref)
        assert worst <= 1, f"t={t}: worst {worst}, {ndiff} channels differ"
        assert ndiff <= max(16, ref.size // 200)


@pytest.mark.parametrize("offset", [4, 8, 12, 16])
def test_device_frames_at_unaligned_offsets(capi, offset):
    """Device destinations that start off a 16-byte boundary, in a frame whose
    width and height are no multiples of 4 or of the 32-pixel tile (302 x 199)
    and in a square one: the same pixels as the host frame, and nothing
    written outside the destination."""
    torch = pytest.importorskip("torch")
    frames = synth.workload("shapes256")
    m = capi.Morph()
    m.load(frames, seed=3, blob_delimiter=1, motion=4, fading=6)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    m.refine(20)
    for res in ((302, 199), (256, 256)):
        m.set(resolution=res)
        fb = m.width * m.height * 4
        buf = torch.zeros(offset + fb + 64, dtype=torch.uint8, device="cuda")
        for t in (0.2, 0.7):
            want = m.render(t)
            m.render_device(t, buf.data_ptr() + offset)
            assert m.lib.am_device_sync(m.h) == capi.AM_OK
            got = buf.cpu().numpy()
            assert not got[:offset].any() and not got[offset + fb:].any(), (res, t)
            assert np.array_equal(got[offset:offset + fb].reshape(m.height, m.width, 4), want), (res, t)


@pytest.mark.parametrize("motion", [2, 3, 4])
def test_render_perlin_step_ramp_matches_oracle(capi, oracle, motion):
    """PERLIN fading where an atom's octave noise falls below -1.2: the
    reference's ramp width s = (slope + 0.1) / 1.1 is then <= 0 and its colour
    weight steps from 0 to 1 at l (morph.cpp:1467-1479).  This seeded case
    (4 ellipses, HSP blobs) has such atoms in the second key-frame pair."""
    frames = synth.workload("ellipses64")
    m = capi.Morph()
    m.load(frames, seed=7, blob_delimiter=capi.HSP, motion=motion, fading=capi.PERLIN)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    m.refine(50)
    w, pts, order = m.export_chains()
    from oracle.oracle import stored_frames
    colors, present = stored_frames(frames, capi.HSP, oracle)
    bbox = _bbox(frames)
    # the case does exercise the step: some frame-1 atom has slope < -0.1
    P = pts.reshape(2, -1)
    x = (P & np.uint64(0xFFFF)).astype(np.float64) + ((P >> np.uint64(32)) & np.uint64(0xFF)) / 256.0
    y = ((P >> np.uint64(16)) & np.uint64(0xFFFF)).astype(np.float64) + ((P >> np.uint64(40)) & np.uint64(0xFF)) / 256.0
    bw, bh = bbox[2] - bbox[0] + 1.0, bbox[3] - bbox[1] + 1.0
    px, py = (x[1] - bbox[0]) / bw * 8.0, (y[1] - bbox[1]) / bh * 8.0
    slopes = [oracle.octave_noise(8, a, b) * 0.5 + 0.5 for a, b in zip(px, py)]
    assert min(slopes) < -0.1
    st = dict(K=2, width=m.width, height=m.height, bbox=bbox, seed=7, motion=motion, fading=capi.PERLIN,
              delimiter=capi.HSP, density=1, colors=colors, present=present, widths=w, pts=pts, blob_order=order,
              frame_keys=np.arange(2, dtype=np.uint64))
    for t in (0.3, 0.55, 0.7, 0.9):
        ref = oracle.render(st, t)
        got = m.render(t)
        worst, ndiff = _lsb(got, ref)
        assert worst <= 1, f"t={t}: worst {worst}, {ndiff} channels differ"


def test_render_independent_of_frame_order(capi):
    """Tile regions are planned from the previous frame's counts; records past
    a region's capacity take the overflow list.  Frames rendered in a shuffled
    order (large jumps, so regions misfit and overflow) equal the same frames
    rendered in time order."""
    frames = synth.workload("shapes256")
    m = capi.Morph()
    m.load(frames, seed=2, blob_delimiter=1, motion=capi.SPLINE, fading=capi.PERLIN)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    m.refine(10)
    ts = [i / 16 for i in range(16)]
    forward = {t: m.render(t) for t in ts}
    order = np.random.default_rng(4).permutation(len(ts))
    for k in order:
        t = ts[k]
        assert np.array_equal(m.render(t), forward[t]), t
    m.close()
