"""Host frames played in order (times get_time(i, n), as the reference's
demo writes them): am_render bins the expected next frame beside the
current frame's resolve, and the next call uses it when it asks for exactly
that time and scene.  Every host frame equals the device frame rendered on
its own at the same time (device frames never bin ahead), through
sequences, jumps, repeats, the cycle's wrap, finite timing, setting and
chain changes between calls, and pinned host memory."""
import numpy as np
import pytest

from atomorph_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def morph(capi):
    m = capi.Morph()
    m.load(synth.workload("shapes256"), seed=3, blob_delimiter=1, motion=capi.SPLINE, fading=capi.PERLIN)
    m.set(motion_noise=2.0)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    m.refine(30, capi.PROPOSAL_RANDOM)
    yield m
    m.close()


def device_frame(m, t):
    import torch
    d = torch.zeros((m.height, m.width, 4), dtype=torch.uint8, device="cuda")
    m.render_device(float(t), d.data_ptr())
    torch.cuda.synchronize()
    return d.cpu().numpy()


def check(m, order, n):
    ts = [m.get_time(i, n) for i in order]
    want = {t: device_frame(m, t) for t in set(ts)}
    for i, t in zip(order, ts):
        assert np.array_equal(m.render(t), want[t]), (i, n, t)


def test_sequences_jumps_repeats_and_wrap(morph):
    check(morph, list(range(24)), 24)
    check(morph, [0, 1, 2, 5, 6, 4, 5, 5, 6, 7, 3, 4], 16)
    check(morph, [5, 6, 7, 0, 1, 2, 7, 0], 8)  # the wrap: after 7/8 the next is 0


def test_finite_timing(morph):
    morph.set(finite=1)
    try:
        check(morph, list(range(12)), 12)
    finally:
        morph.set(finite=0)


def test_changes_between_calls(capi, morph):
    n = 20
    for i in range(4):
        morph.render(morph.get_time(i, n))
    # a setting changes after frame 3 bound frame 4 ahead
    morph.set(feather=2)
    t = morph.get_time(4, n)
    got = morph.render(t)
    assert np.array_equal(got, device_frame(morph, t))
    morph.render(morph.get_time(5, n))
    morph.set(feather=0)
    t = morph.get_time(6, n)
    assert np.array_equal(morph.render(t), device_frame(morph, t))
    # the chains change after frame 7 bound frame 8 ahead
    morph.render(morph.get_time(7, n))
    morph.refine(3, capi.PROPOSAL_RANDOM)
    t = morph.get_time(8, n)
    assert np.array_equal(morph.render(t), device_frame(morph, t))
    # a blob drawn alone and the positions readout between calls
    morph.render(morph.get_time(9, n))
    morph.blob_pixels(0, morph.get_time(10, n))
    morph.positions(morph.get_time(10, n))
    for i in (10, 11):
        t = morph.get_time(i, n)
        assert np.array_equal(morph.render(t), device_frame(morph, t))


def test_pinned_host_frames(capi, morph):
    import torch
    n = 16
    buf = torch.zeros((morph.height, morph.width, 4), dtype=torch.uint8).pin_memory()
    for i in range(n):
        t = morph.get_time(i, n)
        assert morph.lib.am_render(morph.h, t, buf.data_ptr(), 0) == capi.AM_OK
        assert np.array_equal(buf.numpy(), device_frame(morph, t)), i
