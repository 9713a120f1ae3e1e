"""Perlin motion perturbation on the GPU (am_set_motion_noise; the reference
moves atoms along their paths only).  Positions equal the oracle's FP32
definition bit for bit and lie within 1/256 px of its FP64 form; frames
rendered with the perturbation match the oracle's within 1 LSB; the
displacement vanishes at key frames."""
import numpy as np
import pytest

from conftest import golden, golden_state, morph_from_golden

pytestmark = pytest.mark.gpu

# FP32 noise against the FP64 accuracy reference: at most one 1/256-px step
POS_TOL_FP64 = 1


@pytest.mark.parametrize("case,amp", [("spline48", 2.0), ("ellipses64", 2.0), ("spline48", 9.5)])
def test_positions_match_fp32_definition_and_fp64_reference(capi, oracle, case, amp):
    g = golden(case)
    m = morph_from_golden(capi, g)
    m.set(motion_noise=amp)
    st = dict(golden_state(g), motion_noise=amp)
    K = int(g["K"])
    worst, moved = 0, 0
    for t in (0.013, 0.21, 0.5 / K, 0.77, 0.999):
        got = m.positions(t)
        ref = oracle.positions(st, t)
        assert np.array_equal(got, ref), (t, int(np.abs(got.astype(np.int64) - ref).max()))
        r64 = oracle.positions(st, t, fp64=True)
        drawn = ref[:, 0] >= 0
        d = np.abs(ref[drawn].astype(np.int64) - r64[drawn])
        worst = max(worst, int(d.max()))
        base = oracle.positions(dict(st, motion_noise=0.0), t)
        moved += int((base[drawn] != ref[drawn]).any(axis=1).sum())
    print(f"{case} A={amp}: max |FP32 - FP64| = {worst} (1/256 px); {moved} displaced atom positions")
    assert worst <= POS_TOL_FP64
    assert moved > 0
    m.close()


def test_displacement_vanishes_at_key_frames(capi, oracle):
    g = golden("spline48")
    m = morph_from_golden(capi, g)
    K = int(g["K"])
    plain = [m.positions(k / K) for k in range(K)]
    m.set(motion_noise=6.0)
    for k in range(K):
        assert np.array_equal(m.positions(k / K), plain[k])
    m.close()


@pytest.mark.parametrize("case", ["spline48", "ellipses64", "features"])
def test_frames_with_motion_noise_match_oracle(capi, oracle, case):
    g = golden(case)
    m = morph_from_golden(capi, g)
    m.set(motion_noise=2.0)
    st = dict(golden_state(g), motion_noise=2.0)
    ts = [0.07, 0.33, 0.58, 0.91]
    ref = oracle.render_many(st, ts, threads=4)
    for i, t in enumerate(ts):
        got = m.render(t).astype(np.int32)
        worst = int(np.abs(got - ref[i].astype(np.int32)).max())
        assert worst <= 1, (case, t, worst)
    # turning it off gives the frames of the paths alone again
    m.set(motion_noise=0.0)
    plain = oracle.render(golden_state(g), 0.33).astype(np.int32)
    assert int(np.abs(m.render(0.33).astype(np.int32) - plain).max()) <= 1
    m.close()


def test_motion_noise_amplitude_is_checked(capi):
    m = capi.Morph()
    assert m.lib.am_set_motion_noise(m.h, -0.5) == capi.AM_ERR_ARG
    assert m.lib.am_set_motion_noise(m.h, 64.5) == capi.AM_ERR_ARG
    assert m.lib.am_set_motion_noise(m.h, 64.0) == capi.AM_OK
    assert m.lib.am_set_motion_noise(m.h, 0.0) == capi.AM_OK
    m.close()
