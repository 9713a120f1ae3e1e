"""The motion perturbation's definition in the oracle (CPU): its FP32 noise
against the FP64 form within one 1/256-px step, zero displacement at key
frames, amplitude bounds, and no effect when off."""
import numpy as np
import pytest

from conftest import golden, golden_state


@pytest.mark.parametrize("case", ["spline48", "ellipses64", "features"])
def test_fp32_definition_within_one_step_of_fp64(oracle, case):
    g = golden(case)
    st = golden_state(g)
    for amp in (2.0, 9.5, 64.0):
        s = dict(st, motion_noise=amp)
        worst, differ, drawn_total = 0, 0, 0
        for t in np.linspace(0.0, 0.999, 23):
            a = oracle.positions(s, t)
            b = oracle.positions(s, t, fp64=True)
            drawn = a[:, 0] >= 0
            d = np.abs(a[drawn].astype(np.int64) - b[drawn])
            worst = max(worst, int(d.max()))
            differ += int((d > 0).sum())
            drawn_total += int(drawn.sum()) * 2
            # the displacement is bounded by the amplitude (noise |n| < 2)
            base = oracle.positions(dict(s, motion_noise=0.0), t)
            assert int(np.abs(a[drawn].astype(np.int64) - base[drawn]).max()) <= 2 * amp * 256 + 1
        assert worst <= 1, (case, amp, worst)
        assert differ <= 0.01 * drawn_total, (case, amp, differ, drawn_total)


def test_no_displacement_at_key_frames_or_when_off(oracle):
    g = golden("spline48")
    st = golden_state(g)
    K = int(g["K"])
    for k in range(K):
        assert np.array_equal(oracle.positions(dict(st, motion_noise=7.0), k / K), oracle.positions(st, k / K))
    for t in (0.1, 0.45, 0.8):
        assert not np.array_equal(oracle.positions(dict(st, motion_noise=7.0), t), oracle.positions(st, t))
        assert np.array_equal(oracle.positions(dict(st, motion_noise=0.0), t), oracle.positions(st, t))


def test_noise_render_is_the_displaced_splat(oracle):
    """With the perturbation on the render differs from the paths alone
    (inside the pair) and equals it at a key frame."""
    g = golden("ellipses64")
    st = golden_state(g)
    a = oracle.render(dict(st, motion_noise=3.0), 0.3)
    b = oracle.render(st, 0.3)
    assert (a != b).any()
    assert np.array_equal(oracle.render(dict(st, motion_noise=3.0), 0.0), oracle.render(st, 0.0))
