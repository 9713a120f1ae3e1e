"""The resolve's exactly rounded channel means (`round_div_by` / `round_div`
in atomorph_gb300/csrc/k_render.cu), restated step for step in numpy float32
arithmetic: an IEEE reciprocal of the weight, a fused multiply-add estimate
of num / den + 1/2, truncation, and one correction on the exact remainder.
For den < 2^24 and quotients below 256 (the packed resolve path: at most 258
contributions of weight <= 65025) the estimate is within 1 of
floor(num / den + 1/2), so the corrected quotient equals the reference's
round-half-away mean exactly, ties included.  CPU only; the GPU render
parity tests exercise the kernel itself."""
import numpy as np


def _exact(num, den):
    return (2 * num + den) // (2 * den)


def _device_formula(num, den):
    rcp = np.float32(1.0) / den.astype(np.float32)                      # __frcp_rn(__uint2float_rn(den))
    nf = num.astype(np.float32)                                           # __uint2float_rn(num)
    est = (nf.astype(np.float64) * rcp.astype(np.float64) + 0.5).astype(np.float32)  # __fmaf_rn(nf, rcp, 0.5f)
    q0 = np.floor(est.astype(np.float64)).astype(np.int64)                # __float2uint_rz
    r2 = 2 * (num - q0 * den)
    q = np.where(r2 < -den, q0 - 1, np.where(r2 >= den, q0 + 1, q0))
    return q, q0


def test_round_div_matches_exact_rounding():
    rng = np.random.default_rng(7)
    for trial in range(12):
        hi = (1 << 24) if trial % 3 else 65025 * 4
        den = rng.integers(1, hi, size=100_000, dtype=np.int64)
        q = rng.integers(0, 256, size=den.size)
        if trial % 2:
            # ties and their neighbours: num / den + 1/2 at or next to an integer
            num = q * den + den // 2 + rng.integers(-1, 2, size=den.size)
        else:
            num = q * den + rng.integers(0, den)
        num = np.clip(num, 0, (1 << 32) - 1)
        got, est = _device_formula(num, den)
        want = _exact(num, den)
        assert np.abs(est - want).max() <= 1
        assert np.array_equal(got, want)


def test_round_div_extremes():
    den = np.array([1, 2, 3, 65025, 258 * 65025, (1 << 24) - 1], dtype=np.int64)
    for q in (0, 1, 127, 254, 255):
        for off in (-1, 0, 1):
            num = np.clip(q * den + den // 2 + off, 0, (1 << 32) - 1)
            got, _ = _device_formula(num, den)
            assert np.array_equal(got, _exact(num, den)), (q, off)
