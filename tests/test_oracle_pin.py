"""Pins the C++ restatement (oracle/oracle.cpp) to the reference.

Every check is bit-exact: against fixtures the unmodified reference produced
(tests/golden, made by tests/golden/make_golden.py), and, where the reference
sources were built into oracle/_ref, against the reference run live on fresh
seeded inputs.
"""
import numpy as np
import pytest

from conftest import golden, golden_state
from oracle import oracle as orc


def test_hsp_matches_reference(oracle):
    g = golden("hsp")
    hsp = np.array([oracle.rgb_to_hsp(int(c)) for c in g["rgb"]], np.uint32)
    back = np.array([oracle.hsp_to_rgb(int(c)) for c in g["rgb"]], np.uint32)
    assert np.array_equal(hsp, g["hsp"])
    assert np.array_equal(back, g["back"])


def test_perlin_matches_reference(oracle):
    g = golden("perlin")
    for si, s in enumerate(g["seeds"]):
        got = np.array([oracle.octave_noise(int(s), x, y, 8) for x, y in g["xy"]])
        assert np.array_equal(got, g["noise"][si])


def test_spline_matches_reference(oracle):
    g = golden("spline")
    got = np.array([oracle.spline(g["pts"], t) for t in g["ts"]])
    assert np.array_equal(got, g["values"])


@pytest.mark.parametrize("case", ["ellipses64", "spline48"])
def test_cost_and_sweeps_match_reference(oracle, case):
    g = golden(case)
    K = int(g["K"])
    e0, ex0 = oracle.energy(g["pts0"], g["widths"], K)
    assert e0 == g["energy0"] and ex0 == int(g["energy0"])
    swept = oracle.sweeps(g["pts0"], g["widths"], K, int(g["sweeps"]), int(g["sweep_seed"]))
    assert np.array_equal(swept, g["pts"])
    assert oracle.energy(swept, g["widths"], K)[0] == g["energy"]
    assert g["energy"] <= g["energy0"]


@pytest.mark.parametrize("case", ["ellipses64", "spline48"])
def test_render_matches_reference(oracle, case):
    g = golden(case)
    st = golden_state(g)
    for t, ref in zip(g["ts"], g["renders"]):
        assert np.array_equal(oracle.render(st, float(t)), ref), f"t={t}"


def test_fluid_step_matches_reference(oracle):
    g = golden("fluid")
    P = g["init"].copy()
    gsx, gsy = int(g["gsx"]), int(g["gsy"])
    grid = np.zeros(13 * gsx * gsy)
    touched = np.zeros(gsx * gsy, np.uint8)
    for s in range(8):
        oracle.fluid_step(P, gsx, gsy, grid, touched, 7 - s, float(g["freedom"]))
        if s == 0:
            assert np.array_equal(P, g["step1"])
    assert np.array_equal(P, g["step8"])


@pytest.mark.parametrize("case", ["ellipses64", "spline48"])
def test_components_give_reference_blob_counts(oracle, case):
    """With blob_threshold 1 and blob_number 1 the reference's greedy merge
    ends at the 4-connected components."""
    g = golden(case)
    for k, img in enumerate(g["frames"]):
        labels, stats = oracle.components(img)
        real = [int(s) for s in g["real_blob_sizes"][k] if s > 0]
        assert len(stats) == len(real)
        assert sorted(int(s) for s in stats[:, 0]) == sorted(real)
        assert int(stats[:, 0].sum()) == g["pixel_counts"][k]
        # after matching every frame holds as many blobs as the largest one
        assert g["blob_counts"][k] == max(len([s for s in row if s > 0]) for row in g["real_blob_sizes"])


@pytest.mark.skipif(not orc.have_reference(), reason="reference sources not built here")
def test_live_reference_pin(oracle):
    """Fresh seeded case, reference run live: chains, sweeps, cost, render."""
    from atomorph_gb300 import synth
    R = orc.Reference()
    r = np.random.default_rng(77)
    frames = [synth.ellipses_frame(56, 5, 3.0, 14.0, r) for _ in range(4)]
    for motion, fading, delim, dens in [(4, 6, 1, 1), (3, 5, 0, 2)]:
        R.new(frames, seed=5, motion=motion, fading=fading, delimiter=delim, density=dens)
        R.prepare()
        w, K = R.widths()
        p0 = R.points()
        R.sweeps(4, 31)
        assert np.array_equal(oracle.sweeps(p0, w, K, 4, 31), R.points())
        assert oracle.energy(R.points(), w, K)[0] == R.energy()
        st = R.state(5, motion, fading, delim, dens, frames)
        for t in (0.05, 0.3, 0.61, 0.9):
            assert np.array_equal(oracle.render(st, t), R.render(t))


def test_render_options_match_reference(oracle):
    """feather, keep_background and show_blobs AVERAGE / DISTINCT (morph.h:
    67-70): the oracle draws the reference's frames from the reference's
    chains and blob colours, bit-exact."""
    g = golden("features")
    st = golden_state(g)
    st["blob_avg"] = g["blob_avg"]
    for (feather, kb, sb), frames in zip(g["options"], g["renders"]):
        st.update(feather=int(feather), keep_background=int(kb), show_blobs=int(sb))
        for t, ref in zip(g["ts"], frames):
            assert np.array_equal(oracle.render(st, float(t)), ref), f"options {(feather, kb, sb)} t={t}"


@pytest.mark.skipif(not orc.have_reference(), reason="reference sources not built here")
def test_live_reference_pin_render_options(oracle):
    """Fresh seeded case with the render options, reference run live."""
    from atomorph_gb300 import synth
    R = orc.Reference()
    r = np.random.default_rng(91)
    frames = [synth.ellipses_frame(48, 4, 3.0, 12.0, r) for _ in range(3)]
    R.new(frames, seed=9, motion=3, fading=5, delimiter=0, density=1)
    R.prepare()
    R.sweeps(3, 7)
    for opts in [(2, 1, 0), (4, 0, 1), (0, 1, 2)]:
        R.options(*opts)
        st = R.state(9, 3, 5, 0, 1, frames)
        st.update(feather=opts[0], keep_background=opts[1], show_blobs=opts[2])
        for t in (0.2, 0.55, 0.85):
            assert np.array_equal(oracle.render(st, t), R.render(t)), (opts, t)


@pytest.mark.parametrize("name", ["empty_middle", "single", "mixed_sizes"])
def test_edge_inputs_render_like_reference(oracle, name):
    """An all-transparent key frame, one key frame, key frames of different
    sizes: the oracle draws the reference's frames from its chains."""
    from oracle.oracle import stored_frames
    g = golden("edges")
    frames = [f[:h, :w] for f, (h, w) in zip(g[f"{name}_frames"], g[f"{name}_sizes"])]
    colors, present = stored_frames(frames, 0, oracle)
    K = len(frames)
    H, W = g[f"{name}_frames"].shape[1:3]
    pts = [np.nonzero(f[..., 3]) for f in frames]
    bx = [int(p[1].min()) for p in pts if len(p[1])] + [int(p[1].max()) for p in pts if len(p[1])]
    by = [int(p[0].min()) for p in pts if len(p[0])] + [int(p[0].max()) for p in pts if len(p[0])]
    st = dict(K=K, width=W, height=H, bbox=np.array([min(bx), min(by), max(bx), max(by)], np.uint32), seed=4,
              motion=3, fading=6, delimiter=0, density=1, colors=colors, present=present,
              widths=g[f"{name}_widths"], pts=g[f"{name}_pts"], blob_order=g[f"{name}_blob_order"],
              frame_keys=np.arange(K, dtype=np.uint64))
    for t, ref in zip(g["ts"], g[f"{name}_renders"]):
        assert np.array_equal(oracle.render(st, float(t)), ref), f"{name} t={t}"
