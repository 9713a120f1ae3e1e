"""The rest of the drop-in boundary: morph::get_pixels(blob, t, to)
(morph.h:29, morph.cpp:452-678) and morph::get_blob (morph.h:40) through the
C ABI and through the C++ class am::morph.

* The GPU's per-blob pixel lists equal the reference's own (tests/golden/
  blob_pixels.npz, made by the unmodified reference) pixel for pixel and in
  order, colours within 1 LSB, with feather 0 and 3.
* Before chains exist a blob's list is its own key-frame pixels.
* A repo-authored C++ program written against include/atomorph_gb300.hpp
  (tests/cpp/morph_roundtrip.cpp) ingests key frames with add_pixel, steps
  the pipeline as the reference's demo does, and reads whole frames and
  every blob's list; frames within 1 LSB of the oracle's render of the chains
  it exported, blob lists equal to the oracle's."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from atomorph_gb300 import synth
from conftest import ROOT, golden, golden_state, morph_from_golden
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def test_blob_pixels_match_reference(capi):
    g = golden("features")
    z = golden("blob_pixels")
    m = morph_from_golden(capi, g)
    checked = 0
    for feather in (0, 3):
        m.set(feather=feather)
        for fe, ti, b, off, n in z["index"]:
            if fe != feather:
                continue
            t = float(z["ts"][ti])
            xy, rgba = m.blob_pixels(int(b), t)
            assert np.array_equal(xy, z["xy"][off:off + n]), (feather, t, b)
            assert int(np.abs(rgba.astype(np.int32) - z["rgba"][off:off + n]).max(initial=0)) <= 1, (feather, t, b)
            checked += 1
    assert checked == len(z["index"])
    # a blob the key frame does not have
    import ctypes as C
    cnt = C.c_size_t()
    nb = m.blob_count(0)
    assert m.lib.am_get_blob_pixels(m.h, nb, 0.05, None, None, 0, C.byref(cnt)) == capi.AM_ERR_NOT_FOUND
    m.close()


def test_blob_pixels_before_chains_are_the_key_frame_pixels(capi, oracle):
    frames = synth.workload("ellipses64")
    m = capi.Morph()
    m.load(frames, seed=7)
    assert m.run_until(capi.STATE_BLOB_MATCHING) == capi.STATE_BLOB_MATCHING
    colors, present = orc.stored_frames(frames, capi.HSP, oracle)
    lab = m.blob_labels(0)
    for b in range(m.blob_count(0)):
        xy, rgba = m.blob_pixels(b, 0.0)
        ys, xs = np.nonzero(lab == b)
        assert np.array_equal(xy[:, 0], xs) and np.array_equal(xy[:, 1], ys)  # ascending position order
        # get_pixel reads the stored HSP colour back as RGB (morph.cpp:378-392)
        want = np.array([oracle.hsp_to_rgb(int(c)) for c in colors[0][ys, xs]], np.uint32).view(np.uint8).reshape(-1, 4)
        assert np.array_equal(rgba, want)
    m.close()


def test_blob_info_against_labels(capi):
    import ctypes as C
    g = golden("ellipses64")
    m = capi.Morph()
    m.load(list(g["frames"]), seed=int(g["seed"]), blob_delimiter=int(g["delimiter"]))
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    w, pts, order = m.export_chains()
    for k in range(2):
        lab = m.blob_labels(k)
        for b in range(m.blob_count(k)):
            grp, sz = C.c_size_t(), C.c_size_t()
            v = np.zeros(6)
            assert m.lib.am_get_blob_info(m.h, k, b, C.byref(grp), C.byref(sz), v.ctypes.data_as(C.POINTER(C.c_double))) == 0
            assert sz.value == int((lab == b).sum())
            assert grp.value == order[k][b]
            if sz.value:
                ys, xs = np.nonzero(lab == b)
                assert abs(v[0] - xs.mean()) < 1e-9 and abs(v[1] - ys.mean()) < 1e-9
    m.close()


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not present")
def test_cpp_program_against_the_header(capi, oracle, tmp_path):
    lib = os.path.join(ROOT, "atomorph_gb300", "lib", "libatomorph_gb300.so")
    exe = tmp_path / "morph_roundtrip"
    subprocess.run(["g++", "-std=c++11", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "morph_roundtrip.cpp"), "-L", os.path.dirname(lib),
                    "-latomorph_gb300", "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)], check=True)
    rng = np.random.default_rng(31)
    frames = [synth.ellipses_frame(48, 4, 4.0, 12.0, rng) for _ in range(3)]
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        np.array([3, 48, 48], np.uint32).tofile(f)
        np.stack(frames).tofile(f)
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([str(exe), str(inp), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    raw = open(out / "chains.bin", "rb").read()
    K, Cn, N = np.frombuffer(raw[:24], np.uint64).astype(int)
    o = 24
    widths = np.frombuffer(raw[o:o + 8 * Cn], np.uint64); o += 8 * Cn
    pts = np.frombuffer(raw[o:o + 8 * K * N], np.uint64); o += 8 * K * N
    order = np.frombuffer(raw[o:o + 4 * K * Cn], np.int32).reshape(K, Cn)
    assert K == 3 and int(widths.sum()) == N
    colors, present = orc.stored_frames(frames, capi.HSP, oracle)
    xs, ys = [], []
    for fr in frames:
        y, x = np.nonzero(fr[..., 3])
        xs += [x.min(), x.max()]
        ys += [y.min(), y.max()]
    st = dict(K=3, width=48, height=48, bbox=np.array([min(xs), min(ys), max(xs), max(ys)]), seed=7,
              motion=capi.SPLINE, fading=capi.PERLIN, delimiter=capi.HSP, density=1, colors=colors, present=present,
              widths=np.array(widths), pts=np.array(pts), blob_order=np.array(order),
              frame_keys=np.arange(3, dtype=np.uint64))
    assert oracle.energy(pts, widths, 3)[1] == float(open(out / "state.txt").read().split()[1])
    for i, t in enumerate((0.1, 0.45, 0.8)):
        got = np.fromfile(out / f"frame_{i}.bin", np.uint8).reshape(48, 48, 4).astype(np.int32)
        assert int(np.abs(got - oracle.render(st, t).astype(np.int32)).max()) <= 1, t
    data = open(out / "blobs.bin", "rb").read()
    nb = int(np.frombuffer(data[:8], np.uint64)[0])
    o = 8
    assert nb == Cn
    for b in range(nb):
        n = int(np.frombuffer(data[o:o + 8], np.uint64)[0]); o += 8
        xy = np.frombuffer(data[o:o + 4 * n], np.uint16).reshape(n, 2); o += 4 * n
        rgba = np.frombuffer(data[o:o + 4 * n], np.uint8).reshape(n, 4); o += 4 * n
        surface, group = np.frombuffer(data[o:o + 16], np.uint64); o += 16
        ref = oracle.blob_pixels(st, b, 0.45)
        assert np.array_equal(xy, ref[0]), b
        assert int(np.abs(rgba.astype(np.int32) - ref[1]).max(initial=0)) <= 1, b
        assert int(group) == int(order[1][b])
