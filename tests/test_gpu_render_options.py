"""Render options on the GPU (morph.h:67-70): feather, keep_background and
show_blobs AVERAGE / DISTINCT in the atom frame (morph.cpp:625-674,
1313-1399, 1431-1465) and feather / keep_background in the fluid draw
(morph.cpp:1187-1299), against the oracle (pinned to the reference by
test_oracle_pin.py) on the same chains and particles.

Tolerance: at most 1 LSB per channel.  The background's PERLIN cross-fade
and the atoms' colour fades run in FP32, the reference's in FP64; means and
feather scaling are exact."""
import ctypes as C

import numpy as np
import pytest

from atomorph_gb300 import synth

pytestmark = pytest.mark.gpu

OPTIONS = [(0, 0, 1), (0, 0, 2), (0, 1, 0), (3, 0, 0), (2, 1, 0), (1, 1, 1), (5, 0, 2), (40, 0, 0), (7, 1, 0)]


def _bbox(frames):
    xs, ys = [], []
    for f in frames:
        y, x = np.nonzero(f[..., 3])
        xs += [x.min(), x.max()]
        ys += [y.min(), y.max()]
    return np.array([min(xs), min(ys), max(xs), max(ys)], np.uint32)


def _blob_avg(m, K, Cn):
    """[K][C] colours am_get_blob_average reports (RGB; the stored colour for
    an RGB delimiter)."""
    out = np.zeros((K, Cn), np.uint32)
    xy = (C.c_uint16 * 2)()
    for k in range(K):
        for b in range(Cn):
            rgba = np.zeros(4, np.uint8)
            if m.lib.am_get_blob_average(m.h, k, b, xy, rgba.ctypes.data_as(C.POINTER(C.c_uint8))) == 0:
                out[k, b] = int(rgba.view(np.uint32)[0])
    return out


@pytest.mark.parametrize("delimiter", [0, 1])
def test_render_options_match_oracle(capi, oracle, delimiter):
    frames = synth.workload("shapes256")
    m = capi.Morph()
    m.load(frames, seed=11, blob_delimiter=delimiter, motion=capi.SPLINE, fading=capi.PERLIN)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    m.refine(30)
    w, pts, order = m.export_chains()
    from oracle.oracle import stored_frames
    colors, present = stored_frames(frames, delimiter, oracle)
    K = len(frames)
    st = dict(K=K, width=m.width, height=m.height, bbox=_bbox(frames), seed=11, motion=capi.SPLINE,
              fading=capi.PERLIN, delimiter=delimiter, density=1, colors=colors, present=present, widths=w, pts=pts,
              blob_order=order, frame_keys=np.arange(K, dtype=np.uint64), blob_avg=_blob_avg(m, K, len(w)))
    for feather, kb, sb in OPTIONS:
        if sb == 1 and delimiter == 1:
            continue  # the oracle takes stored (HSP) blob colours; the API reports RGB
        m.set(feather=feather, keep_background=kb, show_blobs=sb)
        st.update(feather=feather, keep_background=kb, show_blobs=sb)
        for t in (0.12, 0.5, 0.83):
            ref = oracle.render(st, t).astype(int)
            got = m.render(t).astype(int)
            d = np.abs(got - ref)
            assert d.max() <= 1, f"options {(feather, kb, sb)} t={t}: worst {d.max()}, {(d > 0).sum()} differ"
            assert (d > 0).sum() <= max(16, ref.size // 200), (feather, kb, sb, t, int((d > 0).sum()))
    m.close()


def test_render_rejects_feather_above_limit(capi):
    m = capi.Morph()
    assert m.lib.am_set_feather(m.h, 97) == capi.AM_ERR_UNSUPPORTED
    assert m.lib.am_set_feather(m.h, 96) == capi.AM_OK
    m.close()


@pytest.mark.parametrize("feather,with_bg", [(0, True), (3, False), (4, True)])
def test_fluid_draw_options_match_oracle(capi, oracle, feather, with_bg):
    rng = np.random.default_rng(5 + feather)
    width, height, sp, n = 120, 90, 1.0, 9000
    P = np.zeros((18, n))
    P[0] = rng.uniform(25, 95, n)
    P[1] = rng.uniform(20, 70, n)
    P[4], P[5] = P[0], P[1]
    P[6] = 1.0
    P[7] = rng.random(n) < 0.9
    P[8] = rng.random(n) < 0.5
    P[9] = rng.choice([0.1, 1.0], n)
    P[10:18] = rng.random((8, n))
    gsx, gsy = width + 20, height + 20
    f = capi.Fluid(gsx, gsy, n)
    f.set(P)
    P0 = f.get()
    bbox = [3, 2, width - 5, height - 4]
    bg = rng.integers(0, 256, (height, width, 4), dtype=np.uint8) if with_bg else None
    t = 0.9
    img = f.render_ex(width, height, sp, bbox, t, feather, bg)
    ref = oracle.draw_fluid(P0.copy(), width, height, sp, bbox, t, feather, bg)
    d = np.abs(img.astype(int) - ref.astype(int))
    print(f"fluid draw feather {feather} background {with_bg}: max diff {d.max()}, {(d > 0).sum()} differ")
    assert d.max() <= 1
    f.close()
