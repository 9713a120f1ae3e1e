"""Frames of key frames made of dust and of stacked atoms.

Dust: scattered opaque pixels, most of them isolated, so every key frame has
hundreds of one-pixel blobs and a 32 x 32 output tile is composited from
about a hundred blob ranks.  Stacks: a big blob matched to a one-pixel blob,
so at that key frame thousands of atoms lie on one pixel, the tile's records
overflow the resolve's record cache and whole warps of records hit one
address (reduced in the warp).  Frames within 1 LSB of the oracle's render of
the same chains: plain, with AVERAGE blob colours, with keep_background, and
at density 2."""
import numpy as np
import pytest

from oracle import oracle as orc
from test_gpu_render_options import _bbox, _blob_avg

pytestmark = pytest.mark.gpu

TS = (0.0, 0.13, 0.5, 0.87)


def dust_frame(size, fill, rng):
    img = np.zeros((size, size, 4), np.uint8)
    on = rng.random((size, size)) < fill
    img[..., :3] = rng.integers(0, 256, (size, size, 3))
    img[..., 3] = np.where(on, 255, 0)
    img[~on, :3] = 0
    return img


@pytest.mark.parametrize("density", [1, 2])
def test_dust_frames_match_the_oracle(capi, oracle, density):
    rng = np.random.default_rng(77)
    frames = [dust_frame(96, 0.12, rng) for _ in range(3)]
    K = len(frames)
    m = capi.Morph()
    m.load(frames, seed=9, blob_delimiter=0, motion=capi.SPLINE, fading=capi.PERLIN, density=density)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    m.refine(10, capi.PROPOSAL_RANDOM)
    print("chains", m.chains, "atoms", m.atoms)
    assert m.chains > 400  # about 100 blob ranks per 32 x 32 tile
    w, pts, order = m.export_chains()
    colors, present = orc.stored_frames(frames, 0, oracle)
    st = dict(K=K, width=m.width, height=m.height, bbox=_bbox(frames), seed=9, motion=capi.SPLINE,
              fading=capi.PERLIN, delimiter=0, density=density, colors=colors, present=present, widths=w, pts=pts,
              blob_order=order, frame_keys=np.arange(K, dtype=np.uint64), blob_avg=_blob_avg(m, K, len(w)))
    for kb, sb in ((0, 0), (0, 1), (1, 0)):
        m.set(keep_background=kb, show_blobs=sb)
        st.update(keep_background=kb, show_blobs=sb)
        for t in TS:
            got = m.render(t).astype(np.int32)
            ref = oracle.render(st, t).astype(np.int32)
            d = np.abs(got - ref)
            assert int(d.max()) <= 1, (kb, sb, t, int(d.max()), int((d > 1).sum()))
            assert got[..., 3].any()
    m.close()


def test_stacked_atoms_match_the_oracle(capi, oracle):
    """A big blob matched to a one-pixel blob: thousands of atoms stacked on
    one pixel at that key frame (whole warps of records on one address)."""
    big = np.zeros((64, 64, 4), np.uint8)
    big[8:56, 8:56] = (200, 40, 90, 255)
    big[8:56, 8:56, :3] += np.random.default_rng(3).integers(0, 40, (48, 48, 3)).astype(np.uint8)
    dot = np.zeros((64, 64, 4), np.uint8)
    dot[30, 33] = (10, 220, 30, 255)
    frames = [big, dot]
    m = capi.Morph()
    m.load(frames, seed=2, blob_delimiter=0, motion=capi.LINEAR, fading=capi.PERLIN)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    w, pts, order = m.export_chains()
    assert m.chains == 1 and int(w[0]) == 48 * 48
    colors, present = orc.stored_frames(frames, 0, oracle)
    st = dict(K=2, width=m.width, height=m.height, bbox=_bbox(frames), seed=2, motion=capi.LINEAR,
              fading=capi.PERLIN, delimiter=0, density=1, colors=colors, present=present, widths=w, pts=pts,
              blob_order=order, frame_keys=np.arange(2, dtype=np.uint64))
    for t in (0.5, 0.497, 0.9, 0.999):
        got = m.render(t).astype(np.int32)
        ref = oracle.render(st, t).astype(np.int32)
        assert int(np.abs(got - ref).max()) <= 1, t
    m.close()


@pytest.mark.parametrize("density", [1, 2])
def test_heavy_tiles_resolved_in_row_bands(capi, oracle, density):
    """A 96 x 96 blob and a 16 x 16 square matched to a 3 x 3 dot and a
    12 x 12 square in one 32 x 32 tile: near the second key frame that tile
    holds over 9,000 atoms of two blob ranks (a heavy tile).  The first
    frames resolve it with one CTA and note it; the same frames again are
    resolved with 31 helper CTAs, one row band each.  Both within 1 LSB of
    the oracle and equal byte for byte."""
    rng = np.random.default_rng(11)
    a = np.zeros((128, 128, 4), np.uint8)
    a[4:100, 4:100] = (200, 40, 90, 255)
    a[4:100, 4:100, :3] += rng.integers(0, 40, (96, 96, 3)).astype(np.uint8)
    a[108:124, 108:124] = (30, 90, 220, 255)
    b = np.zeros((128, 128, 4), np.uint8)
    b[60:63, 60:63] = (210, 50, 80, 255)
    b[40:52, 40:52] = (40, 100, 210, 255)
    frames = [a, b]
    m = capi.Morph()
    m.load(frames, seed=5, blob_delimiter=0, motion=capi.LINEAR, fading=capi.PERLIN, density=density)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    w, pts, order = m.export_chains()
    assert m.chains == 2 and int(w.max()) >= 96 * 96 * density
    colors, present = orc.stored_frames(frames, 0, oracle)
    st = dict(K=2, width=m.width, height=m.height, bbox=_bbox(frames), seed=5, motion=capi.LINEAR,
              fading=capi.PERLIN, delimiter=0, density=density, colors=colors, present=present, widths=w,
              pts=pts, blob_order=order, frame_keys=np.arange(2, dtype=np.uint64))
    ts = (0.5, 0.47, 0.53, 0.2)
    assert m.heavy_tiles() == (0, 0)
    solo = m.render(ts[0])  # nothing noted yet: one CTA per tile
    tiles, helpers = m.heavy_tiles()
    assert tiles >= 1 and helpers == 0
    banded = [m.render(t) for t in ts]
    tiles2, helpers = m.heavy_tiles()
    assert tiles2 >= 1 and helpers == 31 * tiles2
    assert np.array_equal(solo, banded[0])
    for t, f in zip(ts, banded):
        ref = oracle.render(st, t).astype(np.int32)
        assert int(np.abs(f.astype(np.int32) - ref).max()) <= 1, t
        assert f[..., 3].any()
    m.close()
