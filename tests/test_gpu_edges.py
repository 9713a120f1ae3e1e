"""Edge inputs through the GPU pipeline: an all-transparent key frame between
two others, a single key frame, key frames of different sizes (fixtures from
the unmodified reference, tests/golden/edges.npz).  Counts are exact; frames
drawn from the reference's chains match its frames within 1 LSB, and frames
drawn from the GPU's own chains match the oracle on those chains."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

CASES = ["empty_middle", "single", "mixed_sizes"]


def _frames(g, name):
    return [f[:h, :w] for f, (h, w) in zip(g[f"{name}_frames"], g[f"{name}_sizes"])]


def _state(oracle, frames, W, H, w, pts, order):
    from oracle.oracle import stored_frames
    colors, present = stored_frames(frames, 0, oracle)
    nz = [np.nonzero(f[..., 3]) for f in frames]
    bx = [int(p[1].min()) for p in nz if len(p[1])] + [int(p[1].max()) for p in nz if len(p[1])]
    by = [int(p[0].min()) for p in nz if len(p[0])] + [int(p[0].max()) for p in nz if len(p[0])]
    return dict(K=len(frames), width=W, height=H, bbox=np.array([min(bx), min(by), max(bx), max(by)], np.uint32),
                seed=4, motion=3, fading=6, delimiter=0, density=1, colors=colors, present=present, widths=w,
                pts=pts, blob_order=order, frame_keys=np.arange(len(frames), dtype=np.uint64))


@pytest.mark.parametrize("name", CASES)
def test_edge_counts_and_chains(capi, oracle, name):
    g = golden("edges")
    frames = _frames(g, name)
    K = len(frames)
    m = capi.Morph()
    m.load(frames, seed=4, blob_delimiter=0, motion=capi.LINEAR, fading=capi.PERLIN)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    for k in range(K):
        assert m.blob_count(k) == g[f"{name}_blob_counts"][k]
        assert m.pixel_count(k) == g[f"{name}_pixel_counts"][k]
    w, pts, order = m.export_chains()
    assert m.chains == len(g[f"{name}_widths"])
    P = pts.reshape(K, -1)
    for k, img in enumerate(frames):
        orig = P[k][((P[k] >> 48) & 3) == 3]
        ys, xs = np.nonzero(img[..., 3])
        assert len(orig) == len(xs)
        assert set(zip((orig & 0xFFFF).tolist(), ((orig >> 16) & 0xFFFF).tolist())) == set(zip(xs.tolist(), ys.tolist()))
    assert m.cost() == oracle.energy(pts, w, K)[1]
    m.refine(20)
    w, pts, order = m.export_chains()
    st = _state(oracle, frames, m.width, m.height, w, pts, order)
    for t in g["ts"]:
        ref = oracle.render(st, float(t)).astype(int)
        got = m.render(float(t)).astype(int)
        assert np.abs(got - ref).max() <= 1, (name, t)
    m.close()


@pytest.mark.parametrize("name", CASES)
def test_edge_frames_from_reference_chains(capi, name):
    g = golden("edges")
    frames = _frames(g, name)
    m = capi.Morph()
    m.load(frames, seed=4, blob_delimiter=0, motion=capi.LINEAR, fading=capi.PERLIN)
    m.import_chains(g[f"{name}_widths"], g[f"{name}_pts"], g[f"{name}_blob_order"])
    for t, ref in zip(g["ts"], g[f"{name}_renders"]):
        d = np.abs(m.render(float(t)).astype(int) - ref.astype(int))
        assert d.max() <= 1, (name, t, int(d.max()))
    m.close()
