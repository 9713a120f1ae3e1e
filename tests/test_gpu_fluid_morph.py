"""The morph's fluid path: draw_fluid against the oracle on the same particle
states (<= 1 LSB), and the particle management invariants of step_fluid over
a rendered cycle (exact active counts per chain, particles of the current
pair only, attractors inside the grid)."""
import numpy as np
import pytest

from atomorph_gb300 import synth

pytestmark = pytest.mark.gpu


def _particles(n, width, height, sp, rng):
    P = np.zeros((18, n))
    P[0] = rng.uniform(5, width * sp + 15, n)   # some beyond the edges on both sides
    P[1] = rng.uniform(5, height * sp + 15, n)
    P[4], P[5] = P[0], P[1]
    P[6] = 1.0
    P[7] = rng.random(n) < 0.9
    P[8] = rng.random(n) < 0.5
    P[9] = rng.choice([0.1, 1.0], n)
    P[10:14] = rng.random((4, n))
    P[14:18] = rng.random((4, n))
    return P


@pytest.mark.parametrize("width,height,sp,n,t", [(96, 80, 1.0, 6000, 0.35), (256, 256, 1.0, 60000, 0.8),
                                                  (200, 120, 0.5, 20000, 0.05)])
def test_fluid_draw_matches_oracle(capi, oracle, width, height, sp, n, t):
    rng = np.random.default_rng(width + n)
    P = _particles(n, width, height, sp, rng)
    gsx, gsy = int(round(width * sp)) + 20, int(round(height * sp)) + 20
    f = capi.Fluid(gsx, gsy, n)
    f.set(P)
    P0 = f.get()  # the FP32 state the GPU holds, as doubles
    bbox = [3, 2, width - 5, height - 4]
    img = f.render(width, height, sp, bbox, t)
    ref_state = P0.copy()
    ref = oracle.draw_fluid(ref_state, width, height, sp, bbox, t)
    d = np.abs(img.astype(int) - ref.astype(int))
    print(f"draw_fluid {width}x{height} sp={sp} n={n}: max diff {d.max()}, "
          f"{(d > 0).mean():.5f} of channels differ")
    assert np.array_equal(img[..., 3] > 0, ref[..., 3] > 0) or d.max() <= 1
    assert d.max() <= 1
    got = f.get()
    act = P0[7] != 0
    assert np.array_equal(got[8][act], np.ones(act.sum()))           # every drawn particle matured
    assert np.abs(got[14:18, act] - ref_state[14:18, act]).max() < 1e-5  # corrected colours
    f.close()


def _surfaces(pts, w, K):
    N = int(w.sum())
    P = pts.reshape(K, N)
    real = ((P >> np.uint64(48)) & np.uint64(3)) == np.uint64(3)  # HAS_PIXEL | HAS_FLUID
    off = np.concatenate([[0], np.cumsum(w)]).astype(np.int64)
    return np.array([[int(real[k, off[c]:off[c + 1]].sum()) for c in range(len(w))] for k in range(K)]), off


def test_fluid_morph_counts_over_a_cycle(capi):
    frames = synth.workload("shapes256")
    m = capi.Morph()
    m.load(frames, seed=7, blob_delimiter=0, motion=capi.LINEAR, fading=capi.PERLIN)
    m.set(fluid=2)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    m.refine(50)
    w, pts, order = m.export_chains()
    K = len(frames)
    S, off = _surfaces(pts, w, K)
    n = int(w.sum())
    frames_n = 12
    for i in range(frames_n):
        time = i / frames_n
        img = m.render(time)
        P = m.fluid_particles()
        assert P.shape[1] == n
        f = int(time * K)
        tl = time * K - f
        act = P[7] != 0
        for c in range(len(w)):
            limit = min(int(np.floor((1 - tl) * S[f, c] + tl * S[(f + 1) % K, c] + 0.5)), int(w[c]))
            assert int(act[off[c]:off[c + 1]].sum()) == limit, (i, c)
        gsx, gsy = m.width + 20, m.height + 20
        assert (P[4][act] >= 1).all() and (P[4][act] <= gsx).all()
        assert (P[5][act] >= 1).all() and (P[5][act] <= gsy).all()
        assert np.isfinite(P[:, act]).all()
        assert img[..., 3].any()
    m.close()


@pytest.mark.parametrize("case,noise", [("ellipses64", 0.0), ("features", 0.0), ("features", 3.0)])
def test_update_particle_targets_match_oracle(capi, oracle, case, noise):
    """update_particle's gravity target and ideal colour (morph.cpp:697-767)
    of every active particle after fluid frames, against the oracle's FP64
    restatement given the columns the particle read: gravity within
    GRAVITY_TOL grid units (FP32 attractor arithmetic), colour channels within
    1/255 + COLOUR_TOL (the FP32 fade is within 1 LSB)."""
    from conftest import golden, golden_state, morph_from_golden
    GRAVITY_TOL, COLOUR_TOL = 1e-3, 1e-6
    g = golden(case)
    m = morph_from_golden(capi, g)
    sp = 1.0
    m.set(fluid=2, fluid_sparseness=sp, motion_noise=noise)
    st = dict(golden_state(g), motion_noise=noise)
    K = int(g["K"])
    w, pts, order = m.export_chains()
    surf, off = _surfaces(pts, w, K)
    col_of = np.repeat(np.arange(len(w)), w.astype(np.int64))
    checked = 0
    for i, t in enumerate([0.1, 0.12, 0.4, 0.42, 0.77]):
        m.render(t)
        P = m.fluid_particles()
        src, dst = m.fluid_links()
        act = np.nonzero(P[7] != 0)[0]
        f = min(int(t * K), K - 1)
        c = col_of[src[act]]
        assert np.array_equal(c, col_of[dst[act]])  # a particle reads columns of its own chain
        ref = oracle.fluid_targets(st, t, sp, src[act], dst[act], surf[f][c], surf[(f + 1) % K][c])
        dg = np.abs(P[4:6, act].T - ref[:, 0:2])
        dc = np.abs(P[10:14, act].T - ref[:, 2:6])
        print(f"{case} A={noise} t={t}: {len(act)} particles, gravity max {dg.max():.2e}, colour max {dc.max():.2e}")
        assert dg.max() <= GRAVITY_TOL
        assert dc.max() <= 1 / 255 + COLOUR_TOL
        checked += len(act)
    assert checked > 0
    m.close()
