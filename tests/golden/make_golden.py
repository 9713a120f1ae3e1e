"""Generates the golden fixtures in this directory from the UNMODIFIED
reference library (oracle/_ref/libamref.so, built from the reference sources
by oracle/Makefile).  Run it where the reference sources are present:

    python tests/golden/make_golden.py

Fixtures (all small, seeded):
  hsp.npz         RGB->HSP and HSP->RGB byte conversions (color.cpp:64-92)
  perlin.npz      8-octave Perlin noise samples (perlin.cpp:57-69)
  spline.npz      cyclic Catmull-Rom samples (spline.cpp:45-57)
  ellipses64.npz  64x64, 2 key frames: reference blobs, chains, cost, 20
                  refinement sweeps, rendered frames (LINEAR, PERLIN, HSP)
  spline48.npz    48x48, 3 key frames: chains and frames (SPLINE, COSINE, RGB,
                  density 2)
  fluid.npz       FluidModel::step on 300 particles for 8 steps
  features.npz    56x56, 4 key frames (SPLINE, PERLIN, HSP): frames rendered
                  with feather, keep_background and show_blobs AVERAGE /
                  DISTINCT (morph.h:67-70), and the blob colours they read

  edges.npz       edge inputs: an all-transparent key frame, a single key
                  frame, key frames of different sizes (counts, chains, frames)
  blob_rules.npz  blob counts under blob_threshold / number / min / max size
  converge256.npz the reference's converged cost (its own morph_asynch to a
                  plateau) on the CPU pipeline's chains of shapes256
  matching.npz    blob matching results (groups per pixel, best blob-map
                  energy, descriptors) on four cases of 2-4 key frames
  blob_pixels.npz morph::get_pixels(blob, t) lists of every blob at four
                  times, feather 0 and 3, on the features case's chains

    python tests/golden/make_golden.py features   # one fixture only (or: edges, blob_rules, converge, matching, blob_pixels)
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from atomorph_gb300 import synth  # noqa: E402
from oracle import oracle as orc  # noqa: E402

RENDER_TS = [0.0, 0.1, 0.37, 0.5, 0.8, 0.99]


def morph_case(R, frames, *, seed, motion, fading, delimiter, density, sweeps, sweep_seed):
    R.new(frames, seed=seed, motion=motion, fading=fading, delimiter=delimiter, density=density)
    R.prepare()
    w, K = R.widths()
    st = R.state(seed, motion, fading, delimiter, density, frames)
    out = dict(frames=np.stack(frames), seed=seed, motion=motion, fading=fading, delimiter=delimiter,
               density=density, K=K, widths=w, pts0=st["pts"], blob_order=st["blob_order"], bbox=st["bbox"],
               colors=st["colors"], present=st["present"], width=st["width"], height=st["height"],
               blob_counts=np.array([R.blob_count(f) for f in range(K)]),
               real_blob_sizes=np.array([sorted(s for g_, s, xy in R.blobs(f) if s > 0) + [0] * (
                   R.blob_count(f) - sum(1 for g_, s, xy in R.blobs(f) if s > 0)) for f in range(K)]),
               pixel_counts=np.array([R.pixel_count(f) for f in range(K)]),
               energy0=R.energy())
    R.sweeps(sweeps, sweep_seed)
    out.update(sweeps=sweeps, sweep_seed=sweep_seed, pts=R.points(), energy=R.energy(), ts=np.array(RENDER_TS),
               renders=np.stack([R.render(t) for t in RENDER_TS]))
    return out


def edges_case(R):
    """Edge inputs: an all-transparent key frame between two others, one key
    frame, key frames of different sizes (LINEAR, PERLIN, RGB): reference
    counts after matching and frames rendered from the reference's chains."""
    rng = np.random.default_rng(3)
    a = synth.ellipses_frame(48, 3, 4.0, 12.0, rng)
    b = synth.ellipses_frame(48, 3, 4.0, 12.0, rng)
    small = synth.ellipses_frame(32, 2, 3.0, 8.0, rng)
    empty = np.zeros((48, 48, 4), np.uint8)
    out = {}
    for name, frames in (("empty_middle", [a, empty, b]), ("single", [a]), ("mixed_sizes", [a, small, b])):
        R.new(frames, seed=4, motion=3, fading=6, delimiter=0, density=1)
        R.prepare()
        w, K = R.widths()
        st = R.state(4, 3, 6, 0, 1, frames)
        canvas = np.zeros((K, st["height"], st["width"], 4), np.uint8)
        for k, f in enumerate(frames):
            canvas[k, :f.shape[0], :f.shape[1]] = f
        out.update({f"{name}_frames": canvas, f"{name}_sizes": np.array([f.shape[:2] for f in frames]),
                    f"{name}_blob_counts": np.array([R.blob_count(f) for f in range(K)]),
                    f"{name}_pixel_counts": np.array([R.pixel_count(f) for f in range(K)]),
                    f"{name}_widths": w, f"{name}_pts": st["pts"], f"{name}_blob_order": st["blob_order"],
                    f"{name}_renders": np.stack([R.render(t) for t in FEATURE_TS])})
    out["ts"] = np.array(FEATURE_TS)
    return out


BLOB_RULES = [(0.05, 1, 1, 2**62), (0.12, 1, 1, 2**62), (1.0, 60, 1, 2**62), (0.12, 1, 8, 2**62),
              (1.0, 1, 1, 200), (0.08, 30, 4, 2**62)]


def blob_rules_case(R):
    """Blob detection outside the component regime (blob_threshold,
    blob_number, blob_min_size, blob_max_size; thread.cpp:225-585): the
    reference's real blob count per key frame for each setting, on two noisy
    96x96 key frames (RGB delimiter)."""
    rng = np.random.default_rng(12)
    frames = [synth.shapes_frame(96, 6, 0.5, rng) for _ in range(2)]
    counts = []
    for thr, bn, mn, mx in BLOB_RULES:
        R.new(frames, seed=3, motion=3, fading=3, delimiter=0, density=1, threshold=thr, blob_number=bn)
        R.lib.ref_set_blob_min_size(R.h, mn)
        R.lib.ref_set_blob_max_size(R.h, mx)
        R.prepare()
        counts.append([sum(1 for g, s, xy in R.blobs(f) if s > 0) for f in range(2)])
    return dict(frames=np.stack(frames), rules=np.array(BLOB_RULES, dtype=np.float64), counts=np.array(counts))


FEATURE_OPTIONS = [(0, 0, 0), (0, 0, 1), (0, 0, 2), (0, 1, 0), (3, 0, 0), (2, 1, 0), (1, 1, 1), (5, 0, 2)]
FEATURE_TS = [0.05, 0.3, 0.61, 0.9]


def features_case(R):
    """Render options (feather, keep_background, show_blobs) on one seeded
    case; the state the oracle needs to draw the same frames."""
    rng = np.random.default_rng(77)
    frames = [synth.ellipses_frame(56, 5, 3.0, 14.0, rng) for _ in range(4)]
    R.new(frames, seed=5, motion=4, fading=6, delimiter=1, density=1)
    R.prepare()
    R.sweeps(4, 31)
    st = R.state(5, 4, 6, 1, 1, frames)
    renders = []
    for feather, kb, sb in FEATURE_OPTIONS:
        R.options(feather, kb, sb)
        renders.append(np.stack([R.render(t) for t in FEATURE_TS]))
    R.options(0, 0, 0)
    return dict(frames=np.stack(frames), options=np.array(FEATURE_OPTIONS), ts=np.array(FEATURE_TS),
                renders=np.stack(renders), K=st["K"], width=st["width"], height=st["height"], bbox=st["bbox"],
                seed=5, motion=4, fading=6, delimiter=1, density=1, colors=st["colors"], present=st["present"],
                widths=st["widths"], pts=st["pts"], blob_order=st["blob_order"], blob_avg=st["blob_avg"])


def converge_case(R, window=10000, rel=2e-5, max_sweeps=200000):
    """C2-style convergence target: the chains the CPU pipeline builds for
    shapes256 (2 key frames of 256x256, about 40k atoms, HSP), refined by the
    reference's own morph_asynch (the unmodified library, ref_sweeps) until a
    window of `window` sweeps gains less than `rel` of the cost.  The chains
    are rebuilt at test time by the same deterministic CPU pipeline; their
    checksum is stored to prove it."""
    O = orc.Oracle()
    frames = synth.workload("shapes256")
    st = orc.pipeline(O, frames, delimiter=1, density=1, seed=5, motion=4, fading=6)
    w, pts, K = st["widths"], st["pts"], st["K"]
    R.new(frames, seed=5, motion=4, fading=6, delimiter=1, density=1, resync=True)
    R.prepare()
    rw, rK = R.widths()
    assert rK == K and np.array_equal(np.sort(rw), np.sort(w)) and np.array_equal(rw, w), (rw, w)
    R.set_points(pts)
    e0 = O.energy(pts, w, K)[1]
    assert int(R.energy()) == e0
    # the first 50 sweeps of the reference and of the oracle's restatement agree bit for bit
    R.sweeps(50, 1)
    assert np.array_equal(R.points(), O.sweeps(pts, w, K, 50, 1))
    done, seed, trace = 50, 2, [(50, int(R.energy()))]
    while done < max_sweeps:
        R.sweeps(window, seed)
        seed += 1
        done += window
        trace.append((done, int(R.energy())))
        if trace[-2][1] - trace[-1][1] < rel * trace[-1][1]:
            break
    cost = trace[-1][1]
    assert O.energy(R.points(), w, K)[1] == cost
    return dict(initial_cost=e0, converged_cost=cost, converged_sweeps=done, trace=np.array(trace, np.int64),
                widths=w, pts_checksum=np.uint64(int(np.bitwise_xor.reduce(pts * np.uint64(0x9E3779B97F4A7C15)))))


MATCH_CASES = [("ellipses64", 7, 1), ("spline48", 3, 0), ("features", 5, 1), ("many96", 11, 0)]


def matching_frames(name):
    if name == "ellipses64":
        return synth.workload("ellipses64")
    if name == "spline48":
        r3 = np.random.default_rng(48)
        return [synth.ellipses_frame(48, 3, 4.0, 12.0, r3) for _ in range(3)]
    if name == "features":
        rng = np.random.default_rng(77)
        return [synth.ellipses_frame(56, 5, 3.0, 14.0, rng) for _ in range(4)]
    rng = np.random.default_rng(96)
    return [synth.ellipses_frame(96, 10, 3.0, 10.0, rng) for _ in range(4)]


def matching_case(R):
    """Blob matching (thread::match, thread.cpp:598-738) of the reference,
    run with a valid bounding box (one synchronize before prepare, as the
    demo's loop gives it): per case the group of every key-frame pixel's
    blob, the reference's best blob-map energy and its blob descriptors
    (running means, stored colour space) by group."""
    O = orc.Oracle()
    out = {}
    for name, seed, delim in MATCH_CASES:
        frames = matching_frames(name)
        R.new(frames, seed=seed, motion=3, fading=6, delimiter=delim, density=1, resync=True)
        R.prepare()
        K = len(frames)
        glab = np.stack([R.group_labels(f) for f in range(K)])
        groups = max(R.blob_count(f) for f in range(K))
        desc = np.zeros((groups, K, 7))
        for f in range(K):
            for g, sz, xy in R.blobs(f):
                desc[g, f, 0] = sz
                desc[g, f, 1:] = xy
        bd = orc.bbox_diag2(frames)
        e = R.blob_energy()
        assert abs(O.blob_energy(desc, bd) - e) <= 1e-9 * max(e, 1.0), (name, O.blob_energy(desc, bd), e)
        out.update({f"{name}_frames": np.stack(frames), f"{name}_group_labels": glab.astype(np.int16),
                    f"{name}_energy": e, f"{name}_desc": desc, f"{name}_delimiter": delim, f"{name}_seed": seed})
    out["cases"] = np.array([c[0] for c in MATCH_CASES])
    return out


BLOB_TS = [0.05, 0.3, 0.61, 0.9]


def blob_pixels_case(R):
    """morph::get_pixels(blob, t) of the reference (morph.cpp:452-678) for
    every blob of the key frame at each time in BLOB_TS, on the features
    case's chains, with feather 0 and 3: pixel lists concatenated, offsets per
    (feather, t, blob)."""
    rng = np.random.default_rng(77)
    frames = [synth.ellipses_frame(56, 5, 3.0, 14.0, rng) for _ in range(4)]
    R.new(frames, seed=5, motion=4, fading=6, delimiter=1, density=1)
    R.prepare()
    R.sweeps(4, 31)
    xy, rgba, index = [], [], []
    for feather in (0, 3):
        R.options(feather, 0, 0)
        for ti, t in enumerate(BLOB_TS):
            f = int(t * 4)
            for b in range(R.blob_count(f)):
                got = R.blob_pixels(b, t)
                n = 0 if got is None else len(got[0])
                index.append((feather, ti, b, sum(len(a) for a in xy), n))
                if got is not None:
                    xy.append(got[0]); rgba.append(got[1])
    R.options(0, 0, 0)
    return dict(ts=np.array(BLOB_TS), index=np.array(index, np.int64), xy=np.concatenate(xy),
                rgba=np.concatenate(rgba))


def main():
    orc.build(with_ref=True)
    R = orc.Reference()
    if sys.argv[1:] == ["blob_pixels"]:
        np.savez_compressed(os.path.join(HERE, "blob_pixels.npz"), **blob_pixels_case(R))
        return
    if sys.argv[1:] == ["matching"]:
        np.savez_compressed(os.path.join(HERE, "matching.npz"), **matching_case(R))
        return
    if sys.argv[1:] == ["converge"]:
        np.savez_compressed(os.path.join(HERE, "converge256.npz"), **converge_case(R))
        return
    if sys.argv[1:] == ["features"]:
        np.savez_compressed(os.path.join(HERE, "features.npz"), **features_case(R))
        return
    if sys.argv[1:] == ["edges"]:
        np.savez_compressed(os.path.join(HERE, "edges.npz"), **edges_case(R))
        return
    if sys.argv[1:] == ["blob_rules"]:
        np.savez_compressed(os.path.join(HERE, "blob_rules.npz"), **blob_rules_case(R))
        return
    L = R.lib
    rng = np.random.default_rng(2024)
    rgb = rng.integers(0, 2**32, 4096, dtype=np.uint64).astype(np.uint32)
    np.savez_compressed(os.path.join(HERE, "hsp.npz"), rgb=rgb,
                        hsp=np.array([L.ref_rgb_to_hsp(int(c)) for c in rgb], np.uint32),
                        back=np.array([L.ref_hsp_to_rgb(int(c)) for c in rgb], np.uint32))
    xy = rng.uniform(0, 9, (512, 2))
    seeds = np.array([1, 7, 8, 12345])
    noise = np.array([[L.ref_octave_noise(int(s), x, y, 8) for x, y in xy] for s in seeds])
    np.savez_compressed(os.path.join(HERE, "perlin.npz"), xy=xy, seeds=seeds, noise=noise)
    pts = rng.uniform(0, 60, (5, 2))
    ts = np.linspace(0, 0.999, 97)
    sp = []
    for t in ts:
        o = np.zeros(2)
        L.ref_spline_eval(pts.ctypes.data_as(orc.f64p), len(pts), t, o.ctypes.data_as(orc.f64p))
        sp.append(o)
    np.savez_compressed(os.path.join(HERE, "spline.npz"), pts=pts, ts=ts, values=np.array(sp))

    frames = synth.workload("ellipses64")
    np.savez_compressed(os.path.join(HERE, "ellipses64.npz"),
                        **morph_case(R, frames, seed=7, motion=3, fading=6, delimiter=1, density=1, sweeps=20,
                                     sweep_seed=123))
    r3 = np.random.default_rng(48)
    frames3 = [synth.ellipses_frame(48, 3, 4.0, 12.0, r3) for _ in range(3)]
    np.savez_compressed(os.path.join(HERE, "spline48.npz"),
                        **morph_case(R, frames3, seed=3, motion=4, fading=5, delimiter=0, density=2, sweeps=5,
                                     sweep_seed=9))

    n, gsx, gsy = 300, 40, 36
    P = np.zeros((18, n))
    P[0] = rng.uniform(6, 33, n); P[1] = rng.uniform(6, 29, n)
    P[4] = P[0] + rng.normal(0, 2, n); P[5] = P[1] + rng.normal(0, 2, n)
    P[6] = 1.0; P[7] = 1.0; P[8] = rng.random(n) < 0.7; P[9] = rng.choice([0.1, 1.0], n)
    P[10:14] = rng.random((4, n)); P[14:18] = rng.random((4, n)); P[7][::13] = 0
    h = L.ref_fluid_new(gsx, gsy, n)
    q = np.zeros((n, 20)); q[:, :18] = P.T
    L.ref_fluid_set(h, q.ctypes.data_as(orc.f64p), n)
    steps = []
    for s in range(8):
        L.ref_fluid_step(h, 7 - s, 4.0, 0.25)
        L.ref_fluid_get(h, q.ctypes.data_as(orc.f64p), n)
        steps.append(q[:, :18].T.copy())
    L.ref_fluid_free(h)
    np.savez_compressed(os.path.join(HERE, "fluid.npz"), init=P, gsx=gsx, gsy=gsy, freedom=4.0,
                        step1=steps[0], step8=steps[-1])
    np.savez_compressed(os.path.join(HERE, "features.npz"), **features_case(R))
    np.savez_compressed(os.path.join(HERE, "edges.npz"), **edges_case(R))
    np.savez_compressed(os.path.join(HERE, "blob_rules.npz"), **blob_rules_case(R))
    np.savez_compressed(os.path.join(HERE, "converge256.npz"), **converge_case(R))
    np.savez_compressed(os.path.join(HERE, "matching.npz"), **matching_case(R))
    np.savez_compressed(os.path.join(HERE, "blob_pixels.npz"), **blob_pixels_case(R))
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
