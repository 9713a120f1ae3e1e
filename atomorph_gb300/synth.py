"""Seeded synthetic key frames for the morph workloads.

No public benchmark or dataset exists for this path; every workload is a set
of RGBA8 key frames of opaque shapes on a transparent background, generated
here from a seed.  Only pixels with alpha > 0 become atoms, as in the
reference demo's loader (demo/main.cpp:96-127).

Workloads (sizes are the ones the benchmark and the tests quote):

* ``ellipses64``   64x64, 2 key frames x 4 filled ellipses, centres uniform in
                   the frame, radii U[6,16] per axis, uniform opaque RGB.
* ``shapes256``    256x256, 2 key frames x U{12..20} ellipses/rectangles,
                   ~35-45k opaque pixels, base colour per shape plus
                   N(0, 12^2) per pixel and channel.
* ``shapes512``    512x512, 2 key frames, ~200k opaque pixels, same style.
* ``shapes1024``   1024x1024, 8 key frames x U{40..80} overlapping
                   ellipses/rectangles covering ~95% (~1M atoms per frame).
* ``batch``        32 jobs, atom counts log-uniform in [2k, 200k], 3..8 key
                   frames, canvas 128/256/512.

The generator is numpy's PCG64 (``numpy.random.default_rng``) seeded with
``1000 * workload_id + 100 * job + frame``.
"""
from __future__ import annotations

import numpy as np

WORKLOAD_IDS = {"ellipses64": 1, "shapes256": 2, "batch": 3, "shapes512": 4, "shapes1024": 5}


def _rng(workload: str, job: int, frame: int) -> np.random.Generator:
    return np.random.default_rng(1000 * WORKLOAD_IDS[workload] + 100 * job + frame)


def _paint(img: np.ndarray, kind: int, cx: float, cy: float, rx: float, ry: float,
           rgb: np.ndarray, jitter: float, rng: np.random.Generator) -> None:
    h, w = img.shape[:2]
    x0, x1 = max(0, int(np.floor(cx - rx))), min(w, int(np.ceil(cx + rx)) + 1)
    y0, y1 = max(0, int(np.floor(cy - ry))), min(h, int(np.ceil(cy + ry)) + 1)
    if x0 >= x1 or y0 >= y1:
        return
    ys, xs = np.mgrid[y0:y1, x0:x1]
    if kind == 0:
        m = ((xs + 0.5 - cx) / rx) ** 2 + ((ys + 0.5 - cy) / ry) ** 2 <= 1.0
    else:
        m = (np.abs(xs + 0.5 - cx) <= rx) & (np.abs(ys + 0.5 - cy) <= ry)
    n = int(m.sum())
    if n == 0:
        return
    col = np.broadcast_to(rgb.astype(np.float64), (n, 3))
    if jitter > 0:
        col = col + rng.normal(0.0, jitter, size=(n, 3))
    col = np.clip(np.rint(col), 0, 255).astype(np.uint8)
    sub = img[y0:y1, x0:x1]
    sub[m, 0:3] = col
    sub[m, 3] = 255


def ellipses_frame(size: int, n: int, rmin: float, rmax: float, rng: np.random.Generator) -> np.ndarray:
    img = np.zeros((size, size, 4), np.uint8)
    for _ in range(n):
        cx, cy = rng.uniform(0, size, 2)
        rx, ry = rng.uniform(rmin, rmax, 2)
        rgb = rng.integers(0, 256, 3)
        _paint(img, 0, cx, cy, rx, ry, rgb, 0.0, rng)
    return img


def shapes_frame(size: int, n: int, coverage: float, rng: np.random.Generator,
                 jitter: float = 12.0) -> np.ndarray:
    """n random ellipses/rectangles whose common scale is chosen so the opaque
    fraction of the canvas is close to ``coverage``."""
    kinds = rng.integers(0, 2, n)
    centres = rng.uniform(0, size, (n, 2))
    aspect = rng.uniform(0.4, 1.0, (n, 2))
    rel = rng.uniform(0.5, 1.5, n)
    rgbs = rng.integers(0, 256, (n, 3))
    jseed = int(rng.integers(0, 2**31))

    # Coverage is estimated on a grid of at most 256x256 cell centres.
    g = min(size, 256)
    step = size / g

    def cover(scale: float) -> float:
        m = np.zeros((g, g), bool)
        for k in range(n):
            rx, ry = scale * rel[k] * aspect[k]
            cx, cy = centres[k]
            x0, x1 = max(0, int((cx - rx) / step) - 1), min(g, int((cx + rx) / step) + 2)
            y0, y1 = max(0, int((cy - ry) / step) - 1), min(g, int((cy + ry) / step) + 2)
            if x0 >= x1 or y0 >= y1:
                continue
            ys, xs = np.mgrid[y0:y1, x0:x1]
            xs = (xs + 0.5) * step
            ys = (ys + 0.5) * step
            if kinds[k] == 0:
                mk = ((xs - cx) / rx) ** 2 + ((ys - cy) / ry) ** 2 <= 1.0
            else:
                mk = (np.abs(xs - cx) <= rx) & (np.abs(ys - cy) <= ry)
            m[y0:y1, x0:x1] |= mk
        return float(m.mean())

    lo, hi = 0.5, float(size)
    for _ in range(18):
        mid = 0.5 * (lo + hi)
        if cover(mid) < coverage:
            lo = mid
        else:
            hi = mid
    scale = 0.5 * (lo + hi)
    img = np.zeros((size, size, 4), np.uint8)
    jrng = np.random.default_rng(jseed)
    for k in range(n):
        rx, ry = scale * rel[k] * aspect[k]
        _paint(img, int(kinds[k]), centres[k][0], centres[k][1], rx, ry, rgbs[k], jitter, jrng)
    return img


def workload(name: str, job: int = 0) -> list[np.ndarray]:
    """Key frames (list of HxWx4 uint8 RGBA arrays) of one job of a workload."""
    if name == "ellipses64":
        return [ellipses_frame(64, 4, 6.0, 16.0, _rng(name, job, f)) for f in range(2)]
    if name == "shapes256":
        out = []
        for f in range(2):
            r = _rng(name, job, f)
            out.append(shapes_frame(256, int(r.integers(12, 21)), 0.61, r))
        return out
    if name == "shapes512":
        out = []
        for f in range(2):
            r = _rng(name, job, f)
            out.append(shapes_frame(512, int(r.integers(12, 21)), 0.76, r))
        return out
    if name == "shapes1024":
        out = []
        for f in range(8):
            r = _rng(name, job, f)
            out.append(shapes_frame(1024, int(r.integers(40, 81)), 0.95, r))
        return out
    if name == "batch":
        r = _rng(name, job, 99)
        atoms = float(np.exp(r.uniform(np.log(2e3), np.log(2e5))))
        frames = int(r.integers(3, 9))
        size = next(s for s in (128, 256, 512) if atoms <= 0.75 * s * s)
        cov = atoms / (size * size)
        out = []
        for f in range(frames):
            rf = _rng(name, job, f)
            out.append(shapes_frame(size, int(rf.integers(3, 13)), cov, rf))
        return out
    raise KeyError(name)


def opaque_count(img: np.ndarray) -> int:
    return int((img[..., 3] > 0).sum())
