"""ORACLE — test infrastructure only.

ctypes bindings for the two CPU checkers built by oracle/Makefile:

* :class:`Oracle` — the C++ restatement (``liboracle.so``), available on every
  machine that ran ``make``.
* :class:`Reference` — the unmodified reference library plus harness
  (``_ref/libamref.so``), available only where the reference sources were
  present at build time.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs may
import this module.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# Where the reference sources are (the fixtures' generator and the live pin
# build the unmodified reference from them); absent on machines without them.
REF_SOURCES = os.environ.get("ATOMORPH_REFERENCE", "/root/reference")

u8p = C.POINTER(C.c_uint8)
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
i32p = C.POINTER(C.c_int32)
f64p = C.POINTER(C.c_double)


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(t)


def build(with_ref: bool | None = None) -> None:
    """Builds liboracle.so (and _ref/libamref.so when the reference sources
    exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if with_ref is None:
        with_ref = os.path.isdir(REF_SOURCES)
    if with_ref:
        subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref", f"REF={REF_SOURCES}"], check=True)


def have_reference() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libamref.so"))


class Scene(C.Structure):
    _fields_ = [
        ("K", C.c_uint32), ("C", C.c_uint32), ("CW", C.c_uint32), ("CH", C.c_uint32),
        ("width", C.c_uint32), ("height", C.c_uint32), ("bbox", C.c_uint32 * 4), ("seed", C.c_uint32),
        ("motion", C.c_uint32), ("fading", C.c_uint32), ("delimiter", C.c_uint32), ("density", C.c_uint32),
        ("colors", u32p), ("present", u8p), ("widths", u64p), ("pts", u64p), ("blob_order", i32p),
        ("frame_keys", u64p), ("feather", C.c_uint32), ("keep_background", C.c_uint32), ("show_blobs", C.c_uint32),
        ("blob_avg", u32p), ("motion_noise", C.c_double),
    ]


def make_scene(state: dict) -> tuple[Scene, list]:
    """Builds an orc_scene from a morph-state dict (see tests/morphstate.py);
    returns the struct and the arrays it points into (keep them alive)."""
    keep = []

    def arr(name, dt):
        a = np.ascontiguousarray(state[name], dtype=dt)
        keep.append(a)
        return a

    colors = arr("colors", np.uint32)
    present = arr("present", np.uint8)
    widths = arr("widths", np.uint64)
    pts = arr("pts", np.uint64)
    order = arr("blob_order", np.int32)
    keys = arr("frame_keys", np.uint64)
    s = Scene()
    s.K, s.C = int(state["K"]), int(len(widths))
    s.CH, s.CW = int(colors.shape[1]), int(colors.shape[2])
    s.width, s.height = int(state["width"]), int(state["height"])
    for i in range(4):
        s.bbox[i] = int(state["bbox"][i])
    s.seed = int(state["seed"])
    s.motion, s.fading = int(state["motion"]), int(state["fading"])
    s.delimiter, s.density = int(state["delimiter"]), int(state["density"])
    s.colors, s.present, s.widths = _p(colors, u32p), _p(present, u8p), _p(widths, u64p)
    s.pts, s.blob_order, s.frame_keys = _p(pts, u64p), _p(order, i32p), _p(keys, u64p)
    # render options (morph.h:67-70); blob_avg: [K][C] stored-space colour of
    # the b-th blob of key frame k (create_color of its mean), for AVERAGE
    s.feather = int(state.get("feather", 0))
    s.keep_background = int(bool(state.get("keep_background", 0)))
    s.show_blobs = int(state.get("show_blobs", 0))
    if state.get("blob_avg") is not None:
        s.blob_avg = _p(arr("blob_avg", np.uint32), u32p)
    # Perlin motion perturbation amplitude in px (not in the reference)
    s.motion_noise = float(state.get("motion_noise", 0.0))
    return s, keep


class Oracle:
    def __init__(self):
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build(with_ref=False)
        L = self.lib = C.CDLL(path)
        L.orc_rgb_to_hsp.restype = C.c_uint32
        L.orc_rgb_to_hsp.argtypes = [C.c_uint32]
        L.orc_hsp_to_rgb.restype = C.c_uint32
        L.orc_hsp_to_rgb.argtypes = [C.c_uint32]
        L.orc_octave_noise.restype = C.c_double
        L.orc_octave_noise.argtypes = [C.c_uint, C.c_double, C.c_double, C.c_int]
        L.orc_spline_eval.argtypes = [f64p, C.c_int, C.c_double, f64p]
        L.orc_energy.restype = C.c_double
        L.orc_energy.argtypes = [u64p, u64p, C.c_uint32, C.c_uint32, u64p]
        L.orc_sweeps.argtypes = [u64p, u64p, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint]
        L.orc_render.argtypes = [C.POINTER(Scene), C.c_double, u8p]
        L.orc_render_many.argtypes = [C.POINTER(Scene), f64p, C.c_uint32, u8p, C.c_uint32]
        L.orc_positions.argtypes = [C.POINTER(Scene), C.c_double, C.c_int, i32p]
        L.orc_fluid_targets.argtypes = [C.POINTER(Scene), C.c_double, C.c_double, C.c_uint32, u32p, u32p, f64p, f64p,
                                        f64p]
        L.orc_blob_pixels.restype = C.c_size_t
        L.orc_blob_pixels.argtypes = [C.POINTER(Scene), C.c_size_t, C.c_double, C.POINTER(C.c_uint16), u8p,
                                      C.c_size_t]
        L.orc_fluid_step.argtypes = [f64p, C.c_uint32, C.c_uint32, C.c_uint32, f64p, u8p, C.c_uint64, C.c_double]
        L.orc_srand.argtypes = [C.c_uint]
        L.orc_draw_fluid.argtypes = [f64p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_double, u32p, C.c_double, u8p]
        L.orc_draw_fluid_ex.argtypes = [f64p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_double, u32p, C.c_double,
                                        C.c_uint32, u8p, u8p]
        L.orc_background.argtypes = [C.POINTER(Scene), C.c_double, u8p]
        L.orc_components.restype = C.c_uint32
        L.orc_components.argtypes = [u8p, u32p, C.c_uint32, C.c_uint32, i32p, f64p, C.c_uint32]
        L.orc_blob_energy.restype = C.c_double
        L.orc_blob_energy.argtypes = [f64p, C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_double]
        L.orc_blob_match.restype = C.c_double
        L.orc_blob_match.argtypes = [f64p, i32p, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint, C.c_double,
                                     C.c_double, C.c_double, C.c_double]
        L.orc_chain_build.restype = C.c_uint64
        L.orc_chain_build.argtypes = [C.POINTER(u64p), u64p, f64p, f64p, C.c_uint32, C.c_uint32, C.c_uint,
                                      u64p, C.c_uint64]
        L.orc_fix_volatiles.argtypes = [f64p, C.c_uint32]

    def rgb_to_hsp(self, c: int) -> int:
        return self.lib.orc_rgb_to_hsp(c)

    def hsp_to_rgb(self, c: int) -> int:
        return self.lib.orc_hsp_to_rgb(c)

    def octave_noise(self, seed, x, y, octaves=8) -> float:
        return self.lib.orc_octave_noise(seed, x, y, octaves)

    def spline(self, xy: np.ndarray, t: float) -> np.ndarray:
        xy = np.ascontiguousarray(xy, np.float64)
        out = np.zeros(2)
        self.lib.orc_spline_eval(_p(xy, f64p), len(xy), t, _p(out, f64p))
        return out

    def energy(self, pts: np.ndarray, widths: np.ndarray, K: int) -> tuple[float, int]:
        pts = np.ascontiguousarray(pts, np.uint64)
        widths = np.ascontiguousarray(widths, np.uint64)
        ex = np.zeros(1, np.uint64)
        e = self.lib.orc_energy(_p(pts, u64p), _p(widths, u64p), len(widths), K, _p(ex, u64p))
        return e, int(ex[0])

    def sweeps(self, pts: np.ndarray, widths: np.ndarray, K: int, n: int, seed: int) -> np.ndarray:
        out = np.ascontiguousarray(pts, np.uint64).copy()
        widths = np.ascontiguousarray(widths, np.uint64)
        self.lib.orc_sweeps(_p(out, u64p), _p(widths, u64p), len(widths), K, n, seed)
        return out

    def render(self, state: dict, t: float) -> np.ndarray:
        s, keep = make_scene(state)
        out = np.zeros((int(state["height"]), int(state["width"]), 4), np.uint8)
        self.lib.orc_render(C.byref(s), t, _p(out, u8p))
        return out

    def render_many(self, state: dict, ts, threads: int = 1) -> np.ndarray:
        s, keep = make_scene(state)
        ts = np.ascontiguousarray(ts, np.float64)
        out = np.zeros((len(ts), int(state["height"]), int(state["width"]), 4), np.uint8)
        self.lib.orc_render_many(C.byref(s), _p(ts, f64p), len(ts), _p(out, u8p), threads)
        return out

    def positions(self, state: dict, t: float, fp64: bool = False) -> np.ndarray:
        """[N, 2] position words (integer part * 256 + fraction byte) of every
        atom column at time t, -1 where the atom is not drawn; fp64 gives the
        motion perturbation's FP64 accuracy reference."""
        s, keep = make_scene(state)
        N = int(np.sum(state["widths"]))
        out = np.zeros((max(N, 1), 2), np.int32)
        self.lib.orc_positions(C.byref(s), t, int(fp64), _p(out, i32p))
        return out[:N]

    def fluid_targets(self, state: dict, t: float, sparseness: float, src, dst, s0, s1) -> np.ndarray:
        """update_particle's gravity target (x, y) and ideal colour (R, G, B, A)
        for particles reading columns src / dst with blob surfaces s0 / s1:
        [n, 6] (morph.cpp:697-767)."""
        s, keep = make_scene(state)
        src = np.ascontiguousarray(src, np.uint32)
        dst = np.ascontiguousarray(dst, np.uint32)
        s0 = np.ascontiguousarray(s0, np.float64)
        s1 = np.ascontiguousarray(s1, np.float64)
        out = np.zeros((len(src), 6))
        self.lib.orc_fluid_targets(C.byref(s), t, sparseness, len(src), _p(src, u32p), _p(dst, u32p), _p(s0, f64p),
                                   _p(s1, f64p), _p(out, f64p))
        return out

    def blob_pixels(self, state: dict, blob: int, t: float):
        """morph::get_pixels(blob, t): ([n, 2] x, y, [n, 4] RGBA) or None."""
        s, keep = make_scene(state)
        n = self.lib.orc_blob_pixels(C.byref(s), blob, t, None, None, 0)
        if n == (1 << 64) - 1:
            return None
        xy = np.zeros((max(n, 1), 2), np.uint16)
        rgba = np.zeros((max(n, 1), 4), np.uint8)
        self.lib.orc_blob_pixels(C.byref(s), blob, t, xy.ctypes.data_as(C.POINTER(C.c_uint16)), _p(rgba, u8p), n)
        return xy[:n], rgba[:n]

    def components(self, img: np.ndarray, stored: np.ndarray | None = None):
        """4-connected components of img's opaque pixels: (labels, stats)."""
        h, w = img.shape[:2]
        present = np.ascontiguousarray(img[..., 3] > 0, np.uint8)
        if stored is None:
            stored = img
        colors = np.ascontiguousarray(stored).view(np.uint32).reshape(h, w).copy()
        labels = np.zeros((h, w), np.int32)
        cap = w * h
        stats = np.zeros((cap, 7))
        n = self.lib.orc_components(_p(present, u8p), _p(colors, u32p), w, h, _p(labels, i32p),
                                    _p(stats, f64p), cap)
        return labels, stats[:n].copy()

    def fluid_step(self, P: np.ndarray, gsx: int, gsy: int, grid: np.ndarray, touched: np.ndarray,
                   steps_left: int, freedom_radius: float) -> None:
        n = P.shape[1]
        self.lib.orc_fluid_step(_p(P, f64p), n, gsx, gsy, _p(grid, f64p), _p(touched, u8p), steps_left,
                                freedom_radius)

    def draw_fluid(self, P: np.ndarray, width: int, height: int, sparseness: float, bbox, t: float,
                   feather: int = 0, background: np.ndarray | None = None) -> np.ndarray:
        """draw_fluid of particles P[18, n] (modified like the reference's:
        colours corrected, particles matured); returns the RGBA8 frame.  With
        `background` (the get_background image) keep_background is on."""
        n = P.shape[1]
        out = np.zeros((height, width, 4), np.uint8)
        bb = np.ascontiguousarray(bbox, np.uint32)
        bg = None if background is None else np.ascontiguousarray(background, np.uint8)
        self.lib.orc_draw_fluid_ex(_p(P, f64p), n, width, height, sparseness, _p(bb, u32p), t, feather,
                                   None if bg is None else _p(bg, u8p), _p(out, u8p))
        return out

    def background(self, state: dict, t: float) -> np.ndarray:
        """The get_background image at time t (morph.cpp:1405-1413, 1431-1465)."""
        s, keep = make_scene(state)
        out = np.zeros((int(state["height"]), int(state["width"]), 4), np.uint8)
        self.lib.orc_background(C.byref(s), t, _p(out, u8p))
        return out

    def srand(self, s: int) -> None:
        self.lib.orc_srand(s)

    def blob_energy(self, desc: np.ndarray, bbox_d: float, weights=(1, 1, 1)) -> float:
        """desc[g, k, 7] blob descriptors (size, x, y, r, g, b, a)."""
        wr, ws, wx = blob_weights(*weights)
        d = np.ascontiguousarray(desc, np.float64)
        return self.lib.orc_blob_energy(_p(d, f64p), d.shape[0], d.shape[1], bbox_d, wr, ws, wx)


def group_desc(colors: np.ndarray, glabels: np.ndarray, groups: int) -> np.ndarray:
    """Blob descriptors by group, [groups, K, 7] = (size, mean x, mean y,
    mean stored r, g, b, a in 0..1), from each key frame's group-label image
    glabels[k] (-1 where no blob) and stored colours colors[k] (uint32 RGBA);
    exact means.  A group without a blob in a frame has size 0 (its other
    fields do not enter blob_distance, thread.cpp:1163-1170)."""
    K = len(glabels)
    d = np.zeros((groups, K, 7))
    for k in range(K):
        lab = glabels[k]
        ys, xs = np.nonzero(lab >= 0)
        g = lab[ys, xs]
        c = colors[k][ys, xs]
        cnt = np.bincount(g, minlength=groups).astype(np.float64)
        nz = cnt > 0
        d[:, k, 0] = cnt
        for j, v in enumerate((xs, ys)):
            d[nz, k, 1 + j] = np.bincount(g, weights=v, minlength=groups)[nz] / cnt[nz]
        for j in range(4):
            ch = ((c >> np.uint32(8 * j)) & np.uint32(255)).astype(np.float64)
            d[nz, k, 3 + j] = np.bincount(g, weights=ch, minlength=groups)[nz] / cnt[nz] / 255.0
    return d


def bbox_diag2(frames) -> float:
    """Squared diagonal of the key frames' pixel bounding box (thread.cpp:1127-1139)."""
    xs, ys = [], []
    for f in frames:
        y, x = np.nonzero(f[..., 3])
        if len(x):
            xs += [int(x.min()), int(x.max())]
            ys += [int(y.min()), int(y.max())]
    return float((max(xs) - min(xs)) ** 2 + (max(ys) - min(ys)) ** 2)


def blob_weights(rgba: int, size: int, xy: int) -> tuple[float, float, float]:
    """thread::set_blob_weights (thread.cpp:1141-1149)."""
    s = rgba * rgba + size * size + xy * xy
    wr = (rgba * rgba) / s
    ws = (size * size) / s
    return wr, ws, 1.0 - (wr + ws)


class Reference:
    """The unmodified reference library driven through ref_harness.cpp."""

    def __init__(self):
        path = os.path.join(HERE, "_ref", "libamref.so")
        L = self.lib = C.CDLL(path)
        L.ref_new.restype = C.c_void_p
        for name, args in [
            ("ref_free", []), ("ref_set_seed", [C.c_uint]), ("ref_set_delimiter", [C.c_uint]),
            ("ref_set_threshold", [C.c_double]), ("ref_set_blob_number", [C.c_size_t]),
            ("ref_set_blob_min_size", [C.c_size_t]), ("ref_set_blob_max_size", [C.c_size_t]),
            ("ref_set_box_samples", [C.c_size_t]), ("ref_set_density", [C.c_uint]),
            ("ref_set_motion", [C.c_uint]), ("ref_set_fading", [C.c_uint]), ("ref_set_fluid", [C.c_uint]),
            ("ref_set_degeneration", [C.c_size_t]), ("ref_set_finite", [C.c_int]),
            ("ref_set_resolution", [C.c_uint, C.c_uint]), ("ref_set_cycle_length", [C.c_size_t]),
            ("ref_set_threads", [C.c_size_t]), ("ref_set_feather", [C.c_size_t]),
            ("ref_set_keep_background", [C.c_int]), ("ref_set_show_blobs", [C.c_uint]),
            ("ref_add_image", [C.c_size_t, u8p, C.c_uint, C.c_uint]),
            ("ref_prepare", [C.c_size_t, C.c_size_t]), ("ref_export_points", [u64p, C.c_size_t]),
            ("ref_import_points", [u64p, C.c_size_t]), ("ref_sweeps", [C.c_size_t, C.c_uint]),
            ("ref_morph_calls", [C.c_size_t]), ("ref_render", [C.c_double, u8p]), ("ref_bbox", [u32p]),
            ("ref_blob_info", [C.c_size_t, C.c_size_t, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), f64p]),
            ("ref_blob_surface", [C.c_size_t, C.c_size_t, u64p]),
            ("ref_stored_pixel", [C.c_size_t, C.c_uint, C.c_uint, u8p]),
        ]:
            f = getattr(L, name)
            f.argtypes = [C.c_void_p] + args
        L.ref_prepare.restype = C.c_uint
        L.ref_energy.restype = C.c_double
        L.ref_energy.argtypes = [C.c_void_p]
        L.ref_blob_energy.restype = C.c_double
        L.ref_blob_energy.argtypes = [C.c_void_p]
        L.ref_chain_count.restype = C.c_size_t
        L.ref_chain_count.argtypes = [C.c_void_p]
        L.ref_chain_widths.restype = C.c_size_t
        L.ref_chain_widths.argtypes = [C.c_void_p, u64p]
        L.ref_frame_count.restype = C.c_size_t
        L.ref_frame_count.argtypes = [C.c_void_p]
        L.ref_blob_count.restype = C.c_size_t
        L.ref_blob_count.argtypes = [C.c_void_p, C.c_size_t]
        L.ref_pixel_count.restype = C.c_size_t
        L.ref_pixel_count.argtypes = [C.c_void_p, C.c_size_t]
        L.ref_blob_surface.restype = C.c_size_t
        L.ref_blob_pixels.restype = C.c_size_t
        L.ref_blob_pixels.argtypes = [C.c_void_p, C.c_size_t, C.c_double, C.POINTER(C.c_uint16), u8p, C.c_size_t]
        L.ref_synchronize.restype = C.c_int
        L.ref_synchronize.argtypes = [C.c_void_p]
        L.ref_state.restype = C.c_uint
        L.ref_state.argtypes = [C.c_void_p]
        L.ref_get_time.restype = C.c_double
        L.ref_get_time.argtypes = [C.c_void_p, C.c_size_t, C.c_size_t]
        L.ref_rgb_to_hsp.restype = C.c_uint32
        L.ref_rgb_to_hsp.argtypes = [C.c_uint32]
        L.ref_hsp_to_rgb.restype = C.c_uint32
        L.ref_hsp_to_rgb.argtypes = [C.c_uint32]
        L.ref_octave_noise.restype = C.c_double
        L.ref_octave_noise.argtypes = [C.c_uint, C.c_double, C.c_double, C.c_int]
        L.ref_spline_eval.argtypes = [f64p, C.c_size_t, C.c_double, f64p]
        L.ref_fluid_new.restype = C.c_void_p
        L.ref_fluid_new.argtypes = [C.c_uint, C.c_uint, C.c_uint]
        L.ref_fluid_free.argtypes = [C.c_void_p]
        L.ref_fluid_set.argtypes = [C.c_void_p, f64p, C.c_uint]
        L.ref_fluid_get.argtypes = [C.c_void_p, f64p, C.c_uint]
        L.ref_fluid_step.argtypes = [C.c_void_p, C.c_size_t, C.c_double, C.c_double]
        self.h = None

    # -- morph handle ------------------------------------------------------
    def new(self, frames, *, seed=0, delimiter=1, density=1, blob_number=1, motion=3, fading=6,
            threshold=1.0, fluid=0, resync=False):
        """A reference morph of `frames`.  resync: synchronize once before
        prepare(), as the demo's loop does (demo/main.cpp:231-233).  The first
        synchronize after ingestion sets the worker's bounding box and then
        clears it (morph.cpp:119-125, thread.cpp:75-80); blob matching run
        before a second synchronize sees a zero bbox diagonal, every blob
        distance is infinite or NaN (thread.cpp:1167), no swap registers as
        a new best and the groups stay at their initial shuffle."""
        if self.h:
            self.lib.ref_free(self.h)
        h = self.h = self.lib.ref_new()
        L = self.lib
        L.ref_set_seed(h, seed)
        L.ref_set_delimiter(h, delimiter)
        L.ref_set_threshold(h, threshold)
        L.ref_set_blob_number(h, blob_number)
        L.ref_set_motion(h, motion)
        L.ref_set_fading(h, fading)
        L.ref_set_density(h, density)
        L.ref_set_fluid(h, fluid)
        mw = mh = 0
        for i, img in enumerate(frames):
            img = np.ascontiguousarray(img, np.uint8)
            L.ref_add_image(h, i, _p(img, u8p), img.shape[1], img.shape[0])
            mw, mh = max(mw, img.shape[1]), max(mh, img.shape[0])
        L.ref_set_resolution(h, mw, mh)
        self.width, self.height, self.K = mw, mh, len(frames)
        if resync:
            L.ref_synchronize(h)
        return self

    def prepare(self, max_match_steps=20000, max_detect_steps=10**9) -> int:
        return self.lib.ref_prepare(self.h, max_detect_steps, max_match_steps)

    def widths(self) -> tuple[np.ndarray, int]:
        n = self.lib.ref_chain_count(self.h)
        w = np.zeros(n, np.uint64)
        K = self.lib.ref_chain_widths(self.h, _p(w, u64p))
        return w, K

    def points(self) -> np.ndarray:
        w, K = self.widths()
        N = int(w.sum())
        out = np.zeros(K * N, np.uint64)
        self.lib.ref_export_points(self.h, _p(out, u64p), N)
        return out

    def set_points(self, pts: np.ndarray) -> None:
        w, K = self.widths()
        pts = np.ascontiguousarray(pts, np.uint64)
        self.lib.ref_import_points(self.h, _p(pts, u64p), int(w.sum()))

    def energy(self) -> float:
        return self.lib.ref_energy(self.h)

    def sweeps(self, n: int, seed: int) -> None:
        self.lib.ref_sweeps(self.h, n, seed)

    def render(self, t: float) -> np.ndarray:
        out = np.zeros((self.height, self.width, 4), np.uint8)
        self.lib.ref_render(self.h, t, _p(out, u8p))
        return out

    def bbox(self) -> np.ndarray:
        b = np.zeros(4, np.uint32)
        self.lib.ref_bbox(self.h, _p(b, u32p))
        return b

    def blob_count(self, f: int) -> int:
        return self.lib.ref_blob_count(self.h, f)

    def pixel_count(self, f: int) -> int:
        return self.lib.ref_pixel_count(self.h, f)

    def blob_energy(self) -> float:
        """The worker's best blob-map energy (thread.cpp:713-716)."""
        return self.lib.ref_blob_energy(self.h)

    def blob_pixels(self, blob: int, t: float):
        """morph::get_pixels(blob, t): ([n, 2] x, y, [n, 4] RGBA) or None."""
        n = self.lib.ref_blob_pixels(self.h, blob, t, None, None, 0)
        if n == (1 << 64) - 1:
            return None
        xy = np.zeros((max(n, 1), 2), np.uint16)
        rgba = np.zeros((max(n, 1), 4), np.uint8)
        self.lib.ref_blob_pixels(self.h, blob, t, xy.ctypes.data_as(C.POINTER(C.c_uint16)), _p(rgba, u8p), n)
        return xy[:n], rgba[:n]

    def group_labels(self, f: int) -> np.ndarray:
        """[H, W] group of the blob holding each pixel of key frame f (-1: none)."""
        out = np.full((self.height, self.width), -1, np.int32)
        for b, (g, s, xy) in enumerate(self.blobs(f)):
            if not s:
                continue
            pos = np.zeros(s, np.uint64)
            self.lib.ref_blob_surface(self.h, f, b, _p(pos, u64p))
            out[(pos // 65536).astype(np.int64), (pos % 65536).astype(np.int64)] = g
        return out

    def blobs(self, f: int):
        """List of (group, surface, [x,y,r,g,b,a]) in blob-vector order."""
        out = []
        for b in range(self.blob_count(f)):
            g, s = C.c_size_t(), C.c_size_t()
            xy = np.zeros(6)
            self.lib.ref_blob_info(self.h, f, b, C.byref(g), C.byref(s), _p(xy, f64p))
            out.append((g.value, s.value, xy))
        return out

    def options(self, feather: int = 0, keep_background: int = 0, show_blobs: int = 0) -> None:
        self.lib.ref_set_feather(self.h, feather)
        self.lib.ref_set_keep_background(self.h, keep_background)
        self.lib.ref_set_show_blobs(self.h, show_blobs)

    def state(self, seed: int, motion: int, fading: int, delimiter: int, density: int, frames) -> dict:
        """Morph state dict of the reference after prepare(), for the
        oracle / GPU renderers (blob_avg: create_color of each blob's mean)."""
        w, K = self.widths()
        C_ = len(w)
        order = np.zeros((K, C_), np.int32)
        avg = np.zeros((K, C_), np.uint32)
        for f in range(K):
            for b, (g, s, xy) in enumerate(self.blobs(f)):
                order[f, b] = g
                c = [_round_away(v * 255.0) & 255 for v in xy[2:6]]
                avg[f, b] = c[0] | (c[1] << 8) | (c[2] << 16) | (c[3] << 24)
        stored = stored_frames(frames, delimiter, self)
        return dict(K=K, width=self.width, height=self.height, bbox=self.bbox(), seed=seed, motion=motion,
                    fading=fading, delimiter=delimiter, density=density, colors=stored[0], present=stored[1],
                    widths=w, pts=self.points(), blob_order=order, frame_keys=np.arange(K, dtype=np.uint64),
                    blob_avg=avg)


def _round_away(x: float) -> int:
    """std::round: halves away from zero (x - floor(x) is exact in double)."""
    f = math.floor(x)
    r = int(f) + (1 if x - f >= 0.5 else 0)
    return r if x >= 0 else -_round_away(-x)


def stored_frames(frames, delimiter: int, conv) -> tuple[np.ndarray, np.ndarray]:
    """Per-frame stored colours (HSP when delimiter == 1, as morph::add_pixel
    stores them, morph.cpp:299-301) on a common canvas, plus presence."""
    H = max(f.shape[0] for f in frames)
    W = max(f.shape[1] for f in frames)
    colors = np.zeros((len(frames), H, W), np.uint32)
    present = np.zeros((len(frames), H, W), np.uint8)
    lut = {}
    for k, img in enumerate(frames):
        h, w = img.shape[:2]
        c = np.ascontiguousarray(img).view(np.uint32).reshape(h, w)
        m = img[..., 3] > 0
        present[k, :h, :w] = m
        if delimiter == 1:
            vals = np.unique(c[m])
            for v in vals:
                v = int(v)
                if v not in lut:
                    lut[v] = conv.lib.orc_rgb_to_hsp(v) if hasattr(conv.lib, "orc_rgb_to_hsp") else conv.lib.ref_rgb_to_hsp(v)
            conv_c = np.vectorize(lambda v: lut[int(v)], otypes=[np.uint32])(c[m]) if m.any() else c[m]
            cc = np.zeros_like(c)
            cc[m] = conv_c
            colors[k, :h, :w] = cc
        else:
            colors[k, :h, :w] = np.where(m, c, 0)
    return colors, present


def pipeline(O, frames, *, delimiter: int, density: int, seed: int, motion: int, fading: int,
             match_steps: int = 20000) -> dict:
    """The reference pipeline up to chains restated on the CPU (components,
    blob matching, chain construction; oracle.cpp): the morph-state dict of
    the chains it builds for `frames` (blob_number 1 regime: one blob per
    4-connected component).  Deterministic for given inputs on any machine."""
    K = len(frames)
    delim = delimiter
    colors, present = stored_frames(frames, delim, O)
    descs, labels_all = [], []
    for k, img in enumerate(frames):
        st_img = colors[k].view(np.uint8).reshape(img.shape)
        lab, stats = O.components(img, st_img)
        labels_all.append(lab)
        d = np.zeros((len(stats), 7))
        d[:, 0] = stats[:, 0]
        d[:, 1:3] = stats[:, 1:3] / stats[:, :1]
        d[:, 3:7] = stats[:, 3:7] / stats[:, :1] / 255.0
        descs.append(d)
    Wb = max(len(d) for d in descs)
    desc = np.zeros((K, Wb, 7))
    for k, d in enumerate(descs):
        desc[k, :len(d)] = d
        desc[k, len(d):, 1:3] = d[:, 1:3].mean(0) if len(d) else 0
    perm = np.tile(np.arange(Wb, dtype=np.int32), (K, 1))
    xs, ys = [], []
    for f in frames:
        y, x = np.nonzero(f[..., 3])
        xs += [int(x.min()), int(x.max())]
        ys += [int(y.min()), int(y.max())]
    bbox = np.array([min(xs), min(ys), max(xs), max(ys)])
    bbox_d = float((bbox[2] - bbox[0]) ** 2 + (bbox[3] - bbox[1]) ** 2)
    wr, ws, wx = blob_weights(1, 1, 1)
    O.lib.orc_blob_match(desc.ctypes.data_as(f64p), perm.ctypes.data_as(i32p), Wb, K, match_steps, 1, bbox_d,
                         wr, ws, wx)
    widths, chains = [], []
    for g in range(Wb):
        keep = []
        cnt = np.zeros(K, np.uint64)
        cx = np.zeros(K)
        cy = np.zeros(K)
        colk = np.zeros((K, 7))
        for k in range(K):
            b = perm[k, g]
            colk[k] = desc[k, b]
            if b < len(descs[k]):
                ys_, xs_ = np.nonzero(labels_all[k] == b)
                pos = (ys_.astype(np.uint64) * 65536 + xs_.astype(np.uint64))
                pos.sort()
            else:
                pos = np.zeros(0, np.uint64)
            keep.append(pos)
            cnt[k] = len(pos)
        O.lib.orc_fix_volatiles(colk.ctypes.data_as(f64p), K)
        cx[:] = colk[:, 1]
        cy[:] = colk[:, 2]
        ptrs = (u64p * K)(*[p.ctypes.data_as(u64p) for p in keep])
        wdt = O.lib.orc_chain_build(ptrs, cnt.ctypes.data_as(u64p), cx.ctypes.data_as(f64p),
                                    cy.ctypes.data_as(f64p), K, density, g, None, 0)
        buf = np.zeros(int(wdt) * K, np.uint64)
        O.lib.orc_chain_build(ptrs, cnt.ctypes.data_as(u64p), cx.ctypes.data_as(f64p),
                              cy.ctypes.data_as(f64p), K, density, g,
                              buf.ctypes.data_as(u64p), int(wdt))
        widths.append(int(wdt))
        chains.append(buf.reshape(K, int(wdt)))
    widths = np.array(widths, np.uint64)
    pts = np.concatenate(chains, axis=1).reshape(-1)
    order = np.zeros((K, Wb), np.int32)
    for k in range(K):
        for g in range(Wb):
            order[k, perm[k, g]] = g
    H = max(f.shape[0] for f in frames)
    W = max(f.shape[1] for f in frames)
    return dict(K=K, width=W, height=H, bbox=bbox, seed=seed, motion=motion,
                fading=fading, delimiter=delim, density=density, colors=colors,
                present=present, widths=widths, pts=pts, blob_order=order,
                frame_keys=np.arange(K, dtype=np.uint64))
