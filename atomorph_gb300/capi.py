"""ctypes binding of the atomorph_gb300 C ABI (include/atomorph_gb300.h).

This is thin glue for Python callers (tests, the benchmark); the
reference-facing host API is the C++ class ``am::morph`` in
include/atomorph_gb300.hpp.  The binding loads the in-tree CUDA library and
raises if it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libatomorph_gb300.so")
HEADER = os.path.join(HERE, "..", "include", "atomorph_gb300.h")

AM_OK, AM_ERR_BUSY, AM_ERR_NOMEM, AM_ERR_CUDA, AM_ERR_TIMEOUT, AM_ERR_ARG, AM_ERR_STATE, AM_ERR_UNSUPPORTED, \
    AM_ERR_NOT_FOUND = range(9)
RGB, HSP, NONE, LINEAR, SPLINE, COSINE, PERLIN = range(7)
STATE_BLOB_DETECTION, STATE_BLOB_UNIFICATION, STATE_BLOB_MATCHING, STATE_ATOM_MORPHING, STATE_DONE = range(5)
PROPOSAL_RANDOM, PROPOSAL_LOCAL, PROPOSAL_LEARNED, PROPOSAL_SCORED = range(4)

u8p = C.POINTER(C.c_uint8)
u64p = C.POINTER(C.c_uint64)
i32p = C.POINTER(C.c_int32)
u32p = C.POINTER(C.c_uint32)
f64p = C.POINTER(C.c_double)
f32p = C.POINTER(C.c_float)
vp = C.c_void_p

_SIGS = {
    "am_create": (C.c_int, [C.POINTER(vp)]),
    "am_destroy": (None, [vp]),
    "am_clear": (C.c_int, [vp]),
    "am_last_error": (C.c_char_p, []),
    "am_version": (C.c_char_p, []),
    "am_add_pixel": (C.c_int, [vp, C.c_size_t, C.c_uint16, C.c_uint16, C.c_uint8, C.c_uint8, C.c_uint8, C.c_uint8]),
    "am_add_pixels": (C.c_int, [vp, C.c_size_t, u8p, C.c_uint32, C.c_uint32]),
    "am_add_frame": (C.c_int, [vp, C.c_size_t]),
    "am_set_seed": (C.c_int, [vp, C.c_uint]),
    "am_set_blob_delimiter": (C.c_int, [vp, C.c_uint]),
    "am_set_blob_threshold": (C.c_int, [vp, C.c_double]),
    "am_set_blob_max_size": (C.c_int, [vp, C.c_size_t]),
    "am_set_blob_min_size": (C.c_int, [vp, C.c_size_t]),
    "am_set_blob_box_grip": (C.c_int, [vp, C.c_uint16]),
    "am_set_blob_box_samples": (C.c_int, [vp, C.c_size_t]),
    "am_set_blob_number": (C.c_int, [vp, C.c_size_t]),
    "am_set_blob_rgba_weight": (C.c_int, [vp, C.c_uint]),
    "am_set_blob_size_weight": (C.c_int, [vp, C.c_uint]),
    "am_set_blob_xy_weight": (C.c_int, [vp, C.c_uint]),
    "am_set_degeneration": (C.c_int, [vp, C.c_size_t]),
    "am_set_motion": (C.c_int, [vp, C.c_uint]),
    "am_set_fading": (C.c_int, [vp, C.c_uint]),
    "am_set_threads": (C.c_int, [vp, C.c_size_t]),
    "am_set_cycle_length": (C.c_int, [vp, C.c_size_t]),
    "am_set_feather": (C.c_int, [vp, C.c_size_t]),
    "am_set_keep_background": (C.c_int, [vp, C.c_int]),
    "am_set_finite": (C.c_int, [vp, C.c_int]),
    "am_set_show_blobs": (C.c_int, [vp, C.c_uint]),
    "am_set_fluid": (C.c_int, [vp, C.c_uint]),
    "am_set_density": (C.c_int, [vp, C.c_uint16]),
    "am_set_resolution": (C.c_int, [vp, C.c_uint16, C.c_uint16]),
    "am_set_proposal": (C.c_int, [vp, C.c_uint]),
    "am_set_sweeps": (C.c_int, [vp, C.c_size_t]),
    "am_set_motion_noise": (C.c_int, [vp, C.c_double]),
    "am_compute": (C.c_int, [vp]),
    "am_iterate": (C.c_int, [vp, C.c_size_t]),
    "am_compute_seconds": (C.c_int, [vp, C.c_double]),
    "am_suspend": (C.c_int, [vp]),
    "am_suspend_timeout": (C.c_int, [vp, C.c_double]),
    "am_is_busy": (C.c_int, [vp]),
    "am_synchronize": (C.c_int, [vp]),
    "am_next_state": (C.c_int, [vp]),
    "am_get_state": (C.c_uint, [vp]),
    "am_get_energy": (C.c_double, [vp]),
    "am_get_cost": (C.c_int, [vp, u64p, f64p]),
    "am_get_cost_noalloc": (C.c_int, [vp, u64p]),
    "am_get_blob_count": (C.c_size_t, [vp, C.c_size_t]),
    "am_get_blob_count_total": (C.c_size_t, [vp]),
    "am_get_pixel_count": (C.c_size_t, [vp, C.c_size_t]),
    "am_get_frame_count": (C.c_size_t, [vp]),
    "am_get_frame_key": (C.c_size_t, [vp, C.c_double]),
    "am_get_width": (C.c_uint16, [vp]),
    "am_get_height": (C.c_uint16, [vp]),
    "am_get_time": (C.c_double, [vp, C.c_size_t, C.c_size_t]),
    "am_get_average_pixel": (C.c_int, [vp, C.c_size_t, C.POINTER(C.c_uint16), u8p]),
    "am_get_blob_average": (C.c_int, [vp, C.c_size_t, C.c_size_t, C.POINTER(C.c_uint16), u8p]),
    "am_get_blob_labels": (C.c_int, [vp, C.c_size_t, i32p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "am_get_atom_count": (C.c_size_t, [vp]),
    "am_get_blob_info": (C.c_int, [vp, C.c_size_t, C.c_size_t, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), f64p]),
    "am_get_blob_pixels": (C.c_int, [vp, C.c_size_t, C.c_double, C.POINTER(C.c_uint16), u8p, C.c_size_t,
                                     C.POINTER(C.c_size_t)]),
    "am_get_chain_count": (C.c_size_t, [vp]),
    "am_render": (C.c_int, [vp, C.c_double, vp, C.c_int]),
    "am_render_many": (C.c_int, [vp, f64p, C.c_size_t, vp]),
    "am_get_positions": (C.c_size_t, [vp, C.c_double, i32p, C.c_size_t]),
    "am_render_many_host": (C.c_int, [vp, f64p, C.c_size_t, vp]),
    "am_export_chains": (C.c_int, [vp, u64p, u64p, i32p]),
    "am_import_chains": (C.c_int, [vp, C.c_size_t, C.c_size_t, u64p, u64p, i32p]),
    "am_refine": (C.c_int, [vp, C.c_size_t, u64p]),
    "am_record_swaps": (C.c_int, [vp, C.c_size_t]),
    "am_record_outcomes": (C.c_int, [vp, C.c_size_t, C.c_uint32]),
    "am_recorded_swaps": (C.c_size_t, [vp, f32p, f32p, C.c_size_t]),
    "am_train_proposal": (C.c_int, [vp, f32p, f32p, C.c_size_t, C.c_size_t, C.c_double, f32p]),
    "am_train_recorded": (C.c_int, [vp, C.c_size_t, C.c_double, f32p]),
    "am_get_proposal_weights": (C.c_int, [vp, f32p, C.c_size_t]),
    "am_set_proposal_weights": (C.c_int, [vp, f32p, C.c_size_t]),
    "am_proposal_forward": (C.c_int, [vp, f32p, C.c_size_t, f32p]),
    "am_proposal_grad": (C.c_int, [vp, f32p, f32p, C.c_size_t, f32p, f32p]),
    "am_fluid_create": (C.c_int, [C.POINTER(vp), C.c_uint32, C.c_uint32, C.c_uint32]),
    "am_fluid_destroy": (None, [vp]),
    "am_fluid_set_particles": (C.c_int, [vp, f64p]),
    "am_fluid_get_particles": (C.c_int, [vp, f64p]),
    "am_fluid_step": (C.c_int, [vp, C.c_size_t, C.c_double]),
    "am_fluid_steps": (C.c_int, [vp, C.c_size_t, C.c_double]),
    "am_fluid_stream": (vp, [vp]),
    "am_fluid_render": (C.c_int, [vp, C.c_uint32, C.c_uint32, C.c_double, C.POINTER(C.c_uint32), C.c_double, u8p]),
    "am_fluid_render_ex": (C.c_int, [vp, C.c_uint32, C.c_uint32, C.c_double, C.POINTER(C.c_uint32), C.c_double,
                                     C.c_size_t, u8p, u8p]),
    "am_set_fluid_sparseness": (C.c_int, [vp, C.c_double]),
    "am_get_fluid_particles": (C.c_size_t, [vp, f64p, C.c_size_t]),
    "am_get_fluid_links": (C.c_size_t, [vp, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.c_size_t]),
    "am_set_tuning": (C.c_int, [vp, C.c_char_p, C.c_double]),
    "am_batch_create": (C.c_int, [C.POINTER(vp), C.POINTER(vp), C.c_size_t]),
    "am_batch_destroy": (None, [vp]),
    "am_batch_refine": (C.c_int, [vp, C.c_size_t, u64p]),
    "am_batch_tune": (C.c_int, [vp, C.c_size_t]),
    "am_batch_refine_guided": (C.c_int, [vp, C.c_size_t, u64p]),
    "am_batch_refine_schedule": (C.c_int, [vp, C.c_size_t, u64p]),
    "am_batch_tune_schedule": (C.c_int, [vp, C.c_size_t, C.POINTER(C.c_size_t)]),
    "am_batch_render": (C.c_int, [vp, f64p, C.c_size_t, C.POINTER(vp), C.c_int]),
    "am_batch_get_tuning": (C.c_int, [vp, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                      C.POINTER(C.c_uint32)]),
    "am_batch_set_tuning": (C.c_int, [vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]),
    "am_get_stream": (vp, [vp]),
    "am_profile_enable": (C.c_int, [vp, C.c_int]),
    "am_profile_read": (C.c_size_t, [vp, C.POINTER(C.c_char_p), f64p, u64p, C.c_size_t]),
    "am_launch_count": (C.c_uint64, []),
    "am_get_heavy_tiles": (C.c_int, [vp, u32p, u32p]),
    "am_device_sync": (C.c_int, [vp]),
}

_lib = None


def load() -> C.CDLL:
    """Loads the CUDA library (built by atomorph_gb300.build); raises if it is
    not there."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"atomorph_gb300 CUDA library not built: {LIB_PATH} (run __graft_entry__.build())")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def declared_symbols() -> list[str]:
    import re
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(am_[a-z_0-9]+)\s*\(", text)))


class AmError(RuntimeError):
    def __init__(self, code: int, what: str):
        msg = (load().am_last_error() or b"").decode(errors="replace")
        super().__init__(f"{what} failed with status {code}: {msg}")
        self.code = code


def _check(rc: int, what: str) -> int:
    if rc != AM_OK:
        raise AmError(rc, what)
    return rc


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(t)


class Morph:
    """One morph handle (the GB300 counterpart of am::morph)."""

    def __init__(self):
        self.lib = load()
        h = vp()
        _check(self.lib.am_create(C.byref(h)), "am_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.am_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- setters: morph.h:52-76 ---------------------------------------------
    def set(self, **kw) -> "Morph":
        for k, v in kw.items():
            f = getattr(self.lib, "am_set_" + k)
            if k == "resolution":
                _check(f(self.h, *v), "am_set_" + k)
            else:
                _check(f(self.h, v), "am_set_" + k)
        return self

    def blob_labels(self, frame: int) -> np.ndarray:
        """[h, w] blob index of every canvas pixel of key frame `frame` (-1: none)."""
        w, h = C.c_uint32(), C.c_uint32()
        _check(self.lib.am_get_blob_labels(self.h, frame, None, C.byref(w), C.byref(h)), "am_get_blob_labels")
        out = np.zeros((h.value, w.value), np.int32)
        _check(self.lib.am_get_blob_labels(self.h, frame, _p(out, i32p), None, None), "am_get_blob_labels")
        return out

    def fluid_particles(self) -> np.ndarray:
        """[18, n] particle fields of the morph's fluid (oracle order)."""
        n = self.lib.am_get_fluid_particles(self.h, None, 0)
        q = np.zeros((max(n, 1), 18))
        if n:
            self.lib.am_get_fluid_particles(self.h, _p(q, f64p), n)
        return q[:n].T.copy()

    def fluid_links(self):
        """(source, destination) column of every particle's last update."""
        n = self.lib.am_get_fluid_links(self.h, None, None, 0)
        s = np.zeros(max(n, 1), np.uint32)
        d = np.zeros(max(n, 1), np.uint32)
        if n:
            self.lib.am_get_fluid_links(self.h, s.ctypes.data_as(C.POINTER(C.c_uint32)),
                                        d.ctypes.data_as(C.POINTER(C.c_uint32)), n)
        return s[:n], d[:n]

    def tune(self, **kw) -> "Morph":
        """Guided-refinement tunables (am_set_tuning): local_self,
        local_target, local_random, learned_keep, learned_adaptive, guided_switch,
        render_pipeline."""
        for k, v in kw.items():
            _check(self.lib.am_set_tuning(self.h, k.encode(), float(v)), "am_set_tuning " + k)
        return self

    def add_image(self, frame: int, img: np.ndarray) -> None:
        img = np.ascontiguousarray(img, np.uint8)
        _check(self.lib.am_add_pixels(self.h, frame, _p(img, u8p), img.shape[1], img.shape[0]), "am_add_pixels")

    def add_pixel(self, frame, x, y, r, g, b, a) -> int:
        return self.lib.am_add_pixel(self.h, frame, x, y, r, g, b, a)

    def add_frame(self, frame) -> int:
        return self.lib.am_add_frame(self.h, frame)

    def load(self, frames, **settings) -> "Morph":
        """Adds key frames 0..K-1 and sets the resolution to their extent, as
        the reference demo's load_files does (demo/main.cpp:135-176)."""
        self.set(**settings)
        w = h = 0
        for i, img in enumerate(frames):
            self.add_image(i, img)
            w, h = max(w, img.shape[1]), max(h, img.shape[0])
        self.set(resolution=(w, h))
        return self

    # -- control -------------------------------------------------------------
    def synchronize(self) -> int:
        return self.lib.am_synchronize(self.h)

    def iterate(self, n: int) -> None:
        _check(self.lib.am_iterate(self.h, n), "am_iterate")

    def compute(self) -> None:
        _check(self.lib.am_compute(self.h), "am_compute")

    def suspend(self, timeout: float | None = None) -> int:
        if timeout is None:
            return self.lib.am_suspend(self.h)
        return self.lib.am_suspend_timeout(self.h, timeout)

    def next_state(self) -> None:
        self.lib.am_next_state(self.h)

    def wait(self, timeout: float = 600.0) -> None:
        """Waits, without interrupting it, until the worker has used up its
        iteration budget and paused (callers of the reference poll is_busy()
        the same way; suspend() would cut the budget short)."""
        import time
        t0 = time.time()
        while self.lib.am_is_busy(self.h):
            if time.time() - t0 > timeout:
                raise TimeoutError("worker still busy")
            time.sleep(0.0005)

    def run_until(self, state: int, max_steps: int = 100000) -> int:
        """Synchronous driver: synchronize, step, synchronize until the worker
        reaches `state` (or max_steps)."""
        _check(self.synchronize(), "am_synchronize")
        steps = 0
        while self.state < state and steps < max_steps:
            self.iterate(1)
            self.wait()
            _check(self.synchronize(), "am_synchronize")
            steps += 1
        return self.state

    # -- readout -------------------------------------------------------------
    @property
    def state(self) -> int:
        return self.lib.am_get_state(self.h)

    @property
    def energy(self) -> float:
        return self.lib.am_get_energy(self.h)

    def cost(self) -> int:
        ex = C.c_uint64()
        _check(self.lib.am_get_cost(self.h, C.byref(ex), None), "am_get_cost")
        return ex.value

    def blob_count(self, frame: int) -> int:
        return self.lib.am_get_blob_count(self.h, frame)

    def pixel_count(self, frame: int) -> int:
        return self.lib.am_get_pixel_count(self.h, frame)

    @property
    def atoms(self) -> int:
        return self.lib.am_get_atom_count(self.h)

    @property
    def chains(self) -> int:
        return self.lib.am_get_chain_count(self.h)

    @property
    def width(self) -> int:
        return self.lib.am_get_width(self.h)

    @property
    def height(self) -> int:
        return self.lib.am_get_height(self.h)

    def get_time(self, i: int, n: int) -> float:
        return self.lib.am_get_time(self.h, i, n)

    def render(self, t: float) -> np.ndarray:
        out = np.zeros((self.height, self.width, 4), np.uint8)
        _check(self.lib.am_render(self.h, t, out.ctypes.data, 0), "am_render")
        return out

    def blob_pixels(self, blob: int, t: float):
        """morph::get_pixels(blob, t): ([n, 2] x, y and [n, 4] RGBA) in the
        reference's order."""
        n = C.c_size_t()
        _check(self.lib.am_get_blob_pixels(self.h, blob, t, None, None, 0, C.byref(n)), "am_get_blob_pixels")
        xy = np.zeros((max(n.value, 1), 2), np.uint16)
        rgba = np.zeros((max(n.value, 1), 4), np.uint8)
        _check(self.lib.am_get_blob_pixels(self.h, blob, t, xy.ctypes.data_as(C.POINTER(C.c_uint16)), _p(rgba, u8p),
                                           n.value, C.byref(n)), "am_get_blob_pixels")
        return xy[:n.value], rgba[:n.value]

    def positions(self, t: float) -> np.ndarray:
        """[N, 2] position words (integer pixel * 256 + fraction byte) of every
        atom column at time t as the render places them; -1 where not drawn."""
        n = self.lib.am_get_positions(self.h, t, None, 0)
        out = np.zeros((max(n, 1), 2), np.int32)
        if n:
            got = self.lib.am_get_positions(self.h, t, _p(out, i32p), n)
            if got != n:
                raise AmError(AM_ERR_CUDA, "am_get_positions")
        return out[:n]

    def render_device(self, t: float, dev_ptr: int) -> None:
        _check(self.lib.am_render(self.h, t, dev_ptr, 1), "am_render")

    def refine(self, sweeps: int, proposal: int | None = None) -> np.ndarray:
        if proposal is not None:
            self.set(proposal=proposal)
        gains = np.zeros(max(sweeps, 1), np.uint64)
        _check(self.lib.am_refine(self.h, sweeps, _p(gains, u64p)), "am_refine")
        return gains[:sweeps]

    def export_chains(self):
        """(widths, pts[K*N], blob_order[K, C])."""
        Cn = self.chains
        N = self.atoms
        K = self.lib.am_get_frame_count(self.h)
        w = np.zeros(max(Cn, 1), np.uint64)
        pts = np.zeros(max(K * N, 1), np.uint64)
        order = np.zeros(max(K * Cn, 1), np.int32)
        _check(self.lib.am_export_chains(self.h, _p(w, u64p), _p(pts, u64p), _p(order, i32p)), "am_export_chains")
        return w[:Cn], pts[:K * N], order[:K * Cn].reshape(K, Cn)

    def import_chains(self, widths, pts, order) -> None:
        widths = np.ascontiguousarray(widths, np.uint64)
        pts = np.ascontiguousarray(pts, np.uint64)
        order = np.ascontiguousarray(order, np.int32)
        K = order.shape[0]
        _check(self.lib.am_import_chains(self.h, K, len(widths), _p(widths, u64p), _p(pts, u64p), _p(order, i32p)),
               "am_import_chains")

    # -- learned proposal -----------------------------------------------------
    def record_swaps(self, cap: int) -> None:
        _check(self.lib.am_record_swaps(self.h, cap), "am_record_swaps")

    def record_outcomes(self, cap: int, every: int = 1) -> None:
        """Plain sweeps log 1 in `every` proposals (pair features, 1 when the swap lowers the cost,
        else 0) for the learned pair proposal; cap 0 stops."""
        _check(self.lib.am_record_outcomes(self.h, cap, every), "am_record_outcomes")

    def recorded_count(self) -> int:
        return int(self.lib.am_recorded_swaps(self.h, None, None, 1 << 62))

    def recorded_swaps(self, cap: int):
        f = np.zeros((cap, 10), np.float32)
        t = np.zeros(cap, np.float32)
        n = self.lib.am_recorded_swaps(self.h, _p(f, f32p), _p(t, f32p), cap)
        return f[:n], t[:n]

    def train_proposal(self, feats, targets, epochs: int = 3, lr: float = 1e-3) -> float:
        feats = np.ascontiguousarray(feats, np.float32)
        targets = np.ascontiguousarray(targets, np.float32)
        loss = C.c_float()
        _check(self.lib.am_train_proposal(self.h, _p(feats, f32p), _p(targets, f32p), len(targets), epochs, lr,
                                          C.byref(loss)), "am_train_proposal")
        return loss.value

    def train_recorded(self, epochs: int = 3, lr: float = 1e-3) -> float:
        """Trains on the recorded samples in device memory; recording stops."""
        loss = C.c_float()
        _check(self.lib.am_train_recorded(self.h, epochs, lr, C.byref(loss)), "am_train_recorded")
        return loss.value

    def proposal_weights(self, w=None):
        if w is None:
            out = np.zeros(4929, np.float32)
            _check(self.lib.am_get_proposal_weights(self.h, _p(out, f32p), 4929), "am_get_proposal_weights")
            return out
        w = np.ascontiguousarray(w, np.float32)
        _check(self.lib.am_set_proposal_weights(self.h, _p(w, f32p), len(w)), "am_set_proposal_weights")
        return w

    def proposal_forward(self, feats):
        feats = np.ascontiguousarray(feats, np.float32)
        out = np.zeros(len(feats), np.float32)
        _check(self.lib.am_proposal_forward(self.h, _p(feats, f32p), len(feats), _p(out, f32p)), "am_proposal_forward")
        return out

    def proposal_grad(self, feats, targets):
        feats = np.ascontiguousarray(feats, np.float32)
        targets = np.ascontiguousarray(targets, np.float32)
        g = np.zeros(4929, np.float32)
        loss = C.c_float()
        _check(self.lib.am_proposal_grad(self.h, _p(feats, f32p), _p(targets, f32p), len(targets), _p(g, f32p),
                                         C.byref(loss)), "am_proposal_grad")
        return g, loss.value

    def profile(self, on: bool) -> None:
        _check(self.lib.am_profile_enable(self.h, 1 if on else 0), "am_profile_enable")

    def profile_read(self) -> dict:
        names = (C.c_char_p * 16)()
        ms = np.zeros(16)
        n = np.zeros(16, np.uint64)
        k = self.lib.am_profile_read(self.h, names, _p(ms, f64p), _p(n, u64p), 16)
        return {names[i].decode(): (float(ms[i]), int(n[i])) for i in range(k)}

    def heavy_tiles(self) -> tuple:
        """(heavy tiles of the last frame that had any, helper CTAs of the last
        resolve): tiles resolved in row bands by helper CTAs."""
        tiles, helpers = C.c_uint32(0), C.c_uint32(0)
        _check(self.lib.am_get_heavy_tiles(self.h, C.byref(tiles), C.byref(helpers)), "am_get_heavy_tiles")
        return tiles.value, helpers.value

    @property
    def stream(self) -> int:
        return self.lib.am_get_stream(self.h) or 0


def launch_count() -> int:
    return load().am_launch_count()


class Fluid:
    """The FP32 GPU fluid solver (counterpart of the reference's FluidModel)."""

    FIELDS = 18

    def __init__(self, gsx: int, gsy: int, n: int):
        self.lib = load()
        h = vp()
        _check(self.lib.am_fluid_create(C.byref(h), gsx, gsy, n), "am_fluid_create")
        self.h, self.n = h, n

    def close(self):
        if self.h:
            self.lib.am_fluid_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set(self, P: np.ndarray) -> None:
        """P: [18, n] fields (oracle order)."""
        q = np.ascontiguousarray(np.asarray(P, np.float64).T)
        _check(self.lib.am_fluid_set_particles(self.h, _p(q, f64p)), "am_fluid_set_particles")

    def get(self) -> np.ndarray:
        q = np.zeros((self.n, 18))
        _check(self.lib.am_fluid_get_particles(self.h, _p(q, f64p)), "am_fluid_get_particles")
        return q.T.copy()

    def step(self, steps_left: int, freedom_radius: float) -> None:
        _check(self.lib.am_fluid_step(self.h, steps_left, freedom_radius), "am_fluid_step")

    def steps(self, n: int, freedom_radius: float) -> None:
        _check(self.lib.am_fluid_steps(self.h, n, freedom_radius), "am_fluid_steps")

    def render(self, width: int, height: int, sparseness: float, bbox, t: float) -> np.ndarray:
        out = np.zeros((height, width, 4), np.uint8)
        bb = (C.c_uint32 * 4)(*[int(v) for v in bbox])
        _check(self.lib.am_fluid_render(self.h, width, height, sparseness, bb, t, _p(out, u8p)), "am_fluid_render")
        return out

    def render_ex(self, width: int, height: int, sparseness: float, bbox, t: float, feather: int = 0,
                  background: np.ndarray | None = None) -> np.ndarray:
        """draw_fluid with feather layers and keep_background over `background`."""
        out = np.zeros((height, width, 4), np.uint8)
        bb = (C.c_uint32 * 4)(*[int(v) for v in bbox])
        bg = None if background is None else np.ascontiguousarray(background, np.uint8)
        _check(self.lib.am_fluid_render_ex(self.h, width, height, sparseness, bb, t, feather,
                                           None if bg is None else _p(bg, u8p), _p(out, u8p)), "am_fluid_render_ex")
        return out


class Batch:
    """Batched refinement and rendering of many morph jobs (am_batch_*)."""

    def __init__(self, jobs):
        self.lib = load()
        self.jobs = list(jobs)  # keeps the handles alive
        arr = (vp * len(self.jobs))(*[j.h for j in self.jobs])
        h = vp()
        _check(self.lib.am_batch_create(C.byref(h), arr, len(self.jobs)), "am_batch_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.am_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def refine(self, sweeps: int) -> np.ndarray:
        """Runs `sweeps` plain sweeps of every job; returns gains [jobs, sweeps]."""
        g = np.zeros((len(self.jobs), sweeps), np.uint64)
        _check(self.lib.am_batch_refine(self.h, sweeps, _p(g, u64p)), "am_batch_refine")
        return g

    def refine_guided(self, sweeps: int) -> np.ndarray:
        """`sweeps` guided sweeps of every job; returns gains [jobs, sweeps]."""
        g = np.zeros((len(self.jobs), sweeps), np.uint64)
        _check(self.lib.am_batch_refine_guided(self.h, sweeps, _p(g, u64p)), "am_batch_refine_guided")
        return g

    def tune_schedule(self, sweeps: int) -> int:
        """Plain sweeps before the guided ones the autotuner picks for a budget."""
        n = C.c_size_t()
        _check(self.lib.am_batch_tune_schedule(self.h, sweeps, C.byref(n)), "am_batch_tune_schedule")
        return n.value

    def refine_schedule(self, sweeps: int) -> np.ndarray:
        g = np.zeros((len(self.jobs), sweeps), np.uint64)
        _check(self.lib.am_batch_refine_schedule(self.h, sweeps, _p(g, u64p)), "am_batch_refine_schedule")
        return g

    def render(self, ts) -> list:
        """Frames of every job at the times ts, batched; one [n, H, W, 4]
        uint8 array per job."""
        ts = np.ascontiguousarray(ts, np.float64)
        outs = [np.zeros((len(ts), j.height, j.width, 4), np.uint8) for j in self.jobs]
        arr = (vp * len(outs))(*[o.ctypes.data for o in outs])
        _check(self.lib.am_batch_render(self.h, _p(ts, f64p), len(ts), arr, 0), "am_batch_render")
        return outs

    def render_device(self, ts, dev_ptrs) -> None:
        """Frames of every job at the times ts into device buffers
        (dev_ptrs[j]: n frames of job j)."""
        ts = np.ascontiguousarray(ts, np.float64)
        arr = (vp * len(dev_ptrs))(*[int(d) for d in dev_ptrs])
        _check(self.lib.am_batch_render(self.h, _p(ts, f64p), len(ts), arr, 1), "am_batch_render")

    def tune(self, trial_sweeps: int = 3) -> dict:
        _check(self.lib.am_batch_tune(self.h, trial_sweeps), "am_batch_tune")
        return self.tuning

    @property
    def tuning(self) -> dict:
        v = [C.c_uint32(0) for _ in range(4)]
        _check(self.lib.am_batch_get_tuning(self.h, *[C.byref(x) for x in v]), "am_batch_get_tuning")
        return dict(threads=v[0].value, ctas_per_sm=v[1].value, chunk=v[2].value, order=v[3].value)

    def set_tuning(self, threads: int, ctas_per_sm: int, chunk: int, order: int) -> None:
        _check(self.lib.am_batch_set_tuning(self.h, threads, ctas_per_sm, chunk, order), "am_batch_set_tuning")
