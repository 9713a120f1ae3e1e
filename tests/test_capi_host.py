"""C ABI checks that need no GPU: the library loads, exports every entry point
include/atomorph_gb300.h declares, and the host-side logic (ingestion,
settings, time mapping) behaves like the reference's am::morph."""
import ctypes as C
import subprocess

import numpy as np
import pytest

from atomorph_gb300 import synth


def test_exports_every_declared_symbol(capi):
    out = subprocess.run(["nm", "-D", "--defined-only", capi.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    declared = capi.declared_symbols()
    assert len(declared) > 50
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    lib = capi.load()
    for s in declared:
        assert getattr(lib, s) is not None


def test_ingest_counts_and_frames(capi):
    frames = synth.workload("ellipses64")
    m = capi.Morph()
    m.load(frames)
    assert m.lib.am_get_frame_count(m.h) == 2
    for k, img in enumerate(frames):
        assert m.pixel_count(k) == synth.opaque_count(img)
    assert (m.width, m.height) == (64, 64)
    # add_frame of an existing key fails (morph.cpp:288), a new key succeeds
    assert m.add_frame(0) == capi.AM_ERR_ARG
    assert m.add_frame(5) == capi.AM_OK
    assert m.pixel_count(5) == 0
    # overwriting a pixel keeps the count (std::map assignment, morph.cpp:310)
    before = m.pixel_count(0)
    ys, xs = np.nonzero(frames[0][..., 3])
    assert m.add_pixel(0, int(xs[0]), int(ys[0]), 1, 2, 3, 255) == capi.AM_OK
    assert m.pixel_count(0) == before
    assert m.add_pixel(0, 200, 3, 1, 2, 3, 255) == capi.AM_OK
    assert m.pixel_count(0) == before + 1


def test_get_time_and_frame_key(capi):
    m = capi.Morph()
    for k in (0, 3, 9):
        m.add_frame(k)
    # morph::get_time (morph.cpp:1522-1538)
    assert m.get_time(5, 10) == 0.5
    assert m.get_time(0, 0) == 0.0
    m.set(finite=1)
    assert m.get_time(0, 1) == pytest.approx((1 - 1 / 3) / 2)
    assert m.get_time(4, 5) == pytest.approx(1 - 1 / 3)
    # morph::get_frame_key (morph.cpp:404-423): t wraps into [0,1)
    lib = m.lib
    assert lib.am_get_frame_key(m.h, 0.0) == 0
    assert lib.am_get_frame_key(m.h, 0.5) == 3
    assert lib.am_get_frame_key(m.h, 0.9) == 9
    assert lib.am_get_frame_key(m.h, -0.1) == 9
    assert lib.am_get_frame_key(m.h, 1.4) == 3


def test_setter_validation_and_density_fluid_coupling(capi):
    m = capi.Morph()
    assert m.lib.am_set_motion(m.h, 99) == capi.AM_ERR_ARG
    assert m.lib.am_set_fading(m.h, 4) == capi.AM_ERR_ARG  # SPLINE is motion-only
    assert m.lib.am_set_proposal(m.h, 7) == capi.AM_ERR_ARG
    # set_fluid/set_density interplay (morph.cpp:1553-1570)
    m.set(density=2)
    m.set(fluid=10)
    m.set(density=3)  # density > 1 with fluid on turns the fluid off
    assert m.lib.am_set_fluid(m.h, 10) == capi.AM_OK
    # tunables: known names in range, unknown names and bad values refused
    for name, v in (("render_pipeline", 0), ("render_pipeline", 1), ("learned_keep", 0.5), ("guided_switch", 0)):
        assert m.lib.am_set_tuning(m.h, name.encode(), float(v)) == capi.AM_OK, name
    assert m.lib.am_set_tuning(m.h, b"no_such_knob", 1.0) == capi.AM_ERR_ARG
    assert m.lib.am_set_tuning(m.h, b"learned_keep", 0.0) == capi.AM_ERR_ARG
    assert m.lib.am_set_tuning(m.h, b"render_pipeline", -1.0) == capi.AM_ERR_ARG


def test_not_busy_without_work(capi):
    m = capi.Morph()
    assert m.lib.am_is_busy(m.h) == 0
    assert m.suspend(0.01) == capi.AM_OK
    assert m.state == capi.STATE_BLOB_DETECTION


def test_heavy_tiles_before_any_frame(capi):
    """No frame rendered: no heavy tiles noted, no helper CTAs launched; a
    null handle is rejected."""
    m = capi.Morph()
    assert m.heavy_tiles() == (0, 0)
    tiles, helpers = C.c_uint32(7), C.c_uint32(7)
    assert m.lib.am_get_heavy_tiles(None, C.byref(tiles), C.byref(helpers)) == capi.AM_ERR_ARG
    assert m.lib.am_get_heavy_tiles(m.h, None, None) == capi.AM_OK
