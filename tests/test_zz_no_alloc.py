"""am_get_cost_noalloc (static device scratch, no allocation) against
am_get_cost on the same chains: exact integers, so equal bit for bit, on two
calls in a row and again after the chains change.  This file is collected
last; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from atomorph_gb300 import synth

pytestmark = pytest.mark.gpu


def _both(capi, m):
    ref = C.c_uint64(0)
    assert m.lib.am_get_cost(m.h, C.byref(ref), None) == capi.AM_OK
    got = []
    for _ in range(2):
        v = C.c_uint64(0)
        rc = m.lib.am_get_cost_noalloc(m.h, C.byref(v))
        assert rc == capi.AM_OK, m.lib.am_last_error()
        got.append(v.value)
    return ref.value, got


@pytest.mark.parametrize("workload,kw", [
    ("ellipses64", dict(seed=1)),
    ("shapes256", dict(seed=3, blob_delimiter=0)),
])
def test_noalloc_cost_matches_existing_entry_point(capi, workload, kw):
    frames = synth.workload(workload)
    m = capi.Morph()
    m.load(frames, **kw)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    ref, got = _both(capi, m)
    assert ref > 0 and got == [ref, ref], (ref, got)
    m.refine(40)
    ref2, got2 = _both(capi, m)
    assert ref2 < ref and got2 == [ref2, ref2], (ref2, got2)
    m.close()


def test_noalloc_cost_of_an_empty_handle_is_zero(capi):
    m = capi.Morph()
    v = C.c_uint64(7)
    assert m.lib.am_get_cost_noalloc(m.h, C.byref(v)) == capi.AM_OK
    assert v.value == 0
    assert m.lib.am_get_cost_noalloc(m.h, None) == capi.AM_ERR_ARG
    m.close()


def _synthetic_chains(rng, K, widths, size=64):
    """Random points (8-byte point words, HAS_PIXEL set) for chains of the
    given widths over K key frames, frame-major."""
    N = int(sum(widths))
    x = rng.integers(0, size, (K, N), dtype=np.uint64)
    y = rng.integers(0, size, (K, N), dtype=np.uint64)
    xf = rng.integers(0, 256, (K, N), dtype=np.uint64)
    yf = rng.integers(0, 256, (K, N), dtype=np.uint64)
    flags = np.uint64(1) << np.uint64(48)
    pts = x | (y << np.uint64(16)) | (xf << np.uint64(32)) | (yf << np.uint64(40)) | flags
    return np.ascontiguousarray(pts.reshape(-1))


@pytest.mark.parametrize("N", [4779, 5461])  # N x 3 key frames = 2048 x 7 + 1 and 2048 x 8 - 1 columns
def test_noalloc_cost_at_chunk_boundaries_with_width_one_chains(capi, oracle, N):
    """Totals one column past and one short of a whole number of 2048-column
    chunks, with chains of width 1 (which cost nothing, thread.cpp:1113)
    spread through the layout: equal to am_get_cost and to the oracle."""
    rng = np.random.default_rng(N)
    K = 3
    frames = [synth.ellipses_frame(64, 3, 4.0, 12.0, rng) for _ in range(K)]
    rest = N - 6
    widths = np.array([1, rest // 2, 1, 1, rest - rest // 2, 1, 1, 1], np.uint64)
    widths = widths[widths > 0]
    assert int(widths.sum()) == N
    pts = _synthetic_chains(rng, K, widths)
    order = np.tile(np.arange(len(widths), dtype=np.int32), (K, 1))
    m = capi.Morph()
    m.load(frames, seed=2)
    m.import_chains(widths, pts, order)
    ref, got = _both(capi, m)
    assert got == [ref, ref], (ref, got)
    assert ref == oracle.energy(pts, widths, K)[1]
    m.close()


def test_noalloc_cost_rejects_chains_beyond_its_scratch(capi):
    """2^27 + 2 columns (one chain of 2^26 + 1 atoms over 2 key frames) is
    past the static scratch: AM_ERR_ARG with a message, before any device
    work; the allocating entry point still answers."""
    rng = np.random.default_rng(5)
    frames = [synth.ellipses_frame(64, 2, 4.0, 12.0, rng) for _ in range(2)]
    N = (1 << 26) + 1
    pts = np.full(2 * N, np.uint64(1) << np.uint64(48), np.uint64)
    m = capi.Morph()
    m.load(frames, seed=2)
    m.import_chains(np.array([N], np.uint64), pts, np.zeros((2, 1), np.int32))
    v = C.c_uint64(7)
    assert m.lib.am_get_cost_noalloc(m.h, C.byref(v)) == capi.AM_ERR_ARG
    assert b"columns" in m.lib.am_last_error()
    assert v.value == 7
    assert m.cost() == 0
    m.close()


def test_noalloc_cost_keeps_the_callers_current_device(capi):
    """The call makes the handle's device current while it runs and puts the
    calling thread's current device back."""
    import torch
    frames = synth.workload("ellipses64")
    m = capi.Morph()
    m.load(frames, seed=1)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    before = torch.cuda.current_device()
    v = C.c_uint64(0)
    assert m.lib.am_get_cost_noalloc(m.h, C.byref(v)) == capi.AM_OK
    assert torch.cuda.current_device() == before
    m.close()
