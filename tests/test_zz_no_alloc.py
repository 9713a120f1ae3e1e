"""am_get_cost_noalloc (static device scratch, no allocation) against
am_get_cost on the same chains: exact integers, so equal bit for bit, on two
calls in a row and again after the chains change.  This file is collected
last; it also passes alone in a fresh process."""
import ctypes as C

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
