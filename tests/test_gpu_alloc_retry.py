"""A failed device allocation is reported once, as AM_ERR_NOMEM, and does not
fail the caller's next call: the runtime's pending error from the failed
cudaMalloc is taken off where the failure is handled."""
import ctypes as C

import numpy as np
import pytest

from atomorph_gb300 import synth

pytestmark = pytest.mark.gpu


def test_render_and_cost_after_a_failed_allocation(capi):
    frames = synth.workload("ellipses64")
    m = capi.Morph()
    m.load(frames, seed=7)
    assert m.run_until(capi.STATE_ATOM_MORPHING) == capi.STATE_ATOM_MORPHING
    first = m.render(0.4)
    cost = m.cost()
    # a fluid grid of 2^17 x 2^17 nodes (about 0.9 TB of node fields) cannot
    # be allocated on any current GPU
    h = C.c_void_p()
    rc = m.lib.am_fluid_create(C.byref(h), 1 << 17, 1 << 17, 16)
    assert rc == capi.AM_ERR_NOMEM and not h.value
    again = m.render(0.4)
    assert np.array_equal(first, again)
    assert m.cost() == cost
    # and a fluid frame of the morph itself allocates its own solver afresh
    m.set(fluid=2)
    out = np.zeros((m.height, m.width, 4), np.uint8)
    assert m.lib.am_render(m.h, 0.3, out.ctypes.data, 0) == capi.AM_OK, m.lib.am_last_error()
    assert out[..., 3].any()
    m.set(fluid=0)
    assert np.array_equal(m.render(0.4), first)
    m.close()
