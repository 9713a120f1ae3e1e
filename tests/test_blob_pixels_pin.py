"""The oracle's morph::get_pixels(blob, t) (morph.cpp:452-678) equals the
reference's own lists (tests/golden/blob_pixels.npz, made by the unmodified
reference) bit for bit, with feather 0 and 3."""
import numpy as np

from conftest import golden, golden_state


def test_oracle_blob_pixels_equal_reference(oracle):
    g = golden("features")
    z = golden("blob_pixels")
    for feather, ti, b, off, n in z["index"]:
        st = dict(golden_state(g), feather=int(feather))
        got = oracle.blob_pixels(st, int(b), float(z["ts"][ti]))
        assert got is not None
        assert np.array_equal(got[0], z["xy"][off:off + n])
        assert np.array_equal(got[1], z["rgba"][off:off + n])
