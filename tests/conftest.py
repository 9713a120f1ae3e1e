import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as orc
    if not os.path.exists(os.path.join(orc.HERE, "liboracle.so")):
        orc.build(with_ref=False)
    return orc.Oracle()


@pytest.fixture(scope="session")
def capi():
    from atomorph_gb300 import capi as capi_mod
    if not os.path.exists(capi_mod.LIB_PATH):
        from atomorph_gb300 import build
        build.build()
    capi_mod.load()
    return capi_mod


def golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def golden_state(g: dict, pts_key: str = "pts") -> dict:
    """Morph-state dict (oracle renderer input) of a golden morph case."""
    return dict(K=int(g["K"]), width=int(g["width"]), height=int(g["height"]), bbox=g["bbox"],
                seed=int(g["seed"]), motion=int(g["motion"]), fading=int(g["fading"]),
                delimiter=int(g["delimiter"]), density=int(g["density"]), colors=g["colors"], present=g["present"],
                widths=g["widths"], pts=g[pts_key], blob_order=g["blob_order"],
                frame_keys=np.arange(int(g["K"]), dtype=np.uint64))


def morph_from_golden(capi_mod, g: dict, pts_key: str = "pts"):
    """A GPU handle with the golden case's key frames, settings and chains."""
    m = capi_mod.Morph()
    m.load(list(g["frames"]), seed=int(g["seed"]), blob_delimiter=int(g["delimiter"]), motion=int(g["motion"]),
           fading=int(g["fading"]), density=int(g["density"]))
    m.import_chains(g["widths"], g[pts_key], g["blob_order"])
    return m
