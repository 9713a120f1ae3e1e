"""The transport-cost bar on a C2-size job: every GPU refinement form ends
within 0.5% of the reference's converged cost from the same chains.

shapes256 (2 key frames of 256x256, about 42k atoms, HSP delimiter): the
chains come from the deterministic CPU pipeline (oracle.pipeline; their
checksum is pinned in tests/golden/converge256.npz), the reference's
converged cost from the unmodified reference library's own morph_asynch
(thread.cpp:990-1041) run to a plateau on those chains.  Each GPU form runs
in blocks until a window of sweeps gains less than 2e-5 of its cost."""
import numpy as np
import pytest

from atomorph_gb300 import synth
from conftest import golden
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

BAR = 1.005          # within 0.5% of the reference's converged cost
WINDOW = 4000        # sweeps per plateau check
REL = 2e-5
MAX_SWEEPS = 120000


def _chains(oracle):
    frames = synth.workload("shapes256")
    st = orc.pipeline(oracle, frames, delimiter=1, density=1, seed=5, motion=4, fading=6)
    return frames, st


def _run_to_plateau(m, kind, B=500):
    c = m.cost()
    trace = [(0, c)]
    sweeps = 0
    while sweeps < MAX_SWEEPS:
        g = m.refine(B, kind)
        sweeps += B
        c -= int(g.sum())
        trace.append((sweeps, c))
        back = next((tr for tr in reversed(trace) if tr[0] <= sweeps - WINDOW), None)
        if back is not None and back[1] - c < REL * c:
            break
    assert m.cost() == c
    return c, sweeps, trace


@pytest.mark.parametrize("kind", ["plain", "guided"])
def test_converged_cost_within_half_percent_of_reference(capi, oracle, kind):
    g = golden("converge256")
    frames, st = _chains(oracle)
    pts = st["pts"]
    chk = int(np.bitwise_xor.reduce(pts * np.uint64(0x9E3779B97F4A7C15)))
    assert chk == int(g["pts_checksum"]) and np.array_equal(st["widths"], g["widths"])
    m = capi.Morph()
    m.load(frames, seed=5, blob_delimiter=1, motion=4, fading=6, density=1)
    m.import_chains(st["widths"], pts, st["blob_order"])
    assert m.cost() == int(g["initial_cost"])
    ref = int(g["converged_cost"])
    k = capi.PROPOSAL_RANDOM if kind == "plain" else capi.PROPOSAL_LOCAL
    c, sweeps, trace = _run_to_plateau(m, k)
    hit = next((s for s, v in trace if v <= BAR * ref), None)
    print(f"{kind}: converged {c} in {sweeps} sweeps ({c / ref:.5f} x reference's {ref}); "
          f"within 0.5% after {hit} sweeps")
    assert c <= BAR * ref, (c, ref, c / ref)
    w, p2, order = m.export_chains()
    assert oracle.energy(p2, w, 2)[1] == c
    m.close()
