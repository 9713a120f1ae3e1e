"""Builds the atomorph_gb300 CUDA library in-tree for sm_103a.

    python -m atomorph_gb300.build

Every translation unit is compiled by nvcc in parallel with
``-gencode arch=compute_103a,code=sm_103a`` and linked into
``atomorph_gb300/lib/libatomorph_gb300.so``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "lib")
LIB = os.path.join(OUT, "libatomorph_gb300.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code keeps every double operation separately rounded (no FMA
# contraction), as the reference's x86 build evaluates it.
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")]

# (source, extra flags).  Colour conversion must round every multiply and add
# separately to reproduce the reference's bytes, so it is built without FMA
# contraction.
UNITS = [
    ("k_colour.cu", ["-fmad=false"]),
    ("k_chains.cu", []),
    ("k_render.cu", []),
    ("k_blobs.cu", []),
    ("k_local.cu", []),
    ("k_mlp.cu", []),
    ("engine.cpp", ["-x", "cu"]),
    ("engine_mlp.cpp", ["-x", "cu"]),
    ("k_fluid.cu", []),
    ("k_fluid_morph.cu", []),
    ("noalloc.cu", []),
    ("k_batch.cu", []),
    ("engine_batch.cpp", ["-x", "cu"]),
    ("capi_batch.cpp", ["-x", "cu", "-Xcompiler", "-fvisibility=default"]),
    ("capi.cpp", ["-x", "cu", "-Xcompiler", "-fvisibility=default"]),
    ("capi_fluid.cpp", ["-x", "cu", "-Xcompiler", "-fvisibility=default"]),
]


def _compile(unit):
    src, extra = unit
    obj = os.path.join(OUT, "obj", src + ".o")
    cmd = [NVCC, *ARCH, *COMMON, *extra, "-c", os.path.join(SRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return src, r.returncode, r.stdout + r.stderr


def build(verbose: bool = False) -> str:
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(UNITS), os.cpu_count() or 4)) as ex:
        results = list(ex.map(_compile, UNITS))
    failed = [(s, log) for s, rc, log in results if rc != 0]
    for s, rc, log in results:
        if verbose or rc:
            sys.stderr.write(f"--- {s} (rc={rc})\n{log}")
    if failed:
        raise RuntimeError("nvcc failed for: " + ", ".join(s for s, _ in failed))
    objs = [os.path.join(OUT, "obj", s + ".o") for s, _ in UNITS]
    tmp = LIB + ".tmp"
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
