"""Drop-in check of the C++ boundary: the reference's own command-line
program (demo/main.cpp, unmodified, compiled from where it lies) builds
against include/atomorph_gb300.hpp and links with the GPU library; the only
change a caller makes is the include (here a one-line atomorph.h that
includes atomorph_gb300.hpp, placed where the demo's "../atomorph.h" looks).
Runs where the reference sources are present; the demo's --help runs
without a GPU."""
import os
import shutil
import subprocess

import pytest

REF = os.environ.get("ATOMORPH_REFERENCE", "/root/reference")  # the reference sources, where present
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "demo")) or shutil.which("g++") is None,
                    reason="reference demo sources or g++ not present")
def test_reference_demo_builds_and_runs_against_gb300_library(tmp_path):
    lib = os.path.join(ROOT, "atomorph_gb300", "lib", "libatomorph_gb300.so")
    if not os.path.exists(lib):
        pytest.skip("library not built")
    demo = tmp_path / "demo"
    demo.mkdir()
    for f in ("main.cpp", "main.h", "options.h", "lodepng.cpp", "lodepng.h"):
        os.symlink(os.path.join(REF, "demo", f), demo / f)  # compiled where it lies, not copied
    (tmp_path / "atomorph.h").write_text('#include "atomorph_gb300.hpp"\n')
    inc = os.path.join(ROOT, "include")
    objs = []
    for src in ("main.cpp", "lodepng.cpp"):
        obj = tmp_path / (src + ".o")
        subprocess.run(["g++", "-std=c++17", "-O1", "-c", str(demo / src), "-I", inc, "-o", str(obj)],
                       check=True, capture_output=True)
        objs.append(str(obj))
    exe = tmp_path / "atomorph"
    subprocess.run(["g++", *objs, "-L", os.path.dirname(lib), "-latomorph_gb300",
                    "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)], check=True, capture_output=True)
    r = subprocess.run([str(exe), "--help"], capture_output=True, text=True, timeout=60)
    assert "Usage:" in r.stdout and "--blob-feather" in r.stdout
