"""The reference-side bridge (integration/gb300_bridge.cpp) compiles against
the reference's own headers (v25/classes.hpp, v25/functions.hpp) and
include/mdsc.h, links against the reference's classes and functions and
libmdsc.so with every symbol resolved, and its host-side conversions
(pack / unpack in rev_II order, dipoles through the body frame) give the
particles back: tests/bridge_check.cpp.  No GPU is involved; skipped where
the reference's sources are absent."""
import os
import subprocess

import pytest

from conftest import REFERENCE, ROOT


def test_bridge_compiles_links_and_round_trips(tmp_path):
    v25 = os.path.join(REFERENCE, "v25")
    if not os.path.isdir(v25):
        pytest.skip("reference sources not present")
    from mdspherocyl_gb300 import build

    lib = build.build()
    libdir = os.path.dirname(lib)
    exe = str(tmp_path / "bridge_check")
    cmd = ["g++", "-O1", "-fopenmp", "-ffp-contract=off", "-w",
           "-I", os.path.join(ROOT, "oracle"),  # the gsl_rng stand-in
           "-I", v25, "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "bridge_check.cpp"),
           os.path.join(ROOT, "integration", "gb300_bridge.cpp"),
           os.path.join(v25, "classes.cpp"), os.path.join(v25, "functions.cpp"), os.path.join(v25, "jacobi.c"),
           "-L", libdir, "-lmdsc", f"-Wl,-rpath,{libdir}", "-Wl,--no-undefined", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60, cwd=str(tmp_path))
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert "round trip OK" in r.stdout
