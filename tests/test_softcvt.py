"""The integer FP64<->FP32 conversions (mdspherocyl_gb300/csrc/softcvt.cuh)
against the IEEE casts, on the CPU: truncating FP64->FP32 bit for bit,
exact FP32->FP64, the two-float split of an FP64 value to 2^-47, and
floor(y) modulo 2^32 (the fixed-point coordinate), over 2e6 random values
across 120 binades."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_soft_conversions(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "softcvt_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-o", str(exe), os.path.join(HERE, "softcvt_check.cpp")],
                   check=True, capture_output=True, timeout=120)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 mismatches" in r.stdout
