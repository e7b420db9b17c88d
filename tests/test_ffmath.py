"""The conditioning's Box-Muller pair in float-float (csrc/ffmath.cuh) against the
double evaluation, on the host: the header compiles for the host with the same
float operations, and every pair its rounding test accepts must round to the
double evaluation's floats (tests/ffmath_check.cpp)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_float_float_normal_pair_rounds_as_double(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "ffmath_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe,
                    os.path.join(HERE, "ffmath_check.cpp"), "-lm"], check=True)
    r = subprocess.run([exe, "3000000"], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
