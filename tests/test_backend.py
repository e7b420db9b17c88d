"""The C++ batch backend (include/gpis_backend.hpp over gpis_backend_*): the
check program compiles against the header here; on a GPU it runs and compares
submitBatch replies with gpis_flights_trace_host on the same flights."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "backend_check.cpp")
BUILD = os.path.join(ROOT, "gpis_extend_gb300", "_build")


def build_check():
    from gpis_extend_gb300 import build
    lib = build.build()
    exe = os.path.join(BUILD, "backend_check")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
                           lib, "-Wl,-rpath," + BUILD, "-lpthread"])
    return exe


def test_backend_check_compiles():
    assert os.path.exists(build_check())


@pytest.mark.gpu
def test_backend_replies_match_trace_host():
    exe = build_check()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout, r.stderr)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr
