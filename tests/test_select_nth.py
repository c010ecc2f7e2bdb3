"""The libstdc++-order selection used by the ShapeDiameter kernel (thea_gb300/csrc/select_nth.cuh), compiled on the host
and checked element for element against this C++ library's std::nth_element (tests/cpp/select_nth_check.cpp)."""

import os
import subprocess

from tests.conftest import ROOT


def test_select_nth_matches_std_nth_element():
    src = os.path.join(ROOT, "tests", "cpp", "select_nth_check.cpp")
    out = os.path.join(ROOT, "tests", "cpp", "_build", "select_nth_check")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    r = subprocess.run(["g++", "-std=c++17", "-O1", src, "-o", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "matches std::nth_element" in r.stdout
