"""The bulk FP32 running sum behind the sample graph's mean separation (thea_gb300/csrc/running_sum.cuh), compiled on
the host and checked bit for bit against the sequential loop (tests/cpp/running_sum_check.cpp)."""

import os
import subprocess

from tests.conftest import ROOT


def test_running_sum_matches_the_sequential_loop():
    src = os.path.join(ROOT, "tests", "cpp", "running_sum_check.cpp")
    out = os.path.join(ROOT, "tests", "cpp", "_build", "running_sum_check")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", src, "-o", out], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([out], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "matches the sequential loop" in r.stdout
