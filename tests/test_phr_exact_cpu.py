"""The exact-float64 helpers of the PHR sweep (trace_gb300/csrc/phr_exact.cuh),
compiled for the host and checked against float64 arithmetic: the barycenter
key bits over edge cases and random pairs, and the float32 cost bound the
sweep's screening relies on."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "trace_gb300", "csrc")


def test_phr_exact_helpers(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "phr_exact_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                    os.path.join(HERE, "cpp", "phr_exact_check.cpp"), "-o", exe, "-lm"], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr
