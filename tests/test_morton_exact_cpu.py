"""The float32-pair Morton quantisation (trace_gb300/csrc/morton_exact.cuh),
compiled for the host and checked against the reference's float64 formula on
random and near-integer triangle bounds in offset, tiny and wide scenes."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "trace_gb300", "csrc")


def test_morton_exact_helpers(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "morton_exact_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                    os.path.join(HERE, "cpp", "morton_exact_check.cpp"), "-o", exe, "-lm"], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr
    decided, deferred, plain, plain_deferred = map(int, out.stdout.split()[1:5])
    assert decided > 0
    # random bounds in scenes near the origin: the float32 path decides nearly all
    assert plain > 0 and plain_deferred <= 0.001 * plain, out.stdout
