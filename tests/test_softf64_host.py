"""The integer-pipe binary64 routines (softf64.cuh) compiled for the host
with g++ and checked bit for bit against the host's IEEE multiply, add,
fused multiply-add and power-of-two scaling (tests/softf64_check.cpp): the
device kernels rely on these routines returning exactly what the FP64
instructions return."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "py-orbit_gb300", "csrc")


@pytest.mark.skipif(shutil.which("g++") is None, reason="no host C++ compiler")
def test_soft_binary64_matches_ieee(tmp_path):
    exe = str(tmp_path / "softf64_check")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                           os.path.join(HERE, "softf64_check.cpp"), "-o", exe])
    out = subprocess.run([exe, "3000000"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0 and out.stdout.strip() == "0", out.stdout + out.stderr
