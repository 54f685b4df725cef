"""The double-precision exp and the divisions by known divisors that the
FP64 cost kernels use (photic_gb300/csrc/photic_fastmath.cuh), compiled for
the host from the same source: divisions bit for bit against IEEE division,
exp within 1 ulp of the host libm's exp (the reference's exp,
model/samodel.c:2899,2931,2934) and identical to it on at least 96 % of
arguments."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_fastmath_host(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "fastmath_check")
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp",
           "-I", os.path.join(ROOT, "photic_gb300", "csrc"),
           os.path.join(ROOT, "tests", "fastmath_check.cpp"), "-o", exe, "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    r = subprocess.run([exe, "18", "20"], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("OK")
