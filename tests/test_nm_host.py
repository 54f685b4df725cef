"""The device Nelder-Mead state machine (photic_gb300/csrc/photic_nm.cuh),
compiled for the host from the same source, reproduces the oracle's nelmin
(the restatement of model/asa047.c:10-502, itself pinned to the reference)
bit for bit: minimiser, minimum, evaluation and restart counts and fault
code, from random starts under the plain, the reference's and a short
tolerance, driven by the oracle's cost.  No GPU needed."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_state_machine_matches_oracle_nelmin(tmp_path, port):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "nm_host_check")
    oracle = os.path.join(ROOT, "oracle")
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off",
           "-I", os.path.join(ROOT, "photic_gb300", "csrc"), "-I", oracle,
           os.path.join(ROOT, "tests", "nm_host_check.cpp"), "-o", exe,
           "-L", oracle, "-lphotic_oracle", "-Wl,-rpath," + oracle, "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    for seed in (1, 2):
        r = subprocess.run([exe, "600", str(seed)], capture_output=True, text=True, timeout=600)
        print(r.stdout)
        assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr
