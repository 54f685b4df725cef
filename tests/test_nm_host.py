"""The device Nelder-Mead state machines, compiled for the host from the same
sources, reproduce the oracle's nelmin (the restatement of
model/asa047.c:10-502, itself pinned to the reference) bit for bit:
minimiser, minimum, evaluation and restart counts and fault code.

* photic_nm.cuh (one lane per pixel, the plain inversion): from random
  starts under the plain, the reference's and a short tolerance, driven by
  the oracle's cost.
* photic_nmgroup.cuh (a group of G lanes per pixel, the temporal and region
  fits): the lanes run one after another at each step; the photic cost at
  n = 6 with one and two coordinates per lane, and coupled valley costs at
  n = 9..33 with one to three coordinates per lane; every lane must take the
  same decisions.
No GPU needed."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(tmp_path, source):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / os.path.splitext(source)[0])
    oracle = os.path.join(ROOT, "oracle")
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off",
           "-I", os.path.join(ROOT, "photic_gb300", "csrc"), "-I", oracle,
           os.path.join(ROOT, "tests", source), "-o", exe,
           "-L", oracle, "-lphotic_oracle", "-Wl,-rpath," + oracle, "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def _run_ok(exe, *args):
    r = subprocess.run([exe, *args], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr


def test_state_machine_matches_oracle_nelmin(tmp_path, port):
    exe = _build(tmp_path, "nm_host_check.cpp")
    for seed in (1, 2):
        _run_ok(exe, "600", str(seed))


def test_group_state_machine_matches_oracle_nelmin(tmp_path, port):
    exe = _build(tmp_path, "nmgroup_host_check.cpp")
    for seed in (1, 2):
        _run_ok(exe, "12", str(seed))
