"""Build libphotic_gb300.so in-tree with nvcc for sm_103a.

The library is plain CUDA C++ behind the C ABI of include/photic.h.  The
translation units are compiled in parallel and linked with a static CUDA
runtime, so the .so has no dependency beyond the driver.  Every unit is
compiled with --fmad=false: no multiply-add pair is fused unless the
source asks for it with an explicit fma, which keeps the double-precision
path in the reference's rounding.  The host side gets -ffp-contract=off for
the same reason: GCC on aarch64 fuses a*b+c by default, which moved the
host-computed band constants and Rrs(440) off the reference's values by an
ulp.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libphotic_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["photic_host.cu", "photic_invert.cu", "photic_guarded.cu", "photic_joint.cu",
           "photic_joint_group.cu", "photic_region.cu",
           "photic_gemm.cu", "photic_mlp.cu", "photic_aux.cu", "photic_ncgrid.cu",
           "photic_scene.cu", "photic_lut.cu"]


def nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build photic_gb300")


def flags(extra=()):
    return (ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                    "-Xcompiler", "-O2", "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"] + list(extra))


def _compile(src: str, extra) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + flags(extra) + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps += [os.path.join(HERE, "..", "include", h) for h in ("photic.h", "photic_nc.h")]
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else [])
