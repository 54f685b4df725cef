"""The link-compatible samodel entry points (include/photic_samodel.h).

CPU checks: the header's model_data / geogrid / scene layouts equal the
reference's model/common.h field for field (compile-time asserts; needs the
reference headers, skipped where they are absent), and the C driver that the
GPU tests run compiles and links against the library's exports.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_MODEL = os.environ.get("PHOTIC_REFERENCE_MODEL_DIR",
                           os.path.join(os.sep, "root", "reference", "model"))
LIB_DIR = os.path.join(ROOT, "photic_gb300")


def _cc():
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    return cc


def test_struct_layouts_match_reference(tmp_path):
    if not os.path.isfile(os.path.join(REF_MODEL, "common.h")):
        pytest.skip("reference headers not present")
    r = subprocess.run([_cc(), "-std=c11", "-c", "-I", REF_MODEL, "-I",
                        os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "dropin", "layout_check.c"),
                        "-o", str(tmp_path / "lc.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def build_driver(out_dir):
    """Compile tests/dropin/dropin_driver.c against the in-tree library."""
    lib = os.path.join(LIB_DIR, "libphotic_gb300.so")
    if not os.path.isfile(lib):
        pytest.skip("libphotic_gb300.so not built")
    exe = os.path.join(str(out_dir), "dropin_driver")
    r = subprocess.run([_cc(), "-std=c11", "-O2", "-Wall", "-Werror", "-I",
                        os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "dropin", "dropin_driver.c"), "-o", exe,
                        "-L", LIB_DIR, "-lphotic_gb300", "-Wl,-rpath," + LIB_DIR, "-lm"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_driver_links(tmp_path):
    build_driver(tmp_path)
