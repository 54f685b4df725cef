"""The relink recipe: photic's own objects, minus model/samodel.c, linked
against libphotic_gb300.so.

The reference builds its program with one compiler line over every source
file (model/makefile:14-15).  Replacing the inversion means taking
samodel.c off that line and linking this library; asa047.c stays, because
model/align.c:377, 437 call nelmin2 / nelmin3 from model/asa047.c:512, 1013.
The test compiles every other reference object from its own sources (the
netCDF and PGPLOT libraries, absent here, are stood in for by
oracle/ref_ncstub.c and tests/dropin/pgplot_stub.c), replaces bam.c -- which
does not compile as shipped -- by a caller making bam.c's samodel() call,
and links: no undefined and no duplicate symbol may remain, and the
inversion entry points must resolve to the library.  CPU only; skipped
where the reference sources are absent."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# the reference's program minus samodel.c (replaced) and bam.c (does not
# compile as shipped; relink_caller.c makes its samodel call)
KEEP = ["common", "nc", "io", "graphics", "colours", "interp", "filllakesutils", "smoothutils",
        "jerlov", "secchi", "linenoise", "asa047", "samodelgraphics", "align", "process",
        "refine", "write", "plot"]


def _ref_model_dir():
    from oracle import oracle as O
    d = os.path.join(O.REFERENCE_ROOT, "model")
    return d if os.path.isfile(os.path.join(d, "samodel.c")) else None


def test_reference_program_relinks_against_the_library(tmp_path):
    model = _ref_model_dir()
    if model is None:
        pytest.skip("reference sources absent")
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no C compiler")
    from photic_gb300 import _lib
    lib = _lib.LIB_PATH
    if not os.path.exists(lib):
        pytest.skip("libphotic_gb300.so not built")
    stub = os.path.join(ROOT, "oracle", "stub")
    flags = ["-O1", "-std=gnu99", "-fcommon", "-w", "-I", stub, "-I", model]
    objs = []
    srcs = [os.path.join(model, f + ".c") for f in KEEP]
    srcs += [os.path.join(ROOT, "oracle", "ref_ncstub.c"),
             os.path.join(ROOT, "tests", "dropin", "pgplot_stub.c"),
             os.path.join(ROOT, "tests", "dropin", "relink_caller.c")]
    for s in srcs:
        o = str(tmp_path / (os.path.basename(s)[:-2] + ".o"))
        r = subprocess.run([cc] + flags + ["-c", s, "-o", o], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        objs.append(o)
    exe = str(tmp_path / "photic_relinked")
    libdir = os.path.dirname(lib)
    r = subprocess.run([cc, "-o", exe] + objs +
                       ["-L", libdir, "-lphotic_gb300", f"-Wl,-rpath,{libdir}", "-lm",
                        "-fopenmp"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr  # undefined or duplicate symbols fail here
    # the inversion's entry points come from the library, not from the objects
    r = subprocess.run(["nm", "-D", "--undefined-only", exe], capture_output=True, text=True)
    undefined = {ln.split()[-1].split("@")[0] for ln in r.stdout.splitlines() if ln.strip()}
    assert "samodel" in undefined
    r = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True)
    exported = {ln.split()[-1] for ln in r.stdout.splitlines() if ln.strip()}
    assert "samodel" in exported
    # nelmin2 / nelmin3 (align.c's optimiser) stay with the reference's asa047
    r = subprocess.run(["nm", exe], capture_output=True, text=True)
    assert " T nelmin2" in r.stdout and " T nelmin3" in r.stdout
