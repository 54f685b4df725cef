"""The C-ABI library: it loads, exports every function include/photic.h
declares, and its host-side set-up agrees with the oracle.  No GPU needed
(only host functions are called)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(photic_[a-z0-9_]+|samodel[a-z_]*|read_nc|write_nc)\s*\(",
                                 txt)))


@pytest.fixture(scope="module")
def lib():
    from photic_gb300 import _lib
    return _lib.lib()


def test_exports_every_declared_symbol(lib):
    for h in os.listdir(os.path.join(ROOT, "include")):
        for name in _declared(h):
            assert hasattr(lib, name), f"{name} declared in include/{h} but not exported"


def test_config_defaults_and_validation(lib):
    from photic_gb300 import _lib as L
    c = L.photic_config()
    lib.photic_config_default(C.byref(c))
    assert c.n_bands == 4 and c.kcount == 2000 and c.konvge == 100 and c.reqmin == 1e-10
    assert list(c.hstarts[:8]) == [40.0, 30.0, 20.0, 15.0, 10.0, 7.5, 2.5, 1.0]
    assert lib.photic_config_check(C.byref(c)) == 0
    c.reqmin = 0.0  # nelmin's ifault 1 condition
    assert lib.photic_config_check(C.byref(c)) == L.ERR_INVALID
    assert b"reqmin" in lib.photic_last_error()
    lib.photic_config_default(C.byref(c))
    c.n_bands = 9
    assert lib.photic_config_check(C.byref(c)) == L.ERR_INVALID


def test_interp_matches_oracle(lib, port):
    X = np.array([443.0, 482.0, 561.0, 655.0])
    Y = np.array([0.011, 0.013, 0.009, 0.001])
    Xp = X.ctypes.data_as(C.POINTER(C.c_double))
    Yp = Y.ctypes.data_as(C.POINTER(C.c_double))
    for x in [400.0, 440.0, 443.0, 482.0, 490.0, 550.0, 640.0, 655.0, 750.0]:
        assert lib.photic_interp_1d(Xp, Yp, 4, x) == port.interp_1d(X, Y, x)


@pytest.mark.parametrize("theta", [35.0, 25.0, 50.0])
def test_band_constants_match_oracle(lib, port, theta):
    import photic_gb300
    cfg = photic_gb300.Config(theta_sun_deg=theta).to_c()
    out = np.zeros((4, 8))
    assert lib.photic_band_constants(C.byref(cfg), out.ctypes.data_as(C.POINTER(C.c_double))) == 0
    np.testing.assert_array_equal(out, port.band_constants(theta_sun=theta))


def test_headers_are_plain_c(tmp_path):
    """The public headers compile as C99 (-pedantic) and as C++: callers in
    the reference's own language include them unchanged."""
    import shutil
    import subprocess
    src = tmp_path / "h.c"
    src.write_text('#include "photic.h"\n#include "photic_nc.h"\n#include "photic_samodel.h"\n'
                   "int main(void) { photic_nc_grid_info i; (void)i; return PHOTIC_ERR_IO; }\n")
    inc = os.path.join(ROOT, "include")
    cc, cxx = shutil.which("gcc") or shutil.which("cc"), shutil.which("g++")
    if cc is None or cxx is None:
        pytest.skip("no C / C++ compiler")
    for cmd in ([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror"],
                [cxx, "-std=c++11", "-Wall", "-Werror", "-x", "c++"]):
        r = subprocess.run(cmd + ["-fsyntax-only", "-I", inc, str(src)], capture_output=True,
                           text=True)
        assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("lbo,sbo", [(0, 1024), (128, 0), (120, 1024), (128, 1000),
                                     (128, 1040), (16384, 16), (-128, 1024)])
def test_gemm_strides_outside_the_tile_are_refused(lib, lbo, sbo):
    """Core-matrix strides that would point the tensor core outside the
    staged shared-memory tile are rejected on the host, before any device
    work (the pointers below are never dereferenced)."""
    from photic_gb300 import _lib as L
    fake = 1 << 20  # 16-byte aligned, never touched
    rc = lib.photic_gemm_bf16_strides(fake, 64, fake, 64, fake, 128, 128, 128, 64, lbo, sbo,
                                      None)
    assert rc == L.ERR_INVALID
    assert b"stride" in lib.photic_last_error()


def test_lookup_table_arguments_are_checked(lib):
    """photic_lut_invert_batch refuses what it cannot run before it touches
    the device: no configuration, an empty table, a negative chain count,
    and every precision but FP64; an empty batch is a no-op."""
    from photic_gb300 import _lib as L
    c = L.photic_config()
    lib.photic_config_default(C.byref(c))
    lc = L.photic_lut_config()
    lib.photic_lut_config_default(C.byref(lc))
    assert lc.n_lut == 16000 and lc.n_chains == 0 and lc.use_noise == 0
    o = L.photic_outputs()
    n_sh, n_ch = C.c_int64(7), C.c_int64(7)
    dummy = C.c_void_p(16)  # never dereferenced: the checks come first

    def call(cfg, lut, npix=4):
        return lib.photic_lut_invert_batch(C.byref(cfg), lut, dummy, npix, None, 0.0,
                                           C.byref(o), None, None, None, C.byref(n_sh),
                                           C.byref(n_ch), None)

    assert call(c, None) == L.ERR_INVALID
    lc.n_lut = 0
    assert call(c, C.byref(lc)) == L.ERR_INVALID
    lc.n_lut, lc.n_chains = 16000, -1
    assert call(c, C.byref(lc)) == L.ERR_INVALID
    lc.n_chains = 0
    for prec in (L.PREC_DF64, L.PREC_FP32, L.PREC_GUARDED):
        c.precision = prec
        assert call(c, C.byref(lc)) == L.ERR_UNSUPPORTED
        assert b"FP64" in lib.photic_last_error()
    c.precision = L.PREC_FP64
    assert call(c, C.byref(lc), npix=0) == L.OK
    assert n_sh.value == 0 and n_ch.value == 0


def test_general_lookup_table_arguments_are_checked(lib):
    """photic_region_lut_invert_batch refuses unsupported configurations
    and bad table settings before it touches the device; an empty grid is a
    no-op."""
    from photic_gb300 import _lib as L
    c = L.photic_config()
    lib.photic_config_default(C.byref(c))
    lc = L.photic_lut_config()
    lib.photic_lut_config_default(C.byref(lc))
    o = L.photic_outputs()
    n_sh, n_ch = C.c_int64(7), C.c_int64(7)
    dummy = C.c_void_p(16)  # never dereferenced: the checks come first
    th = (C.c_double * 2)(35.0, 40.0)

    def call(cfg, lut, S=1, ns=2, nbt=3, nrows=4, ncols=4):
        return lib.photic_region_lut_invert_batch(C.byref(cfg), lut, dummy, S, th, nrows, ncols,
                                                  ns, nbt, None, None, 0.0, C.byref(o), None,
                                                  None, None, C.byref(n_sh), C.byref(n_ch), None)

    assert call(c, C.byref(lc), ns=3) == L.ERR_UNSUPPORTED
    assert call(c, C.byref(lc), nbt=4) == L.ERR_UNSUPPORTED
    assert call(c, C.byref(lc), S=9) == L.ERR_UNSUPPORTED
    assert call(c, C.byref(lc), S=4) == L.ERR_UNSUPPORTED  # 9 regions x 4 scenes x 4 bands > 128
    assert call(c, None) == L.ERR_INVALID
    lc.n_lut = 0
    assert call(c, C.byref(lc)) == L.ERR_INVALID
    lc.n_lut = 16000
    c.precision = L.PREC_DF64
    assert call(c, C.byref(lc)) == L.ERR_UNSUPPORTED
    c.precision = L.PREC_FP64
    assert call(c, C.byref(lc), nrows=0) == L.OK
    assert n_sh.value == 0 and n_ch.value == 0
