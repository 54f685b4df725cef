"""ctypes front end of the CPU oracles (test infrastructure only).

Two libraries sit behind the same calls:

* ``port``      -- oracle/libphotic_oracle.so, the C restatement in
                   photic_oracle.c of the reference's samodel_Rrs /
                   samodel_error / nelmin / samodel_optimise.  It builds on
                   any host and is the oracle on the GPU machine.
* ``reference`` -- oracle/_ref/libphotic_ref.so, the reference's own
                   model/samodel.c, asa047.c and common.c compiled in place
                   (only where the reference sources are available).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this
module; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "libphotic_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libphotic_ref.so")
NOUT = 44

# Output record columns shared by the oracles and the GPU path.
COL = dict(H=0, B=1, cost=2, rrs_error=3, K_min=4, iod=5, evals_kept=6, evals=7,
           converged=8, status=9, n_scenes=10, P=11, G=19, X=27, restarts=35,
           kept_start=36, ifault=37)

OLI_BANDS = (443.0, 482.0, 561.0, 655.0)
DEFAULT_HSTARTS = (40.0, 30.0, 20.0, 15.0, 10.0, 7.5, 2.5, 1.0)

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)
_i32p = C.POINTER(C.c_int32)


# Where the reference checkout is read from when the reference is compiled
# in place (PHOTIC_REFERENCE overrides; absent on machines without it).
REFERENCE_ROOT = os.environ.get("PHOTIC_REFERENCE", "/root/reference")


def build(ref: bool = True) -> None:
    """Compile the port (and the reference harness when its sources exist)."""
    targets = ["all"] if ref else ["libphotic_oracle.so"]
    ref_dir = os.path.join(REFERENCE_ROOT, "model")
    extra = [f"REF_DIR={ref_dir}"] if ref and os.path.isfile(os.path.join(ref_dir, "samodel.c")) \
        else []
    subprocess.run(["make", "-s", "-C", HERE] + targets + extra, check=True)


def _ptr(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class _Lib:
    def __init__(self, path: str, prefix: str):
        self.path = path
        self.lib = C.CDLL(path)
        self.prefix = prefix

    def fn(self, name):
        return getattr(self.lib, self.prefix + name)


_port = None
_ref = None


def port() -> _Lib:
    global _port
    if _port is None:
        if not os.path.exists(PORT_SO):
            build(ref=False)
        _port = _Lib(PORT_SO, "po_")
        L = _port.lib
        L.po_cost.restype = C.c_double
        L.po_interp_1d.restype = C.c_double
        L.po_invert_batch.argtypes = [C.c_int, _dp, C.c_double, C.c_double, C.c_double, _fp,
                                      C.c_int64, C.c_float, C.c_double, C.c_int, C.c_int,
                                      C.c_int, _dp, _dp, C.c_double, C.c_int, _dp]
        L.po_joint_invert_batch.argtypes = [C.c_int, _dp, C.c_double, C.c_double, _i32p, _dp,
                                            _fp, C.c_int64, C.c_float, C.c_int, C.c_double,
                                            C.c_int, C.c_int, C.c_int, _dp, C.c_int, _dp]
        L.po_generate_single.argtypes = [C.c_uint64, C.c_int64, C.c_int64, C.c_int, _dp,
                                         C.c_double, C.c_double, C.c_double, C.c_double,
                                         C.c_float, _fp, _dp]
        L.po_joint_counts.argtypes = [C.c_uint64, C.c_int64, C.c_int, C.c_int, _i32p]
        L.po_generate_joint.argtypes = [C.c_uint64, C.c_int64, C.c_int, _dp, C.c_double,
                                        C.c_double, C.c_double, C.c_double, C.c_double,
                                        C.c_float, _i32p, _dp, _fp, _dp]
        L.po_cost.argtypes = [C.c_int, _dp, C.c_double, C.c_double, C.c_double, _dp, _dp, _dp,
                              _dp]
        L.po_nelmin_pixel.argtypes = [C.c_int, _dp, C.c_double, C.c_double, _dp, _dp, _dp,
                                      C.c_double, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _ip]
        L.po_band_constants.argtypes = [C.c_int, _dp, C.c_double, C.c_double, _dp]
        L.po_interp_1d.argtypes = [_dp, _dp, C.c_int, C.c_double]
        L.po_philox4x32.argtypes = [C.c_uint32] * 6 + [C.POINTER(C.c_uint32)]
        L.po_region_invert_batch.argtypes = [C.c_int, _dp, C.c_double, C.c_double, C.c_double,
                                             _fp, C.c_int, C.c_int, C.c_float, C.c_double,
                                             C.c_int, C.c_int, C.c_int, _dp]
        L.po_depth_sigma.argtypes = [C.c_int, _dp, C.c_double, C.c_double, _fp, C.c_int64, _fp,
                                     _dp, C.c_int, C.c_uint64, C.c_double, C.c_int, C.c_int,
                                     C.c_int, _dp, _i32p, _dp, _dp, _fp]
    return _port


def reference_available() -> bool:
    return os.path.exists(REF_SO)


def reference() -> _Lib:
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            raise FileNotFoundError(
                "oracle/_ref/libphotic_ref.so is not built (needs the reference sources)")
        _ref = _Lib(REF_SO, "photic_ref_")
        L = _ref.lib
        L.photic_ref_cost.restype = C.c_double
        L.photic_ref_interp_1d.restype = C.c_double
        L.photic_ref_invert_batch.argtypes = [C.c_int, _dp, C.c_double, C.c_double, C.c_double,
                                              _fp, C.c_longlong, C.c_float, C.c_int, C.c_double,
                                              C.c_int, C.c_int, C.c_int, _dp]
        L.photic_ref_joint_invert_batch.argtypes = [C.c_int, _dp, C.c_double, C.c_double, _ip,
                                                    _dp, _fp, C.c_longlong, C.c_float, C.c_int,
                                                    C.c_double, C.c_int, C.c_int, C.c_int, _dp]
        L.photic_ref_cost.argtypes = [C.c_int, _dp, C.c_double, C.c_double, C.c_double, _dp,
                                      _dp, C.c_int, _dp, _dp]
        L.photic_ref_nelmin.argtypes = [C.c_int, _dp, C.c_double, C.c_double, _dp, _dp, _dp,
                                        C.c_double, C.c_int, C.c_int, _dp, _dp, _ip, _ip, _ip]
        L.photic_ref_band_constants.argtypes = [C.c_int, _dp, C.c_double, C.c_double, _dp]
        L.photic_ref_interp_1d.argtypes = [_dp, _dp, C.c_int, C.c_double]
    return _ref


# --------------------------------------------------------------------------
# Calls with identical meaning on both libraries.
# --------------------------------------------------------------------------

def invert_batch(rrs, *, wl=OLI_BANDS, theta_sun=35.0, theta_view=0.0, h_tide=0.0,
                 nodata=-9999.0, reqmin=1e-10, konvge=100, kcount=2000, hstarts=None,
                 seeds=None, seed_step_scale=1.0, nthreads=0, which="port"):
    """Invert [npix, n_bands] float32 spectra; returns [npix, NOUT] float64.

    ``which="reference"`` runs the reference's own samodel_optimise with the
    tolerances swapped in at its nelmin call; ``reqmin=None`` keeps the
    reference's hard-coded 1e-2 / 100 / 5000 there.
    """
    rrs = _f32(rrs)
    npix, nb = rrs.shape
    wl = _f64(wl)
    out = np.zeros((npix, NOUT), dtype=np.float64)
    if which == "reference":
        L = reference().lib
        override = 0 if reqmin is None else 1
        L.photic_ref_invert_batch(nb, _ptr(wl, _dp), theta_sun, theta_view, h_tide,
                                  _ptr(rrs, _fp), npix, nodata, override,
                                  1e-2 if reqmin is None else reqmin, konvge, kcount, nthreads,
                                  _ptr(out, _dp))
        return out
    L = port().lib
    if reqmin is None:
        reqmin, konvge, kcount = 1e-2, 100, 5000
    hs = _f64(hstarts) if hstarts is not None else None
    sd = _f64(seeds) if seeds is not None else None
    rc = L.po_invert_batch(nb, _ptr(wl, _dp), theta_sun, theta_view, h_tide, _ptr(rrs, _fp),
                           npix, nodata, reqmin, konvge, kcount,
                           0 if hs is None else len(hs), _ptr(hs, _dp), _ptr(sd, _dp),
                           seed_step_scale, nthreads, _ptr(out, _dp))
    if rc:
        raise ValueError(f"po_invert_batch failed ({rc})")
    return out


def joint_invert_batch(scene_offsets, theta_sun, rrs, *, wl=OLI_BANDS, theta_view=0.0,
                       h_tide=0.0, nodata=-9999.0, layout=0, reqmin=1e-10, konvge=100,
                       kcount=2000, hstarts=None, nthreads=0, which="port"):
    offs = np.ascontiguousarray(scene_offsets, dtype=np.int32)
    th = _f64(theta_sun)
    rrs = _f32(rrs)
    npix = len(offs) - 1
    wl = _f64(wl)
    out = np.zeros((npix, NOUT), dtype=np.float64)
    if which == "reference":
        if layout != 0:
            raise ValueError("the reference implements only the shared-bottom layout")
        L = reference().lib
        L.photic_ref_joint_invert_batch(rrs.shape[1], _ptr(wl, _dp), theta_view, h_tide,
                                        offs.ctypes.data_as(_ip), _ptr(th, _dp),
                                        _ptr(rrs, _fp), npix, nodata, 1, reqmin, konvge,
                                        kcount, nthreads, _ptr(out, _dp))
        return out
    L = port().lib
    hs = _f64(hstarts) if hstarts is not None else None
    rc = L.po_joint_invert_batch(rrs.shape[1], _ptr(wl, _dp), theta_view, h_tide,
                                 offs.ctypes.data_as(_i32p), _ptr(th, _dp), _ptr(rrs, _fp),
                                 npix, nodata, layout, reqmin, konvge, kcount,
                                 0 if hs is None else len(hs), _ptr(hs, _dp),
                                 nthreads, _ptr(out, _dp))
    if rc:
        raise ValueError(f"po_joint_invert_batch failed ({rc})")
    return out


def cost(rrs_measured, params, *, wl=OLI_BANDS, theta_sun=35.0, theta_view=0.0, h_tide=0.0,
         which="port"):
    """Cost, modelled Rrs and K of one 6-parameter vector for one spectrum."""
    r = _f64(rrs_measured)
    p = _f64(params)
    wl = _f64(wl)
    nb = len(wl)
    rm = np.zeros(nb)
    K = np.zeros(nb)
    if which == "reference":
        c = reference().lib.photic_ref_cost(nb, _ptr(wl, _dp), theta_sun, theta_view, h_tide,
                                            _ptr(r, _dp), _ptr(p, _dp), len(p), _ptr(rm, _dp),
                                            _ptr(K, _dp))
    else:
        c = port().lib.po_cost(nb, _ptr(wl, _dp), theta_sun, theta_view, h_tide, _ptr(r, _dp),
                               _ptr(p, _dp), _ptr(rm, _dp), _ptr(K, _dp))
    return c, rm, K


def nelmin(rrs_measured, start, step, *, wl=OLI_BANDS, theta_sun=35.0, theta_view=0.0,
           reqmin=1e-10, konvge=100, kcount=2000, which="port"):
    r = _f64(rrs_measured)
    st = _f64(start).copy()
    sp = _f64(step)
    wl = _f64(wl)
    xmin = np.zeros(6)
    y = C.c_double()
    ic, nr, fl = C.c_int(), C.c_int(), C.c_int()
    f = (reference().lib.photic_ref_nelmin if which == "reference"
         else port().lib.po_nelmin_pixel)
    f(len(wl), _ptr(wl, _dp), theta_sun, theta_view, _ptr(r, _dp), _ptr(st, _dp),
      _ptr(sp, _dp), reqmin, konvge, kcount, _ptr(xmin, _dp), C.byref(y), C.byref(ic),
      C.byref(nr), C.byref(fl))
    return xmin, y.value, ic.value, nr.value, fl.value


def band_constants(*, wl=OLI_BANDS, theta_sun=35.0, theta_view=0.0, which="port"):
    wl = _f64(wl)
    out = np.zeros((len(wl), 8))
    f = (reference().lib.photic_ref_band_constants if which == "reference"
         else port().lib.po_band_constants)
    f(len(wl), _ptr(wl, _dp), theta_sun, theta_view, _ptr(out, _dp))
    return out


def interp_1d(X, Y, x, which="port"):
    X = _f64(X)
    Y = _f64(Y)
    f = (reference().lib.photic_ref_interp_1d if which == "reference"
         else port().lib.po_interp_1d)
    return f(_ptr(X, _dp), _ptr(Y, _dp), len(X), x)


# --------------------------------------------------------------------------
# Synthetic generator (port only; the reference has none).
# --------------------------------------------------------------------------

def generate_single(seed, npix, *, pix0=0, wl=OLI_BANDS, theta_sun=35.0, theta_view=0.0,
                    mask_frac=0.15, noise_sigma=2e-4, nodata=-9999.0):
    wl = _f64(wl)
    rrs = np.zeros((npix, len(wl)), dtype=np.float32)
    truth = np.zeros((npix, 5))
    port().lib.po_generate_single(seed, pix0, npix, len(wl), _ptr(wl, _dp), theta_sun,
                                  theta_view, mask_frac, noise_sigma, nodata, _ptr(rrs, _fp),
                                  _ptr(truth, _dp))
    return rrs, truth


def generate_joint(seed, npix, *, kmin=2, kmax=8, wl=OLI_BANDS, theta_view=0.0,
                   theta_sun_range=(25.0, 50.0), mask_frac=0.0, noise_sigma=2e-4,
                   nodata=-9999.0):
    wl = _f64(wl)
    counts = np.zeros(npix, dtype=np.int32)
    port().lib.po_joint_counts(seed, npix, kmin, kmax, counts.ctypes.data_as(_i32p))
    offs = np.zeros(npix + 1, dtype=np.int32)
    offs[1:] = np.cumsum(counts)
    nobs = int(offs[-1])
    th = np.zeros(nobs)
    rrs = np.zeros((nobs, len(wl)), dtype=np.float32)
    truth = np.zeros((nobs, 5))
    port().lib.po_generate_joint(seed, npix, len(wl), _ptr(wl, _dp), theta_view,
                                 theta_sun_range[0], theta_sun_range[1], mask_frac, noise_sigma,
                                 nodata, offs.ctypes.data_as(_i32p), _ptr(th, _dp),
                                 _ptr(rrs, _fp), _ptr(truth, _dp))
    return offs, th, rrs, truth


def philox4x32(c, k):
    out = (C.c_uint32 * 4)()
    port().lib.po_philox4x32(*(list(c) + list(k)), out)
    return list(out)


def depth_sigma(rrs, depth, r_sigma, *, n_samples=128, seed=1, wl=OLI_BANDS, theta_sun=35.0,
                theta_view=0.0, reqmin=1e-10, konvge=100, kcount=2000, sample_depth=None,
                nthreads=0):
    """Depth uncertainty (model/samodel.c:1368-1479) with Philox draws; returns
    (depth_sigma [npix] f32, table [120], sample_pixel [120*n], sample_depth)."""
    rrs = _f32(rrs)
    npix, nb = rrs.shape
    dep = np.ascontiguousarray(depth, dtype=np.float32)
    rs = _f64(r_sigma)
    wl = _f64(wl)
    ns = 120 * n_samples
    spix = np.zeros(ns, dtype=np.int32)
    sdep = np.zeros(ns)
    table = np.zeros(120)
    sig = np.zeros(npix, dtype=np.float32)
    sin = _f64(sample_depth) if sample_depth is not None else None
    rc = port().lib.po_depth_sigma(nb, _ptr(wl, _dp), theta_sun, theta_view, _ptr(rrs, _fp),
                                   npix, dep.ctypes.data_as(_fp), _ptr(rs, _dp), n_samples,
                                   seed, reqmin, konvge, kcount, nthreads, _ptr(sin, _dp),
                                   spix.ctypes.data_as(_i32p), _ptr(sdep, _dp), _ptr(table, _dp),
                                   sig.ctypes.data_as(_fp))
    if rc:
        raise ValueError("po_depth_sigma failed")
    return sig, table, spix, sdep


def region_depth_sigma(grid, depth, r_sigma, *, n_spatial=2, n_bottoms=3, n_samples=128,
                       seed=1, wl=OLI_BANDS, theta_sun=35.0, theta_view=0.0, nodata=-9999.0,
                       reqmin=None, konvge=100, kcount=2000, sample_depth=None, nthreads=0):
    """The depth uncertainty for the general fit: grid [(n_scenes,) nrows,
    ncols, n_bands], depth [nrows*ncols] (positive, 0 not fitted), r_sigma
    [n_scenes, n_bands]; reqmin None: the reference's tolerances.  Returns
    (depth_sigma, table [120], sample_pixel [120*n], sample_depth)."""
    g = _f32(grid)
    if g.ndim == 3:
        g = g[None]
    S, nr, nc, nb = g.shape
    npix = nr * nc
    dep = np.ascontiguousarray(depth, dtype=np.float32).reshape(-1)
    rs = _f64(np.asarray(r_sigma, dtype=np.float64).reshape(S, nb))
    th = _f64(np.broadcast_to(np.asarray(theta_sun, dtype=np.float64), (S,)))
    wl = _f64(wl)
    if reqmin is None:
        reqmin, konvge, kcount = 1e-2, 100, 5000
    ns = 120 * n_samples
    spix = np.zeros(ns, dtype=np.int32)
    sdep = np.zeros(ns)
    table = np.zeros(120)
    sig = np.zeros(npix, dtype=np.float32)
    sin = _f64(sample_depth) if sample_depth is not None else None
    L = port().lib
    L.po_region_depth_sigma.argtypes = [C.c_int, _dp, _dp, C.c_double, _fp, C.c_int, C.c_int,
                                        C.c_int, C.c_float, C.c_int, C.c_int, _fp, _dp, C.c_int,
                                        C.c_uint64, C.c_double, C.c_int, C.c_int, C.c_int, _dp,
                                        _i32p, _dp, _dp, _fp]
    rc = L.po_region_depth_sigma(nb, _ptr(wl, _dp), _ptr(th, _dp), theta_view, _ptr(g, _fp), S,
                                 nr, nc, nodata, n_spatial, n_bottoms, dep.ctypes.data_as(_fp),
                                 _ptr(rs, _dp), n_samples, seed, reqmin, konvge, kcount,
                                 nthreads, _ptr(sin, _dp), spix.ctypes.data_as(_i32p),
                                 _ptr(sdep, _dp), _ptr(table, _dp), sig.ctypes.data_as(_fp))
    if rc:
        raise ValueError("po_region_depth_sigma failed")
    return sig, table, spix, sdep


def region_invert_batch(grid, *, wl=OLI_BANDS, theta_sun=35.0, theta_view=0.0, h_tide=0.0,
                        nodata=-9999.0, reqmin=1e-10, konvge=100, kcount=2000, n_spatial=2,
                        n_bottoms=1, h_empirical=None, nthreads=0, which="port"):
    """The general fit of a grid: [nrows, ncols, n_bands] (one scene) or
    [n_scenes, nrows, ncols, n_bands] float32 with theta_sun one sun zenith
    per scene; each pixel alone (n_spatial = 1) or with its 3 x 3
    neighbourhood (n_spatial = 2), n_bottoms bottom types (sand, seagrass,
    coral) mixed per region; h_empirical (None or [nrows*ncols] with NaN for
    none) gives per-pixel empirical depths.  Returns [nrows*ncols, NOUT]
    (o[38] regions, o[39] origin, o[40..42] bottom shares (%), o[43] bottom
    type)."""
    g = np.ascontiguousarray(grid, dtype=np.float32)
    if g.ndim == 3:
        g = g[None]
    ns, nrows, ncols, nb = g.shape
    override = reqmin is not None  # None: the reference's own 1e-2 / 100 / 5000
    if not override:
        reqmin, konvge, kcount = 1e-2, 100, 5000
    th = _f64(np.broadcast_to(np.asarray(theta_sun, dtype=np.float64), (ns,)))
    wl = _f64(wl)
    he = _f64(h_empirical) if h_empirical is not None else None
    out = np.zeros((nrows * ncols, NOUT), dtype=np.float64)
    if which == "reference":
        f = reference().lib.photic_ref_region_fit_batch
        f.argtypes = [C.c_int, _dp, _dp, C.c_double, C.c_double, _fp, C.c_int, C.c_int, C.c_int,
                      C.c_float, C.c_int, C.c_int, _dp, C.c_int, C.c_double, C.c_int, C.c_int,
                      C.c_int, _dp]
        rc = f(nb, _ptr(wl, _dp), _ptr(th, _dp), theta_view, h_tide, g.ctypes.data_as(_fp), ns,
               nrows, ncols, nodata, n_spatial, n_bottoms, _ptr(he, _dp), 1 if override else 0,
               reqmin, konvge, kcount, nthreads, _ptr(out, _dp))
    else:
        f = port().lib.po_region_fit_batch
        f.argtypes = [C.c_int, _dp, _dp, C.c_double, C.c_double, _fp, C.c_int, C.c_int, C.c_int,
                      C.c_float, C.c_int, C.c_int, _dp, C.c_double, C.c_int, C.c_int, C.c_int,
                      _dp]
        rc = f(nb, _ptr(wl, _dp), _ptr(th, _dp), theta_view, h_tide, g.ctypes.data_as(_fp), ns,
               nrows, ncols, nodata, n_spatial, n_bottoms, _ptr(he, _dp), reqmin, konvge, kcount,
               nthreads, _ptr(out, _dp))
    if rc:
        raise ValueError("region_invert_batch failed")
    return out


def region_cost(rrs, params, *, origin=0, n_bottoms=1, wl=OLI_BANDS, theta_sun=35.0,
                theta_view=0.0, h_tide=0.0):
    """samodel_error of one parameter vector for a pixel given as its regions'
    spectra rrs [R, n_bands] or [R, S, n_bands]; returns (cost, details[5],
    modelled Rrs [R, S, n_bands])."""
    r = _f64(rrs)
    if r.ndim == 2:
        r = r[:, None, :]
    R, S, nb = r.shape
    r = np.ascontiguousarray(r)
    th = _f64(np.broadcast_to(np.asarray(theta_sun, dtype=np.float64), (S,)))
    p = _f64(params)
    wl = _f64(wl)
    det = np.zeros(5)
    rm = np.zeros((R, S, nb))
    f = port().lib.po_region_cost
    f.restype = C.c_double
    f.argtypes = [C.c_int, _dp, _dp, C.c_double, C.c_double, _dp, C.c_int, C.c_int, C.c_int,
                  C.c_int, _dp, _dp, _dp]
    c = f(nb, _ptr(wl, _dp), _ptr(th, _dp), theta_view, h_tide, _ptr(r, _dp), R, S, origin,
          n_bottoms, _ptr(p, _dp), _ptr(det, _dp), _ptr(rm, _dp))
    return c, det, rm



# --------------------------------------------------------------------------
# netCDF short packing (model/nc.c:251-320): the port's restatement and the
# reference's own write_nc / read_nc through the in-memory netCDF stand-in.
# --------------------------------------------------------------------------
_i16p = C.POINTER(C.c_int16)


def nc_compress(grid, spval, which="port"):
    """compress_2d over a row-major grid: (packed int16, add_offset,
    scale_factor, missing_value); with which="reference" the values the
    reference's write_nc put in its file."""
    g = _f32(grid)
    packed = np.zeros(g.shape, dtype=np.int16)
    off, sc, sp = C.c_float(), C.c_float(), C.c_float()
    mv = C.c_int16()
    if which == "port":
        L = port().lib
        L.po_nc_compress(_ptr(g, _fp), C.c_int64(g.size), C.c_double(spval), _ptr(packed, _i16p),
                         C.byref(off), C.byref(sc), C.byref(mv))
        return packed, off.value, sc.value, mv.value
    L = reference().lib
    nrows, ncols = g.shape
    lons = np.arange(ncols, dtype=np.float32)
    lats = np.arange(nrows, dtype=np.float32)
    rc = L.photic_ref_nc_write(_ptr(g, _fp), C.c_int(ncols), C.c_int(nrows), _ptr(lons, _fp),
                               _ptr(lats, _fp), C.c_double(spval), _ptr(packed, _i16p),
                               C.byref(off), C.byref(sc), C.byref(mv), C.byref(sp))
    if rc:
        raise RuntimeError(f"reference write_nc harness failed ({rc})")
    return packed, off.value, sc.value, mv.value


def nc_decompress(packed, add_offset, scale_factor, missing_value=-32768, spval=-9999.0,
                  which="port", has_missing=True, has_spval=True):
    """decompress_2d of a row-major packed grid; with which="reference" the
    grid (and spval) the reference's read_nc returns for a file holding it,
    with or without the missing_value / decompressed_missing_value
    attributes."""
    p = np.ascontiguousarray(packed, dtype=np.int16)
    out = np.zeros(p.shape, dtype=np.float32)
    if which == "port":
        mv = missing_value if has_missing else -32768
        sp = float(np.float32(spval)) if has_spval else 0.0
        port().lib.po_nc_decompress(_ptr(p, _i16p), C.c_int64(p.size), C.c_float(add_offset),
                                    C.c_float(scale_factor), C.c_int16(mv), C.c_double(sp),
                                    _ptr(out, _fp))
        return out, sp
    L = reference().lib
    nrows, ncols = p.shape
    lons = np.arange(ncols, dtype=np.float32)
    lats = np.arange(nrows, dtype=np.float32)
    spo = C.c_double()
    rc = L.photic_ref_nc_read(_ptr(p, _i16p), C.c_int(ncols), C.c_int(nrows), _ptr(lons, _fp),
                              _ptr(lats, _fp), C.c_float(add_offset), C.c_float(scale_factor),
                              C.c_int(int(has_missing)), C.c_int16(missing_value),
                              C.c_int(int(has_spval)), C.c_float(spval), _ptr(out, _fp),
                              C.byref(spo))
    if rc:
        raise RuntimeError(f"reference read_nc harness failed ({rc})")
    return out, spo.value


def nc_reference_layout(grid, spval=-9999.0):
    """The dimensions, variables and attributes (in call order) of the file
    the reference's write_nc writes for a grid."""
    nc_compress(grid, spval, which="reference")
    buf = C.create_string_buffer(1 << 16)
    reference().lib.photic_ref_nc_layout(buf, C.c_int(len(buf)))
    return buf.value.decode().splitlines()


# --------------------------------------------------------------------------
# Spatially coherent scene and the pixel loop with the dynamic lookup table
# (model/samodel.c:649-1215).
# --------------------------------------------------------------------------
_i64p = C.POINTER(C.c_int64)


def generate_field(seed, nrows, ncols, *, row0=0, n_rows=None, wl=OLI_BANDS, theta_sun=35.0,
                   theta_view=0.0, mask_frac=0.1, noise_sigma=1e-4, nodata=-9999.0):
    """Rows [row0, row0 + n_rows) of a nrows x ncols scene whose parameters
    are smooth fields; returns ([n_rows*ncols, n_bands] float32 spectra,
    [n_rows*ncols, 5] truth H P G X B)."""
    n_rows = nrows - row0 if n_rows is None else n_rows
    wl = _f64(wl)
    n = n_rows * ncols
    rrs = np.zeros((n, len(wl)), dtype=np.float32)
    truth = np.zeros((n, 5))
    L = port().lib
    L.po_generate_field.argtypes = [C.c_uint64, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                    C.c_int, _dp, C.c_double, C.c_double, C.c_double,
                                    C.c_double, C.c_float, _fp, _dp]
    L.po_generate_field(seed, nrows, ncols, row0, n_rows, len(wl), _ptr(wl, _dp), theta_sun,
                        theta_view, mask_frac, noise_sigma, nodata, _ptr(rrs, _fp),
                        _ptr(truth, _dp))
    return rrs, truth


def lut_key(rrs, *, nodata=-9999.0, rrs_noise=None):
    """The spectral index samodel() sorts the pixels by, per pixel."""
    rrs = _f32(rrs)
    L = port().lib
    L.po_lut_key.restype = C.c_float
    L.po_lut_key.argtypes = [_fp, C.c_int, C.c_float, _dp]
    nz = _f64(rrs_noise) if rrs_noise is not None else None
    nb = rrs.shape[1]
    return np.array([L.po_lut_key(_ptr(rrs[p], _fp), nb, nodata, _ptr(nz, _dp))
                     for p in range(rrs.shape[0])], dtype=np.float32)


def lut_invert(rrs, *, wl=OLI_BANDS, theta_sun=35.0, theta_view=0.0, h_tide=0.0,
               nodata=-9999.0, rrs_noise=None, empirical=None, empirical_nodata=-9999.0,
               reqmin=None, konvge=100, kcount=2000, n_lut=16000, n_chains=1, nthreads=0):
    """samodel()'s loop with the dynamic lookup table over [npix, n_bands]
    float32 spectra, the sorted shallow pixels cut into n_chains slices;
    empirical ([npix] floats, empirical_nodata for none) orders the pixels and
    starts their fits as the reference's empirical depth grid does.
    reqmin None: the reference's tolerances (1e-2 / 100 / 5000).  Returns
    (records [npix, NOUT], source [npix] (-1 fitted, -2 masked, else the
    pixel whose fit served it), order [n_shallow], chain_stats [n_chains, 4]
    (served, fitted, final match and entry thresholds))."""
    rrs = _f32(rrs)
    npix, nb = rrs.shape
    wl = _f64(wl)
    if reqmin is None:
        reqmin, konvge, kcount = 1e-2, 100, 5000
    out = np.zeros((npix, NOUT))
    source = np.zeros(npix, dtype=np.int64)
    order = np.zeros(max(npix, 1), dtype=np.int64)
    n_sh = C.c_int64(0)
    stats = np.zeros((max(1, n_chains), 4))
    nz = _f64(rrs_noise) if rrs_noise is not None else None
    em = _f32(empirical).reshape(-1) if empirical is not None else None
    L = port().lib
    L.po_lut_invert.argtypes = [C.c_int, _dp, C.c_double, C.c_double, C.c_double, _fp,
                                C.c_int64, C.c_float, _dp, _fp, C.c_float, C.c_double, C.c_int,
                                C.c_int, C.c_int, C.c_int64, C.c_int, _i64p, _i64p, _dp, _i64p,
                                _dp]
    rc = L.po_lut_invert(nb, _ptr(wl, _dp), theta_sun, theta_view, h_tide, _ptr(rrs, _fp), npix,
                         nodata, _ptr(nz, _dp), _ptr(em, _fp), empirical_nodata, reqmin, konvge,
                         kcount, n_lut, n_chains, nthreads, _ptr(order, _i64p), C.byref(n_sh),
                         _ptr(out, _dp), _ptr(source, _i64p), _ptr(stats, _dp))
    if rc:
        raise ValueError(f"po_lut_invert failed ({rc})")
    S = n_sh.value
    return out, source, order[:S], stats[:min(n_chains, max(S, 1))]


def glut_invert(grid, *, wl=OLI_BANDS, theta_sun=35.0, theta_view=0.0, h_tide=0.0,
                nodata=-9999.0, n_spatial=2, n_bottoms=3, rrs_noise=None, empirical=None,
                empirical_nodata=-9999.0, reqmin=None, konvge=100, kcount=2000, n_lut=16000,
                n_chains=1, nthreads=0):
    """samodel()'s loop with the dynamic lookup table in the general
    configuration: grid [nrows, ncols, n_bands] or [n_scenes, nrows, ncols,
    n_bands] float32, 3 x 3 regions (n_spatial 2), n_bottoms bottom types,
    one sun zenith per scene (theta_sun scalar or sequence), rrs_noise
    [n_scenes, n_bands] (the spectral-angle order), empirical [nrows,
    ncols].  Returns (records [npix, NOUT], source, order, chain_stats) as
    lut_invert."""
    g = _f32(grid)
    if g.ndim == 3:
        g = g[None]
    S, nr, nc, nb = g.shape
    npix = nr * nc
    wl = _f64(wl)
    th = _f64(np.broadcast_to(np.asarray(theta_sun, dtype=np.float64), (S,)))
    if reqmin is None:
        reqmin, konvge, kcount = 1e-2, 100, 5000
    out = np.zeros((npix, NOUT))
    source = np.zeros(npix, dtype=np.int64)
    order = np.zeros(max(npix, 1), dtype=np.int64)
    n_sh = C.c_int64(0)
    stats = np.zeros((max(1, n_chains), 4))
    nz = _f64(np.asarray(rrs_noise, dtype=np.float64).reshape(S, nb)) if rrs_noise is not None \
        else None
    em = _f32(empirical).reshape(-1) if empirical is not None else None
    L = port().lib
    L.po_glut_invert.argtypes = [C.c_int, _dp, _dp, C.c_double, C.c_double, _fp, C.c_int,
                                 C.c_int, C.c_int, C.c_float, C.c_int, C.c_int, _dp, _fp,
                                 C.c_float, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int64,
                                 C.c_int, _i64p, _i64p, _dp, _i64p, _dp]
    rc = L.po_glut_invert(nb, _ptr(wl, _dp), _ptr(th, _dp), theta_view, h_tide, _ptr(g, _fp), S,
                          nr, nc, nodata, n_spatial, n_bottoms, _ptr(nz, _dp), _ptr(em, _fp),
                          empirical_nodata, reqmin, konvge, kcount, n_lut, n_chains, nthreads,
                          _ptr(order, _i64p), C.byref(n_sh), _ptr(out, _dp), _ptr(source, _i64p),
                          _ptr(stats, _dp))
    if rc:
        raise ValueError(f"po_glut_invert failed ({rc})")
    S_ = n_sh.value
    return out, source, order[:S_], stats[:min(n_chains, max(S_, 1))]


def reference_samodel_stack(grid, *, wl=OLI_BANDS, theta_sun=35.0, theta_view=0.0,
                            nodata=-9999.0, r_sigma=None, empirical=None,
                            empirical_nodata=-9999.0, n_spatial=1, n_bottoms=1):
    """The reference's own samodel() over [n_scenes, nrows, ncols, n_bands]
    co-registered scenes (one sun zenith each, r_sigma [n_scenes, n_bands])
    on one thread; returns the [10, nrows, ncols] grids as
    reference_samodel_grid."""
    g = _f32(grid)
    S, nr, nc, nb = g.shape
    wl = _f64(wl)
    th = _f64(np.broadcast_to(np.asarray(theta_sun, dtype=np.float64), (S,)))
    out = np.zeros((10, nr, nc), dtype=np.float32)
    rs = _f64(np.asarray(r_sigma, dtype=np.float64).reshape(S, nb)) if r_sigma is not None \
        else None
    em = _f32(empirical).reshape(nr, nc) if empirical is not None else None
    L = reference().lib
    L.photic_ref_samodel_stack.argtypes = [C.c_int, _dp, _dp, C.c_double, _fp, C.c_int, C.c_int,
                                           C.c_int, C.c_float, _dp, _fp, C.c_float, C.c_int,
                                           C.c_int, _fp]
    rc = L.photic_ref_samodel_stack(nb, _ptr(wl, _dp), _ptr(th, _dp), theta_view, _ptr(g, _fp),
                                    S, nr, nc, nodata, _ptr(rs, _dp), _ptr(em, _fp),
                                    empirical_nodata, n_spatial, n_bottoms, _ptr(out, _fp))
    if rc:
        raise ValueError(f"photic_ref_samodel_stack failed ({rc})")
    return out


def reference_samodel_grid(grid, *, wl=OLI_BANDS, theta_sun=35.0, theta_view=0.0,
                           nodata=-9999.0, r_sigma=None, empirical=None,
                           empirical_nodata=-9999.0, n_spatial=1, n_bottoms=1):
    """The reference's own samodel() with its lookup table over a
    [nrows, ncols, n_bands] grid on one thread; returns [10, nrows, ncols]
    float32 grids as samodel() leaves them (depth negative below the datum,
    depth sigma, model error, bottom albedo, sand, seagrass, coral, K_min,
    bottom type, index of optical depth)."""
    grid = _f32(grid)
    nr, nc, nb = grid.shape
    wl = _f64(wl)
    out = np.zeros((10, nr, nc), dtype=np.float32)
    rs = _f64(r_sigma) if r_sigma is not None else None
    em = _f32(empirical).reshape(nr, nc) if empirical is not None else None
    L = reference().lib
    L.photic_ref_samodel_grid.argtypes = [C.c_int, _dp, C.c_double, C.c_double, _fp, C.c_int,
                                          C.c_int, C.c_float, _dp, _fp, C.c_float, C.c_int,
                                          C.c_int, _fp]
    rc = L.photic_ref_samodel_grid(nb, _ptr(wl, _dp), theta_sun, theta_view, _ptr(grid, _fp),
                                   nr, nc, nodata, _ptr(rs, _dp), _ptr(em, _fp),
                                   empirical_nodata, n_spatial, n_bottoms, _ptr(out, _fp))
    if rc:
        raise ValueError(f"photic_ref_samodel_grid failed ({rc})")
    return out
