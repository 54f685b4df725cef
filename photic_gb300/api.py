"""Python host layer over the C ABI (include/photic.h).

This is the user-facing mirror of the reference's per-pixel operator,
``samodel_optimise`` (model/samodel.c:1768) applied over a scene the way
the pixel loop of ``samodel`` does (model/samodel.c:901-1166): give it the
band reflectances of many pixels, get back depth, P, G, X, bottom albedo,
the model error and the convergence flag of every pixel.  Configuration
names follow the reference (reqmin / konvge / kcount of nelmin, depth starts
``hstarts``, subsurface ``theta_sun`` / ``theta_view``).

Device memory and streams come from PyTorch; every computation runs in the
CUDA library, and an error from it raises :class:`PhoticError`.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Dict, Optional, Sequence

import torch

from . import _lib as L
from ._lib import PhoticError  # noqa: F401

PRECISIONS = {"fp64": L.PREC_FP64, "df64": L.PREC_DF64, "fp32": L.PREC_FP32,
              "guarded": L.PREC_GUARDED}
LAYOUTS = {"reference": L.LAYOUT_REFERENCE, "scene_b": L.LAYOUT_SCENE_B}
OUTPUT_FIELDS = ("depth", "depth_f64", "P", "G", "X", "bottom_albedo", "model_error",
                 "rrs_error", "K_min", "iod", "evals", "evals_kept", "status", "params")
# extra outputs of the bottom-mixture fit (region_fit)
MIX_FIELDS = ("bottom_percent", "bottom_type")
_DTYPES = {"depth_f64": torch.float64, "evals": torch.int32, "evals_kept": torch.int32,
           "status": torch.int32, "params": torch.float64}


@dataclass
class Config:
    """Mirror of ``photic_config``; the defaults are the plain-method
    workload: OLI-like bands, sun 35 deg, nadir, reqmin 1e-10, kcount 2000
    and the reference's eight cold depth starts (model/samodel.c:2216)."""
    wavelengths: Sequence[float] = (443.0, 482.0, 561.0, 655.0)
    theta_sun_deg: float = 35.0
    theta_view_deg: float = 0.0
    h_tide: float = 0.0
    nodata_value: float = -9999.0
    reqmin: float = 1.0e-10
    konvge: int = 100
    kcount: int = 2000
    hstarts: Sequence[float] = (40.0, 30.0, 20.0, 15.0, 10.0, 7.5, 2.5, 1.0)
    early_exit_per_scene: float = 2.5
    precision: str = "fp64"
    layout: str = "reference"
    block_threads: int = 0
    blocks_per_sm: int = 0
    seed_step_scale: float = 1.0

    @classmethod
    def reference_default(cls, **kw) -> "Config":
        """The tolerances the reference hard-codes (model/samodel.c:2142-2144)."""
        kw.setdefault("reqmin", 1.0e-2)
        kw.setdefault("konvge", 100)
        kw.setdefault("kcount", 5000)
        return cls(**kw)

    @property
    def n_bands(self) -> int:
        return len(self.wavelengths)

    def to_c(self) -> L.photic_config:
        c = L.photic_config()
        L.lib().photic_config_default(C.byref(c))
        c.n_bands = len(self.wavelengths)
        if c.n_bands > L.MAX_BANDS:
            raise ValueError(f"at most {L.MAX_BANDS} bands")
        for i, w in enumerate(self.wavelengths):
            c.wavelengths[i] = float(w)
        c.theta_sun_deg = float(self.theta_sun_deg)
        c.theta_view_deg = float(self.theta_view_deg)
        c.h_tide = float(self.h_tide)
        c.nodata_value = float(self.nodata_value)
        c.reqmin = float(self.reqmin)
        c.konvge = int(self.konvge)
        c.kcount = int(self.kcount)
        if len(self.hstarts) > L.MAX_HSTARTS:
            raise ValueError(f"at most {L.MAX_HSTARTS} depth starts")
        c.n_hstarts = len(self.hstarts)
        for i, h in enumerate(self.hstarts):
            c.hstarts[i] = float(h)
        c.early_exit_per_scene = float(self.early_exit_per_scene)
        c.precision = PRECISIONS[self.precision]
        c.layout = LAYOUTS[self.layout]
        c.block_threads = int(self.block_threads)
        c.blocks_per_sm = int(self.blocks_per_sm)
        c.seed_step_scale = float(self.seed_step_scale)
        return c


def version() -> str:
    return L.lib().photic_version().decode()


def _stream_handle(stream: Optional[torch.cuda.Stream]) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def _ptr(t: Optional[torch.Tensor]) -> Optional[int]:
    return None if t is None else int(t.data_ptr())


def _check_cuda(t: torch.Tensor, name: str, dtype) -> None:
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")


def alloc_outputs(npix: int, device, fields: Sequence[str] = OUTPUT_FIELDS,
                  n_obs: Optional[int] = None) -> Dict[str, torch.Tensor]:
    out = {}
    for f in fields:
        if f == "params":
            if n_obs is None:
                out[f] = torch.empty(npix, 6, dtype=torch.float64, device=device)
            continue
        if f == "bottom_percent":
            out[f] = torch.empty(npix, 3, dtype=torch.float32, device=device)
            continue
        n = n_obs if (n_obs is not None and f in ("P", "G", "X")) else npix
        out[f] = torch.empty(n, dtype=_DTYPES.get(f, torch.float32), device=device)
    return out


def _outputs_struct(out: Dict[str, torch.Tensor]) -> L.photic_outputs:
    s = L.photic_outputs()
    for f in OUTPUT_FIELDS + MIX_FIELDS:
        setattr(s, f, _ptr(out.get(f)))
    return s


def fallbacks_first(seeds: torch.Tensor) -> torch.Tensor:
    """A pixel order for :func:`invert` that takes the cold-start fallbacks
    of a seeded batch (NaN seeds, several times longer to fit) first."""
    return torch.argsort((~torch.isnan(seeds[:, 0])).to(torch.int8), stable=True).to(torch.int32)


def invert(rrs: torch.Tensor, config: Optional[Config] = None, *,
           seeds: Optional[torch.Tensor] = None, order: Optional[torch.Tensor] = None,
           out: Optional[Dict[str, torch.Tensor]] = None,
           fields: Sequence[str] = OUTPUT_FIELDS,
           stream: Optional[torch.cuda.Stream] = None) -> Dict[str, torch.Tensor]:
    """Fit every pixel of ``rrs`` ([npix, n_bands] float32, CUDA).

    ``seeds`` ([npix, 6] float64) starts a pixel's single fit from the given
    vector (H, 100B, q, 100P, 100G, 100X); NaN in column 0 keeps that pixel
    on the cold multi-start.  ``order`` (int32 permutation of the pixels)
    is the order the work queue hands them out in; results stay at each
    pixel's index.  Asynchronous on ``stream``; call :func:`sync` to surface
    device-side errors.
    """
    cfg = config or Config()
    _check_cuda(rrs, "rrs", torch.float32)
    if rrs.dim() != 2 or rrs.shape[1] != cfg.n_bands:
        raise ValueError(f"rrs must be [npix, {cfg.n_bands}]")
    npix = rrs.shape[0]
    if seeds is not None:
        _check_cuda(seeds, "seeds", torch.float64)
        if tuple(seeds.shape) != (npix, 6):
            raise ValueError("seeds must be [npix, 6]")
    if order is not None:
        _check_cuda(order, "order", torch.int32)
        if order.numel() != npix:
            raise ValueError("order must hold one entry per pixel")
    if out is None:
        out = alloc_outputs(npix, rrs.device, fields)
    c = cfg.to_c()
    os_ = _outputs_struct(out)
    L.check(L.lib().photic_invert_batch_ordered(C.byref(c), _ptr(rrs), npix, cfg.n_bands, 1,
                                                _ptr(seeds), _ptr(order), C.byref(os_),
                                                _stream_handle(stream)))
    return out


def lut_invert(rrs: torch.Tensor, config: Optional[Config] = None, *, n_lut: int = 16000,
               n_chains: int = 0, rrs_noise: Optional[Sequence[float]] = None,
               empirical: Optional[torch.Tensor] = None, empirical_nodata: float = -9999.0,
               fields: Sequence[str] = OUTPUT_FIELDS, stream: Optional[torch.cuda.Stream] = None
               ) -> Dict[str, torch.Tensor]:
    """samodel()'s pixel loop with its dynamic lookup table
    (model/samodel.c:649-1215) over ``rrs`` ([npix, n_bands] float32, CUDA):
    the shallow pixels sorted by spectral index (times the spectral angle
    to ``rrs_noise`` when every band of it is at least 1e-6), cut into
    ``n_chains`` contiguous slices (0: eight per resident lane), each run as
    the reference runs them on one thread -- served from its table of
    ``n_lut`` fits when a stored spectrum matches, else fitted (hot-started
    from the previous pixel when the last two were continuous).  Use
    ``Config.reference_default()`` for the reference's tolerances.  Returns
    the outputs plus "source" (int64: -2 masked, -1 fitted, else the pixel
    whose fit served it), "order" (the sorted shallow pixels) and
    "chain_stats" ([n_chains, 4]: served, fitted, final match and entry
    thresholds).  ``empirical`` ([npix] float32, CUDA; ``empirical_nodata``
    for none) is the reference's empirical depth grid: it orders the pixels
    and starts their fits.  Synchronises the stream once (to size the
    order)."""
    cfg = config or Config()
    _check_cuda(rrs, "rrs", torch.float32)
    if rrs.dim() != 2 or rrs.shape[1] != cfg.n_bands:
        raise ValueError(f"rrs must be [npix, {cfg.n_bands}]")
    if not rrs.is_contiguous():
        raise ValueError("rrs must be contiguous")
    npix = rrs.shape[0]
    if empirical is not None:
        _check_cuda(empirical, "empirical", torch.float32)
        if empirical.numel() != npix or not empirical.is_contiguous():
            raise ValueError("empirical must be a contiguous [npix] tensor")
    out = alloc_outputs(npix, rrs.device, fields)
    source = torch.empty(npix, dtype=torch.int64, device=rrs.device)
    order = torch.empty(max(npix, 1), dtype=torch.int64, device=rrs.device)
    lc = L.photic_lut_config()
    L.lib().photic_lut_config_default(C.byref(lc))
    lc.n_lut = int(n_lut)
    lc.n_chains = int(n_chains)
    if rrs_noise is not None:
        lc.use_noise = 1
        for b, v in enumerate(rrs_noise):
            lc.rrs_noise[b] = float(v)
    c = cfg.to_c()
    max_chains = int(n_chains) if n_chains else int(L.lib().photic_lut_default_chains(C.byref(c)))
    if max_chains < 1:
        raise PhoticError(L.ERR_CUDA, "no chain count for this configuration: "
                          + L.lib().photic_last_error().decode(errors="replace"))
    stats = torch.zeros(max(1, min(max_chains, npix)), 4, dtype=torch.float64, device=rrs.device)
    os_ = _outputs_struct(out)
    n_sh, n_ch = C.c_int64(0), C.c_int64(0)
    L.check(L.lib().photic_lut_invert_batch(C.byref(c), C.byref(lc), _ptr(rrs), npix,
                                            _ptr(empirical), float(empirical_nodata),
                                            C.byref(os_), _ptr(source), _ptr(order),
                                            _ptr(stats), C.byref(n_sh), C.byref(n_ch),
                                            _stream_handle(stream)))
    out["source"] = source
    out["order"] = order[:n_sh.value]
    out["chain_stats"] = stats[:n_ch.value]
    return out


def region_depth_sigma(grid: torch.Tensor, depth: torch.Tensor, r_sigma,
                       config: Optional[Config] = None, *, n_spatial: int = 2,
                       n_bottoms: int = 3, theta_sun: Optional[Sequence[float]] = None,
                       n_samples: int = 128, seed: int = 1,
                       stream: Optional[torch.cuda.Stream] = None) -> Dict[str, torch.Tensor]:
    """The reference's depth uncertainty for the general fit
    (model/samodel.c:1368-1479 with regions, mixtures or scene stacks): the
    samples of ``depth_sigma``, each sampled pixel's regions of every scene
    of ``grid`` ([(n_scenes,) nrows, ncols, n_bands]) moved by n *
    ``r_sigma`` ([n_scenes, n_bands]) and refitted by the general fit.
    ``depth``: [nrows * ncols] float32, positive, 0 = not fitted.  Returns
    sigma, table, sample_pixel and sample_depth as ``depth_sigma``."""
    cfg = config or Config()
    _check_cuda(grid, "grid", torch.float32)
    _check_cuda(depth, "depth", torch.float32)
    g4 = grid if grid.dim() == 4 else grid.unsqueeze(0)
    if g4.dim() != 4 or g4.shape[3] != cfg.n_bands or not g4.is_contiguous():
        raise ValueError(f"grid must be a contiguous [(n_scenes,) nrows, ncols, {cfg.n_bands}]")
    S, nrows, ncols = int(g4.shape[0]), int(g4.shape[1]), int(g4.shape[2])
    vals = [float(v) for row in r_sigma for v in row]
    if len(vals) != S * cfg.n_bands:
        raise ValueError("r_sigma must be [n_scenes, n_bands]")
    ns = 120 * n_samples
    dev = grid.device
    out = {"sigma": torch.empty(nrows * ncols, dtype=torch.float32, device=dev),
           "table": torch.empty(120, dtype=torch.float64, device=dev),
           "sample_pixel": torch.empty(ns, dtype=torch.int32, device=dev),
           "sample_depth": torch.empty(ns, dtype=torch.float64, device=dev)}
    c = cfg.to_c()
    th = (C.c_double * S)(*([cfg.theta_sun_deg] * S if theta_sun is None else
                            [float(t) for t in theta_sun]))
    rs = (C.c_double * len(vals))(*vals)
    L.check(L.lib().photic_region_depth_sigma(
        C.byref(c), _ptr(g4), S, th, nrows, ncols, int(n_spatial), int(n_bottoms), _ptr(depth),
        rs, int(n_samples), int(seed), _ptr(out["sigma"]), _ptr(out["table"]),
        _ptr(out["sample_pixel"]), _ptr(out["sample_depth"]), _stream_handle(stream)))
    return out


def region_invert(grid: torch.Tensor, config: Optional[Config] = None, *,
                  fields: Sequence[str] = OUTPUT_FIELDS,
                  stream: Optional[torch.cuda.Stream] = None) -> Dict[str, torch.Tensor]:
    """Spatial-region fit (model/samodel.c:2957-3027, n_spatial = 2) of a
    [nrows, ncols, n_bands] float32 grid: every pixel with its 3 x 3
    neighbourhood, one depth / albedo / q per region, shared P, G, X,
    depth- and bottom-continuity terms; depth is the origin-weighted mean.
    Outputs are per pixel ([nrows * ncols]); bits 24-27 of status hold the
    region count."""
    cfg = config or Config()
    _check_cuda(grid, "grid", torch.float32)
    if grid.dim() != 3 or grid.shape[2] != cfg.n_bands:
        raise ValueError(f"grid must be [nrows, ncols, {cfg.n_bands}]")
    nrows, ncols = int(grid.shape[0]), int(grid.shape[1])
    out = alloc_outputs(nrows * ncols, grid.device, [f for f in fields if f != "params"])
    c = cfg.to_c()
    os_ = _outputs_struct(out)
    L.check(L.lib().photic_region_invert_batch(C.byref(c), _ptr(grid), nrows, ncols, 2,
                                               C.byref(os_), _stream_handle(stream)))
    return out


def region_fit(grid: torch.Tensor, config: Optional[Config] = None, *, n_spatial: int = 2,
               n_bottoms: int = 3, theta_sun: Optional[Sequence[float]] = None,
               h_empirical: Optional[torch.Tensor] = None,
               fields: Sequence[str] = OUTPUT_FIELDS + MIX_FIELDS,
               stream: Optional[torch.cuda.Stream] = None) -> Dict[str, torch.Tensor]:
    """The reference's default inversion call (model/bam.c:3236-3241 with
    n_spatial = 2, n_bottoms = 3): every pixel of a [nrows, ncols, n_bands]
    (one scene) or [n_scenes, nrows, ncols, n_bands] float32 grid, fitted
    alone (``n_spatial`` = 1) or with its 3 x 3 neighbourhood (2),
    ``n_bottoms`` bottom types (sand, seagrass, coral) mixed in every region,
    the scenes jointly (each with its own P, G, X and sun zenith
    ``theta_sun``, default the config's).  ``h_empirical`` ([nrows * ncols]
    float64, NaN for none) gives empirical depths (single depth start; deeper
    than 8 m: sand alone).  Outputs per pixel (P, G, X: [npix, n_scenes]),
    with ``bottom_percent`` [npix, 3] and ``bottom_type``."""
    cfg = config or Config()
    _check_cuda(grid, "grid", torch.float32)
    g4 = grid if grid.dim() == 4 else grid.unsqueeze(0)
    if g4.dim() != 4 or g4.shape[3] != cfg.n_bands:
        raise ValueError(f"grid must be [(n_scenes,) nrows, ncols, {cfg.n_bands}]")
    S, nrows, ncols = int(g4.shape[0]), int(g4.shape[1]), int(g4.shape[2])
    if h_empirical is not None:
        _check_cuda(h_empirical, "h_empirical", torch.float64)
    out = alloc_outputs(nrows * ncols, grid.device, [f for f in fields if f != "params"],
                        n_obs=nrows * ncols * S if S > 1 else None)
    c = cfg.to_c()
    th = (C.c_double * S)(*([cfg.theta_sun_deg] * S if theta_sun is None else
                            [float(t) for t in theta_sun]))
    os_ = _outputs_struct(out)
    L.check(L.lib().photic_region_fit_batch(C.byref(c), _ptr(g4), S, th, nrows, ncols,
                                            int(n_spatial), int(n_bottoms), _ptr(h_empirical),
                                            C.byref(os_), _stream_handle(stream)))
    if S > 1:
        for f in ("P", "G", "X"):
            if f in out:
                out[f] = out[f].view(nrows * ncols, S)
    return out


def region_lut_invert(grid: torch.Tensor, config: Optional[Config] = None, *,
                      n_spatial: int = 2, n_bottoms: int = 3,
                      theta_sun: Optional[Sequence[float]] = None, n_lut: int = 16000,
                      n_chains: int = 0, rrs_noise=None, empirical: Optional[torch.Tensor] = None,
                      empirical_nodata: float = -9999.0,
                      fields: Sequence[str] = OUTPUT_FIELDS + MIX_FIELDS,
                      stream: Optional[torch.cuda.Stream] = None) -> Dict[str, torch.Tensor]:
    """samodel()'s pixel loop with its dynamic lookup table in the general
    configuration (model/samodel.c:649-1352): the fit of ``region_fit``
    (``n_spatial``, ``n_bottoms``, the scenes of a [n_scenes, nrows, ncols,
    n_bands] grid with sun zeniths ``theta_sun``) for each pixel its table
    cannot serve, the sorted shallow pixels cut into ``n_chains`` slices (0:
    eight per resident warp), each run as the reference runs them on one
    thread.  ``rrs_noise`` ([n_scenes, n_bands]) orders by the spectral
    angle too; ``empirical`` ([nrows * ncols] float32, CUDA) is the
    reference's empirical depth grid.  Use ``Config.reference_default()``
    for the reference's tolerances.  Returns the outputs (P, G, X: [npix,
    n_scenes]) plus "source", "order" and "chain_stats" as ``lut_invert``.
    Synchronises the stream once (to size the order)."""
    cfg = config or Config()
    _check_cuda(grid, "grid", torch.float32)
    g4 = grid if grid.dim() == 4 else grid.unsqueeze(0)
    if g4.dim() != 4 or g4.shape[3] != cfg.n_bands or not g4.is_contiguous():
        raise ValueError(f"grid must be a contiguous [(n_scenes,) nrows, ncols, {cfg.n_bands}]")
    S, nrows, ncols = int(g4.shape[0]), int(g4.shape[1]), int(g4.shape[2])
    npix = nrows * ncols
    if empirical is not None:
        _check_cuda(empirical, "empirical", torch.float32)
        if empirical.numel() != npix or not empirical.is_contiguous():
            raise ValueError("empirical must be a contiguous [nrows * ncols] tensor")
    out = alloc_outputs(npix, grid.device, [f for f in fields if f != "params"],
                        n_obs=npix * S if S > 1 else None)
    source = torch.empty(npix, dtype=torch.int64, device=grid.device)
    order = torch.empty(max(npix, 1), dtype=torch.int64, device=grid.device)
    lc = L.photic_lut_config()
    L.lib().photic_lut_config_default(C.byref(lc))
    lc.n_lut = int(n_lut)
    lc.n_chains = int(n_chains)
    c = cfg.to_c()
    th = (C.c_double * S)(*([cfg.theta_sun_deg] * S if theta_sun is None else
                            [float(t) for t in theta_sun]))
    noise = None
    if rrs_noise is not None:
        vals = [float(v) for row in rrs_noise for v in row]
        if len(vals) != S * cfg.n_bands:
            raise ValueError("rrs_noise must be [n_scenes, n_bands]")
        noise = (C.c_double * len(vals))(*vals)
    max_chains = int(n_chains) if n_chains else int(L.lib().photic_region_lut_default_chains(
        C.byref(c), S, int(n_spatial), int(n_bottoms)))
    if max_chains < 1:
        raise PhoticError(L.ERR_CUDA, "no chain count for this configuration: "
                          + L.lib().photic_last_error().decode(errors="replace"))
    stats = torch.zeros(max(1, min(max_chains, npix)), 4, dtype=torch.float64, device=grid.device)
    os_ = _outputs_struct(out)
    n_sh, n_ch = C.c_int64(0), C.c_int64(0)
    L.check(L.lib().photic_region_lut_invert_batch(
        C.byref(c), C.byref(lc), _ptr(g4), S, th, nrows, ncols, int(n_spatial), int(n_bottoms),
        noise, _ptr(empirical), float(empirical_nodata), C.byref(os_), _ptr(source),
        _ptr(order), _ptr(stats), C.byref(n_sh), C.byref(n_ch), _stream_handle(stream)))
    if S > 1:
        for f in ("P", "G", "X"):
            if f in out:
                out[f] = out[f].view(npix, S)
    out["source"] = source
    out["order"] = order[:n_sh.value]
    out["chain_stats"] = stats[:n_ch.value]
    return out


def depth_sigma(rrs: torch.Tensor, depth: torch.Tensor, r_sigma: Sequence[float],
                config: Optional[Config] = None, *, n_samples: int = 128, seed: int = 1,
                stream: Optional[torch.cuda.Stream] = None) -> Dict[str, torch.Tensor]:
    """The reference's depth uncertainty (model/samodel.c:1368-1479) on the
    GPU: per 0.25 m depth interval, ``n_samples`` pixels of the interval are
    refitted with their spectra moved by n * ``r_sigma`` (n uniform in
    [-1, 1]); each pixel gets its interval's standard deviation of refitted
    depths.  ``depth`` ([npix] float32, positive, 0 = not fitted) is the
    scene's fit.  Returns sigma [npix], table [120], sample_pixel and
    sample_depth [120 * n_samples]."""
    cfg = config or Config()
    _check_cuda(rrs, "rrs", torch.float32)
    _check_cuda(depth, "depth", torch.float32)
    npix = rrs.shape[0]
    if depth.numel() != npix or len(r_sigma) != cfg.n_bands:
        raise ValueError("depth must be [npix] and r_sigma one value per band")
    dev = rrs.device
    out = {"sigma": torch.empty(npix, dtype=torch.float32, device=dev),
           "table": torch.empty(120, dtype=torch.float64, device=dev),
           "sample_pixel": torch.empty(120 * n_samples, dtype=torch.int32, device=dev),
           "sample_depth": torch.empty(120 * n_samples, dtype=torch.float64, device=dev)}
    rs = (C.c_double * cfg.n_bands)(*[float(v) for v in r_sigma])
    c = cfg.to_c()
    L.check(L.lib().photic_depth_sigma(C.byref(c), _ptr(rrs), npix, _ptr(depth), rs,
                                       int(n_samples), int(seed), _ptr(out["sigma"]),
                                       _ptr(out["table"]), _ptr(out["sample_pixel"]),
                                       _ptr(out["sample_depth"]), _stream_handle(stream)))
    return out


def cost(rrs: torch.Tensor, params: torch.Tensor, config: Optional[Config] = None, *,
         stream: Optional[torch.cuda.Stream] = None):
    """samodel_error of [n, 6] parameter vectors against [n, n_bands]
    spectra; returns (cost [n] f64, modelled Rrs [n, n_bands] f64)."""
    cfg = config or Config()
    _check_cuda(rrs, "rrs", torch.float32)
    _check_cuda(params, "params", torch.float64)
    n = rrs.shape[0]
    c_out = torch.empty(n, dtype=torch.float64, device=rrs.device)
    rm = torch.empty(n, cfg.n_bands, dtype=torch.float64, device=rrs.device)
    c = cfg.to_c()
    L.check(L.lib().photic_cost_batch(C.byref(c), _ptr(rrs), _ptr(params), n, _ptr(c_out),
                                      _ptr(rm), _stream_handle(stream)))
    return c_out, rm


def generate_scene(npix: int, seed: int = 20260101, config: Optional[Config] = None, *,
                   pix0: int = 0, mask_frac: float = 0.15, noise_sigma: float = 2.0e-4,
                   device="cuda", with_truth: bool = True,
                   stream: Optional[torch.cuda.Stream] = None):
    """Synthetic scene of the plain-method workload, generated on the GPU.
    Returns (rrs [npix, n_bands] f32, truth [npix, 5] f64 = H, P, G, X, B)."""
    cfg = config or Config()
    rrs = torch.empty(npix, cfg.n_bands, dtype=torch.float32, device=device)
    truth = torch.empty(npix, 5, dtype=torch.float64, device=device) if with_truth else None
    c = cfg.to_c()
    L.check(L.lib().photic_generate_scene(C.byref(c), seed, pix0, npix, mask_frac, noise_sigma,
                                          _ptr(rrs), _ptr(truth), _stream_handle(stream)))
    return rrs, truth


def generate_field(nrows: int, ncols: int, seed: int = 20261201, config: Optional[Config] = None,
                   *, row0: int = 0, n_rows: Optional[int] = None, mask_frac: float = 0.1,
                   noise_sigma: float = 1.0e-4, device="cuda", with_truth: bool = True,
                   stream: Optional[torch.cuda.Stream] = None):
    """Spatially coherent synthetic scene (smooth depth, one water mass,
    three bottom classes), rows [row0, row0 + n_rows) of nrows x ncols,
    generated on the GPU.  Returns (rrs [n_rows * ncols, n_bands] f32,
    truth [n_rows * ncols, 5] f64 = H, P, G, X, B)."""
    cfg = config or Config()
    n_rows = nrows - row0 if n_rows is None else n_rows
    n = n_rows * ncols
    rrs = torch.empty(n, cfg.n_bands, dtype=torch.float32, device=device)
    truth = torch.empty(n, 5, dtype=torch.float64, device=device) if with_truth else None
    c = cfg.to_c()
    L.check(L.lib().photic_generate_field(C.byref(c), seed, nrows, ncols, row0, n_rows,
                                          mask_frac, noise_sigma, _ptr(rrs), _ptr(truth),
                                          _stream_handle(stream)))
    return rrs, truth


def joint_invert(offsets: torch.Tensor, theta_sun: torch.Tensor, rrs: torch.Tensor,
                 config: Optional[Config] = None, *,
                 out: Optional[Dict[str, torch.Tensor]] = None,
                 fields: Sequence[str] = OUTPUT_FIELDS,
                 stream: Optional[torch.cuda.Stream] = None) -> Dict[str, torch.Tensor]:
    """Temporal joint fit (model/samodel.c:2463-2491 with n_scenes = k).

    Pixel p owns observations offsets[p] .. offsets[p+1]-1 (int32 CSR);
    observation o has spectrum rrs[o] (float32, [n_obs, n_bands]) and
    subsurface sun zenith theta_sun[o] (float64, degrees).  Per-pixel
    outputs are [npix]; P, G, X are per observation ([n_obs]).
    ``config.layout`` selects shared (B, q) -- the reference's -- or
    per-scene B ("scene_b")."""
    cfg = config or Config()
    _check_cuda(offsets, "offsets", torch.int32)
    _check_cuda(theta_sun, "theta_sun", torch.float64)
    _check_cuda(rrs, "rrs", torch.float32)
    npix = offsets.numel() - 1
    n_obs = rrs.shape[0]
    if rrs.dim() != 2 or rrs.shape[1] != cfg.n_bands or theta_sun.numel() != n_obs:
        raise ValueError("rrs must be [n_obs, n_bands] and theta_sun [n_obs]")
    if out is None:
        out = alloc_outputs(npix, rrs.device, fields, n_obs=n_obs)
    c = cfg.to_c()
    os_ = _outputs_struct(out)
    L.check(L.lib().photic_joint_invert_batch(C.byref(c), _ptr(offsets), _ptr(theta_sun),
                                              _ptr(rrs), npix, n_obs, C.byref(os_),
                                              _stream_handle(stream)))
    return out


def generate_joint(npix: int, seed: int = 20260202, config: Optional[Config] = None, *,
                   kmin: int = 2, kmax: int = 8, theta_sun_range=(25.0, 50.0),
                   mask_frac: float = 0.0, noise_sigma: float = 2.0e-4, device="cuda",
                   stream: Optional[torch.cuda.Stream] = None):
    """Synthetic multi-scene stacks (temporal workload): per pixel k scenes
    with k ~ U{kmin..kmax}, shared depth, per-scene P, G, X, B and sun
    zenith.  Returns (offsets, theta_sun, rrs, truth)."""
    cfg = config or Config()
    h = _stream_handle(stream)
    counts = torch.empty(npix, dtype=torch.int32, device=device)
    L.check(L.lib().photic_joint_counts(seed, npix, kmin, kmax, _ptr(counts), h))
    offsets = torch.zeros(npix + 1, dtype=torch.int32, device=device)
    offsets[1:] = torch.cumsum(counts, 0, dtype=torch.int32)
    n_obs = int(offsets[-1].item())
    theta = torch.empty(n_obs, dtype=torch.float64, device=device)
    rrs = torch.empty(n_obs, cfg.n_bands, dtype=torch.float32, device=device)
    truth = torch.empty(n_obs, 5, dtype=torch.float64, device=device)
    c = cfg.to_c()
    L.check(L.lib().photic_generate_joint(C.byref(c), seed, npix, _ptr(offsets),
                                          float(theta_sun_range[0]), float(theta_sun_range[1]),
                                          mask_frac, noise_sigma, _ptr(theta), _ptr(rrs),
                                          _ptr(truth), h))
    return offsets, theta, rrs, truth


def sync(stream: Optional[torch.cuda.Stream] = None) -> None:
    """Wait for ``stream`` and raise if the device recorded an error."""
    L.check(L.lib().photic_sync(_stream_handle(stream)))


class JointGraph:
    """The temporal joint fit captured once as a CUDA graph for a fixed
    pixel count and observation count.  One replay runs the binning by
    scene count, the eight per-k kernels (parallel branches of the graph)
    and the workspace allocation, whatever the per-pixel counts in the
    offsets are.  Inputs live in the static tensors ``offsets``,
    ``theta_sun`` and ``rrs``; :meth:`run` copies new ones in (optional)
    and replays; outputs are the static tensors of ``out``.

    The library's per-device state is set up by an eager call before the
    capture, so the capture itself makes no synchronous allocation."""

    def __init__(self, npix: int, n_obs: int, config: Optional[Config] = None, *,
                 fields: Sequence[str] = OUTPUT_FIELDS, device=None):
        self.cfg = config or Config()
        dev = device or torch.device("cuda", torch.cuda.current_device())
        self.offsets = torch.zeros(npix + 1, dtype=torch.int32, device=dev)
        self.theta_sun = torch.full((n_obs,), 35.0, dtype=torch.float64, device=dev)
        self.rrs = torch.full((n_obs, self.cfg.n_bands), 0.01, dtype=torch.float32, device=dev)
        # a valid CSR layout for the warm-up: pixel p owns observation p
        # while there are observations
        self.offsets[1:] = torch.clamp(torch.arange(1, npix + 1, device=dev), max=n_obs).int()
        self.out = alloc_outputs(npix, dev, fields, n_obs=n_obs)
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            joint_invert(self.offsets, self.theta_sun, self.rrs, self.cfg, out=self.out,
                         stream=side)
        sync(side)
        torch.cuda.current_stream(dev).wait_stream(side)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            joint_invert(self.offsets, self.theta_sun, self.rrs, self.cfg, out=self.out)

    def run(self, offsets: Optional[torch.Tensor] = None,
            theta_sun: Optional[torch.Tensor] = None,
            rrs: Optional[torch.Tensor] = None) -> Dict[str, torch.Tensor]:
        if offsets is not None:
            self.offsets.copy_(offsets)
        if theta_sun is not None:
            self.theta_sun.copy_(theta_sun)
        if rrs is not None:
            self.rrs.copy_(rrs)
        self.graph.replay()
        return self.out
