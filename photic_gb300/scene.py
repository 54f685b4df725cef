"""The reference's SCENE command (model/bam.c:1300-1543) on the host side:
parse the command text into the scene record, map it onto a
:class:`~photic_gb300.api.Config`, and read the named band files into the
inversion's device layout, so a real LANDSAT / Sentinel scene given the way
the reference's command files give it can be fed to the fit."""
from __future__ import annotations

import ctypes as C
import os
from typing import Callable, Dict, Optional

from . import _lib as L
from .api import Config

MAX_STRING_LEN = 2048
MAX_GRIDS = 265
MAX_BANDS = 64
NAME_LEN = 256
GIVEN = {"RINF": 1, "HTIDE": 2, "K": 4, "RSIGMA": 8, "KSIGMA": 16}


class photic_scene(C.Structure):
    """include/photic_samodel.h (the reference's scene, model/common.h:194-218)"""
    _fields_ = [
        ("scene_name", C.c_char * MAX_STRING_LEN),
        ("n_bands", C.c_int),
        ("nrows", C.c_int),
        ("ncols", C.c_int),
        ("band_indexes", C.c_int * MAX_GRIDS),
        ("wavelengths", C.c_int * MAX_GRIDS),
        ("theta_w", C.c_double),
        ("theta_v", C.c_double),
        ("H_tide", C.c_double),
        ("R_inf", C.c_double * MAX_GRIDS),
        ("R_sigma", C.c_double * MAX_GRIDS),
        ("K", C.c_double * MAX_GRIDS),
        ("K_sigma", C.c_double * MAX_GRIDS),
        ("ratio_min", C.c_double),
        ("ratio_max", C.c_double),
        ("slope_min", C.c_double),
        ("slope_max", C.c_double),
        ("pgx_present", C.c_int),
        ("ps_p", C.c_int),
        ("ps_g", C.c_int),
        ("ps_x", C.c_int),
    ]


class photic_scene_spec(C.Structure):
    _fields_ = [
        ("scene", photic_scene),
        ("band_names", (C.c_char * NAME_LEN) * MAX_BANDS),
        ("pgx_names", (C.c_char * NAME_LEN) * 3),
        ("given", C.c_int32),
    ]


def _bind():
    lib = L.lib()
    lib.photic_parse_scene.restype = C.c_int
    lib.photic_parse_scene.argtypes = [C.c_char_p, C.POINTER(photic_scene_spec)]
    lib.photic_config_from_scene.restype = C.c_int
    lib.photic_config_from_scene.argtypes = [C.POINTER(photic_scene), C.POINTER(L.photic_config)]
    return lib


def parse(line: str) -> Dict:
    """The record the reference's run_scene fills from one SCENE line."""
    lib = _bind()
    spec = photic_scene_spec()
    L.check(lib.photic_parse_scene(line.encode(), C.byref(spec)))
    s = spec.scene
    nb = s.n_bands
    given = {k for k, bit in GIVEN.items() if spec.given & bit}
    return {"name": s.scene_name.decode(), "n_bands": nb,
            "bands": [spec.band_names[n].value.decode() for n in range(nb)],
            "wavelengths": [s.wavelengths[n] for n in range(nb)],
            "theta_view": s.theta_v, "theta_sun": s.theta_w, "h_tide": s.H_tide,
            "R_inf": [s.R_inf[n] for n in range(nb)], "K": [s.K[n] for n in range(nb)],
            "R_sigma": [s.R_sigma[n] for n in range(nb)],
            "K_sigma": [s.K_sigma[n] for n in range(nb)],
            "pgx": [spec.pgx_names[c].value.decode() for c in range(3)],
            "pgx_present": bool(s.pgx_present), "given": sorted(given), "_spec": spec}


def config(rec: Dict, **overrides) -> Config:
    """The inversion's configuration for a parsed scene (the library's
    photic_config_from_scene): bands, wavelengths, subsurface sun and view
    zenith, tidal height."""
    lib = _bind()
    c = L.photic_config()
    L.check(lib.photic_config_from_scene(C.byref(rec["_spec"].scene), C.byref(c)))
    cfg = Config(wavelengths=tuple(c.wavelengths[b] for b in range(c.n_bands)),
                 theta_sun_deg=c.theta_sun_deg, theta_view_deg=c.theta_view_deg,
                 h_tide=c.h_tide)
    for k, v in overrides.items():
        setattr(cfg, k, v)
    return cfg


def load(line: str, band_file: Callable[[str], str], device=None, **overrides):
    """Parse a SCENE line, read its band grids (``band_file`` maps a band name
    to its netCDF file) into the device layout [nrows * ncols, n_bands], and
    return (config, rrs, info, lons, lats, record)."""
    from .ncgrid import read_bands
    rec = parse(line)
    cfg = config(rec, **overrides)
    rrs, info, lons, lats = read_bands([band_file(b) for b in rec["bands"]], device=device)
    return cfg, rrs, info, lons, lats, rec
