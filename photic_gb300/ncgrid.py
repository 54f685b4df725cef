"""The reference's netCDF grid files (model/nc.c) on both sides of the
inversion: band grids read straight into the device layout ``invert``
takes, result grids written from device tensors.  Packing and unpacking
run on the GPU (include/photic_nc.h); the container functions
``read_info``, ``read_raw`` and ``write_raw`` need no GPU.

    rrs, info, lons, lats = read_bands(["b1.nc", "b2.nc", "b3.nc", "b4.nc"])
    out = photic_gb300.invert(rrs, cfg)
    write_grid("depth.nc", out["depth"].view(info["nrows"], info["ncols"]),
               lons, lats, spval=info["spval"])
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Dict, Optional, Sequence, Tuple

import numpy as np

from . import _lib as L

_INFO_FIELDS = ("ncols", "nrows", "add_offset", "scale_factor", "missing_value",
                "has_missing_value", "spval", "has_spval", "format")


def _info_dict(i: L.photic_nc_grid_info) -> Dict:
    return {k: getattr(i, k) for k in _INFO_FIELDS}


def _info_struct(d: Dict) -> L.photic_nc_grid_info:
    i = L.photic_nc_grid_info()
    i.ncols, i.nrows = int(d["ncols"]), int(d["nrows"])
    i.add_offset = float(d["add_offset"])
    i.scale_factor = float(d["scale_factor"])
    i.missing_value = int(d.get("missing_value", -32768))
    i.has_missing_value = int(d.get("has_missing_value", 1))
    i.spval = float(d.get("spval", 0.0))
    i.has_spval = int(d.get("has_spval", 1))
    i.format = int(d.get("format", 0))
    return i


def _path(p) -> bytes:
    return os.fsencode(p)


def read_info(path) -> Dict:
    """Dimensions and packing attributes of a grid file."""
    i = L.photic_nc_grid_info()
    L.check(L.lib().photic_nc_read_info(_path(path), C.byref(i)))
    return _info_dict(i)


def read_raw(path) -> Tuple[np.ndarray, np.ndarray, np.ndarray, Dict]:
    """(packed int16 [nrows, ncols] in host order, lons, lats, info)."""
    info = read_info(path)
    nr, nc = info["nrows"], info["ncols"]
    be = np.empty((nr, nc), dtype=">i2")
    lons = np.empty(nc, dtype=np.float32)
    lats = np.empty(nr, dtype=np.float32)
    i = L.photic_nc_grid_info()
    L.check(L.lib().photic_nc_read_raw(_path(path), C.byref(i), be.ctypes.data,
                                       lons.ctypes.data, lats.ctypes.data))
    return be.astype(np.int16), lons, lats, _info_dict(i)


def write_raw(path, packed: np.ndarray, lons, lats, add_offset: float, scale_factor: float,
              missing_value: int = -32768, spval: float = 0.0, fmt: int = 0) -> None:
    """A grid file with write_nc's layout around an already packed grid."""
    p = np.ascontiguousarray(packed, dtype=">i2")
    nr, nc = p.shape
    lo = np.ascontiguousarray(lons, dtype=np.float32)
    la = np.ascontiguousarray(lats, dtype=np.float32)
    if lo.size != nc or la.size != nr:
        raise ValueError("lons / lats do not match the grid")
    i = _info_struct({"ncols": nc, "nrows": nr, "add_offset": add_offset,
                      "scale_factor": scale_factor, "missing_value": missing_value,
                      "spval": spval, "format": fmt})
    L.check(L.lib().photic_nc_write_raw(_path(path), C.byref(i), p.ctypes.data, lo.ctypes.data,
                                        la.ctypes.data))


def _stream(stream) -> Optional[int]:
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def pack(grid, spval: float, stream=None):
    """compress_2d of a device float32 tensor: (packed big-endian bytes as a
    uint8 device tensor of 2 * numel, info dict)."""
    import torch
    g = grid.contiguous()
    if g.dtype != torch.float32 or not g.is_cuda:
        raise TypeError("grid must be a float32 CUDA tensor")
    out = torch.empty(2 * g.numel(), dtype=torch.uint8, device=g.device)
    i = L.photic_nc_grid_info()
    L.check(L.lib().photic_nc_pack(g.data_ptr(), g.numel(), float(spval), out.data_ptr(),
                                   C.byref(i), _stream(stream)))
    return out, _info_dict(i)


def unpack_bands(packed: Sequence, infos: Sequence[Dict], npix: int, stream=None):
    """decompress_2d of several packed grids (uint8 device tensors, big-endian)
    into one float32 [npix, n_bands] device tensor."""
    import torch
    nb = len(packed)
    if nb != len(infos) or not 1 <= nb <= L.MAX_BANDS:
        raise ValueError("one info per packed grid, 1..8 grids")
    dev = packed[0].device
    out = torch.empty(npix, nb, dtype=torch.float32, device=dev)
    ptrs = (C.c_void_p * nb)(*[p.data_ptr() for p in packed])
    st = (L.photic_nc_grid_info * nb)(*[_info_struct(d) for d in infos])
    L.check(L.lib().photic_nc_unpack_bands(ptrs, st, nb, npix, out.data_ptr(), _stream(stream)))
    return out


def read_bands(paths: Sequence, device=None, stream=None):
    """The band files of one scene: (rrs float32 [nrows * ncols, n_bands] on
    the device, band 0's info, lons, lats)."""
    import torch
    nb = len(paths)
    info0 = read_info(paths[0])
    npix = info0["nrows"] * info0["ncols"]
    dev = torch.device(device) if device is not None else torch.device("cuda",
                                                                       torch.cuda.current_device())
    rrs = torch.empty(npix, nb, dtype=torch.float32, device=dev)
    lons = np.empty(info0["ncols"], dtype=np.float32)
    lats = np.empty(info0["nrows"], dtype=np.float32)
    arr = (C.c_char_p * nb)(*[_path(p) for p in paths])
    i = L.photic_nc_grid_info()
    L.check(L.lib().photic_nc_read_bands(arr, nb, rrs.data_ptr(), npix, C.byref(i),
                                         lons.ctypes.data, lats.ctypes.data, _stream(stream)))
    return rrs, _info_dict(i), lons, lats


def write_grid(path, grid, lons, lats, spval: float, stream=None) -> None:
    """write_nc of a device float32 grid [nrows, ncols]."""
    import torch
    g = grid.contiguous()
    if g.dtype != torch.float32 or not g.is_cuda or g.dim() != 2:
        raise TypeError("grid must be a 2-D float32 CUDA tensor")
    nr, nc = g.shape
    lo = np.ascontiguousarray(lons, dtype=np.float32)
    la = np.ascontiguousarray(lats, dtype=np.float32)
    if lo.size != nc or la.size != nr:
        raise ValueError("lons / lats do not match the grid")
    L.check(L.lib().photic_nc_write_grid(_path(path), g.data_ptr(), nc, nr, lo.ctypes.data,
                                         la.ctypes.data, float(spval), _stream(stream)))
