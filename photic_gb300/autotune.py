"""Launch-shape autotuner: picks ``block_threads`` and ``blocks_per_sm``
for the inversion and the temporal joint fit on the device at hand.

The timing loop is native (photic_autotune in include/photic.h): each
candidate runs once untimed and once under CUDA events on a seeded
synthetic sample of the workload.  This module adds a persistent cache so a
process tunes a (device, workload) pair once: entries are keyed by the
device name and SM count, the kind (invert / joint), precision, band count
and layout, and stored as JSON at ``$PHOTIC_TUNE_CACHE`` or
``~/.cache/photic_gb300/launch_shapes.json``.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import json
import os
from typing import Callable, Dict, Optional, Tuple

from . import _lib as L
from .api import Config

KINDS = {"invert": L.TUNE_INVERT, "joint": L.TUNE_JOINT}


def cache_path() -> str:
    p = os.environ.get("PHOTIC_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "photic_gb300", "launch_shapes.json")


def cache_key(device: str, sms: int, kind: str, cfg: Config) -> str:
    return (f"{device}|sm{sms}|{kind}|{cfg.precision}|bands{cfg.n_bands}|{cfg.layout}")


def _load(path: str) -> Dict[str, dict]:
    try:
        with open(path) as f:
            d = json.load(f)
        return d if isinstance(d, dict) else {}
    except (OSError, ValueError):
        return {}


def _store(path: str, d: Dict[str, dict]) -> None:
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + f".tmp{os.getpid()}"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def measure(cfg: Config, kind: str = "invert",
            sample_npix: int = 1 << 17) -> Tuple[Tuple[int, int], list]:
    """Run the native tuner; returns ((block_threads, blocks_per_sm), table
    of (block_threads, blocks_per_sm, ms) per candidate)."""
    c = cfg.to_c()
    res = (C.c_double * (3 * 32))()
    n = C.c_int32(0)
    L.check(L.lib().photic_autotune(C.byref(c), KINDS[kind], int(sample_npix), res, 32,
                                    C.byref(n)))
    table = [(int(res[3 * i]), int(res[3 * i + 1]), float(res[3 * i + 2]))
             for i in range(n.value)]
    return (int(c.block_threads), int(c.blocks_per_sm)), table


def _device() -> Tuple[str, int]:
    import torch
    p = torch.cuda.get_device_properties(torch.cuda.current_device())
    return p.name, int(p.multi_processor_count)


def tuned(cfg: Optional[Config] = None, kind: str = "invert", *, sample_npix: int = 1 << 17,
          use_cache: bool = True, retune: bool = False,
          measure_fn: Optional[Callable] = None, device: Optional[Tuple[str, int]] = None
          ) -> Config:
    """``cfg`` with the tuned launch shape for ``kind``; tunes on a miss.
    ``measure_fn`` and ``device`` replace the GPU measurement and the device
    query (for tests of the cache logic)."""
    if kind not in KINDS:
        raise ValueError(f"kind must be one of {sorted(KINDS)}")
    cfg = cfg or Config()
    name, sms = device or _device()
    key = cache_key(name, sms, kind, cfg)
    path = cache_path()
    db = _load(path) if use_cache else {}
    hit = db.get(key)
    if hit is None or retune:
        shape, table = (measure_fn or measure)(cfg, kind, sample_npix)
        hit = {"block_threads": shape[0], "blocks_per_sm": shape[1], "table": table,
               "sample_npix": sample_npix}
        if use_cache:
            db[key] = hit
            _store(path, db)
    return dataclasses.replace(cfg, block_threads=int(hit["block_threads"]),
                               blocks_per_sm=int(hit["blocks_per_sm"]))
