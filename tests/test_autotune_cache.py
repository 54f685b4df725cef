"""Cache logic of the launch-shape autotuner (photic_gb300/autotune.py),
with the GPU measurement replaced by a stub."""
import json

import pytest

from photic_gb300 import Config
from photic_gb300 import autotune as A


def test_tune_caches_per_device_and_workload(tmp_path, monkeypatch):
    monkeypatch.setenv("PHOTIC_TUNE_CACHE", str(tmp_path / "shapes.json"))
    calls = []

    def fake(cfg, kind, n):
        calls.append((kind, cfg.precision, n))
        return (256, 3) if kind == "invert" else (128, 6), [(64, 0, 2.0), (256, 3, 1.0)]

    dev = ("GB300-test", 152)
    c = A.tuned(Config(), "invert", sample_npix=1000, measure_fn=fake, device=dev)
    assert (c.block_threads, c.blocks_per_sm) == (256, 3)
    c = A.tuned(Config(), "invert", sample_npix=1000, measure_fn=fake, device=dev)
    assert len(calls) == 1                       # served from the cache
    j = A.tuned(Config(), "joint", measure_fn=fake, device=dev)
    assert (j.block_threads, j.blocks_per_sm) == (128, 6) and len(calls) == 2
    A.tuned(Config(precision="df64"), "invert", measure_fn=fake, device=dev)
    A.tuned(Config(), "invert", measure_fn=fake, device=("other", 132))
    assert len(calls) == 4
    A.tuned(Config(), "invert", measure_fn=fake, device=dev, retune=True)
    assert len(calls) == 5
    db = json.load(open(tmp_path / "shapes.json"))
    assert len(db) == 4
    key = A.cache_key("GB300-test", 152, "invert", Config())
    assert db[key]["table"] == [[64, 0, 2.0], [256, 3, 1.0]]
    # the other fields of the config are kept
    c = A.tuned(Config(reqmin=1e-2, theta_sun_deg=40.0), "invert", measure_fn=fake, device=dev)
    assert c.reqmin == 1e-2 and c.theta_sun_deg == 40.0


def test_corrupt_cache_is_ignored(tmp_path, monkeypatch):
    p = tmp_path / "shapes.json"
    p.write_text("{not json")
    monkeypatch.setenv("PHOTIC_TUNE_CACHE", str(p))
    c = A.tuned(Config(), "invert", measure_fn=lambda cfg, k, n: ((64, 2), []),
                device=("x", 1))
    assert c.block_threads == 64 and json.load(open(p))


def test_bad_kind():
    with pytest.raises(ValueError):
        A.tuned(Config(), "gemm", measure_fn=lambda *a: ((64, 2), []), device=("x", 1))
