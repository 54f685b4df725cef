"""The native launch-shape autotuner on the GPU: every candidate runs, the
choice is one of them, and fits do not depend on the launch shape."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_autotune_invert_and_joint(gpu, tmp_path, monkeypatch):
    from photic_gb300 import autotune as A
    monkeypatch.setenv("PHOTIC_TUNE_CACHE", str(tmp_path / "shapes.json"))
    cfg = gpu.Config()
    shape, table = A.measure(cfg, "invert", sample_npix=1 << 14)
    assert len(table) == 12 and all(ms > 0 for _, _, ms in table)
    assert shape in [(b, s) for b, s, _ in table]
    assert min(table, key=lambda r: r[2])[:2] == shape
    shape_j, table_j = A.measure(cfg, "joint", sample_npix=1 << 11)
    assert len(table_j) == 5 and shape_j[1] in (2, 3, 4, 6, 8)

    rrs, _ = gpu.generate_scene(1 << 14, seed=123)
    tuned = A.tuned(cfg, "invert", sample_npix=1 << 14)
    a = gpu.invert(rrs, cfg, fields=("depth_f64", "evals", "status"))
    b = gpu.invert(rrs, tuned, fields=("depth_f64", "evals", "status"))
    odd = gpu.Config(block_threads=64, blocks_per_sm=1)
    c = gpu.invert(rrs, odd, fields=("depth_f64", "evals", "status"))
    gpu.sync()
    for f in ("depth_f64", "evals", "status"):
        assert torch.equal(a[f], b[f]) and torch.equal(a[f], c[f]), f
