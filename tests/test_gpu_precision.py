"""The precision policies of the inversion against the FP64 oracle.

FP64 is the drop-in and the headline: faithful to the oracle except on the
last-ulp pixels (tests/test_gpu_invert.py).  The FP32 forward model with the
special-function unit -- the bulk of the arithmetic in FP32 -- keeps the simplex and every decision in FP64 but feeds them costs accurate to
~1e-6 relative, so the Nelder-Mead path departs from the oracle's wherever
two vertex costs are that close; this test measures how far its fits land
from the oracle's, and checks that it runs the same pixels to valid fits.
The guarded policy's decision tally shows how often its double-float screen
has to defer to FP64."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NTHREADS = os.cpu_count() or 1


def test_fp32_forward_model_measured(gpu, port):
    rrs, _ = port.generate_single(20260101, 8192, pix0=3_000_000)
    ref = port.invert_batch(rrs, nthreads=NTHREADS)
    out = gpu.invert(torch.tensor(rrs, device="cuda"), gpu.Config(precision="fp32"))
    gpu.sync()
    out = {k: v.cpu().numpy() for k, v in out.items()}
    st = out["status"] & 0xFF
    np.testing.assert_array_equal(st, ref[:, 9].astype(np.int32))
    fit = st == 0
    d = np.abs(out["depth_f64"][fit] - ref[fit, 0])
    print(f"fp32 forward model: {d.size} px, identical {np.mean(d == 0):.4f}, median |dH| "
          f"{np.median(d):.3g} m, p90 {np.quantile(d, 0.9):.3g} m, p99 {np.quantile(d, 0.99):.3g} m, "
          f"within 1 cm {np.mean(d <= 0.01):.4f}")
    # every fitted pixel gets a finite, positive depth and a converged share
    # like the oracle's
    assert np.all(np.isfinite(out["depth_f64"][fit])) and np.all(out["depth_f64"][fit] > 0)
    conv = ((out["status"][fit] >> 8) & 1).mean()
    assert abs(conv - ref[fit, 8].mean()) < 0.05


def test_guarded_decision_tally(gpu, port):
    from photic_gb300 import _lib as L
    rrs, _ = gpu.generate_scene(1 << 15, seed=20260101, pix0=123)
    stats = torch.zeros(5, dtype=torch.int64, device="cuda")
    L.check(L.lib().photic_set_guard_stats(stats.data_ptr()))
    g = gpu.invert(rrs, gpu.Config(precision="guarded"), fields=("depth_f64", "status"))
    gpu.sync()
    L.check(L.lib().photic_set_guard_stats(None))
    f = gpu.invert(rrs, gpu.Config(precision="fp64"), fields=("depth_f64", "status"))
    gpu.sync()
    s = stats.cpu().numpy().astype(float)
    dec = s[:3].sum()
    print(f"guarded: {dec:.3g} decisions: {s[0] / dec:.4f} on known exact values, "
          f"{s[1] / dec:.4f} on the double-float screen, {s[2] / dec:.4f} deferred to FP64; "
          f"{s[3] / s[4]:.4f} of busy lane-trips waiting")
    assert dec > 0 and s[1] > 0 and s[4] > 0
    # the decisions, hence the fits, are the FP64 kernel's (test_gpu_guarded.py
    # has the bar: at least 99.9 % identical depths)
    assert (g["depth_f64"] == f["depth_f64"]).float().mean().item() >= 0.999
