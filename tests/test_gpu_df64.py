"""Double-float (PHOTIC_PREC_DF64) path against the FP64 oracle.

The cost is evaluated with ~48-bit double-float arithmetic on the FP32
pipes; it must agree with the double-precision cost to 1e-12 relative.
That is not enough to reproduce every Nelder-Mead trajectory: on about 1 %
of pixels a decision between two costs that tie to ~1e-14 goes the other
way and the fit ends elsewhere on the (underdetermined) solution curve.
So this mode is held to median |dH| <= 1 cm and >= 97 % of pixels within
1 cm; only the FP64 mode meets the p99 <= 5 cm bar (test_gpu_invert.py)."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NTHREADS = os.cpu_count() or 1


def test_cost_df64_matches_oracle(gpu, port, golden_dir):
    g = np.load(os.path.join(golden_dir, "cost_nelmin.npz"))
    rng = np.random.default_rng(5)
    rrs, truth = port.generate_single(99, 2048, mask_frac=0.0)
    params = np.column_stack([truth[:, 0], 100 * truth[:, 4], np.ones(2048), 100 * truth[:, 1],
                              100 * truth[:, 2], 100 * truth[:, 3]])
    params *= rng.uniform(0.5, 1.5, size=params.shape)
    rrs = np.concatenate([g["rrs"], rrs])
    params = np.concatenate([g["params"], params])
    c, _ = gpu.cost(torch.tensor(rrs, device="cuda"), torch.tensor(params, device="cuda"),
                    gpu.Config(precision="df64"))
    c = c.cpu().numpy()
    ref = np.array([port.cost(rrs[i].astype(np.float64), params[i])[0] for i in range(len(c))])
    rel = np.abs(c - ref) / np.abs(ref)
    assert rel.max() <= 1e-12, (rel.max(), np.argmax(rel))


@pytest.mark.parametrize("npix", [33, 4096])
def test_invert_df64_parity(gpu, port, npix):
    rrs, _ = port.generate_single(20260101, npix, pix0=9000)
    out = gpu.invert(torch.tensor(rrs, device="cuda"), gpu.Config(precision="df64"))
    gpu.sync()
    ref = port.invert_batch(rrs, nthreads=NTHREADS)
    st = out["status"].cpu().numpy() & 0xFF
    np.testing.assert_array_equal(st, ref[:, 9].astype(np.int32))
    fit = st == 0
    d = np.abs(out["depth_f64"].cpu().numpy()[fit] - ref[fit, 0])
    med, p99 = np.median(d), np.quantile(d, 0.99)
    within = np.mean(d <= 0.01)
    print(f"df64 npix={npix}: median {med:.3g} p99 {p99:.3g} within1cm {within:.4f}")
    assert med <= 0.01 and within >= 0.97, (med, p99, within)
