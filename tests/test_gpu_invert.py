"""GPU parity of the plain-method inversion against the oracle.

The oracle is the C restatement (oracle/photic_oracle.c), pinned bit for bit
to the reference on the host that builds it; here it runs on the same host
as the GPU, so both use that host's libm.  The FP64 kernel evaluates the
cost in the reference's operation order; its only differences from the
oracle are the last-ulp differences between CUDA's and glibc's exp / log /
pow, which can flip a near-tie Nelder-Mead decision on a small fraction of
pixels.  The bar is therefore distributional: median |dH| <= 1 cm and
p99 |dH| <= 5 cm against the FP64 oracle, plus identical masks.
"""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NTHREADS = os.cpu_count() or 1


def _stats(h_gpu, h_ref, mask):
    d = np.abs(h_gpu[mask] - h_ref[mask])
    return np.median(d), np.quantile(d, 0.99), np.mean(d == 0.0)


def test_generator_matches_oracle(gpu, port):
    rrs, truth = gpu.generate_scene(4096, seed=20260101, pix0=12345)
    torch.cuda.synchronize()
    ref, tref = port.generate_single(20260101, 4096, pix0=12345)
    g = rrs.cpu().numpy()
    np.testing.assert_allclose(truth.cpu().numpy(), tref, rtol=1e-15, atol=0)
    same = np.mean(g == ref)
    assert same > 0.999, same
    np.testing.assert_allclose(g, ref, rtol=2.5e-7, atol=1e-9)


def test_cost_matches_oracle(gpu, port, golden_dir):
    g = np.load(os.path.join(golden_dir, "cost_nelmin.npz"))
    rrs = torch.tensor(g["rrs"], device="cuda")
    prm = torch.tensor(g["params"], device="cuda")
    c, rm = gpu.cost(rrs, prm)
    c = c.cpu().numpy()
    rm = rm.cpu().numpy()
    for i in range(len(c)):
        oc, orm, _ = port.cost(g["rrs"][i].astype(np.float64), g["params"][i])
        assert abs(c[i] - oc) <= 1e-13 * abs(oc), (i, c[i], oc)
        np.testing.assert_allclose(rm[i], orm, rtol=1e-13)


def _run_invert(gpu, rrs_np, **cfgkw):
    cfg = gpu.Config(**cfgkw)
    out = gpu.invert(torch.tensor(rrs_np, device="cuda"), cfg)
    gpu.sync()
    return {k: v.cpu().numpy() for k, v in out.items()}


@pytest.mark.parametrize("npix", [1, 7, 33, 4096])
def test_invert_fp64_parity(gpu, port, npix):
    rrs, _ = port.generate_single(20260101, npix, pix0=5000)
    out = _run_invert(gpu, rrs)
    ref = port.invert_batch(rrs, nthreads=NTHREADS)
    st = out["status"] & 0xFF
    np.testing.assert_array_equal(st, ref[:, 9].astype(np.int32))
    fit = st == 0
    if fit.sum() == 0:
        return
    med, p99, same = _stats(out["depth_f64"], ref[:, 0], fit)
    assert med <= 0.01 and p99 <= 0.05, (med, p99, same)
    if npix >= 1000:
        # identical trajectories on the great majority of pixels; the rest
        # sit on near-flat valleys where a last-ulp libm difference decides
        # a comparison
        assert same >= 0.97, same
        conv = ((out["status"] >> 8) & 1).astype(bool)
        assert np.mean(conv[fit] == (ref[fit, 8] == 1)) >= 0.97
        same_evals = np.mean(out["evals"][fit] == ref[fit, 7])
        assert same_evals >= 0.97, same_evals
    # where the trajectories agree, every output agrees to float rounding
    agree = fit & (out["depth_f64"] == ref[:, 0])
    for k, col in [("P", 11), ("G", 19), ("X", 27), ("bottom_albedo", 1),
                   ("model_error", 2), ("rrs_error", 3), ("K_min", 4), ("iod", 5)]:
        np.testing.assert_allclose(out[k][agree], ref[agree, col].astype(np.float32),
                                   rtol=2e-6, atol=1e-7, err_msg=k)


def test_invert_fp64_golden(gpu, golden_dir):
    g = np.load(os.path.join(golden_dir, "single_scene.npz"))
    out = _run_invert(gpu, g["rrs"])
    ref = g["ref"]  # columns: H B cost rrs_err Kmin iod evk ev conv status P G X
    st = out["status"] & 0xFF
    np.testing.assert_array_equal(st, ref[:, 9].astype(np.int32))
    fit = st == 0
    med, p99, same = _stats(out["depth_f64"], ref[:, 0], fit)
    assert med <= 0.01 and p99 <= 0.05 and same >= 0.97, (med, p99, same)


def test_invert_reference_tolerances(gpu, port):
    rrs, _ = port.generate_single(77, 1024)
    out = _run_invert(gpu, rrs, reqmin=1e-2, konvge=100, kcount=5000)
    ref = port.invert_batch(rrs, reqmin=None, nthreads=NTHREADS)
    fit = (out["status"] & 0xFF) == 0
    med, p99, same = _stats(out["depth_f64"], ref[:, 0], fit)
    assert med <= 0.01 and p99 <= 0.05, (med, p99, same)


def test_invert_masks_and_edges(gpu, port):
    rrs, _ = port.generate_single(9, 256, mask_frac=0.0)
    rrs[::5] = -9999.0                      # nodata
    rrs[1::5, 2] = -0.01                    # negative band
    rrs[2::5, 0] = np.float32(-9999.0 * (1 + 5e-7))  # within the 1e-6 nodata tolerance
    out = _run_invert(gpu, rrs)
    ref = port.invert_batch(rrs, nthreads=NTHREADS)
    np.testing.assert_array_equal(out["status"] & 0xFF, ref[:, 9].astype(np.int32))
    m = (out["status"] & 0xFF) == 1
    assert np.all(out["depth"][m] == 0) and np.all(out["evals"][m] == 0)


def test_invert_strided_layout_matches_contiguous(gpu, port):
    import ctypes as C
    from photic_gb300 import _lib as L
    rrs, _ = port.generate_single(21, 500)
    a = _run_invert(gpu, rrs)
    planes = torch.tensor(np.ascontiguousarray(rrs.T), device="cuda")  # [band][pixel]
    out = gpu.api.alloc_outputs(500, "cuda")
    cfg = gpu.Config().to_c()
    os_ = gpu.api._outputs_struct(out)
    L.check(L.lib().photic_invert_batch(C.byref(cfg), planes.data_ptr(), 500, 1, 500, None,
                                        C.byref(os_), torch.cuda.current_stream().cuda_stream))
    gpu.sync()
    np.testing.assert_array_equal(out["depth_f64"].cpu().numpy(), a["depth_f64"])


def test_invert_empty_and_seeded(gpu, port):
    out = gpu.invert(torch.zeros(0, 4, device="cuda"))
    gpu.sync()
    assert out["depth"].numel() == 0
    rrs, truth = port.generate_single(31, 256, mask_frac=0.0)
    seeds = np.column_stack([truth[:, 0], 100 * truth[:, 4], np.ones(256), 100 * truth[:, 1],
                             100 * truth[:, 2], 100 * truth[:, 3]])
    seeds[::4, 0] = np.nan  # these stay on the cold start
    o = gpu.invert(torch.tensor(rrs, device="cuda"), seeds=torch.tensor(seeds, device="cuda"))
    gpu.sync()
    ref = port.invert_batch(rrs, seeds=seeds, nthreads=NTHREADS)
    h = o["depth_f64"].cpu().numpy()
    fit = (o["status"].cpu().numpy() & 0xFF) == 0
    med, p99, same = _stats(h, ref[:, 0], fit)
    assert med <= 0.01 and p99 <= 0.05, (med, p99, same)


def test_invert_order_is_a_permutation_of_work(gpu):
    """A queue order changes only which lane fits which pixel: every
    pixel's outputs stay bit for bit, at its own index."""
    rrs, _ = gpu.generate_scene(20000, seed=314, pix0=777)
    fields = ("depth_f64", "evals", "status", "params")
    a = gpu.invert(rrs, fields=fields)
    order = torch.randperm(20000, device="cuda", generator=torch.Generator("cuda").manual_seed(1))
    b = gpu.invert(rrs, order=order.to(torch.int32), fields=fields)
    gpu.sync()
    for f in fields:
        assert torch.equal(torch.nan_to_num(a[f]), torch.nan_to_num(b[f])), f


def test_empty_inputs_are_no_ops(gpu):
    """Zero pixels: every batched entry point returns without launching."""
    cfg = gpu.Config()
    e = torch.empty(0, 4, dtype=torch.float32, device="cuda")
    out = gpu.invert(e, cfg)
    assert all(v.numel() == 0 for v in out.values())
    offs = torch.zeros(1, dtype=torch.int32, device="cuda")
    th = torch.empty(0, dtype=torch.float64, device="cuda")
    gpu.joint_invert(offs, th, e, cfg)
    gpu.region_invert(torch.empty(0, 5, 4, dtype=torch.float32, device="cuda"), cfg)
    c, rm = gpu.cost(e, torch.empty(0, 6, dtype=torch.float64, device="cuda"), cfg)
    assert c.numel() == 0
    gpu.sync()
