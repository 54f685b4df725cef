"""Temporal joint fit on the GPU against the oracle (FP64).

Pixels carry 2..8 scenes (ragged, CSR); n = 3 + 3k unknowns in the
reference's layout (shared H, B, q) or 1 + 4k with a bottom albedo per
scene.  The oracle is the C restatement, itself pinned bit for bit to the
reference's joint fit (tests/test_oracle_vs_reference.py)."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NTHREADS = os.cpu_count() or 1


def test_joint_generator_matches_oracle(gpu, port):
    offs, th, rrs, truth = gpu.generate_joint(512, seed=77)
    torch.cuda.synchronize()
    o_offs, o_th, o_rrs, o_truth = port.generate_joint(77, 512)
    np.testing.assert_array_equal(offs.cpu().numpy(), o_offs)
    np.testing.assert_array_equal(th.cpu().numpy(), o_th)
    np.testing.assert_allclose(truth.cpu().numpy(), o_truth, rtol=1e-15)
    g = rrs.cpu().numpy()
    assert np.mean(g == o_rrs) > 0.999
    np.testing.assert_allclose(g, o_rrs, rtol=2.5e-7, atol=1e-9)


@pytest.mark.parametrize("layout,npix", [("reference", 600), ("scene_b", 300)])
def test_joint_fp64_parity(gpu, port, layout, npix):
    offs, th, rrs, _ = port.generate_joint(20260202, npix)
    cfg = gpu.Config(layout=layout)
    out = gpu.joint_invert(torch.tensor(offs, device="cuda"), torch.tensor(th, device="cuda"),
                           torch.tensor(rrs, device="cuda"), cfg)
    gpu.sync()
    out = {k: v.cpu().numpy() for k, v in out.items()}
    ref = port.joint_invert_batch(offs, th, rrs, layout=0 if layout == "reference" else 1,
                                  nthreads=NTHREADS)
    st = out["status"] & 0xFF
    np.testing.assert_array_equal(st, ref[:, 9].astype(np.int32))
    fit = st == 0
    d = np.abs(out["depth_f64"][fit] - ref[fit, 0])
    same = np.mean(d == 0)
    print(f"joint {layout}: same {same:.4f} median {np.median(d):.3g} p99 "
          f"{np.quantile(d, 0.99):.3g} within1cm {np.mean(d <= 0.01):.4f}")
    assert np.median(d) <= 0.01
    assert np.quantile(d, 0.99) <= 0.05
    assert same >= 0.90
    # per-observation P/G/X where the trajectories agree
    agree = np.where(fit & (out["depth_f64"] == ref[:, 0]))[0]
    for p in agree[:50]:
        k = offs[p + 1] - offs[p]
        np.testing.assert_allclose(out["P"][offs[p]:offs[p + 1]], ref[p, 11:11 + k].astype(np.float32),
                                   rtol=2e-6)


def test_joint_invalid_and_masked(gpu, port):
    offs, th, rrs, _ = port.generate_joint(5, 64)
    offs = offs.copy()
    rrs = rrs.copy()
    rrs[offs[3]] = -9999.0          # one scene of pixel 3 is nodata -> masked
    t = torch.tensor
    out = gpu.joint_invert(t(offs, device="cuda"), t(th, device="cuda"), t(rrs, device="cuda"))
    gpu.sync()
    st = out["status"].cpu().numpy() & 0xFF
    assert st[3] == 1
    # a pixel with zero scenes is rejected
    offs2 = np.concatenate([[0], offs]).astype(np.int32)
    out2 = gpu.joint_invert(t(offs2, device="cuda"), t(th, device="cuda"), t(rrs, device="cuda"))
    with pytest.raises(gpu.PhoticError):
        gpu.sync()
    assert (out2["status"].cpu().numpy()[0] & 0xFF) == 2


def test_joint_graph_replay_matches_eager(gpu):
    """All ragged pixels in one graph: the captured fit (binning + eight
    per-k kernels on parallel branches) replays on new inputs of the same
    sizes and gives the eager call's results bit for bit."""
    offs, th, rrs, _ = gpu.generate_joint(700, seed=4242)
    n_obs = rrs.shape[0]
    cfg = gpu.Config()
    g = gpu.JointGraph(700, n_obs, cfg)
    fields = ("depth_f64", "P", "status", "evals")
    for scale in (1.0, 1.02):
        r = (rrs * scale).contiguous()
        out = g.run(offs, th, r)
        gpu.sync()
        ref = gpu.joint_invert(offs, th, r, cfg)
        gpu.sync()
        for f in fields:
            assert torch.equal(out[f], ref[f]), f
    # another CSR layout with the same totals: reverse the per-pixel counts
    counts = (offs[1:] - offs[:-1]).flip(0)
    offs2 = torch.zeros_like(offs)
    offs2[1:] = torch.cumsum(counts, 0, dtype=torch.int32)
    out = g.run(offs2, th, rrs)
    gpu.sync()
    ref = gpu.joint_invert(offs2, th, rrs, cfg)
    gpu.sync()
    for f in fields:
        assert torch.equal(out[f], ref[f]), f
