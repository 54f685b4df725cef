"""Spatial-region fit (3 x 3 neighbourhoods, model/samodel.c:2957-3027) on
the GPU against the oracle, itself pinned bit for bit to the reference's
extract_Rrs_data + samodel_optimise (tests/test_oracle_vs_reference.py,
tests/golden/regions.npz).  A grid with masked pixels and edges gives
ragged region counts (1..9); the bar is the FP64 one: identical results
except where a last-ulp libm difference decides a Nelder-Mead comparison."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kcount", [400, 2000])
def test_region_fit_matches_oracle(gpu, port, kcount):
    nr, nc = 20, 16
    rrs, _ = port.generate_single(20260707, nr * nc, pix0=31, mask_frac=0.15)
    grid = rrs.reshape(nr, nc, 4)
    cfg = gpu.Config(kcount=kcount)
    out = gpu.region_invert(torch.tensor(grid, device="cuda"), cfg)
    gpu.sync()
    out = {k: v.cpu().numpy() for k, v in out.items()}
    ref = port.region_invert_batch(grid, kcount=kcount, nthreads=os.cpu_count() or 1)
    st = out["status"]
    np.testing.assert_array_equal(st & 0xFF, ref[:, 9].astype(np.int32))
    fit = (st & 0xFF) == 0
    np.testing.assert_array_equal((st[fit] >> 24) & 0xF, ref[fit, 38].astype(np.int32))
    assert len(np.unique(ref[fit, 38])) > 1  # ragged region counts
    d = np.abs(out["depth_f64"][fit] - ref[fit, 0])
    same = d == 0
    print(f"regions kcount {kcount}: same {same.mean():.3f} median {np.median(d):.3g} "
          f"p99 {np.quantile(d, 0.99):.3g}")
    assert same.mean() >= 0.9 and np.median(d) <= 0.01 and np.quantile(d, 0.99) <= 0.05
    # where the trajectories agree, every product agrees
    # (total evaluations also count the starts that were not kept, whose
    # trajectories may split on a last-ulp difference without changing the
    # result)
    assert np.mean(out["evals"][fit][same] == ref[fit, 7][same]) >= 0.95
    for f, c, tol in (("evals_kept", 6, 0), ("model_error", 2, 1e-6), ("P", 11, 1e-6),
                      ("X", 27, 1e-6), ("K_min", 4, 1e-6), ("iod", 5, 1e-5),
                      ("bottom_albedo", 1, 1e-6)):
        a, b = out[f][fit][same].astype(np.float64), ref[fit, c][same]
        if tol == 0:
            np.testing.assert_array_equal(a, b, err_msg=f)
        else:
            np.testing.assert_allclose(a, b.astype(np.float32), rtol=tol, err_msg=f)
