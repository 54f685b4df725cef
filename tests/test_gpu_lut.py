"""samodel()'s pixel loop with its dynamic lookup table on the GPU
(photic_lut_invert_batch) against the oracle's restatement -- itself pinned
bit for bit to the reference's own samodel() with LUT 1 on one thread
(tests/test_lut_oracle.py) -- and against that reference fixture
(tests/golden/lut.npz) directly.

The order of the pixels is integer work and must be identical.  The loop
is a chain: every fit hot-starts from the previous pixel's, and a served
pixel takes a stored fit, so one last-ulp difference between the device's
and the host's exp / log / pow in one fit moves every later hot start of
that chain until a discontinuity restarts it cold.  The bars are therefore
on the distributions: the share of identical depths, the median |dH|, and
the served share against the oracle's (and the reference's), with the
statistics printed."""
import os

import numpy as np
import pytest
import torch

from tests.test_lut_oracle import fixture_case

pytestmark = pytest.mark.gpu

NTHREADS = os.cpu_count() or 1


def _ref_cfg(gpu):
    return gpu.Config.reference_default()


def _run(gpu, rrs, n_chains, rrs_noise=None, empirical=None):
    em = None if empirical is None else torch.tensor(empirical, device="cuda")
    out = gpu.lut_invert(torch.tensor(rrs, device="cuda"), _ref_cfg(gpu), n_chains=n_chains,
                         rrs_noise=rrs_noise, empirical=em)
    gpu.sync()
    return {k: v.cpu().numpy() for k, v in out.items()}


def _stats(name, h_gpu, h_ref, src_gpu, src_ref, fit):
    d = np.abs(np.asarray(h_gpu, np.float64)[fit] - np.asarray(h_ref, np.float64)[fit])
    sg, sr = np.mean(src_gpu[fit] >= 0), np.mean(src_ref[fit] >= 0)
    print(f"{name}: {fit.sum()} px, identical depth {np.mean(d == 0):.4f}, median |dH| "
          f"{np.median(d):.3g} m, p90 {np.quantile(d, 0.9):.3g} m; served GPU {sg:.4f} "
          f"oracle {sr:.4f}")
    return d, sg, sr


def test_field_generator_matches_oracle(gpu, port):
    n = 64
    rrs, truth = gpu.generate_field(n, n, seed=20261265)
    gpu.sync()
    want, wt = port.generate_field(20261265, n, n)
    got = rrs.cpu().numpy()
    same = np.mean(got == want)
    rel = np.abs(got.astype(np.float64) - want) / np.maximum(np.abs(want), 1e-30)
    print(f"field generator: identical {same:.5f}, max rel diff {rel.max():.2g}")
    assert same >= 0.99 and rel.max() < 1e-5
    np.testing.assert_allclose(truth.cpu().numpy(), wt, rtol=1e-12)


@pytest.mark.parametrize("case", ["plain", "noise", "emp"])
def test_order_matches_oracle(gpu, port, golden_dir, case):
    """The spectral-index order, with the reference's merge tree where NaN
    keys (masked pixels under the spectral angle) occur, or the empirical
    depths' order, bit for bit."""
    rrs, rs, em, _, _ = fixture_case(golden_dir, case)
    o = _run(gpu, rrs, 1, rs, em)
    ref, src, order, _ = port.lut_invert(rrs, rrs_noise=rs, empirical=em, n_chains=1,
                                         nthreads=1)
    np.testing.assert_array_equal(o["order"], order)
    np.testing.assert_array_equal(o["source"] == -2, src == -2)
    np.testing.assert_array_equal(o["status"] & 0xFF, ref[:, 9].astype(np.int32))


@pytest.mark.parametrize("case", ["plain", "noise", "emp"])
def test_one_chain_against_reference(gpu, port, golden_dir, case):
    """One chain is the reference's samodel() on one thread: its fixture."""
    rrs, rs, em, ref_grids, _ = fixture_case(golden_dir, case)
    o = _run(gpu, rrs, 1, rs, em)
    ref_depth = -ref_grids[0].reshape(-1)
    _, src_o, _, _ = port.lut_invert(rrs, rrs_noise=rs, empirical=em, n_chains=1, nthreads=1)
    fit = (o["status"] & 0xFF) == 0
    d, sg, sr = _stats(f"one chain vs reference ({case})", o["depth"], ref_depth, o["source"],
                       src_o, fit)
    assert np.median(d) <= 0.01
    assert np.mean(d == 0) >= 0.5
    assert abs(sg - sr) <= 0.05


def test_chains_against_oracle(gpu, port):
    """32 chains over a 128 x 128 scene against the oracle's 32 chains."""
    n, C = 128, 32
    rrs, _ = port.generate_field(20261212, n, n)
    o = _run(gpu, rrs, C)
    ref, src, order, stats = port.lut_invert(rrs, n_chains=C, nthreads=NTHREADS)
    np.testing.assert_array_equal(o["order"], order)
    assert o["chain_stats"].shape == (C, 4)
    fit = ref[:, 9] == 0
    d, sg, sr = _stats("32 chains vs oracle", o["depth_f64"], ref[:, 0], o["source"], src, fit)
    assert np.median(d) <= 0.01
    assert np.mean(d == 0) >= 0.5
    assert abs(sg - sr) <= 0.05
    # per chain: served + fitted = the slice
    S = order.size
    lens = np.array([(c + 1) * S // C - c * S // C for c in range(C)])
    np.testing.assert_array_equal(o["chain_stats"][:, 0] + o["chain_stats"][:, 1], lens)


def test_served_pixels_carry_their_source(gpu, port):
    n = 96
    rrs, _ = port.generate_field(9090, n, n)
    o = _run(gpu, rrs, 4)
    s = np.where(o["source"] >= 0)[0]
    assert s.size > 0
    src = o["source"][s]
    for f in ("depth_f64", "P", "G", "X", "bottom_albedo", "rrs_error", "K_min", "iod"):
        np.testing.assert_array_equal(o[f][s], o[f][src], err_msg=f)
    np.testing.assert_array_equal(o["params"][s], o["params"][src])
    assert np.all(o["status"][s] & 0x200) and np.all(o["evals"][s] == 0)
    assert np.all(o["source"][src] == -1)  # entries are fits
    fitted = o["source"] == -1
    assert np.all((o["status"][fitted] & 0x200) == 0) and np.all(o["evals"][fitted] > 0)
    # the model error of a served pixel is its spectral difference, within
    # the match threshold's floor or above it
    assert np.all(o["model_error"][s] >= 0)


def test_default_chains(gpu, port):
    """n_chains = 0: eight chains per resident lane of the kernel."""
    n = 256
    rrs, _ = gpu.generate_field(n, n, seed=555)
    out = gpu.lut_invert(rrs, _ref_cfg(gpu))
    gpu.sync()
    st = out["status"].cpu().numpy()
    src = out["source"].cpu().numpy()
    fit = (st & 0xFF) == 0
    assert fit.mean() > 0.8
    S = int(out["order"].numel())
    C = int(out["chain_stats"].shape[0])
    assert C == min(S, int(gpu.api.L.lib().photic_lut_default_chains(
        __import__("ctypes").byref(_ref_cfg(gpu).to_c()))))
    print(f"default chains: {C} chains over {S} shallow pixels, served "
          f"{np.mean(src[fit] >= 0):.4f}")


def test_eight_bands(gpu, port):
    """The 8-band instantiation of the lookup-table kernel (bands 1..3 of an
    OLCI-like set carry the spectral index and the difference)."""
    wl8 = (412.5, 442.5, 490.0, 510.0, 560.0, 620.0, 665.0, 708.75)
    n, C = 48, 4
    rrs, _ = port.generate_field(4848, n, n, wl=wl8)
    cfg = gpu.Config.reference_default(wavelengths=wl8)
    out = gpu.lut_invert(torch.tensor(rrs, device="cuda"), cfg, n_chains=C)
    gpu.sync()
    o = {k: v.cpu().numpy() for k, v in out.items()}
    ref, src, order, _ = port.lut_invert(rrs, wl=wl8, n_chains=C, nthreads=NTHREADS)
    np.testing.assert_array_equal(o["order"], order)
    fit = ref[:, 9] == 0
    d, sg, sr = _stats("8 bands, 4 chains vs oracle", o["depth_f64"], ref[:, 0], o["source"], src,
                       fit)
    assert np.median(d) <= 0.01
    assert np.mean(d == 0) >= 0.5
    assert abs(sg - sr) <= 0.05


def test_edges(gpu, port):
    """No pixels, every pixel masked, and more chains than shallow pixels
    (the chain count clamps to the pixels, as in the oracle)."""
    cfg = _ref_cfg(gpu)
    out = gpu.lut_invert(torch.empty(0, 4, device="cuda"), cfg)
    gpu.sync()
    assert out["order"].numel() == 0 and out["chain_stats"].shape[0] == 0
    assert out["depth"].numel() == 0
    o = _run(gpu, np.full((50, 4), -9999.0, np.float32), 0)
    assert o["order"].size == 0 and o["chain_stats"].shape[0] == 0
    assert np.all(o["source"] == -2) and np.all((o["status"] & 0xFF) == 1)
    rrs, _ = port.generate_field(99, 3, 3)
    rrs[4] = -9999.0
    for C in (1, 64):
        o = _run(gpu, rrs, C)
        ref, src, order, st = port.lut_invert(rrs, n_chains=C, nthreads=1)
        np.testing.assert_array_equal(o["order"], order)
        assert o["chain_stats"].shape[0] == st.shape[0] == min(C, order.size)
        np.testing.assert_array_equal(o["source"] < 0, src < 0)
        np.testing.assert_array_equal(o["status"] & 0xFF, ref[:, 9].astype(np.int32))
        fit = ref[:, 9] == 0
        d = np.abs(o["depth_f64"][fit] - ref[fit, 0])
        assert np.median(d) <= 0.01, d
