"""samodel()'s pixel loop with its dynamic lookup table in the general
configuration on the GPU (photic_region_lut_invert_batch: 3 x 3 regions,
mixtures of bottom types, the spectral-angle order, empirical depths,
stacks of scenes) against the oracle's restatement -- pinned bit for bit to
the reference's own samodel() (tests/test_glut_oracle.py) -- and against the
reference's grids (tests/golden/glut.npz), directly and through the
samodel() drop-in called from C.

The order of the pixels is integer work and must be identical.  A chain
hot-starts every fit from the previous pixel's, so one last-ulp difference
between the device's and the host's exp / log / pow in one fit moves the
later hot starts of that chain until a discontinuity restarts it cold; the
bars are on the distributions (identical depths, median |dH|, the served
share), with the statistics printed."""
import os

import numpy as np
import pytest
import torch

from tests.test_glut_oracle import CASES, glut_case

pytestmark = pytest.mark.gpu

NTHREADS = os.cpu_count() or 1
KEPT_COLS = {0: "depth", 2: "rrs_error", 3: "bottom_albedo", 7: "K_min", 9: "iod"}


def _run(gpu, grids, ths, ns, nbt, rs, em, n_chains):
    cfg = gpu.Config.reference_default()
    emp = None if em is None else torch.tensor(np.ascontiguousarray(em.reshape(-1)),
                                               device="cuda")
    out = gpu.region_lut_invert(torch.tensor(np.ascontiguousarray(grids), device="cuda"), cfg,
                                n_spatial=ns, n_bottoms=nbt, theta_sun=[float(t) for t in ths],
                                n_chains=n_chains, rrs_noise=rs, empirical=emp,
                                empirical_nodata=9999.0)
    gpu.sync()
    return {k: v.cpu().numpy() for k, v in out.items()}


_ORACLE = {}


def _oracle(port, grids, ths, ns, nbt, rs, em, n_chains, key=None):
    if key is not None and (key, n_chains) in _ORACLE:
        return _ORACLE[(key, n_chains)]
    r = port.glut_invert(grids, theta_sun=ths, n_spatial=ns, n_bottoms=nbt, rrs_noise=rs,
                         empirical=em, empirical_nodata=9999.0, n_chains=n_chains,
                         nthreads=NTHREADS)
    if key is not None:
        _ORACLE[(key, n_chains)] = r
    return r


def _check_grids(label, mine, want, same_idx):
    """The other grids on the pixels whose float depths agree: nearly all
    the same fit -- a fit can differ below the float depth's last bit and
    still move its Rrs error or shares in the sixth digit."""
    for name, a, b in zip(label, mine, want):
        a, b = a[same_idx], b[same_idx]
        ident = np.mean(a == b)
        print(f"  {name}: identical on {ident:.4f} of the pixels whose depths agree")
        assert ident >= 0.95, name
        np.testing.assert_allclose(a, b, rtol=1e-3, atol=1e-3, err_msg=name)


def _stats(name, h_gpu, h_ref, src_gpu, src_ref, fit):
    d = np.abs(np.asarray(h_gpu, np.float64)[fit] - np.asarray(h_ref, np.float64)[fit])
    sg, sr = np.mean(src_gpu[fit] >= 0), np.mean(src_ref[fit] >= 0)
    print(f"{name}: {fit.sum()} px, identical depth {np.mean(d == 0):.4f}, median |dH| "
          f"{np.median(d):.3g} m, p90 {np.quantile(d, 0.9):.3g} m; served GPU {sg:.4f} "
          f"oracle {sr:.4f}")
    return d, sg, sr


@pytest.mark.parametrize("case", CASES)
def test_order_matches_oracle(gpu, port, golden_dir, case):
    grids, ths, ns, nbt, rs, em, _, _ = glut_case(golden_dir, case)
    o = _run(gpu, grids, ths, ns, nbt, rs, em, 1)
    ref, src, order, _ = _oracle(port, grids, ths, ns, nbt, rs, em, 1, key=case)
    np.testing.assert_array_equal(o["order"], order)
    np.testing.assert_array_equal(o["source"] == -2, src == -2)
    np.testing.assert_array_equal(o["status"] & 0xFF, ref[:, 9].astype(np.int32))


@pytest.mark.parametrize("case", CASES)
def test_one_chain_against_reference(gpu, port, golden_dir, case):
    """One chain is the reference's samodel() on one thread: its grids."""
    grids, ths, ns, nbt, rs, em, ref_grids, kept = glut_case(golden_dir, case)
    o = _run(gpu, grids, ths, ns, nbt, rs, em, 1)
    _, src_o, _, _ = _oracle(port, grids, ths, ns, nbt, rs, em, 1, key=case)
    fit = (o["status"] & 0xFF) == 0
    d, sg, sr = _stats(f"one chain vs reference ({case})", o["depth"],
                       -ref_grids[list(kept).index(0)].reshape(-1), o["source"], src_o, fit)
    assert np.median(d) <= 0.01
    assert np.mean(d == 0) >= 0.5
    assert abs(sg - sr) <= 0.05
    same = np.where(fit)[0][d == 0]
    ks = [k for k in KEPT_COLS if k != 0]
    _check_grids([KEPT_COLS[k] for k in ks], [o[KEPT_COLS[k]] for k in ks],
                 [ref_grids[list(kept).index(k)].reshape(-1) for k in ks], same)


def test_chains_against_oracle(gpu, port):
    """16 chains over a 28 x 28 scene (3 x 3 regions, three bottom types)
    against the oracle's 16 chains."""
    n, C = 28, 16
    grid = port.generate_field(20261414, n, n)[0].reshape(1, n, n, 4)
    o = _run(gpu, grid, (35.0,), 2, 3, None, None, C)
    ref, src, order, stats = _oracle(port, grid, (35.0,), 2, 3, None, None, C)
    np.testing.assert_array_equal(o["order"], order)
    assert o["chain_stats"].shape == (C, 4)
    fit = ref[:, 9] == 0
    d, sg, sr = _stats("16 chains vs oracle", o["depth_f64"], ref[:, 0], o["source"], src, fit)
    assert np.median(d) <= 0.01
    assert np.mean(d == 0) >= 0.5
    assert abs(sg - sr) <= 0.05
    S = order.size
    lens = np.array([(c + 1) * S // C - c * S // C for c in range(C)])
    np.testing.assert_array_equal(o["chain_stats"][:, 0] + o["chain_stats"][:, 1], lens)


def test_served_pixels_carry_their_source(gpu, port, golden_dir):
    grids, ths, ns, nbt, rs, em, _, _ = glut_case(golden_dir, "r2b3_s2")
    o = _run(gpu, grids, ths, ns, nbt, rs, em, 2)
    s = np.where(o["source"] >= 0)[0]
    assert s.size > 0
    src = o["source"][s]
    for f in ("depth_f64", "bottom_albedo", "rrs_error", "K_min", "iod", "bottom_type"):
        np.testing.assert_array_equal(o[f][s], o[f][src], err_msg=f)
    for f in ("P", "G", "X", "bottom_percent"):
        np.testing.assert_array_equal(o[f][s], o[f][src], err_msg=f)
    assert o["P"].shape[1] == 2
    assert np.all(o["status"][s] & 0x200) and np.all(o["evals"][s] == 0)
    assert np.all((o["status"][s] >> 24) == (o["status"][src] >> 24))  # same region count
    assert np.all(o["source"][src] == -1)


def test_default_chains(gpu, port):
    """n_chains = 0: eight chains per resident warp of the kernel."""
    n = 40
    grid = port.generate_field(9191, n, n)[0].reshape(1, n, n, 4)
    o = _run(gpu, grid, (35.0,), 2, 3, None, None, 0)
    fit = (o["status"] & 0xFF) == 0
    assert fit.mean() > 0.8
    import ctypes
    c = gpu.Config.reference_default().to_c()
    dflt = gpu.api.L.lib().photic_region_lut_default_chains(ctypes.byref(c), 1, 2, 3)
    assert dflt > 0 and o["chain_stats"].shape[0] == min(o["order"].size, dflt)


@pytest.fixture(scope="module")
def driver(tmp_path_factory, gpu):
    from tests.test_dropin_layout import build_driver
    return build_driver(tmp_path_factory.mktemp("dropin_glut"))


@pytest.mark.parametrize("case", ["r2b3", "r2b3_emp", "r2b3_s2"])
def test_samodel_dropin_general_lookup_table(driver, golden_dir, tmp_path, case):
    """The samodel() drop-in called from C in the reference's general
    configurations, one chain (PHOTIC_LUT_CHAINS=1), against the reference's
    own samodel() grids: depth, the model-error grid, albedo, the bottom
    shares and type, K_min and IOD."""
    import subprocess
    grids, ths, ns, nbt, rs, em, ref_grids, kept = glut_case(golden_dir, case)
    S, n = grids.shape[0], grids.shape[1]
    params = np.zeros((S * n * n, 6))
    for s in range(S):
        params[s, 1] = ths[s]
        params[s, 2:6] = 0.0 if rs is None else rs[s]
    if em is not None:
        params[:n * n, 0] = em.reshape(-1)
    inp, out = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(inp, "wb") as f:
        np.array([4, S * n * n, n, n], dtype=np.int32).tofile(f)
        np.array([443.0, 482.0, 561.0, 655.0]).tofile(f)
        np.array([35.0, 0.0]).tofile(f)
        np.ascontiguousarray(grids, dtype=np.float32).tofile(f)
        params.tofile(f)
    mode = f"gridx:{ns}:{nbt}:{S}:{1 if em is not None else 0}"
    r = subprocess.run([driver, mode, inp, out], capture_output=True, text=True, timeout=600,
                       cwd=str(tmp_path), env={**os.environ, "PHOTIC_LUT_CHAINS": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    g = np.fromfile(out, dtype=np.float32).reshape(10, n * n)
    ref = {int(k): ref_grids[i].reshape(-1) for i, k in enumerate(kept)}
    fit = ref[0] != 0
    d = np.abs(g[0, fit] - ref[0][fit])
    same = d == 0
    print(f"samodel() general lookup table ({case}) vs the reference's: {fit.sum()} px, "
          f"identical depth {same.mean():.4f}, median |dH| {np.median(d):.3g} m")
    assert np.median(d) <= 0.01 and same.mean() >= 0.5
    np.testing.assert_array_equal(g[0, ~fit], 0)
    ks = (2, 3, 4, 5, 6, 7, 8, 9)
    _check_grids([str(k) for k in ks], [g[k, fit] for k in ks], [ref[k][fit] for k in ks],
                 np.where(same)[0])
