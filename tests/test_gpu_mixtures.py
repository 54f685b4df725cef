"""The general fit of samodel()'s pixel loop on the GPU: bottom mixtures
(sand, seagrass, coral), pixels alone or with 3 x 3 regions, empirical
depths and scene stacks, against the reference-made golden fixture
(tests/golden/bottoms.npz) and the oracle, itself pinned bit for bit to the
reference (tests/test_oracle_vs_reference.py).  The bar is the
median |dH| <= 1 cm and p99 <= 5 cm, with the bottom shares and types of the
pixels whose fits agree."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NTHREADS = os.cpu_count() or 1


def _fit(gpu, grid, **kw):
    out = gpu.region_fit(torch.tensor(grid, device="cuda"), gpu.Config(kcount=kw.pop("kcount", 2000)),
                         **kw)
    gpu.sync()
    return {k: v.cpu().numpy() for k, v in out.items()}


def _compare(name, out, ref, cols, converged_p99=True, min_same=0.85):
    """Masks, region counts and the depth bar.  The p99 bar is taken over the
    pixels whose fits converged (nelmin ifault 0) on both sides: a fit cut
    off by the evaluation budget stops wherever the budget ran out, and a
    last-ulp difference earlier on its path moves that point."""
    c = {k: cols.index(k) for k in cols}
    st = out["status"]
    np.testing.assert_array_equal(st & 0xFF, ref[:, c[9]].astype(np.int32))
    fit = (st & 0xFF) == 0
    np.testing.assert_array_equal((st[fit] >> 24) & 0xF, ref[fit, c[38]].astype(np.int32))
    d = np.abs(out["depth_f64"][fit] - ref[fit, 0])
    conv = (((st[fit] >> 8) & 1) == 1) & (ref[fit, c[8]] == 1)
    same = d == 0
    agree = np.where(fit)[0][same]
    pct = out["bottom_percent"]
    type_same = np.mean(out["bottom_type"][agree] == ref[agree, c[43]])
    pct_err = np.abs(pct[agree] - ref[agree][:, [c[40], c[41], c[42]]]).max() if agree.size else 0.0
    dc = d[conv] if conv.any() else np.zeros(1)
    print(f"{name}: {d.size} px, same {same.mean():.4f}, median |dH| {np.median(d):.3g} m, "
          f"p99 {np.quantile(d, 0.99):.3g} m; converged on both sides {conv.mean():.3f}: "
          f"p99 {np.quantile(dc, 0.99):.3g} m; bottom type identical {type_same:.4f}, "
          f"max |share diff| {pct_err:.2g} % where the fits agree")
    assert np.median(d) <= 0.01, name
    if converged_p99:
        assert np.quantile(dc, 0.99) <= 0.05, name
    assert same.mean() >= min_same, name
    assert type_same == 1.0 and pct_err <= 1e-3, name
    return fit


def _host_vs_golden(port, name, grid, ref, cols, **kw):
    """The oracle built on this host against the reference's fixture made
    on x86-64: both run the reference's arithmetic in C, so any difference
    is the two hosts' libm, the same last-ulp sensitivity the GPU meets."""
    o = port.region_invert_batch(grid, nthreads=NTHREADS, **kw)
    fit = o[:, 9] == 0
    d = np.abs(o[fit, 0] - ref[fit, 0])
    print(f"  host oracle vs x86 fixture ({name}): same {np.mean(d == 0):.4f}, "
          f"p99 {np.quantile(d, 0.99):.3g} m")


@pytest.mark.parametrize("key", ["ref_s1", "ref_s1_emp", "ref_s2", "ref_s2_emp"])
def test_mixture_golden(gpu, port, golden_dir, key):
    """n_bottoms = 3 (the reference's default) against the reference itself."""
    g = np.load(os.path.join(golden_dir, "bottoms.npz"))
    ns = 1 if key.startswith("ref_s1") else 2
    he = None
    if key.endswith("_emp"):
        he = torch.tensor(g["h_empirical"], device="cuda")
    out = _fit(gpu, g["grid"], n_spatial=ns, n_bottoms=3, h_empirical=he,
               kcount=int(g["kcount"]))
    fit = _compare(f"golden {key}", out, g[key], list(g["cols"]))
    _host_vs_golden(port, key, g["grid"], g[key], list(g["cols"]), n_spatial=ns, n_bottoms=3,
                    kcount=int(g["kcount"]),
                    h_empirical=g["h_empirical"] if key.endswith("_emp") else None)
    assert len(np.unique(out["bottom_type"][fit])) > 1


def test_scene_stack_golden(gpu, port, golden_dir):
    """Two scenes, 3 x 3 regions, three bottom types (n = 9 + 54 + 6)
    against the reference's own fit."""
    g = np.load(os.path.join(golden_dir, "bottoms.npz"))
    out = _fit(gpu, g["stack"], n_spatial=2, n_bottoms=3, theta_sun=list(g["stack_theta_sun"]),
               kcount=int(g["kcount"]))
    cols = list(g["cols"]) + [12, 20, 28]
    ref = g["ref_stack"]
    fit = _compare("golden two-scene stack", out, ref, cols, min_same=0.8)
    _host_vs_golden(port, "two-scene stack", g["stack"], ref, cols,
                    theta_sun=g["stack_theta_sun"], kcount=int(g["kcount"]), n_spatial=2,
                    n_bottoms=3)
    agree = fit & (out["depth_f64"] == ref[:, 0])
    for s, (c, name) in enumerate(((11, "P"), (12, "P"))):
        np.testing.assert_allclose(out["P"][agree, s], ref[agree, cols.index(c)].astype(np.float32),
                                   rtol=2e-6)


@pytest.mark.parametrize("n_spatial,n_bottoms,side", [(1, 3, 48), (1, 2, 32), (2, 3, 14)])
def test_mixture_distribution(gpu, port, n_spatial, n_bottoms, side):
    """Larger grids against the oracle at the plain-method tolerances."""
    rrs, truth = port.generate_single(20261212 + n_bottoms, side * side, pix0=9,
                                      mask_frac=0.15)
    grid = rrs.reshape(side, side, 4)
    he = truth[:, 0] * np.random.default_rng(7).uniform(0.7, 1.3, truth.shape[0])
    he[::2] = np.nan
    for h in (None, he):
        out = _fit(gpu, grid, n_spatial=n_spatial, n_bottoms=n_bottoms,
                   h_empirical=None if h is None else torch.tensor(h, device="cuda"))
        ref = port.region_invert_batch(grid, n_spatial=n_spatial, n_bottoms=n_bottoms,
                                       h_empirical=h, nthreads=NTHREADS)
        _compare(f"mixtures n_spatial {n_spatial} n_bottoms {n_bottoms} "
                 f"{'empirical' if h is not None else 'cold'}", out, ref, list(range(port.NOUT)))


def test_one_bottom_alone_matches_plain_kernel(gpu, port):
    """n_spatial = 1, n_bottoms = 1 is the plain method: the warp-per-pixel
    general kernel and the thread-per-pixel inversion give the same fits bit
    for bit."""
    rrs, _ = port.generate_single(5150, 1500, pix0=77)
    a = _fit(gpu, rrs.reshape(30, 50, 4), n_spatial=1, n_bottoms=1)
    b = gpu.invert(torch.tensor(rrs, device="cuda"))
    gpu.sync()
    b = {k: v.cpu().numpy() for k, v in b.items()}
    np.testing.assert_array_equal(a["status"] & 0xFFFF, b["status"] & 0xFFFF)
    for f in ("depth_f64", "P", "G", "X", "bottom_albedo", "model_error", "evals"):
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)
    fit = (a["status"] & 0xFF) == 0
    assert np.all(a["bottom_type"][fit] == 1) and np.all(a["bottom_percent"][fit, 0] == 100)


def test_scene_stack_matches_joint_kernel(gpu, port):
    """A stack of k scenes fitted alone with one bottom type is the temporal
    joint fit: the general kernel and the lane-group joint kernel agree."""
    k, side = 3, 12
    grids, ths = [], [27.0, 36.0, 45.0]
    for s in range(k):
        r, _ = port.generate_single(6100 + s, side * side, pix0=5, mask_frac=0.0,
                                    theta_sun=ths[s])
        grids.append(r.reshape(side, side, 4))
    grid = np.stack(grids)
    a = _fit(gpu, grid, n_spatial=1, n_bottoms=1, theta_sun=ths)
    offs = np.arange(0, k * side * side + 1, k, dtype=np.int32)
    rr = np.stack([g.reshape(-1, 4) for g in grids], 1).reshape(-1, 4)
    th = np.tile(np.array(ths), side * side)
    t = lambda x: torch.tensor(x, device="cuda")
    b = gpu.joint_invert(t(offs), t(th), t(rr), gpu.Config())
    gpu.sync()
    fit = (a["status"] & 0xFF) == 0
    same = np.mean(a["depth_f64"][fit] == b["depth_f64"].cpu().numpy()[fit])
    print(f"stack vs joint kernel: identical depths {same:.4f}")
    assert same >= 0.97
