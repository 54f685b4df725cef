"""The oracle's restatement of samodel()'s pixel loop with its dynamic
lookup table in the general configurations -- 3 x 3 regions, mixtures of
bottom types, the spectral-angle order, empirical depths, stacks of scenes
(model/samodel.c:649-1352, 1768-2115, 2792-2842, 3031-3139) -- against the
reference itself.

The pin: the reference's own samodel() with LUT 1 on one OpenMP thread
(deterministic) over spatially coherent scenes, tests/golden/glut.npz made
by tests/golden/make_golden.py; one chain of the oracle is that run, and
every kept grid must agree bit for bit.  Then the chains: n chains are the
loop run alone on each contiguous slice of the sorted pixels."""
import os

import numpy as np
import pytest

# kept grid -> oracle record column: depth, model error (the Rrs error),
# albedo, sand, seagrass, coral, K_min, bottom type, IOD
GRID_COLS = {0: 0, 2: 3, 3: 1, 4: 40, 5: 41, 6: 42, 7: 4, 8: 43, 9: 5}
CASES = ["r2b3", "r1b3", "r2b2_noise", "r2b3_emp", "r2b3_s2"]


def glut_case(golden_dir, case):
    """(grids [S, n, n, 4], sun zeniths, n_spatial, n_bottoms, noise or None,
    empirical or None (nodata 9999), the reference's grids, kept grid
    indices)."""
    g = np.load(os.path.join(golden_dir, "glut.npz"))
    ns, nbt = (int(v) for v in g[f"{case}_config"])
    rs = g[f"{case}_r_sigma"] if f"{case}_r_sigma" in g else None
    em = g[f"{case}_empirical"] if f"{case}_empirical" in g else None
    return (g[f"{case}_grid"], g[f"{case}_theta_sun"], ns, nbt, rs, em, g[f"{case}_ref"],
            g["grids"])


def compare_grids(out, ref_grids, kept, label):
    fit = out[:, 9] == 0
    for k, want in zip(kept, ref_grids):
        col = GRID_COLS[int(k)]
        mine = out[:, col].astype(np.float32)
        want = want.reshape(-1)
        if k == 0:
            want = -want
        same = mine[fit] == want[fit]
        assert same.all(), (label, int(k), int((~same).sum()))


def _run(port, case, golden_dir, **kw):
    grids, ths, ns, nbt, rs, em, ref, kept = glut_case(golden_dir, case)
    return port.glut_invert(grids, theta_sun=ths, n_spatial=ns, n_bottoms=nbt, rrs_noise=rs,
                            empirical=em, empirical_nodata=9999.0, **kw), ref, kept


@pytest.mark.parametrize("case", CASES)
def test_oracle_glut_matches_reference_fixture(port, golden_dir, case):
    (out, src, order, stats), ref, kept = _run(port, case, golden_dir, n_chains=1, nthreads=1)
    compare_grids(out, ref, kept, case)
    fit = out[:, 9] == 0
    served = np.mean(src[fit] >= 0)
    print(f"{case}: {fit.sum()} shallow pixels, served {served:.3f}, final thresholds "
          f"{stats[0, 2]:.3f}/{stats[0, 3]:.3f}")
    s = np.where(src >= 0)[0]
    np.testing.assert_array_equal(out[s, 0], out[src[s], 0])
    # a served pixel takes a fit with its own region count
    np.testing.assert_array_equal(out[s, 38], out[src[s], 38])


def test_oracle_glut_matches_reference_live(port):
    if not port.reference_available():
        pytest.skip("reference sources not available on this host")
    n = 14
    grids = np.stack([port.generate_field(4141, n, n, theta_sun=t)[0].reshape(n, n, 4)
                      for t in (30.0, 45.0)])
    ref = port.reference_samodel_stack(grids, theta_sun=(30.0, 45.0), n_spatial=2, n_bottoms=2)
    out, src, order, stats = port.glut_invert(grids, theta_sun=(30.0, 45.0), n_spatial=2,
                                              n_bottoms=2, n_chains=1, nthreads=1)
    keep = [0, 2, 3, 4, 5, 6, 7, 8, 9]
    compare_grids(out, ref[keep], keep, "live")


def test_glut_key_sums_scenes(port):
    """The order key of a stack: blue, green and red summed over the scenes
    (each value not nodata) before the norm."""
    n = 8
    a = port.generate_field(5, n, n)[0]
    b = port.generate_field(5, n, n, theta_sun=50.0)[0]
    b[3, 1] = -9999.0  # a nodata blue in the second scene is left out of the sum
    grids = np.stack([a.reshape(n, n, 4), b.reshape(n, n, 4)])
    out, src, order, _ = port.glut_invert(grids, theta_sun=(35.0, 50.0), n_chains=1,
                                          nthreads=1, n_spatial=1, n_bottoms=1)
    s = a.astype(np.float32) + np.where(b == -9999.0, np.float32(0), b).astype(np.float32)
    key = np.sqrt(np.sum(s[:, 1:4].astype(np.float64) ** 2, axis=1)).astype(np.float32)
    shallow = np.array([p for p in range(n * n)
                        if not ((a[p] < 0).any() or (b[p] < 0).any())])
    want = shallow[np.argsort(key[shallow], kind="stable")]
    np.testing.assert_array_equal(order, want)


def test_glut_chains_are_independent_slices(port, golden_dir):
    (out, src, order, stats), _, _ = _run(port, "r2b3", golden_dir, n_chains=3, nthreads=3)
    grids, ths, ns, nbt, rs, em, _, _ = glut_case(golden_dir, "r2b3")
    S = order.size
    for c in range(3):
        sl = order[c * S // 3:(c + 1) * S // 3]
        assert np.all(src[sl][src[sl] >= 0] >= 0)
        assert set(src[sl][src[sl] >= 0]).issubset(set(sl))  # served from its own chain
        np.testing.assert_array_equal(stats[c, 0] + stats[c, 1], sl.size)


def test_oracle_glut_eight_bands_matches_reference_live(port):
    """Eight OLCI-like bands (the order and the spectral difference use
    bands 1..3 of them), 3 x 3 regions, two bottom types, against the
    reference's own samodel().  The wavelengths are whole nanometres: a
    scene record holds them as int (model/common.h:200)."""
    if not port.reference_available():
        pytest.skip("reference sources not available on this host")
    wl8 = (412.0, 442.0, 490.0, 510.0, 560.0, 620.0, 665.0, 709.0)
    n = 10
    grid = port.generate_field(8181, n, n, wl=wl8)[0].reshape(1, n, n, 8)
    ref = port.reference_samodel_stack(grid, wl=wl8, n_spatial=2, n_bottoms=2)
    out, src, order, stats = port.glut_invert(grid, wl=wl8, n_spatial=2, n_bottoms=2,
                                              n_chains=1, nthreads=1)
    keep = [0, 2, 3, 4, 5, 6, 7, 8, 9]
    compare_grids(out, ref[keep], keep, "eight bands")
    assert (out[:, 9] == 0).sum() > 50


def test_oracle_glut_edges_match_reference_live(port):
    """Edges of the general loop against the reference: a 3 x 3 grid, whose
    clamped neighbourhoods repeat pixels (the corner's 3 x 3 region list
    holds its own spectrum four times, extract_Rrs_data's clamping,
    model/samodel.c:2974-2992), with a nodata pixel in the middle that every
    neighbourhood leaves out."""
    if not port.reference_available():
        pytest.skip("reference sources not available on this host")
    n = 3
    grid = port.generate_field(3131, n, n, mask_frac=0.0)[0].reshape(1, n, n, 4)
    grid[0, 1, 1, 2] = -9999.0
    ref = port.reference_samodel_stack(grid, n_spatial=2, n_bottoms=3)
    out, src, order, stats = port.glut_invert(grid, n_spatial=2, n_bottoms=3, n_chains=1,
                                              nthreads=1)
    keep = [0, 2, 3, 4, 5, 6, 7, 8, 9]
    compare_grids(out, ref[keep], keep, "3x3")
    assert order.size == 8 and src[4] == -2
    assert out[0, 38] == 8  # the corner: 9 clamped slots less the nodata centre


def test_oracle_glut_all_masked(port):
    n = 4
    grid = np.full((1, n, n, 4), -9999.0, np.float32)
    out, src, order, stats = port.glut_invert(grid, n_chains=3, nthreads=1)
    assert order.size == 0 and np.all(src == -2) and np.all(out[:, 9] == 1)
