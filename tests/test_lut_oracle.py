"""The oracle's restatement of samodel()'s pixel loop with its dynamic
lookup table (model/samodel.c:649-1215) against the reference itself.

The pin: the reference's own samodel() with LUT 1, run on one OpenMP thread
(deterministic), on spatially coherent scenes -- tests/golden/lut.npz, made
by tests/golden/make_golden.py -- and, where the reference sources are
present, live on another scene.  One chain of the oracle is the reference
on one thread; every grid must agree bit for bit.  Then the property the GPU
path builds on: n chains are n independent runs of the same loop on
contiguous slices of the sorted pixels."""
import os

import numpy as np
import pytest

# grids of samodel() kept in the fixture and the oracle record column of each
GRID_COLS = {0: 0, 2: 3, 3: 1, 7: 4, 9: 5}  # depth, model error (Rrs), albedo, K_min, IOD


def _compare_grids(out, ref_grids, kept, label):
    fit = out[:, 9] == 0
    for k, g in zip(kept, ref_grids):
        col = GRID_COLS[int(k)]
        mine = out[:, col].astype(np.float32)
        want = g.reshape(-1)
        if k == 0:
            want = -want
        same = mine[fit] == want[fit]
        assert same.all(), (label, int(k), int((~same).sum()))


def fixture_case(golden_dir, case):
    """(spectra [npix, 4], noise spectrum or None, empirical depths or None,
    the reference's grids, kept grid indices) of one case of lut.npz."""
    g = np.load(os.path.join(golden_dir, "lut.npz"))
    grid = g[f"{case}_grid"]
    n = grid.shape[0]
    rs = g[f"{case}_r_sigma"] if f"{case}_r_sigma" in g else None
    em = g[f"{case}_empirical"].reshape(-1) if f"{case}_empirical" in g else None
    return grid.reshape(n * n, 4), rs, em, g[f"{case}_ref"], g["grids"]


@pytest.mark.parametrize("case", ["plain", "noise", "emp"])
def test_oracle_lut_matches_reference_fixture(port, golden_dir, case):
    rrs, rs, em, ref_grids, kept = fixture_case(golden_dir, case)
    out, src, order, stats = port.lut_invert(rrs, rrs_noise=rs, empirical=em, n_chains=1,
                                             nthreads=1)
    _compare_grids(out, ref_grids, kept, case)
    fit = out[:, 9] == 0
    served = np.mean(src[fit] >= 0)
    print(f"{case}: {fit.sum()} shallow pixels, served from the table {served:.4f}, "
          f"final thresholds {stats[0, 2]:.3f}/{stats[0, 3]:.3f}")
    assert served > 0.01
    # served pixels carry their source's fit
    s = np.where(src >= 0)[0]
    np.testing.assert_array_equal(out[s, 0], out[src[s], 0])
    assert np.all(src[src >= 0] != s) if s.size else True


def test_oracle_lut_matches_reference_live(port):
    if not port.reference_available():
        pytest.skip("reference sources not available on this host")
    n = 40
    rrs, _ = port.generate_field(777, n, n)
    ref = port.reference_samodel_grid(rrs.reshape(n, n, 4))
    out, src, order, stats = port.lut_invert(rrs, n_chains=1, nthreads=1)
    _compare_grids(out, ref[[0, 2, 3, 7, 9]], [0, 2, 3, 7, 9], "live")


def test_oracle_order_is_the_stable_key_order(port):
    rrs, _ = port.generate_field(31, 32, 32)
    rrs[5] = rrs[9]  # a tie: equal spectra keep pixel order
    out, src, order, _ = port.lut_invert(rrs, n_chains=1, nthreads=1)
    keys = port.lut_key(rrs)
    shallow = np.where(out[:, 9] == 0)[0]
    want = shallow[np.argsort(keys[shallow], kind="stable")]
    np.testing.assert_array_equal(order, want)
    assert list(order).index(5) < list(order).index(9)
    assert np.all(src[out[:, 9] == 1] == -2)


def test_chains_are_independent_slices(port):
    """n chains = the loop run alone on each contiguous slice of the order."""
    n, C = 48, 5
    rrs, _ = port.generate_field(4242, n, n)
    out, src, order, stats = port.lut_invert(rrs, n_chains=C, nthreads=4)
    S = order.size
    for c in range(C):
        sl = order[c * S // C:(c + 1) * S // C]
        o1, s1, ord1, st1 = port.lut_invert(rrs[sl], n_chains=1, nthreads=1)
        np.testing.assert_array_equal(ord1, np.arange(sl.size))  # the slice keeps its order
        np.testing.assert_array_equal(out[sl], o1)
        mapped = np.where(s1 >= 0, sl[np.maximum(s1, 0)], s1)
        np.testing.assert_array_equal(src[sl], mapped)
        np.testing.assert_array_equal(stats[c], st1[0])


def test_oracle_lut_eight_bands_matches_reference_live(port):
    """Eight OLCI-like bands, whole nanometres (a scene record holds them as
    int, model/common.h:200): the order and the spectral difference use
    bands 1..3 of them."""
    if not port.reference_available():
        pytest.skip("reference sources not available on this host")
    wl8 = (412.0, 442.0, 490.0, 510.0, 560.0, 620.0, 665.0, 709.0)
    n = 32
    rrs, _ = port.generate_field(8282, n, n, wl=wl8)
    ref = port.reference_samodel_grid(rrs.reshape(n, n, 8), wl=wl8)
    out, src, order, stats = port.lut_invert(rrs, wl=wl8, n_chains=1, nthreads=1)
    _compare_grids(out, ref[[0, 2, 3, 7, 9]], [0, 2, 3, 7, 9], "eight bands")
    assert np.mean(src[out[:, 9] == 0] >= 0) > 0.01
