"""The C restatement against the reference compiled from its own sources,
on fresh inputs (skipped where the reference sources are not present)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.skipif(not O.reference_available(),
                                reason="oracle/_ref not built (reference sources absent)")


@pytest.mark.parametrize("seed", [1, 2])
def test_invert_bit_exact(seed):
    rrs, _ = O.generate_single(seed, 600)
    a = O.invert_batch(rrs)
    b = O.invert_batch(rrs, which="reference")
    cols = list(range(0, 11)) + [11, 19, 27]
    assert np.array_equal(a[:, cols], b[:, cols])


def test_invert_edge_spectra_bit_exact():
    rng = np.random.default_rng(3)
    rrs = rng.uniform(1e-5, 0.05, size=(300, 4)).astype(np.float32)  # arbitrary, not physical
    rrs[::10, 1] = 0.0
    rrs[5::10, 0] = 1e-6
    a = O.invert_batch(rrs)
    b = O.invert_batch(rrs, which="reference")
    cols = list(range(0, 11)) + [11, 19, 27]
    assert np.array_equal(a[:, cols], b[:, cols], equal_nan=True)


def test_joint_bit_exact():
    offs, th, rrs, _ = O.generate_joint(11, 80)
    a = O.joint_invert_batch(offs, th, rrs)
    b = O.joint_invert_batch(offs, th, rrs, which="reference")
    assert np.array_equal(a[:, :35], b[:, :35])


def test_interp_1d_bit_exact():
    X = np.array([443.0, 482.0, 561.0, 655.0])
    Y = np.array([0.011, 0.013, 0.009, 0.001])
    for x in [400.0, 440.0, 443.0, 443.001, 482.0, 490.0, 550.0, 640.0, 655.0, 700.0, 750.0]:
        assert O.interp_1d(X, Y, x) == O.interp_1d(X, Y, x, which="reference")


def test_regions_bit_exact():
    """The spatial-region restatement against the compiled reference."""
    if not O.reference_available():
        pytest.skip("reference library not built")
    rrs, _ = O.generate_single(31, 9 * 31, pix0=100, mask_frac=0.2)
    grid = rrs.reshape(9, 31, 4)
    cols = [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 19, 27, 38, 39]
    a = O.region_invert_batch(grid, reqmin=1e-2, konvge=100, kcount=5000, nthreads=8)
    b = O.region_invert_batch(grid, reqmin=1e-2, konvge=100, kcount=5000, nthreads=8,
                              which="reference")
    np.testing.assert_array_equal(a[:, cols], b[:, cols])


@pytest.mark.parametrize("n_spatial,n_bottoms", [(1, 2), (1, 3), (2, 2), (2, 3)])
def test_bottom_mixtures_bit_exact(n_spatial, n_bottoms):
    """Sand/seagrass/coral mixtures per region (the reference's default
    n_bottoms = 3), alone and with 3 x 3 regions, with and without empirical
    depths (pixels deeper than 8 m are fitted with sand alone)."""
    rrs, truth = O.generate_single(41 + n_bottoms, 8 * 13, pix0=500, mask_frac=0.15)
    grid = rrs.reshape(8, 13, 4)
    he = truth[:, 0] * np.random.default_rng(n_bottoms).uniform(0.7, 1.3, truth.shape[0])
    he[::3] = np.nan
    cols = [c for c in range(O.NOUT) if c not in (36, 37)]  # kept start / ifault: port only
    for h in (None, he):
        a = O.region_invert_batch(grid, kcount=600, n_spatial=n_spatial, n_bottoms=n_bottoms,
                                  h_empirical=h, nthreads=8)
        b = O.region_invert_batch(grid, kcount=600, n_spatial=n_spatial, n_bottoms=n_bottoms,
                                  h_empirical=h, nthreads=8, which="reference")
        np.testing.assert_array_equal(a[:, cols], b[:, cols])
        fit = a[:, 9] == 0
        assert len(np.unique(a[fit, 43])) > 1  # several bottom types win


@pytest.mark.parametrize("n_scenes,n_spatial,n_bottoms", [(2, 1, 1), (2, 1, 3), (2, 2, 3),
                                                          (3, 2, 1)])
def test_scene_stacks_bit_exact(n_scenes, n_spatial, n_bottoms):
    """Several scenes of one place (their own sun zeniths and masks), fitted
    jointly with regions and bottom mixtures: n = R + 2 Nb R + 3 Ns."""
    grids = []
    for s in range(n_scenes):
        r, _ = O.generate_single(900 + s, 6 * 8, pix0=300, mask_frac=0.1, theta_sun=28.0 + 6 * s)
        grids.append(r.reshape(6, 8, 4))
    grid = np.stack(grids)
    th = [28.0 + 6 * s for s in range(n_scenes)]
    cols = [c for c in range(O.NOUT) if c not in (36, 37)]
    a = O.region_invert_batch(grid, theta_sun=th, kcount=500, n_spatial=n_spatial,
                              n_bottoms=n_bottoms, nthreads=8)
    b = O.region_invert_batch(grid, theta_sun=th, kcount=500, n_spatial=n_spatial,
                              n_bottoms=n_bottoms, nthreads=8, which="reference")
    np.testing.assert_array_equal(a[:, cols], b[:, cols])
    assert np.all(a[a[:, 9] == 0, 10] == n_scenes)


def test_depth_sigma_statistics_bit_exact():
    """The depth uncertainty's per-interval statistic (model/samodel.c:
    1459-1460) -- the reference's vec_mean2_double / vec_stddev_double with
    samples at 0 (no pixel found) and within 1e-4 of 0 left out -- against the
    oracle's restatement, which the GPU's table reproduces given the same
    refitted depths (tests/test_gpu_depth_sigma.py)."""
    import ctypes as C
    ref = O.reference().lib.photic_ref_depth_sigma_stat
    ref.restype = C.c_double
    ref.argtypes = [C.POINTER(C.c_double), C.c_int]
    rng = np.random.default_rng(17)
    n_samples, n_int = 32, 40
    samples = rng.uniform(0.1, 30.0, size=(n_int, n_samples))
    samples[rng.uniform(size=samples.shape) < 0.3] = 0.0      # intervals with misses
    samples[3] = 0.0                                           # an empty interval
    samples[4, :5] = 5e-5                                      # inside the 1e-4 tolerance
    samples[5, 1:] = 0.0                                       # a single refit
    samples[6] = np.float32(7.3)                               # all equal
    depth = np.full(16, 0.0, dtype=np.float32)
    depth[0] = n_int / 4.0 + 0.1                               # intervals up to n_int / 4 m
    rrs = np.full((16, 4), 0.01, dtype=np.float32)
    _, table, _, _ = O.depth_sigma(rrs, depth, [2e-4] * 4, n_samples=n_samples, seed=3,
                                   sample_depth=np.pad(samples, ((0, 120 - n_int), (0, 0))).ravel())
    for k in range(n_int):
        v = np.ascontiguousarray(samples[k])
        want = ref(v.ctypes.data_as(C.POINTER(C.c_double)), n_samples)
        assert table[k] == want, (k, table[k], want)
