"""netCDF short-packed grids on the GPU: photic_nc_pack and
photic_nc_unpack_bands against the oracle's compress_2d / decompress_2d
(pinned bit for bit to the reference's model/nc.c by tests/test_ncgrid.py),
bit for bit, on the quirk grids and on a grid of many tiles; the file paths
read_bands / write_grid; and the reference's own entry points read_nc /
write_nc called through the C ABI with the reference's float** grids."""
import ctypes as C

import numpy as np
import pytest

from tests.test_ncgrid import SPVAL, quirk_grids

pytestmark = pytest.mark.gpu


def _be_to_i16(t):
    return np.frombuffer(t.cpu().numpy().tobytes(), dtype=">i2").astype(np.int16)


def _big_grid(seed=21):
    rng = np.random.default_rng(seed)
    nr, nc = 2049, 2100  # 1051 tiles of 4096 cells (two scan chunks), ragged last tile
    g = (40.0 * np.exp(-np.linspace(0.0, 3.0, nr * nc)) + rng.normal(0, 0.8, nr * nc))
    g = g.astype(np.float32).reshape(nr, nc)
    g[rng.random(g.shape) < 0.05] = SPVAL
    g[0, 0] = SPVAL
    g[0, 1] = 55.0  # first compared cell is the maximum
    return g


@pytest.mark.parametrize("name,grid", quirk_grids() + [("big", _big_grid())],
                         ids=[n for n, _ in quirk_grids()] + ["big"])
def test_pack_matches_oracle(gpu, port, name, grid):
    import torch
    from photic_gb300 import ncgrid as N
    want, off, sc, mv = port.nc_compress(grid, SPVAL)
    packed, info = N.pack(torch.from_numpy(grid).cuda(), SPVAL)
    gpu.sync()
    np.testing.assert_array_equal(_be_to_i16(packed).reshape(grid.shape), want)
    assert np.float32(info["add_offset"]).tobytes() == np.float32(off).tobytes()
    assert np.float32(info["scale_factor"]).tobytes() == np.float32(sc).tobytes()
    assert info["missing_value"] == mv == -32768 and info["spval"] == SPVAL


@pytest.mark.parametrize("nb", [1, 3, 4, 8])
def test_unpack_bands_matches_oracle(gpu, port, nb):
    import torch
    from photic_gb300 import ncgrid as N
    rng = np.random.default_rng(nb)
    npix = 300_001
    packed, infos, want = [], [], []
    for b in range(nb):
        p = rng.integers(-32768, 32768, npix).astype(np.int16)
        p[rng.random(npix) < 0.05] = -32768
        off, sc = float(rng.uniform(-1, 1)), float(rng.uniform(1e-5, 1e-3))
        mv = -32768 if b % 2 == 0 else int(p[7])
        want.append(port.nc_decompress(p, off, sc, mv, SPVAL)[0])
        packed.append(torch.from_numpy(np.frombuffer(p.astype(">i2").tobytes(),
                                                     dtype=np.uint8).copy()).cuda())
        infos.append({"ncols": npix, "nrows": 1, "add_offset": off, "scale_factor": sc,
                      "missing_value": mv, "spval": SPVAL})
    out = N.unpack_bands(packed, infos, npix)
    gpu.sync()
    got = out.cpu().numpy()
    for b in range(nb):
        assert got[:, b].tobytes() == want[b].tobytes(), b


def test_scene_files_to_device_and_back(gpu, port, tmp_path):
    import torch
    from photic_gb300 import ncgrid as N
    rng = np.random.default_rng(7)
    nr, nc = 97, 131
    lons = np.linspace(150.0, 150.5, nc).astype(np.float32)
    lats = np.linspace(-23.5, -23.2, nr).astype(np.float32)
    paths, want = [], []
    for b in range(4):
        g = rng.uniform(0.001, 0.03, (nr, nc)).astype(np.float32)
        g[rng.random(g.shape) < 0.03] = SPVAL
        p, off, sc, mv = port.nc_compress(g, SPVAL)
        path = str(tmp_path / f"band{b}.nc")
        N.write_raw(path, p, lons, lats, off, sc, mv, SPVAL)
        paths.append(path)
        want.append(port.nc_decompress(p, off, sc, mv, SPVAL)[0].reshape(-1))
    rrs, info, lo, la = N.read_bands(paths)
    gpu.sync()
    assert (info["ncols"], info["nrows"]) == (nc, nr) and info["spval"] == SPVAL
    np.testing.assert_array_equal(lo, lons)
    np.testing.assert_array_equal(la, lats)
    got = rrs.cpu().numpy()
    for b in range(4):
        assert got[:, b].tobytes() == want[b].tobytes(), b
    # the inversion takes the tensor as it is; masked cells keep nodata
    out = gpu.invert(rrs[:4096], gpu.Config(nodata_value=SPVAL))
    gpu.sync()
    st = out["status"].cpu().numpy() & 0xFF
    assert ((st == 1) == (got[:4096] == np.float32(SPVAL)).any(axis=1)).all()
    # a result grid back to a file
    depth = torch.from_numpy(rng.uniform(0.5, 25.0, (nr, nc)).astype(np.float32)).cuda()
    depth[3, :5] = SPVAL
    N.write_grid(str(tmp_path / "depth.nc"), depth, lons, lats, SPVAL)
    p, lo2, la2, inf2 = N.read_raw(str(tmp_path / "depth.nc"))
    wp, off, sc, mv = port.nc_compress(depth.cpu().numpy(), SPVAL)
    np.testing.assert_array_equal(p, wp)
    assert np.float32(inf2["add_offset"]) == np.float32(off)
    assert np.float32(inf2["scale_factor"]) == np.float32(sc)
    np.testing.assert_array_equal(lo2, lons)


def test_reference_entry_points(gpu, port, tmp_path):
    from photic_gb300 import _lib as L
    from photic_gb300 import ncgrid as N
    lib = L.lib()
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    grid = quirk_grids()[1][1]  # first cell is the maximum
    nr, nc = grid.shape
    lons = np.linspace(0.0, 1.0, nc).astype(np.float32)
    lats = np.linspace(0.0, 1.0, nr).astype(np.float32)
    keep = [np.ascontiguousarray(grid[i]) for i in range(nr)]
    rows = (C.POINTER(C.c_float) * nr)(*[k.ctypes.data_as(C.POINTER(C.c_float)) for k in keep])
    path = str(tmp_path / "ref_api.nc").encode()
    lib.write_nc(path, rows, nc, nr, lons.ctypes.data_as(C.POINTER(C.c_float)),
                 lats.ctypes.data_as(C.POINTER(C.c_float)), SPVAL)
    p, lo, la, info = N.read_raw(path.decode())
    want, off, sc, mv = port.nc_compress(grid, SPVAL)
    np.testing.assert_array_equal(p, want)
    g = C.POINTER(C.POINTER(C.c_float))()
    ncols, nrows = C.c_int(), C.c_int()
    plons, plats = C.POINTER(C.c_float)(), C.POINTER(C.c_float)()
    spval = C.c_double()
    lib.read_nc(path, C.byref(g), C.byref(ncols), C.byref(nrows), C.byref(plons),
                C.byref(plats), C.byref(spval))
    assert (ncols.value, nrows.value) == (nc, nr) and spval.value == SPVAL
    back = np.array([[g[i][j] for j in range(nc)] for i in range(nr)], dtype=np.float32)
    wback, _ = port.nc_decompress(want, off, sc, mv, SPVAL)
    assert back.tobytes() == wback.tobytes()
    assert np.array([plons[j] for j in range(nc)], np.float32).tobytes() == lons.tobytes()
    for i in range(nr):
        libc.free(C.cast(g[i], C.c_void_p))
    libc.free(C.cast(g, C.c_void_p))
    libc.free(C.cast(plons, C.c_void_p))
    libc.free(C.cast(plats, C.c_void_p))


def test_scene_command_feeds_the_inversion(gpu, port, tmp_path):
    """A scene given the reference's way -- a SCENE line naming its band grids
    (model/bam.c:1300-1543) and the grids as netCDF files -- read into the
    device layout and inverted: the same fits as the unpacked bands inverted
    directly, and the configuration the line gives (sun 31.5 deg)."""
    import torch
    from photic_gb300 import ncgrid as N
    from photic_gb300 import scene as S
    nr, nc = 24, 32
    rrs, _ = port.generate_single(4711, nr * nc, mask_frac=0.1, theta_sun=31.5)
    lons = np.linspace(150.0, 150.3, nc).astype(np.float32)
    lats = np.linspace(-24.0, -23.8, nr).astype(np.float32)
    names = ["coastal", "blue", "green", "red"]
    for b, n in enumerate(names):
        band = np.ascontiguousarray(rrs[:, b].reshape(nr, nc))
        N.write_grid(str(tmp_path / f"{n}.nc"), torch.from_numpy(band).cuda(), lons, lats,
                     -9999.0)
    line = ("SCENE NAME oli BANDS coastal blue green red WAVELENGTHS 443 482 561 655 "
            "THETAVIEW 0 THETASUN 31.5 HTIDE 0.25")
    cfg, dev_rrs, info, _, _, rec = S.load(line, lambda n: str(tmp_path / f"{n}.nc"))
    assert rec["bands"] == names and cfg.theta_sun_deg == 31.5 and cfg.h_tide == 0.25
    assert info["nrows"] == nr and info["ncols"] == nc
    out = gpu.invert(dev_rrs, cfg)
    ref = gpu.invert(dev_rrs.clone(), gpu.Config(theta_sun_deg=31.5, h_tide=0.25))
    gpu.sync()
    for f in ("depth_f64", "status", "P"):
        assert torch.equal(out[f], ref[f]), f
    st = out["status"].cpu().numpy() & 0xFF
    assert (st == 0).sum() > 0.8 * nr * nc
