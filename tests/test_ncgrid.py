"""netCDF short-packed grids (model/nc.c), without a GPU.

* The oracle's restatement of compress_2d / decompress_2d is pinned bit for
  bit to the reference's own write_nc / read_nc (model/nc.c), compiled from
  its sources with an in-memory stand-in for libnetcdf (oracle/ref_ncstub.c),
  on grids that reach every branch: spval cells, NaN, infinities, a first
  cell that is the maximum (the one-pass min/max never compares it with the
  maximum, so its quotient overflows short), all-negative, constant and
  all-missing grids, and files without the optional attributes.
* The container the library writes has the dimensions, variables and
  attributes the reference's write_nc defines, read back by scipy's
  independent netCDF reader; files scipy writes (CDF-1 and CDF-2) read back
  through the library.
* Malformed or foreign files fail with PHOTIC_ERR_IO and a message.
"""
import os

import numpy as np
import pytest

netcdf = pytest.importorskip("scipy.io").netcdf_file

SPVAL = -9999.0


def quirk_grids(seed=11):
    rng = np.random.default_rng(seed)
    out = []
    g = rng.uniform(-3.0, 45.0, (37, 53)).astype(np.float32)
    g[rng.random(g.shape) < 0.1] = SPVAL
    out.append(("random", g))
    h = g.copy()
    h[0, 0] = 80.0                      # the first cell is the maximum
    out.append(("first_is_max", h))
    out.append(("negative", -rng.uniform(0.5, 9.0, (9, 11)).astype(np.float32)))
    out.append(("constant", np.full((4, 6), 7.25, np.float32)))
    one = np.full((5, 5), SPVAL, np.float32)
    one[2, 3] = 12.5
    out.append(("single", one))
    out.append(("all_missing", np.full((3, 4), SPVAL, np.float32)))
    n = rng.uniform(0.0, 20.0, (8, 8)).astype(np.float32)
    n[1, 1] = np.nan
    n[5, 2] = np.nan
    out.append(("nan", n))
    i = rng.uniform(0.0, 20.0, (6, 7)).astype(np.float32)
    i[3, 3] = np.inf
    out.append(("inf", i))
    j = rng.uniform(0.0, 20.0, (6, 7)).astype(np.float32)
    j[2, 5] = -np.inf
    out.append(("minus_inf", j))
    d = (np.linspace(60.0, 0.0, 4096 * 3 + 77) + rng.normal(0, 0.5, 4096 * 3 + 77))
    out.append(("descending", d.astype(np.float32).reshape(1, -1)))
    return out


@pytest.fixture(scope="module")
def ref(port):
    from oracle import oracle as O
    if not O.reference_available():
        pytest.skip("reference sources not built here")
    return O


@pytest.mark.parametrize("name,grid", quirk_grids(), ids=[n for n, _ in quirk_grids()])
def test_compress_matches_reference(ref, name, grid):
    a = ref.nc_compress(grid, SPVAL)
    b = ref.nc_compress(grid, SPVAL, which="reference")
    np.testing.assert_array_equal(a[0], b[0])
    assert np.float32(a[1]).tobytes() == np.float32(b[1]).tobytes()
    assert np.float32(a[2]).tobytes() == np.float32(b[2]).tobytes()
    assert a[3] == b[3] == -32768
    if name == "first_is_max":
        # the reference's quirk, reproduced: the first cell wraps
        q = np.float32(np.float32(80.0) - np.float32(a[1])) / np.float32(a[2])
        assert a[0][0, 0] == np.int16(np.int64(np.rint(q)) & 0xFFFF if np.rint(q) < 2**31 else 0)


@pytest.mark.parametrize("has_missing,has_spval", [(True, True), (False, True), (True, False),
                                                   (False, False)])
def test_decompress_matches_reference(ref, has_missing, has_spval):
    rng = np.random.default_rng(5)
    p = rng.integers(-32768, 32768, (23, 31)).astype(np.int16)
    p[rng.random(p.shape) < 0.1] = -32768
    p[0, :3] = 1234
    for off, sc, mv in ((3.5, 0.00125, -32768), (-2.0, 1.0e-4, 1234), (0.0, 0.0, -32768)):
        a = ref.nc_decompress(p, off, sc, mv, SPVAL, has_missing=has_missing,
                              has_spval=has_spval)
        b = ref.nc_decompress(p, off, sc, mv, SPVAL, which="reference",
                              has_missing=has_missing, has_spval=has_spval)
        assert a[0].tobytes() == b[0].tobytes()
        assert a[1] == b[1]


def _layout_from_file(path):
    f = netcdf(path, "r", mmap=False, maskandscale=False)
    tcode = {"f": 5, "h": 3}
    lines = [f"dim {k} {v}" for k, v in f.dimensions.items()]
    owners = {"NC_GLOBAL": f._attributes}
    for name, v in f.variables.items():
        lines.append(f"var {name} {tcode[v.typecode()]} " + " ".join(v.dimensions))
        owners[name] = v._attributes
    atts = {}
    for owner, d in owners.items():
        for k, val in d.items():
            if isinstance(val, bytes):
                atts.setdefault(owner, []).append(f"att {owner} {k} 2 {len(val)} {val.decode()}")
            else:
                t = 3 if np.asarray(val).dtype == np.int16 else 5
                atts.setdefault(owner, []).append(f"att {owner} {k} {t} {np.asarray(val).size}")
    f.close()
    return lines, atts


def test_container_layout_is_write_nc_layout(ref, tmp_path, monkeypatch):
    from photic_gb300 import ncgrid as N
    grid = quirk_grids()[0][1]
    want = ref.nc_reference_layout(grid, SPVAL)
    packed, off, sc, mv = ref.nc_compress(grid, SPVAL)
    monkeypatch.chdir(tmp_path)
    nr, nc = grid.shape
    N.write_raw("photic_ref_grid.nc", packed, np.arange(nc), np.arange(nr), off, sc, mv, SPVAL)
    lines, atts = _layout_from_file("photic_ref_grid.nc")
    assert [l for l in want if not l.startswith("att ")] == lines
    want_atts = {}
    for l in want:
        if l.startswith("att "):
            want_atts.setdefault(l.split()[1], []).append(l)
    assert want_atts == atts


@pytest.mark.parametrize("version", [1, 2])
def test_container_round_trips_with_scipy(tmp_path, version):
    from photic_gb300 import ncgrid as N
    rng = np.random.default_rng(version)
    packed = rng.integers(-32768, 32768, (13, 27)).astype(np.int16)
    lons = np.linspace(140.0, 141.0, 27).astype(np.float32)
    lats = np.linspace(-20.0, -19.5, 13).astype(np.float32)
    # library -> scipy
    p = str(tmp_path / "lib.nc")
    N.write_raw(p, packed, lons, lats, 1.5, 2.0e-3, -32768, SPVAL, fmt=version)
    f = netcdf(p, "r", mmap=False, maskandscale=False)
    assert f.version_byte == version
    np.testing.assert_array_equal(f.variables["bathy"].data, packed)
    np.testing.assert_array_equal(f.variables["lons"].data, lons)
    np.testing.assert_array_equal(f.variables["lats"].data, lats)
    b = f.variables["bathy"]
    assert b.add_offset == np.float32(1.5) and b.scale_factor == np.float32(2.0e-3)
    assert b.missing_value == -32768 and b.decompressed_missing_value == np.float32(SPVAL)
    f.close()
    # scipy -> library, attributes in other numeric types, one optional one absent
    q = str(tmp_path / "scipy.nc")
    w = netcdf(q, "w", version=version)
    w.createDimension("lons", 27)
    w.createDimension("lats", 13)
    w.createVariable("lats", "f4", ("lats",))[:] = lats
    w.createVariable("lons", "f4", ("lons",))[:] = lons
    v = w.createVariable("bathy", "i2", ("lats", "lons"))
    v[:] = packed
    v.add_offset = np.float64(-0.25)
    v.scale_factor = np.float64(1.0 / 3.0)
    v.missing_value = np.int32(77)
    w.close()
    got, lo, la, info = N.read_raw(q)
    np.testing.assert_array_equal(got, packed)
    np.testing.assert_array_equal(lo, lons)
    np.testing.assert_array_equal(la, lats)
    assert info["format"] == version and (info["ncols"], info["nrows"]) == (27, 13)
    assert info["add_offset"] == np.float32(-0.25)
    assert info["scale_factor"] == np.float32(1.0 / 3.0)
    assert info["has_missing_value"] == 1 and info["missing_value"] == 77
    assert info["has_spval"] == 0 and info["spval"] == 0.0


def test_container_errors(tmp_path):
    from photic_gb300 import ncgrid as N
    from photic_gb300._lib import ERR_IO, PhoticError

    def fails(path, text):
        with pytest.raises(PhoticError) as e:
            N.read_info(path)
        assert e.value.code == ERR_IO and text in str(e.value), str(e.value)

    fails(str(tmp_path / "absent.nc"), "cannot open")
    h5 = tmp_path / "h5.nc"
    h5.write_bytes(b"\x89HDF\r\n\x1a\n" + bytes(64))
    fails(str(h5), "HDF5")
    (tmp_path / "text.nc").write_bytes(b"ncols 5\nnrows 5\n")
    fails(str(tmp_path / "text.nc"), "not a netCDF file")
    good = tmp_path / "good.nc"
    N.write_raw(str(good), np.zeros((3, 4), np.int16), np.arange(4), np.arange(3), 0.0, 1.0)
    raw = good.read_bytes()
    (tmp_path / "trunc.nc").write_bytes(raw[:40])
    fails(str(tmp_path / "trunc.nc"), "truncated")
    (tmp_path / "short_data.nc").write_bytes(raw[:-8])
    with pytest.raises(PhoticError) as e:
        N.read_raw(str(tmp_path / "short_data.nc"))
    assert e.value.code == ERR_IO and "truncated variable data" in str(e.value)
    w = netcdf(str(tmp_path / "nooff.nc"), "w")
    w.createDimension("lons", 2)
    w.createDimension("lats", 2)
    w.createVariable("lats", "f4", ("lats",))[:] = [0, 1]
    w.createVariable("lons", "f4", ("lons",))[:] = [0, 1]
    w.createVariable("bathy", "i2", ("lats", "lons"))[:] = [[1, 2], [3, 4]]
    w.close()
    fails(str(tmp_path / "nooff.nc"), "add_offset")
    w = netcdf(str(tmp_path / "float.nc"), "w")
    w.createDimension("lons", 2)
    w.createDimension("lats", 2)
    w.createVariable("lats", "f4", ("lats",))[:] = [0, 1]
    w.createVariable("lons", "f4", ("lons",))[:] = [0, 1]
    w.createVariable("bathy", "f4", ("lats", "lons"))[:] = [[1, 2], [3, 4]]
    w.close()
    fails(str(tmp_path / "float.nc"), "bathy must be short")
