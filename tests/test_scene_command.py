"""The SCENE command (model/bam.c:1300-1543) parsed into the scene record
and the inversion's configuration; host functions only.  The reference's
command interpreter (bam.c) does not compile as shipped, so the expected
records below are read off its run_scene: the grammar, the int wavelengths,
the optional items and the KSIGMA default of K / 10."""
import ctypes as C

import pytest

LINE = ("SCENE NAME LC08_2019 BANDS b1 b2 b3 b4 WAVELENGTHS 443.6 482 561.2 654.9 "
        "THETAVIEW 0.5 THETASUN 31.25 RINF 0.004 0.0038 0.0021 0.0004 HTIDE 0.8 "
        "K 0.05 0.04 0.07 0.4 RSIGMA 0.0002 0.00019 0.00015 0.0001 P p1 G g1 X x1")


@pytest.fixture(scope="module")
def scene():
    from photic_gb300 import scene as S
    return S


def test_full_line(scene):
    r = scene.parse(LINE)
    assert r["name"] == "LC08_2019" and r["n_bands"] == 4
    assert r["bands"] == ["b1", "b2", "b3", "b4"]
    assert r["wavelengths"] == [443, 482, 561, 654]      # int, as the record stores them
    assert r["theta_view"] == 0.5 and r["theta_sun"] == 31.25 and r["h_tide"] == 0.8
    assert r["R_inf"] == [0.004, 0.0038, 0.0021, 0.0004]
    assert r["K"] == [0.05, 0.04, 0.07, 0.4]
    assert r["K_sigma"] == [k / 10.0 for k in r["K"]]   # KSIGMA absent: K / 10
    assert r["pgx"] == ["p1", "g1", "x1"] and r["pgx_present"]
    assert r["given"] == ["HTIDE", "K", "RINF", "RSIGMA"]
    cfg = scene.config(r)
    assert cfg.wavelengths == (443.0, 482.0, 561.0, 654.0)
    assert cfg.theta_sun_deg == 31.25 and cfg.theta_view_deg == 0.5 and cfg.h_tide == 0.8


def test_minimal_line_and_aliases(scene):
    r = scene.parse("SCENE NAME s BANDS a b c WAVELENGTHS 490 560 665 THETAV 0 THETAW 40")
    assert r["n_bands"] == 3 and r["given"] == [] and not r["pgx_present"]
    assert r["R_inf"] == [0.0] * 3 and r["K_sigma"] == [0.0] * 3 and r["h_tide"] == 0.0
    assert scene.config(r).theta_sun_deg == 40.0


def test_reference_tokenizer(scene):
    """Every space splits (model/bam.c:6610-6624): a doubled space is an empty
    token, which here becomes an extra, empty band name."""
    r = scene.parse("SCENE NAME s BANDS a  b WAVELENGTHS 443 482 561 THETAVIEW 0 THETASUN 35")
    assert r["bands"] == ["a", "", "b"]


@pytest.mark.parametrize("line", [
    "SCENE s BANDS a WAVELENGTHS 443 THETAVIEW 0 THETASUN 35",
    "SCENE NAME s a b WAVELENGTHS 443 482 THETAVIEW 0 THETASUN 35",
    "SCENE NAME s BANDS a b THETAVIEW 0 THETASUN 35",
    "SCENE NAME s BANDS a b WAVELENGTHS 443 482 THETASUN 35",
    "SCENE NAME s BANDS a b WAVELENGTHS 443 482 THETAVIEW 0 HTIDE 1",
])
def test_malformed_lines_are_refused(scene, line):
    from photic_gb300 import _lib as L
    with pytest.raises(L.PhoticError):
        scene.parse(line)


def test_config_needs_two_to_eight_bands(scene):
    from photic_gb300 import _lib as L
    r = scene.parse("SCENE NAME s BANDS a WAVELENGTHS 560 THETAVIEW 0 THETASUN 35")
    with pytest.raises(L.PhoticError):
        scene.config(r)
