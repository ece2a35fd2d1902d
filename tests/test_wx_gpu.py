"""The wx.* operator surface on the GPU engine (cpp/main.cpp:62-494): lmweather's twelve scripted known-answer tests
run through the registrations (tests/wx_scripts.py), the file checks and the rerun byte-identity of test.sh:141-163,
its error cases (test.sh:176-213) with the reference's messages, and the builders' initial states against the class
API given the same grids."""
import ctypes
import math
import os

import numpy as np
import pytest

import wx_scripts
from sphere_cases import williamson2, williamson6

pytestmark = pytest.mark.gpu


@pytest.fixture
def wx(engine):
    from lmweather_gb300.wx import Wx

    with Wx() as w:
        yield w


@pytest.mark.parametrize("script", wx_scripts.SCRIPTS, ids=[s.__name__ for s in wx_scripts.SCRIPTS])
def test_reference_script(wx, script, tmp_path):
    script(wx, str(tmp_path))


def _rows(path):
    with open(path) as f:
        return [ln.split() for ln in f if ln.strip()]


def test_result_files_and_rerun(engine, tmp_path):
    """test.sh:141-163: the files the scripts write, their layouts, Parseval on the solid-body spectrum, and every file
    byte-identical when the scripts run again in a fresh host."""
    from lmweather_gb300.wx import Wx

    runs = []
    for k in range(2):
        d = tmp_path / f"run{k}"
        d.mkdir()
        with Wx() as w:
            wx_scripts.determinism(w, str(d))
            wx_scripts.sphere_spectrum(w, str(d))
        runs.append(d)
    names = sorted(os.listdir(runs[0]))
    assert names == sorted(["determinism_plane.csv", "determinism_sphere.csv", "determinism_zonal.csv", "spectrum_winds.csv",
                            "spectrum_solid.csv", "spectrum_mode.csv", "spectrum_day1.csv", "spectrum_day5.csv"])
    for n in names:
        assert (runs[0] / n).read_bytes() == (runs[1] / n).read_bytes(), n
    d = runs[0]
    assert {len(r) for r in _rows(d / "determinism_sphere.csv")} == {8}
    assert {len(r) for r in _rows(d / "determinism_plane.csv")} == {6}
    assert len(_rows(d / "determinism_sphere.csv")) == 2048
    assert len(_rows(d / "spectrum_winds.csv")) == 21 and {len(r) for r in _rows(d / "spectrum_winds.csv")} == {3}
    assert abs(sum(float(r[1]) for r in _rows(d / "spectrum_solid.csv")) - 75.0) <= 1e-6


DEEP = "(" * 300 + "1" + ")" * 300
ERRORS = [
    ("bad_expression", lambda wx: wx.sphere(10).fields("2 +* 3", "0", "0"), "expression"),
    ("unknown_name", lambda wx: wx.sphere(10).fields("foo", "0", "0"), "unknown name"),
    ("mode_range", lambda wx: wx.sphere(10).mode(40, 0, 1.0, 100.0), "truncation"),
    ("bad_wave", lambda wx: wx.sphere(10).fields("1000", "0", "0").perturb(1.0, 1, 0), "max_wave"),
    ("zero_height", lambda wx: wx.sphere(10).fields("0", "0", "0").stable_dt(), "must be positive"),
    ("unstable_dt", lambda wx: wx.plane(20, 10, 1000000.0, 500000.0).depth(100.0).fields("cos(x / 100000.0)", "0", "0").run_dt(5000000.0, 50000.0),
     "stability limit"),
    ("unstable_sphere_dt", lambda wx: wx.sphere(21).williamson2(0.0).run_dt(86400.0, 86400.0), "stability limit"),
    ("blow_up", lambda wx: wx.plane(20, 10, 1000000.0, 500000.0).depth(100.0).fields("-150.0 * cos(2.0 * pi * x / lx)", "0", "0").run(50000000.0),
     "blew up"),
    ("nan_longitude", lambda wx: wx.sphere(10).fields("1000", "0", "0").height_at(10.0, float("nan")), "longitude"),
    ("wrapped_int", lambda wx: wx.sphere(10).mode(4294967298, 0, 1.0, 100.0), "out of range"),
    ("infinite_depth", lambda wx: wx.plane(10, 10, 1000000.0, 500000.0).depth(float("inf")), "depth"),
    ("depth_late", lambda wx: wx.plane(10, 10, 1000000.0, 500000.0).perturb(1.0, 1).depth(100.0), "before fields"),
    ("negative_depth", lambda wx: wx.plane(10, 10, 1000000.0, 500000.0).depth(-5.0), "depth"),
    ("negative_viscosity", lambda wx: wx.plane(10, 10, 1000000.0, 500000.0).viscosity(-1.0), "viscosity"),
    ("outside_domain", lambda wx: wx.plane(10, 10, 1000000.0, 500000.0).h_at(2000000.0, 0.0), "outside the domain"),
    ("bad_harmonic", lambda wx: wx.plane(10, 10, 1000000.0, 500000.0).zonal_amplitude(9, 2), "out of range"),
    ("bad_crest", lambda wx: wx.sphere(10).fields("1000", "0", "0").wave_crest(0, 45.0), "zonal wavenumber"),
    ("pole_wind", lambda wx: wx.sphere(10).fields("1000", "0", "0").u_at(90.0, 0.0), "inside"),
    ("bad_part", lambda wx: wx.sphere(10).fields("1000", "0", "0").mode_coefficient(1, 0, "abs"), "part must be"),
    ("no_rossby_radius", lambda wx: wx.plane(10, 10, 1000000.0, 500000.0).rossby_radius(), "f0 is zero"),
    ("deep_expression", lambda wx: wx.sphere(10).fields(DEEP, "0", "0"), "nested too deeply"),
    ("huge_number", lambda wx: wx.sphere(10).fields("1e400", "0", "0"), "out of range"),
    ("nonfinite_result", lambda wx: wx.sphere(10).fields("0", "0", "0").error_l2(), "not finite"),
    ("no_tracer", lambda wx: wx.sphere(10).fields("1000", "0", "0").tracer_at(0.0, 0.0), "no tracer"),
    ("advect_no_tracer", lambda wx: wx.sphere(10).fields("1000", "0", "0").advect_only().run(3600.0), "set a tracer first"),
    ("tracer_nonfinite", lambda wx: wx.sphere(10).fields("1000", "0", "0").tracer("1 / (lat - lat)"), "not finite"),
    ("orography_nonfinite", lambda wx: wx.sphere(10).orography("1 / (lat - lat)"), "not finite"),
    ("row_outside", lambda wx: wx.plane(10, 10, 1000000.0, 500000.0).save_row(10, "/tmp/never-written.csv"), "row outside the grid"),
    ("wide_column", lambda wx: wx.plane(10, 10, 1000000.0, 500000.0).save_column(4294967296, "/tmp/never-written.csv"), "column outside the grid"),
]


def _accelerated(wx):
    s = wx.sphere(21).fields("5960.0 - 1500.0 * pow(2.718281828459045, -((lon - 3.0) * (lon - 3.0) * cos(lat) * cos(lat) + lat * lat) / 0.1)", "0", "0")
    s.run_dt(5.0 * 86400.0, 0.97 * s.stable_dt() * 1.8856180831641)


ERRORS.append(("accelerated", _accelerated, "the flow accelerated"))


@pytest.mark.parametrize("name, call, fragment", ERRORS, ids=[e[0] for e in ERRORS])
def test_reference_error_cases(wx, name, call, fragment):
    from lmweather_gb300.wx import WxError

    with pytest.raises(WxError, match=fragment):
        call(wx)


def test_result_not_finite_names_the_method(wx):
    from lmweather_gb300.wx import WxError

    with pytest.raises(WxError, match=r"^Sphere.error_l2: the result is not finite$"):
        wx.sphere(10).fields("0", "0", "0").error_l2()


def _grids(lib, handle, nlat, nlon):
    out = []
    for which in range(4):
        g = np.zeros((nlat, nlon))
        assert lib.lmw_sphere_grid(ctypes.c_void_p(handle), 0, which, g.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), g.size) == 0
        out.append(g)
    return out


@pytest.mark.parametrize("builder", ["williamson2", "williamson6"])
def test_builders_match_the_class_api(engine, wx, builder):
    """A builder's state equals the class API's given the builder's formulas evaluated in numpy (libm rounding of the
    trigonometry differs in the last bits: 1e-12 of the field)."""
    lib = engine.load_library()
    if builder == "williamson2":
        o = wx.sphere(42).williamson2(0.05)
        c = williamson2(engine.Sphere(42), 0.05)
    else:
        o = wx.sphere(42).williamson6()
        c = williamson6(engine.Sphere(42))
    a = _grids(lib, o.engine_handle(), 64, 128)
    b = [c.grid_height(), c.grid_u(), c.grid_v(), c.grid_vorticity()]
    for x, y in zip(a, b):
        assert np.abs(x - y).max() <= 1e-12 * np.abs(y).max()
    assert math.isclose(o.energy(), c.energy(), rel_tol=1e-12)


def test_wx_objects_and_engine_handles(wx):
    s = wx.sphere(21)
    p = wx.plane(16, 8, 1.0e6, 5.0e5)
    assert s.type == "Sphere" and p.type == "Plane"
    assert s.truncation() == 21 and s.nlat() == 32 and s.nlon() == 64
    assert s.williamson2(0.0) == s  # builders return the receiver
    assert p.depth(50.0).coriolis(1e-4, 0.0) == p
    assert s.engine_handle() and p.engine_handle()
    assert math.isclose(p.wave_speed(), math.sqrt(9.81 * 50.0))
    assert math.isclose(p.rossby_radius(), math.sqrt(9.81 * 50.0) / 1e-4)
