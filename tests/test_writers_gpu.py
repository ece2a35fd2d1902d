"""The wx layer's text files written from device state (cpp/main.cpp:328-335, 357-384, 464-494): the layouts
test.sh checks (sphere 8 columns and nlat x nlon points, plane 6 columns, spectrum "n ke pe" with the Parseval sum
75 = 15^2/3 for solid-body rotation), values equal to the engine's own grids to the 10 printed digits, byte-identical
files on a rerun, and the reference's error texts."""
import math

import numpy as np
import pytest

from sphere_cases import fields, williamson6

pytestmark = pytest.mark.gpu

# "%.10g" keeps ten significant digits: the printed value is within 5e-10 of the value, relative
RTOL = 6e-10


def _rows(path):
    with open(path) as f:
        lines = f.read().split("\n")
    return lines, [list(map(float, ln.split())) for ln in lines if ln.strip()]


def test_sphere_csv_layout_and_values(engine, tmp_path):
    s = williamson6(engine.Sphere(21))
    s.run(43200.0, 1200.0)
    a, b = tmp_path / "a.csv", tmp_path / "b.csv"
    s.save_csv(str(a))
    t = williamson6(engine.Sphere(21))
    t.run(43200.0, 1200.0)
    t.save_csv(str(b))
    assert a.read_bytes() == b.read_bytes()  # seeded runs repeat bit for bit (tests/determinism.lms)
    lines, rows = _rows(a)
    assert len(rows) == 64 * 32 and {len(r) for r in rows} == {8}
    assert sum(1 for ln in lines if not ln.strip()) == 32 + 1  # a blank line after each latitude row, then EOF
    data = np.array(rows).reshape(32, 64, 8)
    mu, _ = s.gauss()
    assert np.allclose(data[:, 0, 1], np.degrees(np.arcsin(mu)), rtol=RTOL, atol=1e-9)
    assert np.allclose(data[0, :, 0], 360.0 * np.arange(64) / 64, rtol=RTOL, atol=1e-9)
    for col, grid in ((2, s.grid_height()), (3, s.grid_u()), (4, s.grid_v()), (5, s.grid_vorticity())):
        assert np.allclose(data[:, :, col], grid, rtol=RTOL, atol=1e-12 * np.abs(grid).max())
    assert np.all(data[:, :, 6] == 0.0) and np.all(data[:, :, 7] == 0.0)  # no tracer, no orography
    z = tmp_path / "z.csv"
    s.save_zonal_mean(str(z))
    _, zr = _rows(z)
    zm = np.array(zr)
    assert zm.shape == (32, 3)
    assert np.allclose(zm[:, 1], s.grid_height().mean(axis=1), rtol=RTOL)
    assert np.allclose(zm[:, 2], s.grid_u().mean(axis=1), rtol=RTOL, atol=1e-9)


def test_sphere_spectrum_file_parseval(engine, tmp_path):
    r = fields(engine.Sphere(21), lambda lo, la: 2000.0 + 0 * la, lambda lo, la: 15.0 * np.cos(la), lambda lo, la: 0 * la)
    path = tmp_path / "spectrum_solid.csv"
    r.save_spectrum(str(path))
    _, rows = _rows(path)
    assert len(rows) == 21 and {len(x) for x in rows} == {3}
    assert [int(x[0]) for x in rows] == list(range(1, 22))
    assert abs(sum(x[1] for x in rows) - 75.0) <= 1e-6  # test.sh:159


def test_plane_csv_row_column(engine, tmp_path):
    p = engine.Plane(40, 20, 4.0e6, 2.0e6, depth=500.0, f0=1e-4, beta=2e-11)
    p.perturb(1.0, 99)
    p.run(86400.0, 0.0)
    a = tmp_path / "plane.csv"
    p.save_csv(str(a))
    lines, rows = _rows(a)
    assert len(rows) == 40 * 20 and {len(r) for r in rows} == {6}
    assert sum(1 for ln in lines if not ln.strip()) == 20 + 1
    data = np.array(rows).reshape(20, 40, 6)
    h, u, v = p.get()
    assert np.allclose(data[:, :, 2], h, rtol=RTOL)
    assert np.allclose(data[:, :, 3], 0.5 * (u + np.roll(u, -1, axis=1)), rtol=RTOL, atol=1e-12)
    assert np.allclose(data[:, :, 4], 0.5 * (v[:-1] + v[1:]), rtol=RTOL, atol=1e-12)
    zc = np.array([[p.zeta_at_corner(i, j) for i in range(41)] for j in range(21)])
    z = 0.25 * (zc[:-1, :-1] + zc[:-1, 1:] + zc[1:, :-1] + zc[1:, 1:])
    assert np.allclose(data[:, :, 5], z, rtol=RTOL, atol=1e-9 * np.abs(z).max())
    r, c = tmp_path / "row.csv", tmp_path / "col.csv"
    p.save_row(7, str(r))
    p.save_column(3, str(c))
    assert np.allclose(np.array(_rows(r)[1])[:, 1], h[7], rtol=RTOL)
    assert np.allclose(np.array(_rows(c)[1])[:, 1], h[:, 3], rtol=RTOL)
    with pytest.raises(ValueError, match="Plane.save_row: row outside the grid"):
        p.save_row(20, str(r))
    with pytest.raises(ValueError, match="Plane.save_column: column outside the grid"):
        p.save_column(-1, str(c))
    with pytest.raises(RuntimeError, match="Plane.save_csv: cannot write"):
        p.save_csv(str(tmp_path / "missing" / "x.csv"))
    s = engine.Sphere(10)
    with pytest.raises(RuntimeError, match="Sphere.save_spectrum: cannot write"):
        s.save_spectrum(str(tmp_path / "missing" / "s.csv"))
