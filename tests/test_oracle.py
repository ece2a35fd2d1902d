"""The CPU oracle pinned against the reference: golden fixtures made by the reference itself
(tests/golden/make_golden.py), the reference compiled from its own sources where the checkout exists, and the
known-answer checks of the reference's native suite (tests/core.cpp:17-121), restated here."""
import math
import platform

import numpy as np
import pytest

from conftest import golden
from oracle_lib import (OracleError, OraclePlane, OracleSphere, RefPlane, RefSphere, _dp, oracle, ref_available)
from plane_cases import plane_adjustment_case, plane_harmonic_case, plane_rossby_case
from sphere_cases import gravity_modes_case, rossby_haurwitz_case, spectrum_case, williamson2_case

X86 = platform.machine() in ("x86_64", "AMD64")


def same(a, b, tol=1e-13):
    """Bitwise where the fixtures were made (x86_64 glibc); within tol elsewhere (libm may differ in the last bit)."""
    a, b = np.asarray(a), np.asarray(b)
    if X86:
        return np.array_equal(a, b)
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() <= tol * scale


@pytest.fixture(scope="module", autouse=True)
def _built(oracle_built):
    return oracle_built


# --------------------------------------------------------------------------------------- transforms
def test_fft_matches_reference_fixtures():
    g = golden("transforms.npz")
    for n in (8, 64, 128, 512):
        for sign, key in ((-1, "fwd"), (1, "bwd")):
            a = g[f"fft{n}_in"].copy()
            assert oracle().or_fft(_dp(a), n, sign) == 0
            assert same(a, g[f"fft{n}_{key}"]), (n, sign)


def test_fft_against_dft_and_inverse():
    # tests/core.cpp:20-37
    n = 64
    k = np.arange(n)
    a = (np.sin(0.3 * k) + 0.1 * k) + 1j * np.cos(1.7 * k)
    ref = np.array([np.sum(a * np.exp(-2j * math.pi * m * k / n)) for m in range(n)])
    b = a.astype(np.complex128).copy()
    oracle().or_fft(_dp(b.view(np.float64)), n, -1)
    assert np.abs(b - ref).max() <= 1e-10
    oracle().or_fft(_dp(b.view(np.float64)), n, +1)
    assert np.abs(b / n - a).max() <= 1e-12
    c = np.zeros(24)
    assert oracle().or_fft(_dp(c), 12, -1) == 1  # not a power of two


def test_gauss_legendre():
    g = golden("transforms.npz")
    for n in (32, 64, 256):
        x, w = np.zeros(n), np.zeros(n)
        oracle().or_gauss_legendre(n, _dp(x), _dp(w))
        assert same(x, g[f"gl{n}_x"]) and same(w, g[f"gl{n}_w"])
    # tests/core.cpp:39-47
    x, w = np.zeros(32), np.zeros(32)
    oracle().or_gauss_legendre(32, _dp(x), _dp(w))
    assert abs(w.sum() - 2) <= 1e-13
    assert abs((w * x ** 10).sum() - 2 / 11) <= 1e-13
    assert abs((w * x ** 62).sum() - 2 / 63) <= 1e-12
    assert np.all(np.diff(x) > 0) and np.abs(x + x[::-1]).max() <= 1e-14


def test_legendre_columns_and_orthonormality():
    g = golden("transforms.npz")
    for row in g["legendre_cols"]:
        m, nmax, mu = int(row[0]), int(row[1]), row[2]
        out = np.zeros(nmax + 2 - m)
        oracle().or_legendre_column(m, nmax, mu, _dp(out))
        assert same(out, row[3:3 + len(out)])
    # tests/core.cpp:49-59
    x, w = np.zeros(40), np.zeros(40)
    oracle().or_gauss_legendre(40, _dp(x), _dp(w))
    for m in range(7):
        cols = []
        for xi in x:
            c = np.zeros(12 + 2 - m)
            oracle().or_legendre_column(m, 12, xi, _dp(c))
            cols.append(c[: 13 - m])
        cols = np.array(cols)
        gram = (cols * w[:, None]).T @ cols
        assert np.abs(gram - np.eye(13 - m)).max() <= 1e-12


# --------------------------------------------------------------------------------------- sphere
def test_sphere_t21_turbulence_matches_reference_run():
    g = golden("sphere_t21_turb.npz")
    s = OracleSphere(21, diffusion=float(g["diffusion"]))
    h, u, v = s.turbulence_grids(int(g["seed"]), float(g["hbar"]), float(g["umax"]), int(g["nforce"]))
    assert same(h, g["h"]) and same(u, g["u"]) and same(v, g["v"])
    s.set_state_grid(h, u, v)
    z, d, f = s.get_state()
    assert same(z, g["zeta0"]) and same(d, g["delta0"]) and same(f, g["phi0"])
    for _ in range(int(g["steps"])):
        s.step(float(g["dt"]))
    z, d, f = s.get_state()
    assert same(z, g["zeta"]) and same(d, g["delta"]) and same(f, g["phi"])
    diag = s.diagnostics()
    for k, v in zip(g["diag_keys"], g["diag1"]):
        assert same(diag[str(k)], v), k


def test_sphere_known_cases_match_reference_runs():
    g = golden("sphere_t21_known.npz")
    s = OracleSphere(21)
    s.set_axis_tilt(float(g["tc2_alpha"]))
    s.set_state_grid(g["tc2_h"], g["tc2_u"], g["tc2_v"])
    s.run(86400.0, 1800.0)
    z, d, f = s.get_state()
    assert same(z, g["tc2_zeta"]) and same(d, g["tc2_delta"]) and same(f, g["tc2_phi"])
    # Williamson TC2 is steady: the height error stays at round-off (sphere_williamson2.lms asserts < 1e-6)
    assert s.diagnostics()["error_l2"] < 1e-10
    t1 = OracleSphere(21)
    t1.set_axis_tilt(float(g["tc1_alpha"]))
    t1.set_state_grid(g["tc1_h"], g["tc1_u"], g["tc1_v"])
    t1.set_tracer_grid(g["tc1_q"])
    t1.set_advect_only(True)
    t1.run(43200.0, 3600.0)
    z, d, f, q = t1.get_state(with_tracer=True)
    assert same(q, g["tc1_qspec"]) and same(z, g["tc1_zeta"])
    t5 = OracleSphere(21)
    t5.set_orography_grid(g["tc5_hs"])
    t5.set_state_grid(g["tc5_h"], g["tc5_u"], np.zeros_like(g["tc5_h"]))
    t5.run(43200.0, 900.0)
    z, d, f = t5.get_state()
    assert same(z, g["tc5_zeta"]) and same(f, g["tc5_phi"])


def test_sphere_core_known_answers():
    # tests/core.cpp:61-100: spectral round trip, solid-body rotation, rest stays at rest, mass conservation
    s = OracleSphere(21)
    seed = 5

    def rnd():
        nonlocal seed
        seed = (seed * 1664525 + 1013904223) & 0xFFFFFFFF
        return (seed >> 8) / 16777216.0 - 0.5

    spec = np.zeros(22 * 22, np.complex128)
    for m in range(22):
        for n in range(m, 22):
            re = rnd()
            im = 0.0 if m == 0 else rnd()
            spec[m * 22 + n] = re + 1j * im
    back = s.analyze_scalar(s.synthesize_scalar(spec))
    assert np.abs(back - spec).max() <= 1e-12
    lat = np.arcsin(s.mu)[:, None]
    h = np.full((s.nlat, s.nlon), 1000.0)
    u = 10 * np.cos(lat) * np.ones((1, s.nlon))
    s.set_state_grid(h, u, np.zeros_like(h))
    z = s.grid_vorticity()
    assert np.abs(z - 2 * 10 * np.sin(lat) / 6.37122e6).max() <= 1e-12
    assert abs(s.diagnostics()["mean_height"] - 1000.0) <= 1e-9
    e = s.diagnostics()["energy"]
    assert abs(e - (0.5 * 1000 * (100.0 * 2.0 / 3.0) + 0.5 * 9.80616 * 1e6)) <= 1e-6 * e
    r = OracleSphere(10)
    r.set_state_grid(np.full((r.nlat, r.nlon), 5000.0), np.zeros((r.nlat, r.nlon)), np.zeros((r.nlat, r.nlon)))
    r.run(86400.0, 1800.0)
    assert r.diagnostics()["max_wind"] <= 1e-9
    r.perturb(20.0, 3, 5)
    m0 = r.diagnostics()["mean_height"]
    r.run(43200.0, 1800.0)
    assert abs(r.diagnostics()["mean_height"] - m0) <= 1e-9
    with pytest.raises(OracleError):
        r.perturb(1.0, 1, 0)
    with pytest.raises(OracleError):
        OracleSphere(2)


def test_sphere_run_guard_messages():
    s = OracleSphere(21)
    g = golden("sphere_t21_turb.npz")
    s.set_state_grid(g["h"], g["u"], g["v"])
    with pytest.raises(OracleError) as e:
        s.run(86400.0, 5000.0)
    assert e.value.code == 1 and "exceeds the RK4 stability limit" in str(e.value)
    with pytest.raises(OracleError) as e:
        s.run(-1.0, 100.0)
    assert "seconds must not be negative" in str(e.value)


@pytest.mark.skipif(not ref_available(), reason="reference checkout not built here")
def test_oracle_bitwise_against_compiled_reference():
    for T in (10, 21):
        o, r = OracleSphere(T, diffusion=2e15), RefSphere(T, diffusion=2e15)
        h, u, v = o.turbulence_grids(3, 9000.0, 25.0, T // 2)
        o.set_state_grid(h, u, v)
        r.set_state_grid(h, u, v)
        o.set_axis_tilt(0.3)
        r.set_axis_tilt(0.3)
        o.perturb(15.0, 4, T - 1)
        r.perturb(15.0, 4, T - 1)
        for _ in range(6):
            o.step(1200.0)
            r.step(1200.0)
        for a, b in zip(o.get_state(), r.get_state()):
            assert np.array_equal(a, b)
        assert o.diagnostics() == r.diagnostics()
    p, q = OraclePlane(40, 24, 4e5, 2.4e5, f0=1e-4, beta=2e-11, viscosity=30.0, drag=1e-6), RefPlane(
        40, 24, 4e5, 2.4e5, f0=1e-4, beta=2e-11, viscosity=30.0, drag=1e-6)
    p.perturb(0.7, 8)
    q.perturb(0.7, 8)
    p.run(5000.0, 0.0)
    q.run(5000.0, 0.0)
    for a, b in zip(p.get(), q.get()):
        assert np.array_equal(a, b)


# --------------------------------------------------------------------------------------- plane
def test_plane_matches_reference_fixtures():
    g = golden("plane_small.npz")
    kw = dict(f0=1e-4, beta=1.6e-11, gravity=9.81, depth=100.0)
    p = OraclePlane(64, 32, 3.2e5, 1.6e5, **kw)
    h, u = p.jet_grids(u0=20.0, width=2.0e4, noise_rms=0.1, seed=5)
    assert same(h, g["h0"]) and same(u, g["u0"])
    p.set(h, u, g["v0"])
    for _ in range(int(g["steps"])):
        p.step(float(g["dt"]))
    for a, k in zip(p.get(), ("h", "u", "v")):
        assert same(a, g[k]), k
    kw2 = dict(f0=5e-5, beta=2e-11, gravity=9.81, depth=50.0, viscosity=200.0, drag=1e-5, linear=True)
    p2 = OraclePlane(48, 24, 2.4e5, 1.2e5, **kw2)
    p2.perturb(0.5, 9)
    for a, k in zip(p2.get(), ("lin_h0", "lin_u0", "lin_v0")):
        assert same(a, g[k]), k
    p2.run(7200.0, 0.0)
    for a, k in zip(p2.get(), ("lin_h", "lin_u", "lin_v")):
        assert same(a, g[k]), k


def test_plane_gravity_wave_known_answer():
    # tests/core.cpp:102-117: a standing wave returns inverted after half a period; mass exact; bad grids throw
    nx, ny, lx, ly, H = 100, 8, 1.0e6, 2.0e4, 100.0
    p = OraclePlane(nx, ny, lx, ly, depth=H, linear=True)
    k, c = 2 * math.pi / lx, math.sqrt(9.81 * H)
    xc = (np.arange(nx) + 0.5) * lx / nx
    h = np.tile(H + np.cos(k * xc), (ny, 1))
    p.set(h, np.zeros((ny, nx)), np.zeros((ny + 1, nx)))
    p.run(math.pi / (c * k), 0.0)
    hh, _, _ = p.get()
    assert abs((hh[ny // 2, 0] - H) - (-math.cos(k * xc[0]))) <= 2e-3
    assert abs(p.diagnostics()["mean_depth"] - H) <= 1e-10
    with pytest.raises(OracleError):
        OraclePlane(2, 2, 1.0, 1.0)


# ------------------------------------------------------------------- plane point and harmonic diagnostics
def _wavy_plane(cls, **extra):
    """A 40 x 24 channel with a seeded smooth state advanced a little, so every field has structure."""
    p = cls(40, 24, 4e5, 2.4e5, f0=1e-4, beta=2e-11, viscosity=30.0, drag=1e-6, **extra)
    p.perturb(0.7, 8)
    p.run(3000.0, 0.0)
    return p


@pytest.mark.skipif(not ref_available(), reason="reference checkout not built here")
def test_plane_probes_and_harmonics_bitwise_against_compiled_reference():
    # cpp/plane.cpp:220-310 restated in the oracle: bilinear probes, corner vorticity, zonal harmonics
    o, r = _wavy_plane(OraclePlane), _wavy_plane(RefPlane)
    pts = [(0.0, 0.0), (4e5, 2.4e5), (1.23e5, 0.77e5), (3.999e5, 1e3), (2e4, 2.39e5), (5e3, 6e3)]
    for x, y in pts:
        assert o.h_at(x, y) == r.h_at(x, y)
        assert o.u_at(x, y) == r.u_at(x, y)
        assert o.v_at(x, y) == r.v_at(x, y)
    for i, j in [(0, 0), (40, 24), (7, 1), (39, 23), (40, 0), (0, 24), (13, 12)]:
        assert o.zeta_at_corner(i, j) == r.zeta_at_corner(i, j)
    for m in (1, 2, 5, 19):
        assert o.harmonic_energy(m) == r.harmonic_energy(m)
        for j in (0, 11, 23):
            assert o.zonal_amplitude(m, j) == r.zonal_amplitude(m, j)
            assert o.zonal_crest(m, j) == r.zonal_crest(m, j)
        for j in (1, 12, 23):
            assert o.v_zonal_crest(m, j) == r.v_zonal_crest(m, j)
    for bad in ((0, 3), (20, 3), (1, -1), (1, 24)):
        with pytest.raises(OracleError) as e:
            r.zonal_amplitude(*bad)
        assert e.value.code == 1 and "out of range" in str(e.value)
        with pytest.raises(OracleError):
            o.zonal_amplitude(*bad)
    with pytest.raises(OracleError):
        r.v_zonal_crest(1, 0)
    with pytest.raises(OracleError):
        o.v_zonal_crest(1, 0)


def test_plane_harmonic_known_answers():
    plane_harmonic_case(OraclePlane)


def test_plane_rossby_known_answers():
    plane_rossby_case(OraclePlane)


def test_plane_adjustment_known_answers():
    plane_adjustment_case(OraclePlane)


# ------------------------------------------------------------------- sphere known answers on the oracle
class _OracleSphereView(OracleSphere):
    """The oracle sphere with the engine's method names, and the exact point probes of cpp/sphere.cpp:592-652
    synthesised from its spectral state (height and the wave crest)."""

    def gauss(self):
        return self.mu, self.w

    def time(self):
        return OracleSphere.time.fget(self)

    def _d(self, key):
        return self.diagnostics()[key]

    def mean_height(self):
        return self._d("mean_height")

    def energy(self):
        return self._d("energy")

    def kinetic_energy(self):
        return self._d("kinetic_energy")

    def potential_energy(self):
        return self._d("potential_energy")

    def potential_enstrophy(self):
        return self._d("enstrophy")

    def max_wind(self):
        return self._d("max_wind")

    def height_error_l2(self):
        return self._d("error_l2")

    def height_error_linf(self):
        return self._d("error_linf")

    def _phi(self):
        return self.get_state()[2]

    def mode_coefficient(self, n, m, imag=False):
        c = self._phi()[m * (self.T + 1) + n] / self.gravity
        return c.imag if imag else c.real

    def _column(self, m, lat):
        col = np.zeros(self.T - m + 2)
        self.lib.or_legendre_column(m, self.T, math.sin(lat), _dp(col))
        return col

    def wave_crest(self, m, lat):
        phi, col = self._phi(), self._column(m, lat)
        g = sum(phi[m * (self.T + 1) + n] * col[n - m] for n in range(m, self.T + 1))
        return -np.angle(g) / m

    def height_at(self, lat, lon):
        phi, f = self._phi(), 0.0
        for m in range(self.T + 1):
            col = self._column(m, lat)
            F = sum(phi[m * (self.T + 1) + n] * col[n - m] for n in range(m, self.T + 1))
            f += (1.0 if m == 0 else 2.0) * (F * np.exp(1j * m * lon)).real
        return f / self.gravity


def _oracle_sphere(T, **kw):
    return _OracleSphereView(T, **kw)


def test_sphere_gravity_modes_known_answers():
    gravity_modes_case(_oracle_sphere)


def test_sphere_spectrum_known_answers():
    spectrum_case(_oracle_sphere)


def test_sphere_rossby_haurwitz_known_answers():
    rossby_haurwitz_case(_oracle_sphere)


def test_sphere_williamson2_known_answers():
    williamson2_case(_oracle_sphere)
