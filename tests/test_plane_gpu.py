"""GPU parity of the C-grid plane (cpp/plane.cpp) through the C ABI: bitwise identical to the reference's
outputs (golden fixtures made by the reference itself, and the oracle at the full 1024 x 512 size)."""
import math

import numpy as np
import pytest

from conftest import golden
from oracle_lib import OraclePlane
from plane_cases import plane_adjustment_case, plane_harmonic_case, plane_rossby_case

pytestmark = pytest.mark.gpu


def test_plane_jet_200_steps_bitwise(engine):
    g = golden("plane_small.npz")
    p = engine.Plane(64, 32, 3.2e5, 1.6e5, f0=1e-4, beta=1.6e-11, gravity=9.81, depth=100.0)
    p.set_h_from_grid(g["h0"]).set_u_from_grid(g["u0"]).set_v_from_grid(g["v0"])
    for _ in range(int(g["steps"])):
        p.step(float(g["dt"]))
    h, u, v = p.get()
    assert np.array_equal(h, g["h"]) and np.array_equal(u, g["u"]) and np.array_equal(v, g["v"])
    assert p.time() == pytest.approx(200 * 60.0)


def test_plane_linear_viscous_drag_run_bitwise(engine):
    g = golden("plane_small.npz")
    p = engine.Plane(48, 24, 2.4e5, 1.2e5, f0=5e-5, beta=2e-11, gravity=9.81, depth=50.0, viscosity=200.0, drag=1e-5,
                     linear=True)
    p.perturb(0.5, 9)
    h, u, v = p.get()
    assert np.array_equal(h, g["lin_h0"])
    p.run(7200.0, 0.0)  # automatic dt from stable_dt, guards every 64 steps
    h, u, v = p.get()
    assert np.array_equal(h, g["lin_h"]) and np.array_equal(u, g["lin_u"]) and np.array_equal(v, g["lin_v"])
    assert p.time() == pytest.approx(float(g["lin_time"]), rel=1e-15)


def test_plane_nonlinear_viscous_run_bitwise(engine):
    g = golden("plane_small.npz")
    p = engine.Plane(40, 20, 2.0e5, 1.0e5, f0=1e-4, beta=0.0, gravity=9.81, depth=80.0, viscosity=50.0, drag=2e-6)
    p.perturb(1.0, 4)
    p.run(3600.0, 20.0)
    h, u, v = p.get()
    assert np.array_equal(h, g["visc_h"]) and np.array_equal(u, g["visc_u"]) and np.array_equal(v, g["visc_v"])
    d = p.diagnostics()
    for k, ref in zip(("mean_depth", "energy", "max_speed", "pv_anomaly_rms"), g["visc_diag"]):
        assert d[k] == pytest.approx(ref, rel=1e-13, abs=1e-300), k


def test_plane_config1_5000_steps_bitwise_against_reference_run(engine):
    # the stated length of the configuration: 5000 RK4 steps of 60 s at 1024 x 512 from the seeded jet, compared with
    # the reference's own run (tests/golden/make_plane_config1.py keeps SHA-256 digests of its h, u, v after 1000
    # and 5000 steps; the plane's parity bar is bitwise)
    import hashlib
    import json
    import os

    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "plane_config1_5000.json")) as f:
        g = json.load(f)

    def digest(a):
        return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()

    nx, ny, L = g["nx"], g["ny"], g["dx"]
    p = engine.Plane(nx, ny, nx * L, ny * L, **g["params"])
    p.jet(*g["jet"])
    h, u, v = p.get()
    assert (digest(h), digest(u), digest(v)) == (g["initial"]["h"], g["initial"]["u"], g["initial"]["v"])
    done = 0
    for cp in g["checkpoints"]:
        p.run((cp["steps"] - done) * g["dt"], g["dt"])
        done = cp["steps"]
        h, u, v = p.get()
        assert h[256, 512] == cp["samples"]["h[256,512]"] and u[128, 100] == cp["samples"]["u[128,100]"], cp["steps"]
        assert (digest(h), digest(u), digest(v)) == (cp["h"], cp["u"], cp["v"]), cp["steps"]
        d = p.diagnostics()
        for k in ("mean_depth", "energy", "max_speed"):
            assert d[k] == pytest.approx(cp["diagnostics"][k], rel=1e-13), (k, cp["steps"])
    assert p.time() == pytest.approx(5000 * 60.0)


def test_plane_config1_full_size_bitwise_against_oracle(engine):
    # 1024 x 512 cells, dx = dy = 5 km, f0 = 1e-4, beta = 1.6e-11, H = 100 m, jet 20 sech^2(y/100 km) + 0.1 m noise
    nx, ny, L = 1024, 512, 5000.0
    kw = dict(f0=1e-4, beta=1.6e-11, gravity=9.81, depth=100.0)
    o = OraclePlane(nx, ny, nx * L, ny * L, **kw)
    h0, u0 = o.jet_grids(u0=20.0, width=1.0e5, noise_rms=0.1, seed=1)
    p = engine.Plane(nx, ny, nx * L, ny * L, **kw)
    p.jet(20.0, 1.0e5, 0.1, 1)
    h, u, v = p.get()
    assert np.array_equal(h, h0) and np.array_equal(u, u0) and not v.any()
    o.set(h0, u0, np.zeros((ny + 1, nx)))
    for _ in range(6):
        o.step(60.0)
        p.step(60.0)
    for a, b in zip(p.get(), o.get()):
        assert np.array_equal(a, b)
    d, od = p.diagnostics(), o.diagnostics()
    # the oracle sums 524288 depths in sequence (3e-14 relative rounding); the device sums in a tree
    assert d["mean_depth"] == pytest.approx(od["mean_depth"], rel=1e-13)
    assert d["energy"] == pytest.approx(od["energy"], rel=1e-13)


def test_plane_run_guards_and_messages(engine):
    p = engine.Plane(64, 32, 3.2e5, 1.6e5, f0=1e-4, depth=100.0)
    p.perturb(0.2, 1)
    limit = p.stable_dt(math.sqrt(0.5))
    with pytest.raises(ValueError, match="exceeds the RK4 stability limit of about"):
        p.run(3600.0, 2 * limit)
    with pytest.raises(ValueError, match="seconds must not be negative"):
        p.run(-5.0, 1.0)
    m0 = p.mean_depth()
    p.run(0.0, 1.0)
    p.run(1800.0, 0.0)
    assert abs(p.mean_depth() - m0) <= 1e-12 * m0
    with pytest.raises(ValueError, match="grid size mismatch"):
        p.set_h_from_grid(np.zeros(5))


def test_plane_gravity_wave_known_answer(engine):
    # tests/core.cpp:102-110: a standing wave is inverted after half a period
    nx, ny, lx, ly, H = 100, 8, 1.0e6, 2.0e4, 100.0
    p = engine.Plane(nx, ny, lx, ly, depth=H, linear=True)
    k, c = 2 * math.pi / lx, math.sqrt(9.81 * H)
    xc = (np.arange(nx) + 0.5) * lx / nx
    p.set_h_from_grid(np.tile(H + np.cos(k * xc), (ny, 1)))
    p.run(math.pi / (c * k), 0.0)
    h, _, _ = p.get()
    assert abs((h[ny // 2, 0] - H) + math.cos(k * xc[0])) <= 2e-3
    assert abs(p.mean_depth() - H) <= 1e-10


def test_plane_deterministic(engine):
    runs = []
    for _ in range(2):
        p = engine.Plane(96, 48, 4.8e5, 2.4e5, f0=1e-4, beta=1e-11)
        p.perturb(0.5, 12)
        p.run(3000.0, 30.0)
        runs.append(p.get())
    for a, b in zip(*runs):
        assert np.array_equal(a, b)


# ------------------------------------------------------------------- point and harmonic diagnostics
def _gpu_plane_class(engine):
    class GpuPlane(engine.Plane):
        def set(self, h, u, v):
            return self.set_h_from_grid(h).set_u_from_grid(u).set_v_from_grid(v)

    return GpuPlane


def test_plane_probes_and_harmonics_against_oracle(engine):
    # cpp/plane.cpp:220-310 on the device: probes and corner vorticity bit for bit (no FMA contraction), harmonics
    # within 1e-13 of the oracle (the device's sin/cos and its summation order differ from libm's in the last bits)
    kw = dict(f0=1e-4, beta=2e-11, viscosity=30.0, drag=1e-6)
    o = OraclePlane(40, 24, 4e5, 2.4e5, **kw).perturb(0.7, 8)
    p = engine.Plane(40, 24, 4e5, 2.4e5, **kw).perturb(0.7, 8)
    o.run(3000.0, 0.0)
    p.run(3000.0, 0.0)
    for a, b in zip(o.get(), p.get()):
        assert np.array_equal(a, b)
    for x, y in [(0.0, 0.0), (4e5, 2.4e5), (1.23e5, 0.77e5), (3.999e5, 1e3), (2e4, 2.39e5), (5e3, 6e3)]:
        assert p.h_at(x, y) == o.h_at(x, y)
        assert p.u_at(x, y) == o.u_at(x, y)
        assert p.v_at(x, y) == o.v_at(x, y)
    for i, j in [(0, 0), (40, 24), (7, 1), (39, 23), (40, 0), (0, 24), (13, 12)]:
        assert p.zeta_at_corner(i, j) == o.zeta_at_corner(i, j)
    # a harmonic is a sum of O(field) terms: its rounding error scales with the field, not with the harmonic
    # (m = 19 of this smooth state is 1e-12 of m = 1), so the bound is relative to the largest harmonic; crests
    # are compared where the harmonic stands well above that rounding
    hmax = max(o.harmonic_energy(m) for m in range(1, 20))
    amax = max(o.zonal_amplitude(m, j) for m in range(1, 20) for j in (0, 11, 23))
    for m in (1, 2, 5, 19):
        assert abs(p.harmonic_energy(m) - o.harmonic_energy(m)) <= 1e-13 * hmax
        for j in (0, 11, 23):
            a = o.zonal_amplitude(m, j)
            assert abs(p.zonal_amplitude(m, j) - a) <= 1e-13 * amax
            if a > 1e-6 * amax:
                assert p.zonal_crest(m, j) == pytest.approx(o.zonal_crest(m, j), rel=1e-9, abs=1e-3)
        for j in (1, 12, 23):
            if m < 19:
                assert p.v_zonal_crest(m, j) == pytest.approx(o.v_zonal_crest(m, j), rel=1e-9, abs=1e-3)
    for bad in ((0, 3), (20, 3), (1, -1), (1, 24)):
        with pytest.raises(ValueError, match="zonal harmonic or row out of range"):
            p.zonal_amplitude(*bad)
    with pytest.raises(ValueError, match="zonal harmonic or v row out of range"):
        p.v_zonal_crest(1, 0)
    with pytest.raises(ValueError, match="zonal harmonic out of range"):
        p.harmonic_energy(20)
    with pytest.raises(ValueError, match="corner outside the grid"):
        p.zeta_at_corner(41, 0)
    with pytest.raises(ValueError, match="point outside the domain"):
        p.h_at(float("nan"), 0.0)


def test_plane_full_size_harmonics_against_oracle(engine):
    # 1024 x 512: one CTA per row on the device against the oracle's sequential sums
    rng = np.random.default_rng(11)
    h = 100.0 + rng.normal(size=(512, 1024))
    u = rng.normal(size=(512, 1024))
    v = np.zeros((513, 1024))
    v[1:512] = rng.normal(size=(511, 1024))
    o = OraclePlane(1024, 512, 5.12e6, 2.56e6, f0=1e-4, beta=1.6e-11).set(h, u, v)
    p = engine.Plane(1024, 512, 5.12e6, 2.56e6, f0=1e-4, beta=1.6e-11)
    p.set_h_from_grid(h).set_u_from_grid(u).set_v_from_grid(v)
    for m in (1, 7, 100, 511):
        assert p.harmonic_energy(m) == pytest.approx(o.harmonic_energy(m), rel=1e-12, abs=1e-300)
        assert p.zonal_amplitude(m, 256) == pytest.approx(o.zonal_amplitude(m, 256), rel=1e-11)


def test_plane_harmonic_known_answers(engine):
    plane_harmonic_case(_gpu_plane_class(engine))


def test_plane_rossby_known_answers(engine):
    plane_rossby_case(_gpu_plane_class(engine))


def test_plane_adjustment_known_answers(engine):
    plane_adjustment_case(_gpu_plane_class(engine))


def _division_inputs(rng, n):
    """Dividends: random bit patterns over every exponent (zeros, subnormals, infinities and NaNs included),
    stencil-like differences of magnitude 1e-12 .. 1e6, and the special values."""
    raw = rng.integers(0, 2 ** 63, n, dtype=np.uint64) | (rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63))
    mag = 10.0 ** rng.uniform(-12, 6, n) * np.where(rng.integers(0, 2, n) == 0, -1.0, 1.0)
    specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 2.2250738585072014e-308, 1.7976931348623157e308,
                         -1.7976931348623157e308, 1.0, -1.0, 3.0, 0.1], np.float64)
    return np.concatenate([raw, mag.view(np.uint64), specials.view(np.uint64)]), mag


def _division_counts(lib, x, divisors):
    import ctypes as C

    counts = np.zeros(2, np.int64)
    d = np.ascontiguousarray(divisors, np.float64)
    st = lib.lmw_division_selftest(x.ctypes.data_as(C.POINTER(C.c_uint64)), x.size, d.ctypes.data_as(C.POINTER(C.c_double)), d.size,
                                   counts.ctypes.data_as(C.POINTER(C.c_longlong)))
    return st, counts


def test_fixed_divisor_division_is_the_ieee_division(engine):
    """The stencil's division by a grid spacing (two-term reciprocal, exact acceptance test) gives the IEEE quotient
    bit for bit on every dividend, and the fast path answers all but a tiny fraction of stencil-like dividends (the
    rest fall back to the IEEE division)."""
    rng = np.random.default_rng(23)
    x, mag = _division_inputs(rng, 1 << 20)
    plane_spacings = [5000.0, 2500.0, 5000.0 ** 2, 2500.0 ** 2, 1.0e5, 1.0e10, 3906.25, 1953.125 ** 2, 1.0e6 / 20, (1.0e6 / 20) ** 2]
    others = [1.0, 3.0, 1.0 / 3.0, 0.1, -7.5, 2.0 ** -1021, 2.0 ** 1021, 1.5 * 2.0 ** 1020, 2.2250738585072014e-308 * 4.0]
    logu = 10.0 ** rng.uniform(-300, 300, 24)
    divisors = np.array(plane_spacings + others + list(logu) + list(-rng.uniform(0.5, 2.0, 4)), np.float64)
    lib = engine.load_library()
    st, counts = _division_counts(lib, x, divisors)
    assert st == 0
    assert counts[0] == 0, f"{counts[0]} quotients differ from the IEEE division"
    # stencil-like dividends by the plane's spacings: the fast path answers them
    st, counts = _division_counts(lib, mag.view(np.uint64), plane_spacings)
    assert st == 0 and counts[0] == 0
    assert counts[1] >= 0.999 * mag.size * len(plane_spacings), counts
    # multiples of the divisor: exact quotients
    mult = np.concatenate([np.arange(-4096, 4097, dtype=np.float64) * 5000.0, np.arange(1, 4097, dtype=np.float64) * 2.5e7])
    st, counts = _division_counts(lib, mult.view(np.uint64), [5000.0, 2.5e7])
    assert st == 0 and counts[0] == 0
    # a divisor whose reciprocal is not a normal number is refused
    st, counts = _division_counts(lib, x[:4], [1.0e308])
    assert st == 1  # LMW_INVALID_ARGUMENT
