"""ctypes bindings of the CPU oracle (oracle/liboracle.so) and, where it was built, of the reference core
compiled from its own sources (oracle/_ref/libref*.so).

Test infrastructure: imported by tests/, the smoke check and bench.py's CPU-baseline leg only.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
_lock = threading.Lock()


def reference_dir() -> str | None:
    """The lmweather checkout the reference-side checks read: $LMW_REFERENCE_DIR, else a checkout named `reference`
    beside this repository; None when neither holds cpp/sphere.cpp (the checks that need it are skipped and the
    committed golden fixtures, made by the reference, stand in)."""
    for cand in (os.environ.get("LMW_REFERENCE_DIR"), os.path.join(os.path.dirname(ROOT), "reference")):
        if cand and os.path.exists(os.path.join(cand, "cpp", "sphere.cpp")):
            return os.path.abspath(cand)
    return None

D = C.c_double
I = C.c_int
P = C.c_void_p
DP = C.POINTER(C.c_double)
U64 = C.c_uint64


def _dp(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(DP)


def build_oracle(with_ref: bool = True) -> None:
    """Compile the oracle (and the reference harness where the reference checkout exists)."""
    ref = reference_dir() if with_ref else None
    target = "all" if ref else "oracle"
    with _lock:
        subprocess.run(["make", "-s", "-C", ORACLE_DIR, target] + ([f"REF={ref}"] if ref else []), check=True)


_ORACLE = None
_REF: dict[str, C.CDLL] = {}


def oracle() -> C.CDLL:
    global _ORACLE
    if _ORACLE is None:
        path = os.path.join(ORACLE_DIR, "liboracle.so")
        if not os.path.exists(path):
            build_oracle(with_ref=False)
        lib = C.CDLL(path)
        sig = {
            "or_fft": (I, [DP, I, I]),
            "or_gauss_legendre": (None, [I, DP, DP]),
            "or_legendre_column": (None, [I, I, D, DP]),
            "or_sphere_new": (P, [I, D, D, D, D, I]),
            "or_sphere_free": (None, [P]),
            "or_sphere_nlat": (I, [P]),
            "or_sphere_nlon": (I, [P]),
            "or_sphere_time": (D, [P]),
            "or_sphere_mu": (DP, [P]),
            "or_sphere_w": (DP, [P]),
            "or_sphere_set_diffusion": (None, [P, D]),
            "or_sphere_set_axis_tilt": (None, [P, D]),
            "or_sphere_set_state_grid": (I, [P, DP, DP, DP]),
            "or_sphere_set_orography_grid": (None, [P, DP]),
            "or_sphere_set_tracer_grid": (None, [P, DP]),
            "or_sphere_set_advect_only": (None, [P, I]),
            "or_sphere_mark_reference": (None, [P]),
            "or_sphere_add_mode": (I, [P, I, I, D, D]),
            "or_sphere_perturb": (I, [P, D, U64, I]),
            "or_sphere_get_state": (None, [P, DP, DP, DP, DP]),
            "or_sphere_set_state": (None, [P, DP, DP, DP, D]),
            "or_sphere_step": (None, [P, D]),
            "or_sphere_run": (I, [P, D, D, C.c_char_p, I]),
            "or_sphere_stable_dt": (D, [P, D, C.POINTER(I)]),
            "or_sphere_mean_height": (D, [P]),
            "or_sphere_kinetic_energy": (D, [P]),
            "or_sphere_potential_energy": (D, [P]),
            "or_sphere_energy": (D, [P]),
            "or_sphere_potential_enstrophy": (D, [P]),
            "or_sphere_max_wind": (D, [P]),
            "or_sphere_height_error_l2": (D, [P]),
            "or_sphere_height_error_linf": (D, [P]),
            "or_sphere_tracer_mean": (D, [P]),
            "or_sphere_tracer_mass": (D, [P]),
            "or_sphere_tracer_error_l2": (D, [P]),
            "or_sphere_spectrum": (None, [P, DP, DP]),
            "or_sphere_grid_height": (None, [P, DP]),
            "or_sphere_grid_u": (None, [P, DP]),
            "or_sphere_grid_v": (None, [P, DP]),
            "or_sphere_grid_vorticity": (None, [P, DP]),
            "or_sphere_grid_tracer": (None, [P, DP]),
            "or_sphere_analyze_scalar": (None, [P, DP, DP]),
            "or_sphere_synthesize_scalar": (None, [P, DP, DP]),
            "or_sphere_analyze_divergence": (None, [P, DP, DP, DP]),
            "or_sphere_turbulence_grids": (None, [P, U64, D, D, I, DP, DP, DP]),
            "or_plane_new": (P, [I, I, D, D, D, D, D, D, D, D, I]),
            "or_plane_free": (None, [P]),
            "or_plane_reset": (None, [P]),
            "or_plane_time": (D, [P]),
            "or_plane_get": (None, [P, DP, DP, DP]),
            "or_plane_set": (None, [P, DP, DP, DP]),
            "or_plane_perturb": (None, [P, D, U64]),
            "or_plane_step": (None, [P, D]),
            "or_plane_run": (I, [P, D, D, C.c_char_p, I]),
            "or_plane_stable_dt": (D, [P, D, C.POINTER(I)]),
            "or_plane_mean_depth": (D, [P]),
            "or_plane_energy": (D, [P]),
            "or_plane_max_speed": (D, [P]),
            "or_plane_pv_anomaly_rms": (D, [P]),
            "or_plane_jet_grids": (None, [P, D, D, D, U64, DP, DP]),
            "or_plane_zeta_at_corner": (D, [P, I, I]),
            "or_plane_probe": (D, [P, I, D, D]),
            "or_plane_zonal_amplitude": (I, [P, I, I, DP]),
            "or_plane_zonal_crest": (I, [P, I, I, DP]),
            "or_plane_v_zonal_crest": (I, [P, I, I, DP]),
            "or_plane_harmonic_energy": (I, [P, I, DP]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _ORACLE = lib
    return _ORACLE


def ref_available(variant: str = "") -> bool:
    return os.path.exists(os.path.join(ORACLE_DIR, "_ref", f"libref{variant}.so"))


def reference(variant: str = "") -> C.CDLL:
    """The reference core built from its own sources: variant "" (no FMA contraction, the bitwise pin),
    "_fma" (contraction allowed) or "_rel" (the reference's Release flags)."""
    if variant not in _REF:
        lib = C.CDLL(os.path.join(ORACLE_DIR, "_ref", f"libref{variant}.so"))
        CP = C.c_char_p
        sig = {
            "ref_fft": (I, [DP, I, I]),
            "ref_gauss_legendre": (None, [I, DP, DP]),
            "ref_legendre_column": (None, [I, I, D, DP]),
            "ref_sphere_new": (P, [I, D, D, D, D, CP, I]),
            "ref_sphere_free": (None, [P]),
            "ref_sphere_nlat": (I, [P]),
            "ref_sphere_nlon": (I, [P]),
            "ref_sphere_time": (D, [P]),
            "ref_sphere_mu_w": (None, [P, DP, DP]),
            "ref_sphere_set_axis_tilt": (None, [P, D]),
            "ref_sphere_set_diffusion": (None, [P, D]),
            "ref_sphere_set_advect_only": (None, [P, I]),
            "ref_sphere_set_state_grid": (I, [P, DP, DP, DP, CP, I]),
            "ref_sphere_set_orography_grid": (I, [P, DP, CP, I]),
            "ref_sphere_set_tracer_grid": (I, [P, DP, CP, I]),
            "ref_sphere_perturb": (I, [P, D, C.c_ulonglong, I, CP, I]),
            "ref_sphere_add_mode": (I, [P, I, I, D, D, CP, I]),
            "ref_sphere_mark_reference": (None, [P]),
            "ref_sphere_get_state": (None, [P, DP, DP, DP, DP]),
            "ref_sphere_set_state": (None, [P, DP, DP, DP, D]),
            "ref_sphere_step": (None, [P, D]),
            "ref_sphere_run": (I, [P, D, D, CP, I]),
            "ref_sphere_stable_dt": (D, [P, D]),
            "ref_sphere_diagnostics": (None, [P, DP]),
            "ref_sphere_spectrum": (None, [P, DP, DP]),
            "ref_sphere_tracer_mean": (D, [P]),
            "ref_sphere_tracer_mass": (D, [P]),
            "ref_sphere_grids": (None, [P, DP, DP, DP, DP]),
            "ref_sphere_analyze_scalar": (None, [P, DP, DP]),
            "ref_sphere_synthesize_scalar": (None, [P, DP, DP]),
            "ref_sphere_analyze_divergence": (None, [P, DP, DP, DP]),
            "ref_plane_new": (P, [I, I, D, D, D, D, D, D, D, D, I, CP, I]),
            "ref_plane_free": (None, [P]),
            "ref_plane_time": (D, [P]),
            "ref_plane_get": (None, [P, DP, DP, DP]),
            "ref_plane_set": (I, [P, DP, DP, DP, CP, I]),
            "ref_plane_perturb": (None, [P, D, C.c_ulonglong]),
            "ref_plane_step": (None, [P, D]),
            "ref_plane_run": (I, [P, D, D, CP, I]),
            "ref_plane_stable_dt": (D, [P, D]),
            "ref_plane_diagnostics": (None, [P, DP]),
            "ref_plane_probe": (D, [P, I, D, D]),
            "ref_plane_zeta_at_corner": (D, [P, I, I]),
            "ref_plane_harmonic": (I, [P, I, I, I, DP, CP, I]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _REF[variant] = lib
    return _REF[variant]


class OracleError(Exception):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


# ---------------------------------------------------------------------------------------------- sphere
class OracleSphere:
    """The oracle's sphere (cpp/sphere.hpp:27-121), spectral state as complex128 arrays of (T+1)^2."""

    def __init__(self, T: int, radius=6.37122e6, omega=7.292e-5, gravity=9.80616, diffusion=0.0, max_truncation=170):
        self.lib = oracle()
        self.h = self.lib.or_sphere_new(T, radius, omega, gravity, diffusion, max_truncation)
        if not self.h:
            raise OracleError(1, "truncation must be between 4 and 170")
        self.T = T
        self.radius, self.omega, self.gravity = radius, omega, gravity
        self.nlat = self.lib.or_sphere_nlat(self.h)
        self.nlon = self.lib.or_sphere_nlon(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.or_sphere_free(self.h)
            self.h = None

    @property
    def nspec(self):
        return (self.T + 1) ** 2

    @property
    def mu(self):
        return np.ctypeslib.as_array(self.lib.or_sphere_mu(self.h), (self.nlat,)).copy()

    @property
    def w(self):
        return np.ctypeslib.as_array(self.lib.or_sphere_w(self.h), (self.nlat,)).copy()

    def grid(self):
        return np.zeros((self.nlat, self.nlon))

    def set_state_grid(self, h, u, v):
        h, u, v = (np.ascontiguousarray(x, dtype=np.float64) for x in (h, u, v))
        self.lib.or_sphere_set_state_grid(self.h, _dp(h), _dp(u), _dp(v))
        return self

    def set_axis_tilt(self, alpha):
        self.lib.or_sphere_set_axis_tilt(self.h, alpha)
        return self

    def set_diffusion(self, nu):
        self.lib.or_sphere_set_diffusion(self.h, nu)
        return self

    def set_orography_grid(self, hs):
        hs = np.ascontiguousarray(hs, dtype=np.float64)
        self.lib.or_sphere_set_orography_grid(self.h, _dp(hs))
        return self

    def set_tracer_grid(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        self.lib.or_sphere_set_tracer_grid(self.h, _dp(q))
        return self

    def set_advect_only(self, on=True):
        self.lib.or_sphere_set_advect_only(self.h, 1 if on else 0)
        return self

    def perturb(self, amp, seed, nmax):
        if self.lib.or_sphere_perturb(self.h, amp, seed, nmax):
            raise OracleError(1, "max_wave must be between 1 and the truncation")
        return self

    def add_mode(self, n, m, amp, depth):
        if self.lib.or_sphere_add_mode(self.h, n, m, amp, depth):
            raise OracleError(1, "mode (n, m) needs 0 <= m <= n <= truncation and n >= 1")
        return self

    def mark_reference(self):
        self.lib.or_sphere_mark_reference(self.h)
        return self

    def get_state(self, with_tracer=False):
        z, d, f, q = (np.zeros(self.nspec, np.complex128) for _ in range(4))
        v = lambda a: a.view(np.float64)
        self.lib.or_sphere_get_state(self.h, _dp(v(z)), _dp(v(d)), _dp(v(f)), _dp(v(q)) if with_tracer else None)
        return (z, d, f, q) if with_tracer else (z, d, f)

    def set_state(self, z, d, f, t=0.0):
        v = lambda a: np.ascontiguousarray(a, np.complex128).view(np.float64)
        zz, dd, ff = v(z), v(d), v(f)
        self.lib.or_sphere_set_state(self.h, _dp(zz), _dp(dd), _dp(ff), t)
        return self

    def step(self, dt):
        self.lib.or_sphere_step(self.h, dt)

    def run(self, seconds, dt=0.0):
        err = C.create_string_buffer(512)
        code = self.lib.or_sphere_run(self.h, seconds, dt, err, 512)
        if code:
            raise OracleError(code, err.value.decode())
        return self

    def stable_dt(self, safety=1.5):
        st = I(0)
        r = self.lib.or_sphere_stable_dt(self.h, safety, C.byref(st))
        if st.value:
            raise OracleError(2, "the height field must be positive to step the model")
        return r

    @property
    def time(self):
        return self.lib.or_sphere_time(self.h)

    def diagnostics(self):
        L = self.lib
        return {
            "mean_height": L.or_sphere_mean_height(self.h),
            "kinetic_energy": L.or_sphere_kinetic_energy(self.h),
            "potential_energy": L.or_sphere_potential_energy(self.h),
            "energy": L.or_sphere_energy(self.h),
            "enstrophy": L.or_sphere_potential_enstrophy(self.h),
            "max_wind": L.or_sphere_max_wind(self.h),
            "error_l2": L.or_sphere_height_error_l2(self.h),
            "error_linf": L.or_sphere_height_error_linf(self.h),
        }

    def spectrum(self):
        ke, pe = np.zeros(self.T + 1), np.zeros(self.T + 1)
        self.lib.or_sphere_spectrum(self.h, _dp(ke), _dp(pe))
        return ke, pe

    def _grid(self, fn):
        g = self.grid()
        fn(self.h, _dp(g))
        return g

    def grid_height(self):
        return self._grid(self.lib.or_sphere_grid_height)

    def grid_u(self):
        return self._grid(self.lib.or_sphere_grid_u)

    def grid_v(self):
        return self._grid(self.lib.or_sphere_grid_v)

    def grid_vorticity(self):
        return self._grid(self.lib.or_sphere_grid_vorticity)

    def grid_tracer(self):
        return self._grid(self.lib.or_sphere_grid_tracer)

    def analyze_scalar(self, grid):
        grid = np.ascontiguousarray(grid, np.float64)
        out = np.zeros(self.nspec, np.complex128)
        self.lib.or_sphere_analyze_scalar(self.h, _dp(grid), _dp(out.view(np.float64)))
        return out

    def synthesize_scalar(self, spec):
        spec = np.ascontiguousarray(spec, np.complex128)
        g = self.grid()
        self.lib.or_sphere_synthesize_scalar(self.h, _dp(spec.view(np.float64)), _dp(g))
        return g

    def analyze_divergence(self, A, B):
        A, B = (np.ascontiguousarray(x, np.float64) for x in (A, B))
        out = np.zeros(self.nspec, np.complex128)
        self.lib.or_sphere_analyze_divergence(self.h, _dp(A), _dp(B), _dp(out.view(np.float64)))
        return out

    def turbulence_grids(self, seed, mean_height=8000.0, max_wind=30.0, nforce=21):
        h, u, v = self.grid(), self.grid(), self.grid()
        self.lib.or_sphere_turbulence_grids(self.h, seed, mean_height, max_wind, nforce, _dp(h), _dp(u), _dp(v))
        return h, u, v


class RefSphere:
    """The reference's own Sphere (built from its sources) behind the same methods as OracleSphere."""

    def __init__(self, T: int, radius=6.37122e6, omega=7.292e-5, gravity=9.80616, diffusion=0.0, variant=""):
        self.lib = reference(variant)
        err = C.create_string_buffer(512)
        self.h = self.lib.ref_sphere_new(T, radius, omega, gravity, diffusion, err, 512)
        if not self.h:
            raise OracleError(1, err.value.decode())
        self.T = T
        self.nlat = self.lib.ref_sphere_nlat(self.h)
        self.nlon = self.lib.ref_sphere_nlon(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_sphere_free(self.h)
            self.h = None

    @property
    def nspec(self):
        return (self.T + 1) ** 2

    def grid(self):
        return np.zeros((self.nlat, self.nlon))

    def _chk(self, code, err):
        if code:
            raise OracleError(code, err.value.decode())

    def set_state_grid(self, h, u, v):
        h, u, v = (np.ascontiguousarray(x, dtype=np.float64) for x in (h, u, v))
        err = C.create_string_buffer(512)
        self._chk(self.lib.ref_sphere_set_state_grid(self.h, _dp(h), _dp(u), _dp(v), err, 512), err)
        return self

    def set_axis_tilt(self, alpha):
        self.lib.ref_sphere_set_axis_tilt(self.h, alpha)
        return self

    def set_diffusion(self, nu):
        self.lib.ref_sphere_set_diffusion(self.h, nu)
        return self

    def set_orography_grid(self, hs):
        hs = np.ascontiguousarray(hs, dtype=np.float64)
        err = C.create_string_buffer(512)
        self._chk(self.lib.ref_sphere_set_orography_grid(self.h, _dp(hs), err, 512), err)
        return self

    def set_tracer_grid(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        err = C.create_string_buffer(512)
        self._chk(self.lib.ref_sphere_set_tracer_grid(self.h, _dp(q), err, 512), err)
        return self

    def set_advect_only(self, on=True):
        self.lib.ref_sphere_set_advect_only(self.h, 1 if on else 0)
        return self

    def perturb(self, amp, seed, nmax):
        err = C.create_string_buffer(512)
        self._chk(self.lib.ref_sphere_perturb(self.h, amp, seed, nmax, err, 512), err)
        return self

    def add_mode(self, n, m, amp, depth):
        err = C.create_string_buffer(512)
        self._chk(self.lib.ref_sphere_add_mode(self.h, n, m, amp, depth, err, 512), err)
        return self

    def get_state(self, with_tracer=False):
        z, d, f, q = (np.zeros(self.nspec, np.complex128) for _ in range(4))
        v = lambda a: a.view(np.float64)
        self.lib.ref_sphere_get_state(self.h, _dp(v(z)), _dp(v(d)), _dp(v(f)), _dp(v(q)) if with_tracer else None)
        return (z, d, f, q) if with_tracer else (z, d, f)

    def set_state(self, z, d, f, t=0.0):
        v = lambda a: np.ascontiguousarray(a, np.complex128).view(np.float64)
        zz, dd, ff = v(z), v(d), v(f)
        self.lib.ref_sphere_set_state(self.h, _dp(zz), _dp(dd), _dp(ff), t)
        return self

    def step(self, dt):
        self.lib.ref_sphere_step(self.h, dt)

    def run(self, seconds, dt=0.0):
        err = C.create_string_buffer(512)
        self._chk(self.lib.ref_sphere_run(self.h, seconds, dt, err, 512), err)
        return self

    def stable_dt(self, safety=1.5):
        return self.lib.ref_sphere_stable_dt(self.h, safety)

    @property
    def time(self):
        return self.lib.ref_sphere_time(self.h)

    def diagnostics(self):
        out = np.zeros(8)
        self.lib.ref_sphere_diagnostics(self.h, _dp(out))
        keys = ["mean_height", "kinetic_energy", "potential_energy", "energy", "enstrophy", "max_wind", "error_l2", "error_linf"]
        return dict(zip(keys, out.tolist()))

    def spectrum(self):
        ke, pe = np.zeros(self.T + 1), np.zeros(self.T + 1)
        self.lib.ref_sphere_spectrum(self.h, _dp(ke), _dp(pe))
        return ke, pe

    def grids(self):
        h, u, v, z = (self.grid() for _ in range(4))
        self.lib.ref_sphere_grids(self.h, _dp(h), _dp(u), _dp(v), _dp(z))
        return h, u, v, z

    def analyze_scalar(self, grid):
        grid = np.ascontiguousarray(grid, np.float64)
        out = np.zeros(self.nspec, np.complex128)
        self.lib.ref_sphere_analyze_scalar(self.h, _dp(grid), _dp(out.view(np.float64)))
        return out

    def synthesize_scalar(self, spec):
        spec = np.ascontiguousarray(spec, np.complex128)
        g = self.grid()
        self.lib.ref_sphere_synthesize_scalar(self.h, _dp(spec.view(np.float64)), _dp(g))
        return g

    def analyze_divergence(self, A, B):
        A, B = (np.ascontiguousarray(x, np.float64) for x in (A, B))
        out = np.zeros(self.nspec, np.complex128)
        self.lib.ref_sphere_analyze_divergence(self.h, _dp(A), _dp(B), _dp(out.view(np.float64)))
        return out


# ---------------------------------------------------------------------------------------------- plane
PLANE_DEFAULTS = dict(gravity=9.81, depth=100.0, f0=0.0, beta=0.0, viscosity=0.0, drag=0.0, linear=False)


class OraclePlane:
    """The oracle's plane (cpp/plane.hpp:20-68); v has ny+1 rows."""

    def __init__(self, nx, ny, lx, ly, **kw):
        p = dict(PLANE_DEFAULTS, **kw)
        self.lib = oracle()
        self.h = self.lib.or_plane_new(nx, ny, lx, ly, p["gravity"], p["depth"], p["f0"], p["beta"], p["viscosity"],
                                       p["drag"], 1 if p["linear"] else 0)
        if not self.h:
            raise OracleError(1, "grid must be at least 4 x 4 and at most 8 million cells")
        self.nx, self.ny, self.params = nx, ny, p

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.or_plane_free(self.h)
            self.h = None

    def get(self):
        h, u, v = np.zeros((self.ny, self.nx)), np.zeros((self.ny, self.nx)), np.zeros((self.ny + 1, self.nx))
        self.lib.or_plane_get(self.h, _dp(h), _dp(u), _dp(v))
        return h, u, v

    def set(self, h, u, v):
        h, u, v = (np.ascontiguousarray(x, np.float64) for x in (h, u, v))
        self.lib.or_plane_set(self.h, _dp(h), _dp(u), _dp(v))
        return self

    def perturb(self, amp, seed):
        self.lib.or_plane_perturb(self.h, amp, seed)
        return self

    def step(self, dt):
        self.lib.or_plane_step(self.h, dt)

    def run(self, seconds, dt=0.0):
        err = C.create_string_buffer(512)
        code = self.lib.or_plane_run(self.h, seconds, dt, err, 512)
        if code:
            raise OracleError(code, err.value.decode())
        return self

    def stable_dt(self, safety=0.5):
        st = I(0)
        r = self.lib.or_plane_stable_dt(self.h, safety, C.byref(st))
        if st.value:
            raise OracleError(2, "the depth must be positive to step the model")
        return r

    @property
    def time(self):
        return self.lib.or_plane_time(self.h)

    def diagnostics(self):
        L = self.lib
        return {
            "mean_depth": L.or_plane_mean_depth(self.h),
            "energy": L.or_plane_energy(self.h),
            "max_speed": L.or_plane_max_speed(self.h),
            "pv_anomaly_rms": L.or_plane_pv_anomaly_rms(self.h),
        }

    def _harm(self, fn, *args):
        out = D(0.0)
        if fn(self.h, *args, C.byref(out)):
            raise OracleError(1, "zonal harmonic or row out of range")
        return out.value

    def h_at(self, x, y):
        return self.lib.or_plane_probe(self.h, 0, x, y)

    def u_at(self, x, y):
        return self.lib.or_plane_probe(self.h, 1, x, y)

    def v_at(self, x, y):
        return self.lib.or_plane_probe(self.h, 2, x, y)

    def zeta_at_corner(self, i, j):
        return self.lib.or_plane_zeta_at_corner(self.h, i, j)

    def zonal_amplitude(self, m, j):
        return self._harm(self.lib.or_plane_zonal_amplitude, m, j)

    def zonal_crest(self, m, j):
        return self._harm(self.lib.or_plane_zonal_crest, m, j)

    def v_zonal_crest(self, m, j):
        return self._harm(self.lib.or_plane_v_zonal_crest, m, j)

    def harmonic_energy(self, m):
        return self._harm(self.lib.or_plane_harmonic_energy, m)

    def jet_grids(self, u0=20.0, width=1.0e5, noise_rms=0.1, seed=1):
        h, u = np.zeros((self.ny, self.nx)), np.zeros((self.ny, self.nx))
        self.lib.or_plane_jet_grids(self.h, u0, width, noise_rms, seed, _dp(h), _dp(u))
        return h, u


class RefPlane:
    def __init__(self, nx, ny, lx, ly, variant="", **kw):
        p = dict(PLANE_DEFAULTS, **kw)
        self.lib = reference(variant)
        err = C.create_string_buffer(512)
        self.h = self.lib.ref_plane_new(nx, ny, lx, ly, p["gravity"], p["depth"], p["f0"], p["beta"], p["viscosity"],
                                        p["drag"], 1 if p["linear"] else 0, err, 512)
        if not self.h:
            raise OracleError(1, err.value.decode())
        self.nx, self.ny, self.params = nx, ny, p

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_plane_free(self.h)
            self.h = None

    def get(self):
        h, u, v = np.zeros((self.ny, self.nx)), np.zeros((self.ny, self.nx)), np.zeros((self.ny + 1, self.nx))
        self.lib.ref_plane_get(self.h, _dp(h), _dp(u), _dp(v))
        return h, u, v

    def set(self, h, u, v):
        h, u, v = (np.ascontiguousarray(x, np.float64) for x in (h, u, v))
        err = C.create_string_buffer(512)
        code = self.lib.ref_plane_set(self.h, _dp(h), _dp(u), _dp(v), err, 512)
        if code:
            raise OracleError(code, err.value.decode())
        return self

    def perturb(self, amp, seed):
        self.lib.ref_plane_perturb(self.h, amp, seed)
        return self

    def step(self, dt):
        self.lib.ref_plane_step(self.h, dt)

    def run(self, seconds, dt=0.0):
        err = C.create_string_buffer(512)
        code = self.lib.ref_plane_run(self.h, seconds, dt, err, 512)
        if code:
            raise OracleError(code, err.value.decode())
        return self

    def stable_dt(self, safety=0.5):
        return self.lib.ref_plane_stable_dt(self.h, safety)

    @property
    def time(self):
        return self.lib.ref_plane_time(self.h)

    def diagnostics(self):
        out = np.zeros(4)
        self.lib.ref_plane_diagnostics(self.h, _dp(out))
        return dict(zip(["mean_depth", "energy", "max_speed", "pv_anomaly_rms"], out.tolist()))

    def _harm(self, which, m, j=0):
        out = D(0.0)
        err = C.create_string_buffer(512)
        code = self.lib.ref_plane_harmonic(self.h, which, m, j, C.byref(out), err, 512)
        if code:
            raise OracleError(code, err.value.decode())
        return out.value

    def h_at(self, x, y):
        return self.lib.ref_plane_probe(self.h, 0, x, y)

    def u_at(self, x, y):
        return self.lib.ref_plane_probe(self.h, 1, x, y)

    def v_at(self, x, y):
        return self.lib.ref_plane_probe(self.h, 2, x, y)

    def zeta_at_corner(self, i, j):
        return self.lib.ref_plane_zeta_at_corner(self.h, i, j)

    def zonal_amplitude(self, m, j):
        return self._harm(0, m, j)

    def zonal_crest(self, m, j):
        return self._harm(1, m, j)

    def v_zonal_crest(self, m, j):
        return self._harm(2, m, j)

    def harmonic_energy(self, m):
        return self._harm(3, m)


def plane_fields_grids(nx, ny, lx, ly, depth, h, u, v):
    """Grids of the wx builder's Plane.fields(h, u, v) (cpp/main.cpp:409-431) from callables f(x, y): h = depth +
    h(x, y) at cell centres, u at the west faces (i dx, y_j), v at the interior south faces (x_i, j dy), walls 0."""
    dx, dy = lx / nx, ly / ny
    xc, yc = (np.arange(nx) + 0.5) * dx, (np.arange(ny) + 0.5) * dy
    hh = depth + np.broadcast_to(h(xc[None, :], yc[:, None]), (ny, nx))
    uu = np.broadcast_to(u((np.arange(nx) * dx)[None, :], yc[:, None]), (ny, nx))
    vv = np.zeros((ny + 1, nx))
    vv[1:ny] = np.broadcast_to(v(xc[None, :], (np.arange(1, ny) * dy)[:, None]), (ny - 1, nx))
    return np.ascontiguousarray(hh, np.float64), np.ascontiguousarray(uu, np.float64), vv
