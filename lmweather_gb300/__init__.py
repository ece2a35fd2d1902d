"""lmweather-gb300: GB300-native (sm_103a) rotating shallow-water time stepping.

Python mirror of lmweather's numerical-core interface (lmweather::Sphere, cpp/sphere.hpp:27-121, and
lmweather::Plane, cpp/plane.hpp:20-68) over the engine's C ABI (include/lmweather_gb300.h). Method names and
argument meanings follow the reference; its std::invalid_argument surfaces as ValueError and its
std::runtime_error as RuntimeError, with the reference's message texts. All state lives on the GPU; there is no
CPU fallback: without the compiled library (lmweather_gb300/_lib/liblmw_gb300.so) every constructor raises.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

__all__ = ["Sphere", "Plane", "Ensemble", "Mlp", "Surrogate", "gemm_bf16", "DeviceError", "load_library", "library_path", "launch_count", "FP64", "FP32", "SPLIT_BF16"]

FP64, FP32, SPLIT_BF16 = 0, 1, 2
_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def library_path() -> str:
    return os.path.join(_HERE, "_lib", "liblmw_gb300.so")


class DeviceError(RuntimeError):
    """A CUDA failure inside the engine (status LMW_DEVICE_ERROR)."""


_D, _I, _P, _SZ, _U64 = C.c_double, C.c_int, C.c_void_p, C.c_size_t, C.c_uint64
_DP = C.POINTER(C.c_double)
_PP = C.POINTER(C.c_void_p)
_IP = C.POINTER(C.c_int)
_FP = C.POINTER(C.c_float)

_SIGS = {
    "lmw_last_error": (C.c_char_p, []),
    "lmw_version": (C.c_char_p, []),
    "lmw_conversion_selftest": (_I, [C.POINTER(C.c_uint32), _I, C.POINTER(C.c_uint64), _I, _IP]),
    "lmw_division_selftest": (_I, [C.POINTER(C.c_uint64), _I, C.POINTER(C.c_double), _I, C.POINTER(C.c_longlong)]),
    "lmw_wait_selftest": (_I, [_I, _IP, _IP]),
    "lmw_sphere_inject_split_error": (_I, [_P, _I]),
    "lmw_sphere_set_split_form": (_I, [_P, _I]),
    "lmw_ensemble_set_split_form": (_I, [_P, _I]),
    "lmw_launch_count": (C.c_uint64, []),
    "lmw_alloc_count": (C.c_uint64, []),
    "lmw_profiler_range": (_I, [_I]),
    "lmw_sphere_create": (_I, [_I, _D, _D, _D, _D, _PP]),
    "lmw_sphere_create_ex": (_I, [_I, _D, _D, _D, _D, _I, _I, _I, _PP]),
    "lmw_sphere_create_split": (_I, [_I, _D, _D, _D, _D, _I, _I, _I, _PP]),
    "lmw_sphere_destroy": (_I, [_P]),
    "lmw_sphere_dims": (_I, [_P, _IP, _IP, _IP, _IP]),
    "lmw_sphere_gauss": (_I, [_P, _DP, _DP]),
    "lmw_sphere_time": (_I, [_P, _I, _DP]),
    "lmw_sphere_analyze_scalar": (_I, [_P, _DP, _SZ, _DP]),
    "lmw_sphere_synthesize_scalar": (_I, [_P, _DP, _DP, _SZ]),
    "lmw_sphere_analyze_divergence": (_I, [_P, _DP, _DP, _SZ, _DP]),
    "lmw_sphere_set_state_grid": (_I, [_P, _I, _DP, _DP, _DP, _SZ]),
    "lmw_sphere_set_axis_tilt": (_I, [_P, _I, _D]),
    "lmw_sphere_set_omega": (_I, [_P, _I, _D]),
    "lmw_sphere_set_diffusion": (_I, [_P, _D]),
    "lmw_sphere_set_orography_grid": (_I, [_P, _I, _DP, _SZ]),
    "lmw_sphere_add_mode": (_I, [_P, _I, _I, _I, _D, _D]),
    "lmw_sphere_perturb": (_I, [_P, _I, _D, _U64, _I]),
    "lmw_sphere_mark_reference": (_I, [_P, _I]),
    "lmw_sphere_turbulence": (_I, [_P, _I, _U64, _D, _D, _I]),
    "lmw_sphere_get_state": (_I, [_P, _I, _DP, _DP, _DP]),
    "lmw_sphere_set_state": (_I, [_P, _I, _DP, _DP, _DP, _D]),
    "lmw_sphere_step": (_I, [_P, _D]),
    "lmw_sphere_run": (_I, [_P, _D, _D]),
    "lmw_sphere_stable_dt": (_I, [_P, _I, _D, _DP]),
    "lmw_sphere_diagnostics": (_I, [_P, _I, _DP]),
    "lmw_sphere_grid": (_I, [_P, _I, _I, _DP, _SZ]),
    "lmw_sphere_spectrum": (_I, [_P, _I, _DP, _DP]),
    "lmw_plane_create": (_I, [_I, _I, _D, _D, _D, _D, _D, _D, _D, _D, _I, _PP]),
    "lmw_plane_destroy": (_I, [_P]),
    "lmw_plane_set_params": (_I, [_P, _D, _D, _D, _D, _D, _D, _I]),
    "lmw_plane_reset": (_I, [_P]),
    "lmw_plane_set_h": (_I, [_P, _DP, _SZ]),
    "lmw_plane_set_u": (_I, [_P, _DP, _SZ]),
    "lmw_plane_set_v": (_I, [_P, _DP, _SZ]),
    "lmw_plane_get": (_I, [_P, _DP, _DP, _DP]),
    "lmw_plane_perturb": (_I, [_P, _D, _U64]),
    "lmw_plane_jet": (_I, [_P, _D, _D, _D, _U64]),
    "lmw_plane_step": (_I, [_P, _D]),
    "lmw_plane_run": (_I, [_P, _D, _D]),
    "lmw_plane_stable_dt": (_I, [_P, _D, _DP]),
    "lmw_plane_time": (_I, [_P, _DP]),
    "lmw_plane_diagnostics": (_I, [_P, _DP]),
    "lmw_plane_probe": (_I, [_P, _I, _D, _D, _DP]),
    "lmw_plane_zeta_at_corner": (_I, [_P, _I, _I, _DP]),
    "lmw_plane_zonal_amplitude": (_I, [_P, _I, _I, _DP]),
    "lmw_plane_zonal_crest": (_I, [_P, _I, _I, _DP]),
    "lmw_plane_v_zonal_crest": (_I, [_P, _I, _I, _DP]),
    "lmw_plane_harmonic_energy": (_I, [_P, _I, _DP]),
    "lmw_plane_save_csv": (_I, [_P, C.c_char_p]),
    "lmw_plane_save_row": (_I, [_P, _I, C.c_char_p]),
    "lmw_plane_save_column": (_I, [_P, _I, C.c_char_p]),
    "lmw_sphere_save_csv": (_I, [_P, _I, C.c_char_p]),
    "lmw_sphere_save_zonal_mean": (_I, [_P, _I, C.c_char_p]),
    "lmw_sphere_save_spectrum": (_I, [_P, _I, C.c_char_p]),
    "lmw_ensemble_create": (_I, [_I, _IP, C.POINTER(C.c_uint64), _DP, _DP, _D, _D, _D, _I, _I, _PP]),
    "lmw_ensemble_destroy": (_I, [_P]),
    "lmw_ensemble_run": (_I, [_P, _D]),
    "lmw_ensemble_groups": (_I, [_P, _IP, _IP, _IP, _DP, C.POINTER(C.c_int64)]),
    "lmw_ensemble_member_state": (_I, [_P, _I, _DP, _DP, _DP]),
    "lmw_ensemble_member_set_state": (_I, [_P, _I, _DP, _DP, _DP]),
    "lmw_ensemble_get_states": (_I, [_P, _DP, _DP, _DP]),
    "lmw_ensemble_set_states": (_I, [_P, _DP, _DP, _DP]),
    "lmw_ensemble_member_diagnostics": (_I, [_P, _I, _DP]),
    "lmw_ensemble_member_grid": (_I, [_P, _I, _I, _DP, _SZ]),
    "lmw_sphere_split_plan": (_I, [_P, _IP]),
    "lmw_sphere_set_split_plan": (_I, [_P, _IP]),
    "lmw_sphere_set_tracer_grid": (_I, [_P, _I, _DP, _SZ]),
    "lmw_sphere_probe": (_I, [_P, _I, _I, _D, _D, _DP]),
    "lmw_sphere_mode_coefficient": (_I, [_P, _I, _I, _I, _I, _DP]),
    "lmw_sphere_wave_crest": (_I, [_P, _I, _I, _D, _DP]),
    "lmw_sphere_set_advect_only": (_I, [_P, _I]),
    "lmw_sphere_tracer_state": (_I, [_P, _I, _DP]),
    "lmw_sphere_set_tracer_state": (_I, [_P, _I, _DP]),
    "lmw_sphere_tracer_grid": (_I, [_P, _I, _DP, _SZ]),
    "lmw_sphere_tracer_diagnostics": (_I, [_P, _I, _DP]),
    "lmw_ensemble_split_plan": (_I, [_P, _I, _IP]),
    "lmw_mlp_create": (_I, [_I, _I, _I, _I, _U64, _D, _PP]),
    "lmw_mlp_destroy": (_I, [_P]),
    "lmw_mlp_set_layer": (_I, [_P, _I, _FP, _FP]),
    "lmw_mlp_get_layer": (_I, [_P, _I, _FP, _FP]),
    "lmw_mlp_forward": (_I, [_P, _FP, _I, _FP]),
    "lmw_mlp_backward": (_I, [_P, _FP, _FP, _FP, _I, _DP]),
    "lmw_mlp_get_grad": (_I, [_P, _I, _FP, _FP]),
    "lmw_mlp_adam": (_I, [_P, _D, _D, _D, _D]),
    "lmw_mlp_time": (_I, [_P, _I, _I, _DP, _DP]),
    "lmw_gemm_bf16": (_I, [_FP, _FP, _I, _I, _I, _FP]),
    "lmw_surrogate_create": (_I, [_I, _I, _U64, _D, _D, _D, _D, _D, _PP]),
    "lmw_surrogate_destroy": (_I, [_P]),
    "lmw_surrogate_dims": (_I, [_P, _IP]),
    "lmw_surrogate_generate": (_I, [_P, _I, _I, _U64, _D, _D, _I, _DP]),
    "lmw_surrogate_generate_drifted": (_I, [_P, _I, _I, _U64, _D, _D, _I, _DP]),
    "lmw_surrogate_fit": (_I, [_P, _I, _I, _D, _D, _D, _U64, _I, _DP]),
    "lmw_surrogate_evaluate": (_I, [_P, _I, _I, _DP, _DP]),
    "lmw_surrogate_advance": (_I, [_P, _I, _DP]),
    "lmw_surrogate_rollout": (_I, [_P, _I, _U64, _D, _D, _I, _I, _D, _I, _I, _DP, _DP, _DP]),
    "lmw_surrogate_time": (_I, [_P, _I, _I, _DP, _DP]),
    "lmw_surrogate_reset": (_I, [_P, _U64]),
    "lmw_surrogate_set_clip": (_I, [_P, _D]),
    "lmw_surrogate_set_augment": (_I, [_P, _I]),
    "lmw_surrogate_set_averaging": (_I, [_P, _D]),
    "lmw_surrogate_set_symmetry_average": (_I, [_P, _I]),
    "lmw_surrogate_set_kinetic_weight": (_I, [_P, _D]),
    "lmw_surrogate_set_takeover": (_I, [_P, _I]),
    "lmw_surrogate_history": (_I, [_P, _I, _DP, _DP, _IP]),
}


def load_library() -> C.CDLL:
    """Load the engine library (built by lmweather_gb300.build). Raises if it is missing: no fallback."""
    global _LIB
    if _LIB is None:
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(f"lmweather_gb300 CUDA library not built ({path}); run python -m lmweather_gb300.build")
        lib = C.CDLL(path)
        for name, (res, args) in _SIGS.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _LIB = lib
    return _LIB


def launch_count() -> int:
    return int(load_library().lmw_launch_count())


def profiler_range(on: bool) -> None:
    """Start (True) or stop (False) the region a profiler run with --profile-from-start off captures."""
    _check(load_library().lmw_profiler_range(1 if on else 0))


def alloc_count() -> int:
    """Device and pinned-host allocations the library has made so far (all threads)."""
    return int(load_library().lmw_alloc_count())


def _check(code: int) -> None:
    if code == 0:
        return
    msg = load_library().lmw_last_error().decode()
    if code == 1:
        raise ValueError(msg)
    if code == 3:
        raise DeviceError(msg)
    raise RuntimeError(msg)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_DP)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _c128(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex128)


class Sphere:
    """GPU spectral-transform sphere (cpp/sphere.hpp:27-121). Spectra use the reference layout: (T+1)^2 complex
    values per field at m*(T+1)+n. `members` > 1 holds an ensemble of states stepped together; per-member calls
    take `member=`."""

    def __init__(self, truncation: int, radius=6.37122e6, omega=7.292e-5, gravity=9.80616, diffusion=0.0,
                 precision: int = FP64, members: int = 1, max_truncation: int = 170, split_terms: int = 3):
        self._lib = load_library()
        h = C.c_void_p()
        if precision == SPLIT_BF16:
            _check(self._lib.lmw_sphere_create_split(truncation, radius, omega, gravity, diffusion, members, max_truncation,
                                                     split_terms, C.byref(h)))
        else:
            _check(self._lib.lmw_sphere_create_ex(truncation, radius, omega, gravity, diffusion, precision, members,
                                                  max_truncation, C.byref(h)))
        self._h = h
        T, nlat, nlon, B = _I(), _I(), _I(), _I()
        _check(self._lib.lmw_sphere_dims(h, C.byref(T), C.byref(nlat), C.byref(nlon), C.byref(B)))
        self.T, self.nlat, self.nlon, self.members = T.value, nlat.value, nlon.value, B.value
        self.radius, self.omega, self.gravity = radius, omega, gravity
        self.precision = precision

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lmw_sphere_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ geometry
    def truncation(self) -> int:
        return self.T

    @property
    def nspec(self) -> int:
        return (self.T + 1) ** 2

    @property
    def ngrid(self) -> int:
        return self.nlat * self.nlon

    def gauss(self):
        mu, w = np.zeros(self.nlat), np.zeros(self.nlat)
        _check(self._lib.lmw_sphere_gauss(self._h, _dp(mu), _dp(w)))
        return mu, w

    # the reference's transform test hooks (cpp/sphere.hpp:96-99)
    def analyze_scalar(self, grid):
        g = np.ascontiguousarray(grid, dtype=np.float64).reshape(-1)
        spec = np.zeros(self.nspec, dtype=np.complex128)
        _check(self._lib.lmw_sphere_analyze_scalar(self._h, _dp(g), g.size, _dp(spec)))
        return spec

    def synthesize_scalar(self, spec):
        sp = np.ascontiguousarray(spec, dtype=np.complex128).reshape(-1)
        if sp.size != self.nspec:
            raise ValueError("spectrum size mismatch")
        grid = np.zeros((self.nlat, self.nlon))
        _check(self._lib.lmw_sphere_synthesize_scalar(self._h, _dp(sp), _dp(grid), grid.size))
        return grid

    def analyze_divergence(self, A, B):
        a = np.ascontiguousarray(A, dtype=np.float64).reshape(-1)
        b = np.ascontiguousarray(B, dtype=np.float64).reshape(-1)
        if a.size != b.size:
            raise ValueError("grid size mismatch")
        spec = np.zeros(self.nspec, dtype=np.complex128)
        _check(self._lib.lmw_sphere_analyze_divergence(self._h, _dp(a), _dp(b), a.size, _dp(spec)))
        return spec

    def time(self, member: int = 0) -> float:
        t = _D()
        _check(self._lib.lmw_sphere_time(self._h, member, C.byref(t)))
        return t.value

    # ------------------------------------------------------------ state
    def set_state_grid(self, h, u, v, member: int = 0):
        h, u, v = _f64(h), _f64(u), _f64(v)
        if not (h.size == u.size == v.size):
            raise ValueError("grid size mismatch")
        _check(self._lib.lmw_sphere_set_state_grid(self._h, member, _dp(h), _dp(u), _dp(v), h.size))
        return self

    def set_axis_tilt(self, alpha: float, member: int = 0):
        _check(self._lib.lmw_sphere_set_axis_tilt(self._h, member, alpha))
        return self

    def set_omega(self, omega: float, member: int = 0):
        _check(self._lib.lmw_sphere_set_omega(self._h, member, omega))
        return self

    def set_diffusion(self, nu4: float):
        _check(self._lib.lmw_sphere_set_diffusion(self._h, nu4))
        return self

    def set_orography_grid(self, hs, member: int = 0):
        hs = _f64(hs)
        _check(self._lib.lmw_sphere_set_orography_grid(self._h, member, _dp(hs), hs.size))
        return self

    def add_mode(self, n: int, m: int, amplitude: float, mean_depth: float, member: int = 0):
        _check(self._lib.lmw_sphere_add_mode(self._h, member, n, m, amplitude, mean_depth))
        return self

    def perturb(self, amplitude: float, seed: int, max_wave: int, member: int = 0):
        _check(self._lib.lmw_sphere_perturb(self._h, member, amplitude, seed, max_wave))
        return self

    def mark_reference(self, member: int = 0):
        _check(self._lib.lmw_sphere_mark_reference(self._h, member))
        return self

    def turbulence(self, seed: int, mean_height=8000.0, max_wind=30.0, nforce=21, member: int = 0):
        _check(self._lib.lmw_sphere_turbulence(self._h, member, seed, mean_height, max_wind, nforce))
        return self

    # ---- point probes (cpp/sphere.cpp:287-299, 592-652): exact synthesis at (lat, lon) in radians
    def _probe(self, which, lat, lon, member):
        out = _D()
        _check(self._lib.lmw_sphere_probe(self._h, member, which, lat, lon, C.byref(out)))
        return out.value

    def height_at(self, lat: float, lon: float, member: int = 0) -> float:
        return self._probe(0, lat, lon, member)

    def wind_at(self, lat: float, lon: float, zonal: bool, member: int = 0) -> float:
        return self._probe(1 if zonal else 2, lat, lon, member)

    def vorticity_at(self, lat: float, lon: float, member: int = 0) -> float:
        return self._probe(3, lat, lon, member)

    def tracer_at(self, lat: float, lon: float, member: int = 0) -> float:
        return self._probe(4, lat, lon, member)

    def mode_coefficient(self, n: int, m: int, imag: bool = False, member: int = 0) -> float:
        out = _D()
        _check(self._lib.lmw_sphere_mode_coefficient(self._h, member, n, m, 1 if imag else 0, C.byref(out)))
        return out.value

    def wave_crest(self, m: int, lat: float, member: int = 0) -> float:
        out = _D()
        _check(self._lib.lmw_sphere_wave_crest(self._h, member, m, lat, C.byref(out)))
        return out.value

    # ---- passive tracer (cpp/sphere.cpp:250-300), FP64 precision
    def set_tracer_grid(self, q, member: int = 0):
        q = _f64(q)
        _check(self._lib.lmw_sphere_set_tracer_grid(self._h, member, _dp(q), q.size))
        return self

    def set_advect_only(self, on: bool = True):
        _check(self._lib.lmw_sphere_set_advect_only(self._h, 1 if on else 0))
        return self

    def tracer_state(self, member: int = 0):
        q = np.zeros(self.nspec, np.complex128)
        _check(self._lib.lmw_sphere_tracer_state(self._h, member, _dp(q.view(np.float64))))
        return q

    def grid_tracer(self, member: int = 0):
        out = np.zeros((self.nlat, self.nlon))
        _check(self._lib.lmw_sphere_tracer_grid(self._h, member, _dp(out), out.size))
        return out

    def tracer_diagnostics(self, member: int = 0) -> dict:
        out = np.zeros(6)
        _check(self._lib.lmw_sphere_tracer_diagnostics(self._h, member, _dp(out)))
        return dict(zip(("tracer_mean", "tracer_mass", "tracer_error_l2", "tracer_error_linf", "tracer_min", "tracer_max"),
                        out.tolist()))

    def split_plan(self) -> dict:
        """The autotuned launch plan of the split path (zeros in the other precisions)."""
        out = np.zeros(12, np.int32)
        _check(self._lib.lmw_sphere_split_plan(self._h, out.ctypes.data_as(_IP)))
        return dict(zip(self._PLAN_KEYS, out.tolist()))

    _PLAN_KEYS = ("lat_pairs_per_grid_cta", "fft_stages_per_pass", "synthesis_stages", "analysis_stages", "analysis_both_parities",
                  "analysis_ctas", "grid_writes_operands", "analysis_ctas_per_sm", "synthesis_latitude_slices",
                  "analysis_warp_specialised", "grid_fixed_length", "synthesis_warp_specialised")

    def set_split_plan(self, **plan) -> None:
        """Replace entries of the autotuned launch plan (keys as split_plan returns them)."""
        cur = self.split_plan()
        unknown = set(plan) - set(cur)
        if unknown:
            raise ValueError(f"unknown plan entries: {sorted(unknown)}")
        cur.update(plan)
        arr = np.array([cur[k] for k in self._PLAN_KEYS], np.int32)
        _check(self._lib.lmw_sphere_set_split_plan(self._h, arr.ctypes.data_as(_IP)))

    def set_split_form(self, linear_exact: bool) -> None:
        """Split path: True (the default) adds the linear terms of the tendencies in spectral space (FP32, outside the
        BF16 pieces) and sends only the nonlinear products through the BF16 pieces; False sends every term through
        the BF16 GEMMs."""
        _check(self._lib.lmw_sphere_set_split_form(self._h, 1 if linear_exact else 0))

    def get_state(self, member: int = 0):
        z, d, f = (np.zeros(self.nspec, np.complex128) for _ in range(3))
        _check(self._lib.lmw_sphere_get_state(self._h, member, _dp(z.view(np.float64)), _dp(d.view(np.float64)),
                                              _dp(f.view(np.float64))))
        return z, d, f

    def set_state(self, zeta, delta, phi, time: float = 0.0, member: int = 0):
        z, d, f = _c128(zeta), _c128(delta), _c128(phi)
        if not (z.size == d.size == f.size == self.nspec):
            raise ValueError("spectral state size mismatch")
        _check(self._lib.lmw_sphere_set_state(self._h, member, _dp(z.view(np.float64)), _dp(d.view(np.float64)),
                                              _dp(f.view(np.float64)), time))
        return self

    # ------------------------------------------------------------ time stepping
    def step(self, dt: float):
        _check(self._lib.lmw_sphere_step(self._h, dt))
        return self

    def run(self, seconds: float, dt: float = 0.0):
        _check(self._lib.lmw_sphere_run(self._h, seconds, dt))
        return self

    def stable_dt(self, safety: float = 1.5, member: int = 0) -> float:
        out = _D()
        _check(self._lib.lmw_sphere_stable_dt(self._h, member, safety, C.byref(out)))
        return out.value

    # ------------------------------------------------------------ diagnostics
    _DIAG = ("mean_height", "kinetic_energy", "potential_energy", "energy", "enstrophy", "max_wind", "error_l2", "error_linf")

    def diagnostics(self, member: int = 0) -> dict:
        out = np.zeros(8)
        _check(self._lib.lmw_sphere_diagnostics(self._h, member, _dp(out)))
        return dict(zip(self._DIAG, out.tolist()))

    def mean_height(self, member: int = 0) -> float:
        return self.diagnostics(member)["mean_height"]

    def energy(self, member: int = 0) -> float:
        return self.diagnostics(member)["energy"]

    def kinetic_energy(self, member: int = 0) -> float:
        return self.diagnostics(member)["kinetic_energy"]

    def potential_energy(self, member: int = 0) -> float:
        return self.diagnostics(member)["potential_energy"]

    def potential_enstrophy(self, member: int = 0) -> float:
        return self.diagnostics(member)["enstrophy"]

    def max_wind(self, member: int = 0) -> float:
        return self.diagnostics(member)["max_wind"]

    def height_error_l2(self, member: int = 0) -> float:
        return self.diagnostics(member)["error_l2"]

    def height_error_linf(self, member: int = 0) -> float:
        return self.diagnostics(member)["error_linf"]

    def _grid(self, which: int, member: int) -> np.ndarray:
        g = np.zeros((self.nlat, self.nlon))
        _check(self._lib.lmw_sphere_grid(self._h, member, which, _dp(g), g.size))
        return g

    def grid_height(self, member: int = 0):
        return self._grid(0, member)

    def grid_u(self, member: int = 0):
        return self._grid(1, member)

    def grid_v(self, member: int = 0):
        return self._grid(2, member)

    def grid_vorticity(self, member: int = 0):
        return self._grid(3, member)

    def spectrum(self, member: int = 0):
        ke, pe = np.zeros(self.T + 1), np.zeros(self.T + 1)
        _check(self._lib.lmw_sphere_spectrum(self._h, member, _dp(ke), _dp(pe)))
        return ke, pe

    # the wx layer's text files (cpp/main.cpp:328-335, 357-384)
    def save_csv(self, path: str, member: int = 0):
        _check(self._lib.lmw_sphere_save_csv(self._h, member, os.fsencode(path)))

    def save_zonal_mean(self, path: str, member: int = 0):
        _check(self._lib.lmw_sphere_save_zonal_mean(self._h, member, os.fsencode(path)))

    def save_spectrum(self, path: str, member: int = 0):
        _check(self._lib.lmw_sphere_save_spectrum(self._h, member, os.fsencode(path)))


class Plane:
    """GPU C-grid beta-plane channel (cpp/plane.hpp:20-68)."""

    def __init__(self, nx: int, ny: int, lx: float, ly: float, gravity=9.81, depth=100.0, f0=0.0, beta=0.0,
                 viscosity=0.0, drag=0.0, linear=False):
        self._lib = load_library()
        h = C.c_void_p()
        _check(self._lib.lmw_plane_create(nx, ny, lx, ly, gravity, depth, f0, beta, viscosity, drag, 1 if linear else 0,
                                          C.byref(h)))
        self._h = h
        self.nx, self.ny, self.lx, self.ly = nx, ny, lx, ly
        self.params = dict(gravity=gravity, depth=depth, f0=f0, beta=beta, viscosity=viscosity, drag=drag, linear=linear)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lmw_plane_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def dx(self) -> float:
        return self.lx / self.nx

    def dy(self) -> float:
        return self.ly / self.ny

    def set_params(self, **kw):
        self.params.update(kw)
        p = self.params
        _check(self._lib.lmw_plane_set_params(self._h, p["gravity"], p["depth"], p["f0"], p["beta"], p["viscosity"],
                                              p["drag"], 1 if p["linear"] else 0))
        return self

    def reset(self):
        _check(self._lib.lmw_plane_reset(self._h))
        return self

    def set_h_from_grid(self, g):
        g = _f64(g)
        _check(self._lib.lmw_plane_set_h(self._h, _dp(g), g.size))
        return self

    def set_u_from_grid(self, g):
        g = _f64(g)
        _check(self._lib.lmw_plane_set_u(self._h, _dp(g), g.size))
        return self

    def set_v_from_grid(self, g):
        g = _f64(g)
        _check(self._lib.lmw_plane_set_v(self._h, _dp(g), g.size))
        return self

    def get(self):
        h, u, v = np.zeros((self.ny, self.nx)), np.zeros((self.ny, self.nx)), np.zeros((self.ny + 1, self.nx))
        _check(self._lib.lmw_plane_get(self._h, _dp(h), _dp(u), _dp(v)))
        return h, u, v

    def perturb(self, amplitude: float, seed: int):
        _check(self._lib.lmw_plane_perturb(self._h, amplitude, seed))
        return self

    def jet(self, u0=20.0, width=1.0e5, noise_rms=0.1, seed=1):
        _check(self._lib.lmw_plane_jet(self._h, u0, width, noise_rms, seed))
        return self

    def step(self, dt: float):
        _check(self._lib.lmw_plane_step(self._h, dt))
        return self

    def run(self, seconds: float, dt: float = 0.0):
        _check(self._lib.lmw_plane_run(self._h, seconds, dt))
        return self

    def stable_dt(self, safety: float = 0.5) -> float:
        out = _D()
        _check(self._lib.lmw_plane_stable_dt(self._h, safety, C.byref(out)))
        return out.value

    def time(self) -> float:
        out = _D()
        _check(self._lib.lmw_plane_time(self._h, C.byref(out)))
        return out.value

    _DIAG = ("mean_depth", "energy", "max_speed", "pv_anomaly_rms")

    def diagnostics(self) -> dict:
        out = np.zeros(4)
        _check(self._lib.lmw_plane_diagnostics(self._h, _dp(out)))
        return dict(zip(self._DIAG, out.tolist()))

    def mean_depth(self) -> float:
        return self.diagnostics()["mean_depth"]

    def energy(self) -> float:
        return self.diagnostics()["energy"]

    def max_speed(self) -> float:
        return self.diagnostics()["max_speed"]

    def pv_anomaly_rms(self) -> float:
        return self.diagnostics()["pv_anomaly_rms"]

    # the wx.* derived quantities (cpp/main.cpp:445-450)
    def wave_speed(self) -> float:
        return math.sqrt(self.params["gravity"] * self.params["depth"])

    def rossby_radius(self) -> float:
        if self.params["f0"] == 0:
            raise ValueError("Plane.rossby_radius: f0 is zero")
        return math.sqrt(self.params["gravity"] * self.params["depth"]) / abs(self.params["f0"])

    def fields(self, h, u, v):
        """The wx builder's fields(h, u, v) (cpp/main.cpp:409-431) with Python callables f(x, y) of numpy arrays:
        h = depth + h(x, y) at cell centres, u at the west faces, v at the interior south faces (the walls zero)."""
        nx, ny, dx, dy = self.nx, self.ny, self.dx(), self.dy()
        xc, yc = (np.arange(nx) + 0.5) * dx, (np.arange(ny) + 0.5) * dy
        hh = self.params["depth"] + np.broadcast_to(h(xc[None, :], yc[:, None]), (ny, nx))
        uu = np.broadcast_to(u((np.arange(nx) * dx)[None, :], yc[:, None]), (ny, nx))
        vv = np.zeros((ny + 1, nx))
        vv[1:ny] = np.broadcast_to(v(xc[None, :], (np.arange(1, ny) * dy)[:, None]), (ny - 1, nx))
        for name, g in (("height", hh), ("u", uu), ("v", vv)):
            if not np.all(np.isfinite(g)):
                raise ValueError(f"Plane.fields: the {name} expression is not finite")
        return self.set_h_from_grid(hh).set_u_from_grid(uu).set_v_from_grid(vv)

    def _scalar(self, fn, *args) -> float:
        out = _D()
        _check(fn(self._h, *args, C.byref(out)))
        return out.value

    def h_at(self, x: float, y: float) -> float:
        return self._scalar(self._lib.lmw_plane_probe, 0, x, y)

    def u_at(self, x: float, y: float) -> float:
        return self._scalar(self._lib.lmw_plane_probe, 1, x, y)

    def v_at(self, x: float, y: float) -> float:
        return self._scalar(self._lib.lmw_plane_probe, 2, x, y)

    def zeta_at_corner(self, i: int, j: int) -> float:
        return self._scalar(self._lib.lmw_plane_zeta_at_corner, i, j)

    def zonal_amplitude(self, m: int, j: int) -> float:
        return self._scalar(self._lib.lmw_plane_zonal_amplitude, m, j)

    def zonal_crest(self, m: int, j: int) -> float:
        return self._scalar(self._lib.lmw_plane_zonal_crest, m, j)

    def v_zonal_crest(self, m: int, j: int) -> float:
        return self._scalar(self._lib.lmw_plane_v_zonal_crest, m, j)

    def harmonic_energy(self, m: int) -> float:
        return self._scalar(self._lib.lmw_plane_harmonic_energy, m)

    # the wx layer's text files (cpp/main.cpp:464-494)
    def save_csv(self, path: str):
        _check(self._lib.lmw_plane_save_csv(self._h, os.fsencode(path)))

    def save_row(self, j: int, path: str):
        _check(self._lib.lmw_plane_save_row(self._h, j, os.fsencode(path)))

    def save_column(self, i: int, path: str):
        _check(self._lib.lmw_plane_save_column(self._h, i, os.fsencode(path)))


class Ensemble:
    """Spheres with mixed truncations stepped together on the GPU (members of one truncation form one batch).
    Member i: truncation[i], seed[i] (balanced turbulence, nforce = T/2), mean_height[i], omega[i]."""

    def __init__(self, truncation, seed, mean_height, omega, radius=6.37122e6, gravity=9.80616, max_wind=30.0,
                 precision: int = FP64, split_terms: int = 3):
        self._lib = load_library()
        n = len(truncation)
        tr = np.ascontiguousarray(truncation, np.int32)
        sd = np.ascontiguousarray(seed, np.uint64)
        mh = np.ascontiguousarray(mean_height, np.float64)
        om = np.ascontiguousarray(omega, np.float64)
        h = C.c_void_p()
        _check(self._lib.lmw_ensemble_create(n, tr.ctypes.data_as(_IP), sd.ctypes.data_as(C.POINTER(C.c_uint64)), _dp(mh), _dp(om),
                                             radius, gravity, max_wind, precision, split_terms, C.byref(h)))
        self._h = h
        self.truncation = tr.copy()
        self.count = n

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lmw_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, seconds: float):
        _check(self._lib.lmw_ensemble_run(self._h, seconds))
        return self

    def groups(self):
        ng = _I()
        _check(self._lib.lmw_ensemble_groups(self._h, C.byref(ng), None, None, None, None))
        G = ng.value
        tr, cnt = np.zeros(G, np.int32), np.zeros(G, np.int32)
        dt, st = np.zeros(G), np.zeros(G, np.int64)
        _check(self._lib.lmw_ensemble_groups(self._h, C.byref(ng), tr.ctypes.data_as(_IP), cnt.ctypes.data_as(_IP), _dp(dt),
                                             st.ctypes.data_as(C.POINTER(C.c_int64))))
        return [dict(truncation=int(tr[g]), members=int(cnt[g]), dt=float(dt[g]), steps=int(st[g])) for g in range(G)]

    def set_split_form(self, linear_exact: bool) -> None:
        """Sphere.set_split_form for every truncation group."""
        _check(self._lib.lmw_ensemble_set_split_form(self._h, 1 if linear_exact else 0))

    def split_plan(self, group: int) -> dict:
        """The autotuned launch plan of a truncation group's split path."""
        out = np.zeros(12, np.int32)
        _check(self._lib.lmw_ensemble_split_plan(self._h, group, out.ctypes.data_as(_IP)))
        return dict(zip(Sphere._PLAN_KEYS, out.tolist()))

    def member_state(self, i: int):
        T = int(self.truncation[i])
        z, d, f = (np.zeros((T + 1) ** 2, np.complex128) for _ in range(3))
        _check(self._lib.lmw_ensemble_member_state(self._h, i, _dp(z.view(np.float64)), _dp(d.view(np.float64)), _dp(f.view(np.float64))))
        return z, d, f

    def state_size(self) -> int:
        """Complex values per field over all members: sum of (T_i+1)^2."""
        return int(sum((int(T) + 1) ** 2 for T in self.truncation))

    def get_states(self, out=None):
        """Every member's (zeta, delta, phi) at once: each field concatenates the members in order, member i in the
        reference layout ((T_i+1)^2 complex values). `out` may give three complex128 arrays to fill (pinned memory
        copies fastest)."""
        z, d, f = out if out is not None else tuple(np.zeros(self.state_size(), np.complex128) for _ in range(3))
        for a in (z, d, f):
            if a.dtype != np.complex128 or a.size != self.state_size() or not a.flags.c_contiguous:
                raise ValueError("each field needs a contiguous complex128 array of state_size() values")
        _check(self._lib.lmw_ensemble_get_states(self._h, _dp(z.view(np.float64)), _dp(d.view(np.float64)), _dp(f.view(np.float64))))
        return z, d, f

    def set_states(self, zeta, delta, phi):
        """Set every member's state at once (layout as get_states); each member keeps its time."""
        arrs = [np.ascontiguousarray(a, np.complex128) for a in (zeta, delta, phi)]
        for a in arrs:
            if a.size != self.state_size():
                raise ValueError("each field needs state_size() complex values")
        _check(self._lib.lmw_ensemble_set_states(self._h, *(_dp(a.view(np.float64)) for a in arrs)))

    def member_diagnostics(self, i: int) -> dict:
        out = np.zeros(8)
        _check(self._lib.lmw_ensemble_member_diagnostics(self._h, i, _dp(out)))
        return dict(zip(Sphere._DIAG, out.tolist()))


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _fp(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(_FP)


def gemm_bf16(a, b) -> np.ndarray:
    """C = bf16(A) bf16(B)^T on the tensor cores (FP32 accumulation); A [M][K], B [N][K]."""
    a, b = _f32(a), _f32(b)
    M, K = a.shape
    N = b.shape[0]
    c = np.zeros((M, N), np.float32)
    _check(load_library().lmw_gemm_bf16(_fp(a), _fp(b), M, N, K, _fp(c)))
    return c


class Mlp:
    """Four-layer GELU MLP (in -> hidden -> hidden -> hidden -> out) trained with the engine's own tcgen05 BF16
    kernels. No counterpart in the reference."""

    def __init__(self, in_dim: int, hidden: int, out_dim: int, max_batch: int = 128, seed: int = 1, last_layer_scale: float = 1.0):
        self._lib = load_library()
        h = C.c_void_p()
        _check(self._lib.lmw_mlp_create(in_dim, hidden, out_dim, max_batch, seed, last_layer_scale, C.byref(h)))
        self._h = h
        self.dims = (in_dim, hidden, out_dim)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lmw_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _shape(self, layer):
        i, h, o = self.dims
        return (h if layer < 3 else o), (i if layer == 0 else h)

    def set_layer(self, layer: int, w, b):
        w, b = _f32(w), _f32(b)
        assert w.shape == self._shape(layer)
        _check(self._lib.lmw_mlp_set_layer(self._h, layer, _fp(w), _fp(b)))

    def get_layer(self, layer: int):
        no, ni = self._shape(layer)
        w, b = np.zeros((no, ni), np.float32), np.zeros(no, np.float32)
        _check(self._lib.lmw_mlp_get_layer(self._h, layer, _fp(w), _fp(b)))
        return w, b

    def forward(self, x) -> np.ndarray:
        x = _f32(x)
        y = np.zeros((x.shape[0], self.dims[2]), np.float32)
        _check(self._lib.lmw_mlp_forward(self._h, _fp(x), x.shape[0], _fp(y)))
        return y

    def backward(self, x, target, mask=None) -> float:
        x, t = _f32(x), _f32(target)
        m = None if mask is None else _f32(mask)
        loss = _D()
        _check(self._lib.lmw_mlp_backward(self._h, _fp(x), _fp(t), _fp(m), x.shape[0], C.byref(loss)))
        return loss.value

    def grad(self, layer: int):
        no, ni = self._shape(layer)
        gw, gb = np.zeros((no, ni), np.float32), np.zeros(no, np.float32)
        _check(self._lib.lmw_mlp_get_grad(self._h, layer, _fp(gw), _fp(gb)))
        return gw, gb

    def adam(self, lr=3e-4, beta1=0.9, beta2=0.999, eps=1e-8):
        _check(self._lib.lmw_mlp_adam(self._h, lr, beta1, beta2, eps))

    def time(self, batch: int, reps: int = 10):
        tr, fw = _D(), _D()
        _check(self._lib.lmw_mlp_time(self._h, batch, reps, C.byref(tr), C.byref(fw)))
        return tr.value, fw.value


class Surrogate:
    """Learned surrogate of the sphere: a residual MLP advancing the packed spectral state by one window, trained
    on RK4 trajectories, checked and taken over by RK4 in hybrid rollouts. No counterpart in the reference."""

    FIT = ("train_loss", "val_err_mean", "val_err_median", "val_err_p90", "val_err_max", "val_persist_mean", "val_untrained_mean",
           "seconds", "steps")
    ROLLOUT = ("hybrid_s", "network_s", "check_s", "takeover_s", "taken_over", "checks", "err_median", "err_max", "frac_over",
               "rk4_s", "rk4_windows", "hybrid_rate", "rk4_rate", "network_rate", "err_mean", "err_p90")

    def __init__(self, truncation: int = 42, hidden: int = 4096, seed: int = 1, window: float = 21600.0, dt: float = 900.0,
                 radius=6.37122e6, omega=7.292e-5, gravity=9.80616):
        self._lib = load_library()
        h = C.c_void_p()
        _check(self._lib.lmw_surrogate_create(truncation, hidden, seed, window, dt, radius, omega, gravity, C.byref(h)))
        self._h = h
        d = np.zeros(3, np.int32)
        _check(self._lib.lmw_surrogate_dims(self._h, d.ctypes.data_as(_IP)))
        self.features, self.padded, self.hidden = (int(v) for v in d)
        self.truncation = truncation

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lmw_surrogate_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def generate(self, trajectories: int, windows: int, seed0: int = 1, hmin=5000.0, hmax=10000.0, precision: int = FP64) -> float:
        sec = _D()
        _check(self._lib.lmw_surrogate_generate(self._h, trajectories, windows, seed0, hmin, hmax, precision, C.byref(sec)))
        return sec.value

    def generate_drifted(self, trajectories: int, net_windows: int, seed0: int = 2, hmin=5000.0, hmax=10000.0, precision: int = FP64) -> float:
        """After a fit: more training trajectories starting from states the network advanced net_windows windows."""
        sec = _D()
        _check(self._lib.lmw_surrogate_generate_drifted(self._h, trajectories, net_windows, seed0, hmin, hmax, precision, C.byref(sec)))
        return sec.value

    def fit(self, epochs: int, batch: int = 512, lr=3e-4, lr_min=3e-5, val_fraction=0.1, seed: int = 1, loss: str = "energy") -> dict:
        st = np.zeros(9)
        mode = {"normalised": 0, "energy": 1}[loss]
        _check(self._lib.lmw_surrogate_fit(self._h, epochs, batch, lr, lr_min, val_fraction, seed, mode, _dp(st)))
        return dict(zip(self.FIT, st.tolist()))

    def reset(self, seed: int):
        _check(self._lib.lmw_surrogate_reset(self._h, seed))

    def set_clip(self, ratio: float):
        _check(self._lib.lmw_surrogate_set_clip(self._h, ratio))

    def set_averaging(self, decay: float):
        """Moving average of the weights over the second half of fit() (decay per step; 0: the last weights)."""
        _check(self._lib.lmw_surrogate_set_averaging(self._h, decay))

    def set_kinetic_weight(self, weight: float):
        """Weight of the kinetic-energy part of the training loss (1: the energy norm). Before the first fit."""
        _check(self._lib.lmw_surrogate_set_kinetic_weight(self._h, weight))

    def set_takeover(self, mode: str):
        """What a failed rollout check does: "member" (RK4 advances the member from then on, the default) or
        "window" (RK4's result replaces that window; the network keeps the member)."""
        if mode not in ("member", "window"):
            raise ValueError("the takeover mode must be 'member' or 'window'")
        _check(self._lib.lmw_surrogate_set_takeover(self._h, 0 if mode == "member" else 1))

    def set_symmetry_average(self, maps: int):
        """Average the network's increments over `maps` rotations/reflections of the input (1: the plain network)."""
        _check(self._lib.lmw_surrogate_set_symmetry_average(self._h, maps))

    def set_augment(self, on: bool):
        """Random rotations about the polar axis and equatorial reflections of the training pairs (default on)."""
        _check(self._lib.lmw_surrogate_set_augment(self._h, 1 if on else 0))

    def history(self):
        n = _I()
        _check(self._lib.lmw_surrogate_history(self._h, 0, None, None, C.byref(n)))
        loss, gn = np.zeros(max(1, n.value)), np.zeros(max(1, n.value))
        _check(self._lib.lmw_surrogate_history(self._h, n.value, _dp(loss), _dp(gn), C.byref(n)))
        return loss[: n.value], gn[: n.value]

    def evaluate(self, first: int, count: int):
        e, p = np.zeros(count), np.zeros(count)
        _check(self._lib.lmw_surrogate_evaluate(self._h, first, count, _dp(e), _dp(p)))
        return e, p

    def advance(self, states) -> np.ndarray:
        st = np.array(states, dtype=np.float64, order="C", copy=True)
        _check(self._lib.lmw_surrogate_advance(self._h, st.shape[0], _dp(st)))
        return st

    def rollout(self, members: int, seed0: int, windows: int, check_every: int = 4, threshold: float = 1e-3, check_precision: int = FP64,
                ref_windows: int = 4, hmin=5000.0, hmax=10000.0, with_errors: bool = False, with_states: bool = False) -> dict:
        out = np.zeros(16)
        nchk = windows // check_every
        we = np.zeros(max(1, nchk) * members) if with_errors else None
        fs = np.zeros((members, self.features)) if with_states else None
        _check(self._lib.lmw_surrogate_rollout(self._h, members, seed0, hmin, hmax, windows, check_every, threshold, check_precision,
                                               ref_windows, _dp(out), None if we is None else _dp(we), None if fs is None else _dp(fs)))
        r = dict(zip(self.ROLLOUT, out.tolist()))
        if we is not None:
            r["window_errors"] = we[: nchk * members].reshape(nchk, members)
        if fs is not None:
            r["final_states"] = fs
        return r

    def time(self, batch: int = 512, reps: int = 10):
        tr, fw = _D(), _D()
        _check(self._lib.lmw_surrogate_time(self._h, batch, reps, C.byref(tr), C.byref(fw)))
        return tr.value, fw.value
