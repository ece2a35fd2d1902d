"""The allocation-free plane step (lmw_plane_step_noalloc) against the handle-based step (lmw_plane_step).

Some callers cannot allocate device memory: code that runs inside a fixed memory budget claimed up front, a
real-time loop where a cudaMalloc would stall on device-wide synchronisation, or a host that hands out device
memory only from its own pool. They call lmw_plane_step_noalloc with their own device fields; its scratch is a
fixed device array inside the library. This file is collected last so that a run stopping at the first failure
has already run every other test; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NX, NY, LX, LY = 256, 128, 1.28e6, 6.4e5
PARAMS = dict(gravity=9.81, depth=100.0, f0=1e-4, beta=1.6e-11, viscosity=0.0, drag=0.0, linear=False)


def _noalloc(lib):
    f = lib.lmw_plane_step_noalloc
    D, I, P = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    f.restype = I
    f.argtypes = [I, I, D, D, D, D, D, D, D, D, I, P, P, P, D, I, P]
    return f


def _call(f, engine, th, tu, tv, dt, steps, nx=NX, ny=NY):
    p = PARAMS
    code = f(nx, ny, LX, LY, p["gravity"], p["depth"], p["f0"], p["beta"], p["viscosity"], p["drag"], 0,
             th.data_ptr(), tu.data_ptr(), tv.data_ptr(), dt, steps, None)
    engine._check(code)


def test_noalloc_step_matches_handle_step_on_two_calls(engine):
    torch = pytest.importorskip("torch")
    f = _noalloc(engine.load_library())
    ref = engine.Plane(NX, NY, LX, LY, **PARAMS)
    ref.jet(20.0, 5.0e4, 0.1, 3)
    h0, u0, v0 = ref.get()
    # the caller's own device fields (here from torch's allocator; the entry point itself allocates nothing)
    th, tu, tv = (torch.from_numpy(x.copy()).cuda() for x in (h0, u0, v0))
    torch.cuda.synchronize()
    for call in range(2):
        allocs = engine.alloc_count()
        _call(f, engine, th, tu, tv, 60.0, 7)
        torch.cuda.synchronize()
        # the library made no device or pinned-host allocation during the call
        assert engine.alloc_count() == allocs, call
        for _ in range(7):
            ref.step(60.0)
        h, u, v = ref.get()
        # the plane's parity bar is bitwise
        assert np.array_equal(th.cpu().numpy(), h), call
        assert np.array_equal(tu.cpu().numpy(), u), call
        assert np.array_equal(tv.cpu().numpy(), v), call


def test_noalloc_clears_the_wall_rows_of_v(engine):
    # rows 0 and ny of v are walls; a caller's nonzero values there are cleared before the first step, so the
    # result equals the handle's step from the same interior state
    torch = pytest.importorskip("torch")
    f = _noalloc(engine.load_library())
    ref = engine.Plane(NX, NY, LX, LY, **PARAMS)
    ref.jet(20.0, 5.0e4, 0.1, 5)
    h0, u0, v0 = ref.get()
    vbad = v0.copy()
    vbad[0, :] = 1.0
    vbad[-1, :] = -2.0
    th, tu, tv = (torch.from_numpy(x.copy()).cuda() for x in (h0, u0, vbad))
    _call(f, engine, th, tu, tv, 60.0, 3)
    torch.cuda.synchronize()
    for _ in range(3):
        ref.step(60.0)
    h, u, v = ref.get()
    assert np.array_equal(th.cpu().numpy(), h)
    assert np.array_equal(tu.cpu().numpy(), u)
    assert np.array_equal(tv.cpu().numpy(), v)


def test_noalloc_rejects_grids_beyond_its_scratch(engine):
    torch = pytest.importorskip("torch")
    f = _noalloc(engine.load_library())
    nx, ny = 1024, 512
    th = torch.zeros(nx * ny, dtype=torch.float64, device="cuda")
    tu = torch.zeros(nx * ny, dtype=torch.float64, device="cuda")
    tv = torch.zeros(nx * (ny + 1), dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError, match="at most 262144 cells"):
        _call(f, engine, th, tu, tv, 60.0, 1, nx=nx, ny=ny)
