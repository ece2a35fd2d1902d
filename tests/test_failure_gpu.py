"""Failure detection of the tensor-core path without a GPU fault: every wait on an mbarrier in the split-precision
kernels is bounded, reports that it ran out in an error word, and the host turns that into an error at its next
step or guard check (the reference's guards, cpp/sphere.cpp:473-483, cover the arithmetic; these cover the device).
The wait is made to run out on a barrier nothing arrives on; the error word is written on the host."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_the_context_stays_usable(engine):
    lib = engine.load_library()
    completed, ran_out = C.c_int(0), C.c_int(0)
    engine._check(lib.lmw_wait_selftest(20000, C.byref(completed), C.byref(ran_out)))
    assert completed.value == 1  # a phase that completes is seen
    assert ran_out.value == 1  # a phase that never completes is given up on after 20 ms
    s = engine.Sphere(21, diffusion=1e16, precision=engine.SPLIT_BF16, split_terms=3)
    s.turbulence(3, 8000.0, 30.0, 10)
    s.step(1200.0)
    assert np.isfinite(s.diagnostics()["energy"])
    with pytest.raises(ValueError, match="timeout must be between"):
        engine._check(lib.lmw_wait_selftest(0, C.byref(completed), C.byref(ran_out)))


def test_a_timed_out_tensor_core_wait_stops_the_run(engine):
    lib = engine.load_library()
    s = engine.Sphere(21, diffusion=1e16, precision=engine.SPLIT_BF16, members=4, split_terms=3)
    for b in range(4):
        s.turbulence(b + 1, 8000.0, 30.0, 10, member=b)
    s.step(1200.0)
    engine._check(lib.lmw_sphere_inject_split_error(s._h, 3))  # the code a consumer's wait writes when it runs out
    with pytest.raises(engine.DeviceError, match="a wait on the tensor cores timed out"):
        s.step(1200.0)
    with pytest.raises(engine.DeviceError, match="timed out"):
        s.run(6 * 3600.0, 1200.0)
    # another engine on the same device is unaffected
    t = engine.Sphere(21, diffusion=1e16, precision=engine.SPLIT_BF16, split_terms=3)
    t.turbulence(1, 8000.0, 30.0, 10)
    t.run(6 * 3600.0, 1200.0)
    assert np.isfinite(t.diagnostics()["energy"])
    f64 = engine.Sphere(21)
    with pytest.raises(ValueError, match="not in split precision"):
        engine._check(lib.lmw_sphere_inject_split_error(f64._h, 3))
