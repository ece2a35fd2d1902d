"""Passive tracer on the GPU (FP64 path) against the reference's own TC1 run (golden) and against the oracle with a
moving flow: cpp/sphere.cpp:250-300 (tracer tendency, advect-only mode, tracer diagnostics)."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def normrel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_tc1_advect_only_against_reference_run(engine):
    g = golden("sphere_t21_known.npz")
    s = engine.Sphere(21)
    s.set_axis_tilt(float(g["tc1_alpha"]))
    s.set_state_grid(g["tc1_h"], g["tc1_u"], g["tc1_v"])
    s.set_tracer_grid(g["tc1_q"])
    s.set_advect_only(True)
    # the tracer starts at the reference's analysis of the bell and equals the grid it was set from (error 0)
    d0 = s.tracer_diagnostics()
    assert d0["tracer_error_l2"] < 1e-14
    s.run(43200.0, 3600.0)
    q = s.tracer_state()
    assert normrel(q, g["tc1_qspec"]) < 1e-12
    z, d, f = s.get_state()
    # the flow is frozen (no diffusion): vorticity unchanged
    assert normrel(z, g["tc1_zeta"]) < 1e-13
    assert abs(s.tracer_diagnostics()["tracer_mean"] - float(g["tc1_tracer_mean"])) <= 1e-12 * abs(float(g["tc1_tracer_mean"]))


def test_tracer_with_moving_flow_against_oracle(engine, oracle_built):
    from oracle_lib import OracleSphere

    g = golden("sphere_t21_known.npz")
    nu = 6.37122e6 ** 4 / (86400.0 * (21 * 22) ** 2)
    s = engine.Sphere(21, diffusion=nu)
    o = OracleSphere(21, diffusion=nu)
    for x in (s, o):
        x.set_axis_tilt(float(g["tc2_alpha"]))
        x.set_state_grid(g["tc2_h"], g["tc2_u"], g["tc2_v"])
        x.set_tracer_grid(g["tc1_q"])
    s.run(43200.0, 1800.0)
    o.run(43200.0, 1800.0)
    zo, do, fo, qo = o.get_state(with_tracer=True)
    assert normrel(s.tracer_state(), qo) < 1e-12
    z, d, f = s.get_state()
    assert normrel(z, zo) < 1e-12 and normrel(f, fo) < 1e-12
    dg = s.tracer_diagnostics()
    assert abs(dg["tracer_mass"] - o.lib.or_sphere_tracer_mass(o.h)) <= 1e-11 * abs(dg["tracer_mass"])
    assert abs(dg["tracer_error_l2"] - o.lib.or_sphere_tracer_error_l2(o.h)) <= 1e-9 * dg["tracer_error_l2"] + 1e-15
    grid_o = o.grid_tracer()
    assert normrel(s.grid_tracer(), grid_o) < 1e-12


def test_tracer_rules(engine):
    s = engine.Sphere(21)
    s.set_state_grid(8000.0 * np.ones((32, 64)), np.zeros((32, 64)), np.zeros((32, 64)))
    s.set_advect_only(True)
    with pytest.raises(ValueError, match="advect_only: set a tracer first"):
        s.run(3600.0, 600.0)
    f = engine.Sphere(21, precision=engine.FP32)
    with pytest.raises(ValueError, match="FP64"):
        f.set_tracer_grid(np.zeros((32, 64)))
