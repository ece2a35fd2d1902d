"""Generate the golden fixtures in tests/golden/ by running the reference core itself.

The reference's cpp/sphere.cpp and cpp/plane.cpp are compiled from the reference checkout by oracle/Makefile
(oracle/_ref/libref.so, no FMA contraction) and driven through their public API. This script runs only where
the reference checkout exists; the fixtures it writes are committed so that the tests need no reference.

    make -C oracle && python tests/golden/make_golden.py
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from oracle_lib import _dp, build_oracle, reference, RefPlane, RefSphere, OracleSphere, OraclePlane  # noqa: E402

A = 6.37122e6
NU4_T42 = A ** 4 / (86400.0 * (42 * 43) ** 2)  # del^4 coefficient with a 1-day e-folding at n = 42


def nu4_for(T: int) -> float:
    return A ** 4 / (86400.0 * (T * (T + 1)) ** 2)


def sphere_case(T, seed, nforce, dt, steps, hbar=8000.0, umax=30.0, diffusion=None, omega=7.292e-5):
    """Balanced turbulence from the project's seeded recipe (grids from the oracle's generator), stepped by the
    reference. Returns the fixture arrays."""
    diffusion = nu4_for(T) if diffusion is None else diffusion
    gen = OracleSphere(T, omega=omega, diffusion=diffusion)
    h, u, v = gen.turbulence_grids(seed, hbar, umax, nforce)
    r = RefSphere(T, omega=omega, diffusion=diffusion)
    r.set_state_grid(h, u, v)
    z0, d0, f0 = r.get_state()
    diag0 = r.diagnostics()
    for _ in range(steps):
        r.step(dt)
    z1, d1, f1 = r.get_state()
    diag1 = r.diagnostics()
    keys = list(diag1.keys())
    return dict(T=T, seed=seed, nforce=nforce, dt=dt, steps=steps, hbar=hbar, umax=umax, diffusion=diffusion, omega=omega,
                h=h, u=u, v=v, zeta0=z0, delta0=d0, phi0=f0, zeta=z1, delta=d1, phi=f1,
                diag_keys=np.array(keys), diag0=np.array([diag0[k] for k in keys]), diag1=np.array([diag1[k] for k in keys]),
                time=r.time)


def main():
    build_oracle(with_ref=True)
    out = {}
    lib = reference()

    # ---- transforms: FFT against the reference, Gauss-Legendre, Legendre columns (cpp/sphere.cpp:21-73)
    rng = np.random.default_rng(20261203)
    for n in (8, 64, 128, 512):
        a = rng.standard_normal(2 * n)
        fwd, bwd = a.copy(), a.copy()
        lib.ref_fft(_dp(fwd), n, -1)
        lib.ref_fft(_dp(bwd), n, +1)
        out[f"fft{n}_in"], out[f"fft{n}_fwd"], out[f"fft{n}_bwd"] = a, fwd, bwd
    for n in (32, 64, 256):
        x, w = np.zeros(n), np.zeros(n)
        lib.ref_gauss_legendre(n, _dp(x), _dp(w))
        out[f"gl{n}_x"], out[f"gl{n}_w"] = x, w
    cols = []
    for m, nmax, mu in ((0, 21, 0.3), (5, 21, -0.77), (21, 21, 0.999), (40, 85, 0.5)):
        c = np.zeros(nmax + 2 - m)
        lib.ref_legendre_column(m, nmax, mu, _dp(c))
        cols.append(np.concatenate([[m, nmax, mu], c]))
    out["legendre_cols"] = np.array([np.pad(c, (0, 100 - len(c))) for c in cols])
    np.savez_compressed(os.path.join(HERE, "transforms.npz"), **out)

    # ---- sphere: seeded balanced turbulence, T21 and T42 (config 0 recipe: nforce 21, nu4 1-day at n=42)
    t21 = sphere_case(21, seed=1, nforce=10, dt=1800.0, steps=48)
    np.savez_compressed(os.path.join(HERE, "sphere_t21_turb.npz"), **t21)
    t42 = sphere_case(42, seed=1, nforce=21, dt=900.0, steps=480, diffusion=NU4_T42)
    np.savez_compressed(os.path.join(HERE, "sphere_t42_turb_480.npz"), **t42)

    # ---- sphere known answers: Williamson TC2 (tilted), TC6 Rossby-Haurwitz, tracer TC1, orography (main.cpp setups)
    cases = {}
    T = 21
    r = RefSphere(T)
    nlat, nlon = r.nlat, r.nlon
    x, wts = np.zeros(nlat), np.zeros(nlat)
    lib.ref_sphere_mu_w(r.h, _dp(x), _dp(wts))
    lat = np.arcsin(x)[:, None]
    lon = (2 * math.pi * np.arange(nlon) / nlon)[None, :]
    g, om = 9.80616, 7.292e-5
    al = 0.05
    u0 = 2 * math.pi * A / (12 * 86400.0)
    h0 = 2.94e4 / g
    uu = u0 * (np.cos(lat) * math.cos(al) + np.sin(lat) * np.cos(lon) * math.sin(al))
    vv = -u0 * np.sin(lon) * math.sin(al) * np.ones_like(lat)
    t = -np.cos(lon) * np.cos(lat) * math.sin(al) + np.sin(lat) * math.cos(al)
    hh = h0 - (A * om * u0 + 0.5 * u0 * u0) * t * t / g
    r.set_axis_tilt(al)
    r.set_state_grid(hh, uu, vv)
    r.run(86400.0, 1800.0)
    z, d, f = r.get_state()
    cases["tc2"] = dict(alpha=al, h=hh, u=uu, v=vv, zeta=z, delta=d, phi=f, diag=np.array(list(r.diagnostics().values())))
    # tracer: cosine bell advected by the TC2 winds (TC1, advect-only)
    R = A / 3
    c = np.cos(lat) * np.cos(lon - 1.5 * math.pi)
    rr = A * np.arccos(np.clip(c, -1, 1))
    qq = np.where(rr < R, 500.0 * (1 + np.cos(math.pi * rr / R)), 0.0)
    r2 = RefSphere(T)
    r2.set_axis_tilt(al)
    r2.set_state_grid(1000.0 * np.ones_like(hh), uu, vv)
    r2.set_tracer_grid(qq)
    r2.set_advect_only(True)
    r2.run(43200.0, 3600.0)
    z, d, f, q = r2.get_state(with_tracer=True)
    cases["tc1"] = dict(alpha=al, h=1000.0 * np.ones_like(hh), u=uu, v=vv, q=qq, zeta=z, delta=d, phi=f, qspec=q,
                        tracer_mean=lib.ref_sphere_tracer_mean(r2.h))
    # orography: TC5 cone, 12 hours
    hs0, Rm, lonc, latc, u5, h5 = 2000.0, math.pi / 9, 1.5 * math.pi, math.pi / 6, 20.0, 5960.0
    rr = np.sqrt(np.minimum(Rm * Rm, (lon - lonc) ** 2 + (lat - latc) ** 2))
    hs = hs0 * (1 - rr / Rm)
    hh5 = h5 - (A * om * u5 + 0.5 * u5 * u5) * np.sin(lat) ** 2 / g - hs
    uu5 = u5 * np.cos(lat) * np.ones_like(lon)
    r3 = RefSphere(T)
    r3.set_orography_grid(hs)
    r3.set_state_grid(hh5, uu5, np.zeros_like(hh5))
    r3.run(43200.0, 900.0)
    z, d, f = r3.get_state()
    cases["tc5"] = dict(hs=hs, h=hh5, u=uu5, zeta=z, delta=d, phi=f, diag=np.array(list(r3.diagnostics().values())))
    flat = {f"{k}_{kk}": vv_ for k, dct in cases.items() for kk, vv_ in dct.items()}
    flat["mu"], flat["w"] = x, wts
    np.savez_compressed(os.path.join(HERE, "sphere_t21_known.npz"), **flat)

    # ---- plane: 64 x 32 jet with noise (config 1 recipe, scaled down), nonlinear, and a linear viscous/drag case
    kw = dict(f0=1e-4, beta=1.6e-11, gravity=9.81, depth=100.0)
    gen = OraclePlane(64, 32, 3.2e5, 1.6e5, **kw)
    h, u = gen.jet_grids(u0=20.0, width=2.0e4, noise_rms=0.1, seed=5)
    v = np.zeros((33, 64))
    p = RefPlane(64, 32, 3.2e5, 1.6e5, **kw)
    p.set(h, u, v)
    for _ in range(200):
        p.step(60.0)
    h1, u1, v1 = p.get()
    pl = dict(h0=h, u0=u, v0=v, h=h1, u=u1, v=v1, diag=np.array(list(p.diagnostics().values())), steps=200, dt=60.0)
    kw2 = dict(f0=5e-5, beta=2e-11, gravity=9.81, depth=50.0, viscosity=200.0, drag=1e-5, linear=True)
    p2 = RefPlane(48, 24, 2.4e5, 1.2e5, **kw2)
    p2.perturb(0.5, 9)
    h2, u2, v2 = p2.get()
    p2.run(7200.0, 0.0)
    h3, u3, v3 = p2.get()
    pl.update(lin_h0=h2, lin_u0=u2, lin_v0=v2, lin_h=h3, lin_u=u3, lin_v=v3, lin_time=p2.time)
    kw3 = dict(f0=1e-4, beta=0.0, gravity=9.81, depth=80.0, viscosity=50.0, drag=2e-6, linear=False)
    p3 = RefPlane(40, 20, 2.0e5, 1.0e5, **kw3)
    p3.perturb(1.0, 4)
    p3.run(3600.0, 20.0)
    h4, u4, v4 = p3.get()
    pl.update(visc_h=h4, visc_u=u4, visc_v=v4, visc_diag=np.array(list(p3.diagnostics().values())))
    np.savez_compressed(os.path.join(HERE, "plane_small.npz"), **pl)
    for fn in sorted(os.listdir(HERE)):
        if fn.endswith(".npz"):
            print(fn, os.path.getsize(os.path.join(HERE, fn)))


if __name__ == "__main__":
    main()
