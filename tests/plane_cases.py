"""Known-answer cases of the reference's plane scripts (tests/plane_harmonic.lms, tests/plane_rossby.lms,
tests/plane_adjustment.lms), restated for any plane class with the reference's interface: the CPU oracle and
the GPU engine run the same checks with the same tolerances."""
import math

import numpy as np

from oracle_lib import plane_fields_grids


def plane_harmonic_case(cls):
    """tests/plane_harmonic.lms restated: energy by zonal harmonic, and a standing gravity wave that swings into
    u = (c a / H) sin(kx) a quarter period later."""
    pi = math.pi
    w = cls(64, 16, 1.0e6, 2.5e5, depth=100.0, linear=True)
    w.set(*plane_fields_grids(64, 16, 1.0e6, 2.5e5, 100.0, lambda x, y: 0 * x, lambda x, y: 3.0 * np.cos(2 * pi * x / 1.0e6),
                              lambda x, y: 0 * x))
    assert abs(w.harmonic_energy(1) - 9.0 / 4.0) <= 1e-9
    assert abs(w.harmonic_energy(2)) <= 1e-9 and abs(w.harmonic_energy(7)) <= 1e-9
    z = cls(64, 16, 1.0e6, 2.5e5, depth=100.0, linear=True)
    z.set(*plane_fields_grids(64, 16, 1.0e6, 2.5e5, 100.0, lambda x, y: 0 * x, lambda x, y: 3.0 * np.cos(2 * pi * x / 1.0e6),
                              lambda x, y: 4.0 * np.sin(4 * pi * x / 1.0e6) * np.sin(pi * y / 2.5e5)))
    sv = sum(math.sin(pi * j / 16.0) ** 2 for j in range(1, 16))
    assert abs(z.harmonic_energy(2) - 16.0 / 4.0 * sv / 16.0) <= 1e-9
    assert abs(z.harmonic_energy(1) - 9.0 / 4.0) <= 1e-9
    g = cls(200, 8, 2.0e6, 4.0e4, depth=100.0, linear=True)
    g.set(*plane_fields_grids(200, 8, 2.0e6, 4.0e4, 100.0, lambda x, y: np.cos(2 * pi * x / 2.0e6), lambda x, y: 0 * x, lambda x, y: 0 * x))
    assert abs(g.harmonic_energy(1)) <= 1e-9
    c = math.sqrt(9.81 * 100.0)
    g.run(0.5 * pi / (c * 2.0 * pi / 2.0e6), 0.0)
    assert abs(g.harmonic_energy(1) - (c / 100.0) ** 2 / 4.0) <= 1e-3


def plane_rossby_case(cls):
    """tests/plane_rossby.lms restated: a quasi-geostrophic wave drifts west at c = -beta / (k^2 + l^2 + 1/Ld^2)
    (-3.359 m/s) for 20 days within 60 km, keeps its amplitude, stays put without beta, and doubles its speed with
    twice the beta."""
    pi, lx, ly, f0, beta, H, g = math.pi, 4.0e6, 2.0e6, 1e-4, 2e-11, 1000.0, 9.81
    k, l = 2 * pi / lx, pi / ly
    ld = math.sqrt(g * H) / abs(f0)
    cp = -beta / (k * k + l * l + 1.0 / (ld * ld))
    assert abs(cp - -3.359) <= 0.002
    grids = plane_fields_grids(60, 30, lx, ly, H, lambda x, y: f0 * 1e5 * np.cos(2 * pi * x / lx) * np.sin(pi * y / ly) / g,
                               lambda x, y: -1e5 * pi / ly * np.cos(2 * pi * x / lx) * np.cos(pi * y / ly),
                               lambda x, y: -1e5 * 2 * pi / lx * np.sin(2 * pi * x / lx) * np.sin(pi * y / ly))

    def wave(b):
        return cls(60, 30, lx, ly, depth=H, f0=f0, beta=b, linear=True).set(*grids)

    m = wave(beta)
    c0, amp0 = m.zonal_crest(1, 15), m.zonal_amplitude(1, 15)
    t = 20.0 * 86400.0
    m.run(t, 0.0)
    diff = (m.zonal_crest(1, 15) - c0) - cp * t
    assert abs(diff - math.floor(diff / lx + 0.5) * lx) <= 60000.0
    assert abs(m.zonal_amplitude(1, 15) / amp0 - 1.0) <= 0.1
    f = wave(0.0)
    fc0 = f.zonal_crest(1, 15)
    f.run(t, 0.0)
    moved = f.zonal_crest(1, 15) - fc0
    assert abs(moved - math.floor(moved / lx + 0.5) * lx) < 0.02 * lx

    def drift(b):
        w = wave(b)
        c = w.zonal_crest(1, 15)
        w.run(2.0 * 86400.0, 0.0)
        s = w.zonal_crest(1, 15) - c
        return s - math.floor(s / lx + 0.5) * lx

    assert abs(drift(2.0 * beta) / drift(beta) - 2.0) <= 0.15


def plane_adjustment_case(cls):
    """tests/plane_adjustment.lms restated: an unbalanced bump in a channel conserves linear PV at every corner and
    settles to eta_n = eta0_n / (1 + (n pi Ld / Ly)^2) in cosine modes (time mean over 10 inertial periods)."""
    pi, ny, ly, f0, H, g = math.pi, 200, 4.0e6, 1e-4, 1000.0, 9.81
    m = cls(8, ny, 40000.0, ly, depth=H, f0=f0, beta=0.0, linear=True)
    m.set(*plane_fields_grids(8, ny, 40000.0, ly, H, lambda x, y: np.exp(-(y - ly / 2) ** 2 / 1.6e11) + 0 * x, lambda x, y: 0 * x,
                              lambda x, y: 0 * x))
    ld = math.sqrt(g * H) / f0
    assert abs(ld - 990515.0) <= 100.0
    d0 = m.diagnostics()
    tin = 2.0 * pi / f0
    m.run(5.0 * tin, 0.0)
    d1 = m.diagnostics()
    assert abs(d1["pv_anomaly_rms"] / d0["pv_anomaly_rms"] - 1.0) <= 1e-3
    assert abs(d1["mean_depth"] - d0["mean_depth"]) <= 1e-11
    ys = [0.5 * ly, 0.5 * ly + 4e5, 0.5 * ly + 8e5, 0.5 * ly + 1.2e6, 0.5 * ly - 6e5]
    acc = np.zeros(len(ys))
    samples = 80
    for _ in range(samples):
        m.run(tin / 8.0, 0.0)
        acc += [m.h_at(20000.0, y) - H for y in ys]
    dy = ly / ny
    yy = (np.arange(ny) + 0.5) * dy
    bump = np.exp(-(yy - ly / 2) ** 2 / 1.6e11)
    pred = np.zeros(len(ys))
    for n in range(ny):
        c = float(np.sum(bump * np.cos(n * pi * (np.arange(ny) + 0.5) / ny)))
        c *= (1.0 if n == 0 else 2.0) / ny
        kk = n * pi / ly
        c /= 1.0 + kk * kk * ld * ld
        pred += [c * math.cos(n * pi * y / ly) for y in ys]
    assert np.all(np.abs(acc / samples - pred) <= 0.015)
    assert 0.25 < pred[0] < 0.4
    d2 = m.diagnostics()
    assert 0.01 < d2["max_speed"] < 0.2
    assert abs(d2["energy"] / d0["energy"] - 1.0) <= 5e-4
