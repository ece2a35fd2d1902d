"""Precision study of the sphere engine: the same seeded state run in FP64, FP32 and split-BF16 (3 and 6 products
per term) for a span of model time; errors of the reduced-precision runs against the FP64 run, and speeds.

    python -m lmweather_gb300.precision --truncation 170 --days 2

The step stays inside the reference's RK4 limit for an 8000 m layer over the whole span (240 s at T170, 150 s at T341; a 450 s step at
T170 exceeds the reference's own limit of 316 s for this state, and at 300 s the limit falls below the step on day 2). Errors: relative L2 (area-weighted, Williamson
normalisation against the FP64 height) and L-infinity of the height, relative drift of energy and potential
enstrophy against FP64.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

A = 6.37122e6
STEP = {42: 900.0, 85: 450.0, 170: 240.0, 341: 150.0}


def weighted_l2(a, b, w):
    wt = w[:, None]
    return float(np.sqrt((wt * (a - b) ** 2).sum() / (wt * b ** 2).sum()))


def study(T: int, days: float, seed: int = 1, modes=("fp64", "fp32", "split3", "split6")) -> dict:
    import lmweather_gb300 as lw

    dt = STEP.get(T, 300.0 * 170 / T)
    nu = A ** 4 / (86400.0 * (T * (T + 1)) ** 2)
    cfg = {"fp64": dict(precision=lw.FP64), "fp32": dict(precision=lw.FP32),
           "split3": dict(precision=lw.SPLIT_BF16, split_terms=3), "split6": dict(precision=lw.SPLIT_BF16, split_terms=6)}
    seconds = days * 86400.0
    out = {"truncation": T, "dt_s": dt, "days": days, "steps": int(round(seconds / dt)), "runs": {}}
    ref = None
    for name in modes:
        s = lw.Sphere(T, diffusion=nu, max_truncation=max(T, 170), **cfg[name])
        s.turbulence(seed, 8000.0, 30.0, T // 2)
        mu, w = s.gauss()
        s.run(64 * dt, dt)  # warm the graphs; the studied span starts after it
        t0 = time.perf_counter()
        s.run(seconds, dt)
        el = time.perf_counter() - t0
        h = s.grid_height()
        d = s.diagnostics()
        rec = {"seconds": el, "sim_days_per_s": days / el, "ms_per_step": el / (seconds / dt) * 1e3}
        if ref is None:
            ref = (h, d)
        else:
            hr, dr = ref
            rec.update(height_l2=weighted_l2(h, hr, w), height_linf=float(np.abs(h - hr).max() / np.abs(hr).max()),
                       energy_drift=abs(d["energy"] - dr["energy"]) / abs(dr["energy"]),
                       enstrophy_drift=abs(d["enstrophy"] - dr["enstrophy"]) / abs(dr["enstrophy"]))
            rec["speedup_vs_fp64"] = out["runs"]["fp64"]["seconds"] / el
        out["runs"][name] = rec
        s.close()
    return out


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--truncation", type=int, default=170)
    ap.add_argument("--days", type=float, default=2.0)
    args = ap.parse_args()
    from lmweather_gb300 import build

    build.build()
    print(json.dumps(study(args.truncation, args.days)))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
