"""Run one named workload for a fixed number of RK4 steps: the command that profiler captures wrap.

    python -m lmweather_gb300.profile --case t42 --steps 4
    ncu --metrics gpu__time_duration.sum --clock-control none --csv python -m lmweather_gb300.profile --case t42 --steps 4

Cases: t42 (config-0 sphere), t85, t170 (dt 240 s), t341 (dt 150 s), plane (1024 x 512 beta-plane jet, dt 60 s),
ens (an ensemble of --members spheres at --truncation, the groups of the benchmark ensemble; --plan forces split
plan entries so a capture can use the plan a benchmark run chose). One untimed warm-up step runs first.
"""
from __future__ import annotations

import argparse
import time

A = 6.37122e6


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="t42", choices=["t42", "t85", "t170", "t341", "plane", "ens", "mlp"])
    ap.add_argument("--batch", type=int, default=512)
    ap.add_argument("--truncation", type=int, default=85)
    ap.add_argument("--members", type=int, default=128)
    ap.add_argument("--split-terms", type=int, default=3)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--precision", type=int, default=0)
    ap.add_argument("--plan", default="", help="split plan entries to force, e.g. analysis_stages=1,analysis_ctas_per_sm=3")
    args = ap.parse_args()
    import lmweather_gb300 as lw
    from lmweather_gb300 import build

    build.build()
    t0 = time.perf_counter()
    if args.case == "plane":
        p = lw.Plane(1024, 512, 1024 * 5000.0, 512 * 5000.0, f0=1e-4, beta=1.6e-11, gravity=9.81, depth=100.0)
        p.jet(20.0, 1.0e5, 0.1, 1)
        p.step(60.0)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            p.step(60.0)
        print(f"plane 1024x512: {args.steps} steps in {time.perf_counter() - t0:.4f} s")
        return 0
    if args.case == "mlp":
        # the surrogate's network at its T42 size: training steps (forward, backward, Adam) on a random batch
        import numpy as np

        rng = np.random.default_rng(1)
        net = lw.Mlp(5676, 4096, 5676, max_batch=args.batch, seed=1, last_layer_scale=0.1)
        x = rng.standard_normal((args.batch, 5676)).astype(np.float32)
        t = 0.1 * rng.standard_normal((args.batch, 5676)).astype(np.float32)
        net.backward(x, t)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            net.backward(x, t)
            net.adam(1e-4)
        print(f"mlp 5676-4096x3-5676 batch {args.batch}: {args.steps} training steps in {time.perf_counter() - t0:.4f} s")
        return 0
    if args.case == "ens":
        T, B = args.truncation, args.members
        nu = A ** 4 / (86400.0 * (T * (T + 1)) ** 2)
        s = lw.Sphere(T, diffusion=nu, precision=args.precision, members=B, split_terms=args.split_terms)
        for b in range(B):
            s.turbulence(b + 1, 5000.0 + 5000.0 * b / B, 30.0, T // 2, member=b)
        if args.plan:
            s.set_split_plan(**{k: int(v) for k, v in (kv.split("=") for kv in args.plan.split(","))})
        if args.precision == lw.SPLIT_BF16:
            print("plan", s.split_plan())
        dt = 0.9 * min(s.stable_dt(1.5, member=b) for b in range(B))
        s.step(dt)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            s.step(dt)
        print(f"ensemble T{T} x {B}: {args.steps} steps in {time.perf_counter() - t0:.4f} s")
        return 0
    # steps inside the reference's RK4 stability limit for an 8000 m layer (316 s at T170 falling below 300 s on day 2; 159 s at T341)
    T, dt = {"t42": (42, 900.0), "t85": (85, 450.0), "t170": (170, 240.0), "t341": (341, 150.0)}[args.case]
    nu = A ** 4 / (86400.0 * (T * (T + 1)) ** 2)
    s = lw.Sphere(T, diffusion=nu, precision=args.precision, max_truncation=max(T, 170), split_terms=args.split_terms)
    s.turbulence(1, 8000.0, 30.0, T // 2)
    s.step(dt)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s.step(dt)
    print(f"sphere T{T}: {args.steps} steps in {time.perf_counter() - t0:.4f} s")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
