"""Benchmark: simulated days per second of the shallow-water time stepping on GB300.

Headline workload (one JSON line on rank 0): the sphere at T42 on the 128 x 64 Gaussian grid, FP64, seeded
balanced turbulence (n <= 21, n^-3 kinetic-energy spectrum, 30 m/s, mean height 8000 m), del^4 diffusion with a
1-day e-folding at n = 42, RK4 dt = 900 s; one benchmark step = one run() of 480 RK4 steps (5 model days) with the
reference's guards every 64 steps. Inputs are synthetic and seeded.

  value     sim-days/s from CUDA events on the engine stream, state resident in HBM, L2 flushed between timed steps
  e2e       the same through the C ABI with host buffers: set_state from pinned host memory, run, get_state
  roofline  the dominant kernel's algorithmic FLOP per launch / its measured launch time, against the measured
            FP64 FMA peak of the device (the plain path computes in FP64 throughout)
  cpu_baseline  the oracle (a restatement of the reference algorithm) timed on a bounded sample on the host

`--impl reference` times the reference's CPU algorithm (the oracle port; the reference checkout itself does not
exist on the GPU host) on the same workload and prints the same line with "impl": "reference".
Under torchrun (N > 1) every rank runs its own replica (weak scaling: members are independent; no collective on
the data path); rank 0 prints the max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

A = 6.37122e6
T42_NU4 = A ** 4 / (86400.0 * (42 * 43) ** 2)
WORKLOAD = {"workload": "sphere_t42_fp64_turbulence", "truncation": 42, "grid": "128x64", "dt_s": 900.0,
            "rk4_steps_per_bench_step": 480, "seed": 1, "nforce": 21, "mean_height_m": 8000.0, "max_wind_ms": 30.0,
            "diffusion_m4s": T42_NU4, "precision": "fp64", "members": 1}
METRIC = "sim-days/s at T42 (plain FP64, 128x64 Gaussian grid, RK4 dt=900 s)"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    def __init__(self, world: int, local: int, backend: str):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.p:
            self.p.terminate()
            self.p.wait(timeout=5)

    def summary(self) -> dict:
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(float(r[2]) for r in rows), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit()) if rows else None}


def peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


# ----------------------------------------------------------------------------------------------- reference arm
def cpu_sample(rk4_steps: int):
    """Time the oracle (the reference algorithm restated in C, one thread: the reference core is single-threaded
    and one member cannot use more) on `rk4_steps` RK4 steps of the headline workload. Returns sim-days/s."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import OracleSphere

    o = OracleSphere(42, diffusion=T42_NU4)
    h, u, v = o.turbulence_grids(1, 8000.0, 30.0, 21)
    o.set_state_grid(h, u, v)
    o.step(900.0)
    t0 = time.perf_counter()
    for _ in range(rk4_steps):
        o.step(900.0)
    dt = time.perf_counter() - t0
    return rk4_steps * 900.0 / 86400.0 / dt, dt


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    from oracle_lib import build_oracle  # noqa: F401  (path set in cpu_sample)

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import build_oracle as bo

    bo(with_ref=False)
    per_step = 64  # bounded sample: 64 of the 480 RK4 steps per benchmark step (~1 s of host time)
    for _ in range(args.warmup):
        cpu_sample(4)
    vals, secs = [], 0.0
    for _ in range(args.steps):
        v, s = cpu_sample(per_step)
        vals.append(v)
        secs += s
    value = statistics.median(vals)
    ms_per_step = 480 * 900.0 / 86400.0 / value * 1e3
    sample = f"{per_step} RK4 steps (dt 900 s) of the 480-step T42 run per benchmark step, oracle port, 1 thread"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "sim-days/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded balanced turbulence)", "config": WORKLOAD,
            "cpu_baseline": {"value": value, "unit": "sim-days/s", "cores": 1, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "sim-days/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------------------------------------- our arm
def run_ours(args, rank, world, local):
    import ctypes

    import numpy as np
    import torch

    torch.cuda.set_device(local)
    from lmweather_gb300 import build as b

    if rank == 0 or world == 1:
        b.build()
    dist = Dist(world, local, "nccl")
    dist.barrier()
    import lmweather_gb300 as lw

    lib = lw.load_library()
    lib.lmw_sphere_stream.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]
    lib.lmw_sphere_kernel_times.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    lib.lmw_fp64_peak.argtypes = [ctypes.POINTER(ctypes.c_double)]

    s = lw.Sphere(42, diffusion=T42_NU4)
    s.turbulence(1 + rank, 8000.0, 30.0, 21)
    z0, d0, f0 = s.get_state()
    sp = ctypes.c_void_p()
    lw._check(lib.lmw_sphere_stream(s._h, ctypes.byref(sp)))
    stream = torch.cuda.ExternalStream(sp.value)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 512 MB > L2 (129 MB)
    seconds = 480 * 900.0

    for _ in range(max(args.warmup, 3)):
        s.set_state(z0, d0, f0)
        s.run(seconds, 900.0)
    torch.cuda.synchronize()

    # --- value: device time of K runs (state resident), L2 flushed between timed steps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches0 = lw.launch_count()
    dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            ev[k][0].record(stream)
            s.run(seconds, 900.0)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    launches = lw.launch_count() - launches0
    dist.barrier()
    dev_ms = sum(a.elapsed_time(b) for a, b in ev)
    dev_ms = dist.max(dev_ms)
    sim_days = args.steps * seconds / 86400.0 * world
    value = sim_days / (dev_ms * 1e-3)
    ms_per_step = dev_ms / args.steps

    # --- e2e: through the C ABI with host buffers (set_state from host, run, get_state to host), wall clock
    zs, ds, fs = (torch.from_numpy(x.view(np.float64).copy()).pin_memory().numpy().view(np.complex128) for x in (z0, d0, f0))
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s.set_state(zs, ds, fs)
        s.run(seconds, 900.0)
        zz, dd, ff = s.get_state()
    t_e2e = dist.max(time.perf_counter() - t0)
    e2e = args.steps * seconds / 86400.0 * world / t_e2e
    nbytes = 3 * s.nspec * 16

    # --- roofline: per-kernel launch times on the engine stream (live, CUDA events)
    ms3 = (ctypes.c_double * 3)()
    lw._check(lib.lmw_sphere_kernel_times(s._h, 900.0, 200, ms3))
    nlat, nlon, ntri = s.nlat, s.nlon, (s.T + 1) * (s.T + 2) // 2
    flops = [12.0 * nlat * ntri, 9 * (nlat // 2) * 5.0 * nlon * math.log2(nlon), 14.0 * nlat * ntri]
    names = ["sph_synth (Legendre synthesis)", "sph_grid (FFTs + products)", "sph_analysis (Legendre analysis + RK4)"]
    top = max(range(3), key=lambda i: ms3[i])
    pk = ctypes.c_double()
    lw._check(lib.lmw_fp64_peak(ctypes.byref(pk)))
    achieved = flops[top] / (ms3[top] * 1e-3) / 1e12
    stage_ms = sum(ms3)
    roofline = {"bound": "fp64", "kernel": names[top], "achieved": achieved, "peak": pk.value, "unit": "TFLOP/s",
                "frac": achieved / pk.value, "traffic": None,
                "peak_source": "measured on this device by lmw_fp64_peak (dependent DFMA chains on every SM)",
                "kernel_ms": {n: ms3[i] for i, n in enumerate(names)}, "flop_per_launch": flops[top],
                "stage_kernel_ms_sum": stage_ms}

    # --- CPU baseline on rank 0 (bounded sample)
    cpu = None
    if rank == 0 and world == 1:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from oracle_lib import build_oracle

        build_oracle(with_ref=False)
        cv, csec = cpu_sample(64)
        cpu = {"value": cv, "unit": "sim-days/s", "cores": 1, "kind": "port",
               "sample": f"64 RK4 steps of the T42 workload ({csec:.1f} s), oracle restatement of the reference, 1 thread"}

    clocks = clk.summary()
    if rank == 0:
        cfg = dict(WORKLOAD)
        cfg["l2"] = "flushed (512 MB write) between timed steps"
        cfg["parallelism"] = f"replicas x{world}" if world > 1 else "single GPU"
        line = {"metric": METRIC, "value": value, "unit": "sim-days/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded balanced turbulence)", "config": cfg,
                "e2e": {"value": e2e, "unit": "sim-days/s", "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes},
                "gpu_launches": int(launches), "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks}
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_ours(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
