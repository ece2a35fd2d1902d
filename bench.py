"""Benchmark: simulated days per second of the shallow-water time stepping on GB300.

Headline workload: the mixed-truncation ensemble of 1024 spheres (512 at T21 on 64 x 32, 384 at T42 on 128 x 64,
128 at T85 on 256 x 128), each member with its own seed (balanced turbulence, n <= T/2, n^-3 kinetic-energy
spectrum, 30 m/s), a mean height drawn uniformly from 5000-10000 m and Omega scaled by 0.5, 1 or 2; del^4
diffusion with a 1-day e-folding at n = T; every truncation at its own stable RK4 step (the reference's
stable_dt(1.5), smallest over the group) with the reference's guards every 64 steps. One benchmark step = one
run() of 2 model days of every member, in split precision (Legendre sums on tcgen05 with BF16 hi/lo products and
FP32 accumulation, FP32 FFTs and products, FP64 state). Inputs are synthetic and seeded.

  value         member-sim-days/s = members x 2 days / device time of the run (CUDA events on the group streams),
                state resident in HBM, L2 flushed (512 MB write) between timed steps
  e2e           the same through the C ABI with host buffers: every member's state from host, run, state to host
  error         split vs FP64 runs of a subset of members: relative L2 height error and Phi error after 2 days
  roofline      the stage kernel with the largest share of device time, its algorithmic bytes per launch over its
                CUDA-event launch time, against the measured HBM copy bandwidth
  cpu_baseline  the oracle (the reference algorithm restated in C) timed per member-step on every host core,
                scaled to the workload's member-step counts
  workloads     the other configurations: T42 plain FP64 (config 0), the 1024 x 512 beta-plane (config 1), the
                T170 and T341 precision studies (config 2), the learned surrogate (config 4, bounded training) and
                the ensemble in the other precisions; configs 0, 1 and the T170 study carry the oracle timed on one
                host core beside them (cpu_1core, a bounded sample of RK4 steps of the same seeded state)

`--impl reference` times the reference's CPU algorithm (the oracle port: the reference checkout is absent on the
GPU host) on the same workload with all host cores and prints the same line with "impl": "reference".
Under torchrun (N > 1) every rank runs its own replica of the ensemble (members are independent: weak scaling, no
collective on the data path); rank 0 prints the max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

A = 6.37122e6
OMEGA = 7.292e-5
DAYS = 2.0
METRIC = "member-sim-days/s, 1024-member T21/T42/T85 ensemble, 2 model days (split-BF16 Legendre on tcgen05, FP64 state)"


def nu4(T):
    return A ** 4 / (86400.0 * (T * (T + 1.0)) ** 2)


def ensemble_specs(seed_base: int = 0):
    import numpy as np

    tr = [21] * 512 + [42] * 384 + [85] * 128
    rng = np.random.default_rng(2026 + seed_base)
    heights = rng.uniform(5000.0, 10000.0, len(tr))
    omegas = [OMEGA * (0.5, 1.0, 2.0)[i % 3] for i in range(len(tr))]
    seeds = [seed_base * 100000 + i + 1 for i in range(len(tr))]
    return tr, seeds, list(heights), omegas


WORKLOAD = {"workload": "ensemble_t21x512_t42x384_t85x128_2days", "members": 1024, "truncations": {"21": 512, "42": 384, "85": 128},
            "grids": {"21": "64x32", "42": "128x64", "85": "256x128"}, "model_days_per_bench_step": DAYS,
            "init": "balanced turbulence, nforce = T/2, max wind 30 m/s, mean height U[5000, 10000] m, Omega x {0.5, 1, 2}",
            "diffusion": "del^4, 1-day e-folding at n = T", "step": "stable_dt(1.5) per truncation, guards every 64 steps"}


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class Dist:
    def __init__(self, world: int, backend: str):
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
    """nvidia-smi clocks and throttle reasons every 200 ms during the timed region."""

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
        pw = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(float(r[2]) for r in rows), "reasons": reasons, "samples": len(rows),
                "power_w_max": max(pw) if pw else None}


def peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


# ----------------------------------------------------------------------------------------------- CPU side (oracle)
# The CPU measurement runs whole RK4 member-steps of the workload on every host core for a measured interval:
# each core holds one member of each truncation (its own seeded state, the workload's steps) and runs member-steps
# in the workload's proportions of member-steps per truncation (T21 512 x 179, T42 384 x 327, T85 128 x 616 at
# the stable steps of the 2-day runs), always the truncation furthest behind its share, so a sample's member-days
# per second estimate the whole workload's. The value is the member-days the cores actually simulated over the
# measured wall time.
_CPU_STATE = {}


def _cpu_init(specs):
    """Pool initialiser: one oracle sphere per truncation from a seeded balanced-turbulence state (the cost of a
    member-step does not depend on the member's mean height or rotation rate)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import OracleSphere

    for T, dt, seed, hbar, om in specs:
        o = OracleSphere(T, omega=om, diffusion=nu4(T))
        h, u, v = o.turbulence_grids(seed, hbar, 30.0, T // 2)
        o.set_state_grid(h, u, v)
        _CPU_STATE[T] = (o, dt)
    _CPU_STATE["done"] = {T: 0 for T, *_ in specs}


def _cpu_run_for(args):
    """Run member-steps for `seconds` of wall time; returns (member-steps per truncation, member-days, elapsed)."""
    seconds, shares = args
    done = _CPU_STATE["done"]
    steps = {T: 0 for T in shares}
    days = 0.0
    t0 = time.perf_counter()
    while True:
        total = sum(done.values()) + 1
        T = max(shares, key=lambda k: shares[k] * total - done[k])
        o, dt = _CPU_STATE[T]
        o.step(dt)
        done[T] += 1
        steps[T] += 1
        days += dt / 86400.0
        el = time.perf_counter() - t0
        if el >= seconds:
            return steps, days, el


class CpuEnsemble:
    """The reference's algorithm (the oracle port) on `cores` host cores, one process per core (spawn)."""

    def __init__(self, group_steps: dict, dts: dict, cores: int):
        total = sum(group_steps.values())
        self.shares = {T: n / total for T, n in group_steps.items()}
        self.cores = cores
        ctx = mp.get_context("spawn")
        specs = [(T, dts[T], 7 + T, 8000.0, OMEGA) for T in sorted(group_steps)]
        self.pool = ctx.Pool(cores, initializer=_cpu_init, initargs=(specs,))
        self.pool.map(_cpu_run_for, [(0.05, self.shares)] * cores)  # every worker built its tables and states

    def run(self, seconds: float) -> dict:
        """All cores run member-steps for `seconds`; member-days simulated over the wall time of the whole pass."""
        t0 = time.perf_counter()
        res = self.pool.map(_cpu_run_for, [(seconds, self.shares)] * self.cores)
        wall = time.perf_counter() - t0
        steps = {T: sum(r[0][T] for r in res) for T in self.shares}
        days = sum(r[1] for r in res)
        return {"value": days / wall, "member_days": days, "wall_s": wall, "member_steps": steps}

    def close(self):
        self.pool.close()
        self.pool.join()


# the 2-day workload's member-step counts and stable steps (the reference's stable_dt(1.5), smallest over the group,
# of the seeded initial states: the same steps the GPU run takes)
GROUP_STEPS = {21: 512 * 179, 42: 384 * 327, 85: 128 * 616}
GROUP_DT = {21: 965.4, 42: 528.4, 85: 280.5}


def cpu_single_rate(config: str, budget_s: float = 2.0) -> dict:
    """1-core sim-days/s of the reference algorithm (the oracle port, one thread, in this process) on a bounded
    sample of a single-run configuration: RK4 steps of the same seeded initial state, timed until `budget_s`."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import OraclePlane, OracleSphere

    if config == "plane":
        o = OraclePlane(1024, 512, 1024 * 5000.0, 512 * 5000.0, f0=1e-4, beta=1.6e-11, gravity=9.81, depth=100.0)
        h, u = o.jet_grids(20.0, 1.0e5, 0.1, 1)
        o.set(h, u, np.zeros((513, 1024)))
        dt = 60.0
    else:
        T, dt = (42, 900.0) if config == "t42" else (170, 240.0)
        o = OracleSphere(T, diffusion=nu4(T))
        h, u, v = o.turbulence_grids(1, 8000.0, 30.0, T // 2)
        o.set_state_grid(h, u, v)
    o.step(dt)
    n, t0 = 0, time.perf_counter()
    while n < 2 or time.perf_counter() - t0 < budget_s:
        o.step(dt)
        n += 1
    el = time.perf_counter() - t0
    return {"value": n * dt / 86400.0 / el, "unit": "sim-days/s", "cores": 1, "kind": "port",
            "sample": f"{n} RK4 steps of {dt:g} s of the same seeded initial state, oracle port, one thread ({el:.1f} s)"}


def build_oracle():
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import build_oracle as bo

    bo(with_ref=False)


def ensemble_member_steps(groups):
    return {g["truncation"]: g["members"] * g["steps"] for g in groups}


def run_reference(args, rank, world):
    """The reference's CPU algorithm on every host core (the reference checkout is absent on the GPU host, so the oracle
    port, bitwise equal to it, runs): each bench step is a timed pass of whole member-steps of the workload."""
    if rank != 0:
        return 0
    build_oracle()
    cores = os.cpu_count() or 1
    cpu = CpuEnsemble(GROUP_STEPS, GROUP_DT, cores)
    for _ in range(args.warmup):
        cpu.run(1.0)
    runs = [cpu.run(args.ref_seconds) for _ in range(args.steps)]
    cpu.close()
    days = sum(r["member_days"] for r in runs)
    wall = sum(r["wall_s"] for r in runs)
    value = days / wall
    steps = {T: sum(r["member_steps"][T] for r in runs) for T in GROUP_STEPS}
    smp = (f"{args.steps} timed passes of {args.ref_seconds:g} s on {cores} cores (oracle port, one process per core): "
           f"{steps[21]} T21, {steps[42]} T42 and {steps[85]} T85 member-steps executed ({days:.3f} member-days in {wall:.1f} s), "
           "in the 2-day workload's proportions of member-steps per truncation")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "member-sim-days/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded balanced turbulence)", "config": WORKLOAD,
            "cpu_baseline": {"value": value, "unit": "member-sim-days/s", "cores": cores, "kind": "port", "sample": smp,
                             "member_steps": {str(k): v for k, v in steps.items()}},
            "e2e": {"value": value, "unit": "member-sim-days/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------------------------------------- GPU side
def run_ours(args, rank, world, local):
    import ctypes

    import numpy as np
    import torch

    cpu_pool = None
    if rank == 0 and world == 1:
        build_oracle()
        # the CPU baseline's worker pool starts (by spawn) before any CUDA work
        cpu_pool = CpuEnsemble(GROUP_STEPS, GROUP_DT, os.cpu_count() or 1)
    torch.cuda.set_device(local)
    from lmweather_gb300 import build as b

    if rank == 0 or world == 1:
        b.build()
    dist = Dist(world, "nccl")
    dist.barrier()
    import lmweather_gb300 as lw

    lib = lw.load_library()
    lib.lmw_ensemble_stream.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    lib.lmw_ensemble_kernel_times.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    prec = {"split3": dict(precision=lw.SPLIT_BF16, split_terms=3), "split6": dict(precision=lw.SPLIT_BF16, split_terms=6),
            "fp32": dict(precision=lw.FP32), "fp64": dict(precision=lw.FP64)}
    tr, seeds, heights, omegas = ensemble_specs(rank)
    ens = lw.Ensemble(tr, seeds, heights, omegas, **prec[args.precision])
    streams = []
    for g in range(len(ens.groups())):
        sp = ctypes.c_void_p()
        lw._check(lib.lmw_ensemble_stream(ens._h, g, ctypes.byref(sp)))
        streams.append(torch.cuda.ExternalStream(sp.value))
    seconds = DAYS * 86400.0
    z0 = ens.get_states()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def reset_states():
        ens.set_states(*z0)

    for _ in range(max(args.warmup, 3)):
        reset_states()
        ens.run(seconds)
    torch.cuda.synchronize()

    # --- value: device time of K two-day runs, every member resident, L2 flushed between timed steps
    dev_ms = 0.0
    launches0 = lw.launch_count()
    dist.barrier()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            reset_states()
            flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e0.record(torch.cuda.current_stream())
            torch.cuda.current_stream().synchronize()
            if k == 0:
                lw.profiler_range(True)  # a profiler run with --profile-from-start off captures the first timed run
            ens.run(seconds)
            if k == 0:
                lw.profiler_range(False)
            ends = []
            for st in streams:
                e = torch.cuda.Event(enable_timing=True)
                e.record(st)
                ends.append(e)
            torch.cuda.synchronize()
            dev_ms += max(e0.elapsed_time(e) for e in ends)
    launches = lw.launch_count() - launches0
    groups = ens.groups()
    if args.precision.startswith("split"):
        for g, grp in enumerate(groups):
            grp["autotuned_plan"] = ens.split_plan(g)
    dist.barrier()
    dev_ms = dist.max(dev_ms)
    member_days = ens.count * DAYS * world
    value = member_days * args.steps / (dev_ms * 1e-3)
    ms_per_step = dev_ms / args.steps

    # --- e2e: host buffers through the C ABI: every member's state in from pinned host memory (one
    # lmw_ensemble_set_states call), run, every member's state out (lmw_ensemble_get_states)
    def pinned_like(a):
        return torch.empty(a.size, dtype=torch.complex128).pin_memory().numpy()

    pin_in = tuple(pinned_like(a) for a in z0)
    for dst, src in zip(pin_in, z0):
        dst[:] = src
    pin_out = tuple(pinned_like(a) for a in z0)
    nbytes = sum(a.nbytes for a in pin_in)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ens.set_states(*pin_in)
        ens.run(seconds)
        ens.get_states(out=pin_out)
    t_e2e = dist.max(time.perf_counter() - t0)
    e2e = member_days * args.steps / t_e2e

    # --- roofline: per-group stage-kernel launch times (CUDA events on the group streams)
    kt = []
    for g, grp in enumerate(groups):
        ms3 = (ctypes.c_double * 3)()
        lw._check(lib.lmw_ensemble_kernel_times(ens._h, g, 50, ms3))
        kt.append(list(ms3))
    names = ["synthesis (split_syn)" if args.precision.startswith("split") else "synthesis (sph_synth)",
             "grid: FFTs + products (split_grid)" if args.precision.startswith("split") else "grid: FFTs + products (sph_grid)",
             "analysis + RK4 (split_ana)" if args.precision.startswith("split") else "analysis + RK4 (sph_analysis)"]
    share = []
    for g, grp in enumerate(groups):
        for k in range(3):
            share.append((kt[g][k] * 4 * grp["steps"], g, k))
    _, gtop, ktop = max(share)
    grp = groups[gtop]
    T, Bm = grp["truncation"], grp["members"]
    nlon = 4
    while nlon < 3 * T + 1:
        nlon *= 2
    nlat, nh, M = nlon // 2, nlon // 4, T + 1
    ntri = M * (M + 1) // 2
    pieces = 3 if args.precision == "split6" else 2
    split = args.precision.startswith("split")
    direct = bool(grp.get("autotuned_plan", {}).get("grid_writes_operands", 0)) if split else False
    # algorithmic bytes of one launch (each operand read once, each result written once). Fourier records: 16
    # floats per (member, latitude pair, m); analysis operands: 14 rows (7 complex quantities) per (member, m,
    # parity) over the nh latitudes in `pieces` BF16 pieces (direct interface), or the FP32 fold (10 complex
    # values per (member, m, latitude pair)); synthesis operands: 12 rows per (member, coefficient) in pieces.
    records = Bm * nh * M * 16 * 4
    a_ops = Bm * M * 2 * 14 * nh * pieces * 2 if direct else Bm * M * 10 * nh * 8
    tables = 2 * pieces * nh * ntri * 2
    s_ops = Bm * 12 * pieces * ntri * 2
    if ktop == 1:
        moved = records + a_ops
        what = ("Fourier records in (16 floats per member, latitude pair and m), analysis operands out ("
                + ("BF16 pieces" if direct else "FP32 fold") + ")")
    elif ktop == 0:
        moved = tables + s_ops + records
        what = "BF16 P and H table pieces and synthesis operands in, Fourier records out"
    else:
        moved = tables + a_ops + Bm * 3 * ntri * 16 * 3 + s_ops
        what = ("BF16 table pieces and analysis operands in, FP64 state read, FP64 RK4 accumulator read and written, "
                "next synthesis operands out")
    # DRAM bytes per launch measured by ncu (cold caches) for the T85 x 128 group's kernels, from
    # profiles/split_kernels_t85x128_ensemble.md; the live bench does not run under the profiler
    ncu_traffic = {(85, 1, 1): 66.2e6, (85, 2, 1): 107.1e6} if args.precision == "split3" else {}
    pk = peaks()
    peak = pk.get("hbm_gbs", 6800.0)
    achieved = moved / (kt[gtop][ktop] * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": f"{names[ktop]} at T{T} x {Bm} members", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": ncu_traffic.get((T, ktop, int(direct))),
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch, cold caches "
                                  "(profiles/split_kernels_t85x128_ensemble.md)" if (T, ktop, int(direct)) in ncu_traffic else None,
                "algorithmic_bytes_per_launch": moved, "bytes_counted": what,
                "launch_ms": kt[gtop][ktop],
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy bandwidth), of measured" if "hbm_gbs" in pk else "fallback 6.8 TB/s",
                "stage_kernel_ms": {f"T{groups[g]['truncation']}": dict(zip(["synthesis", "grid", "analysis"], kt[g])) for g in range(len(groups))}}

    # --- accuracy of the headline precision: split vs FP64 on a subset (8 members of each truncation)
    sub = [i for T in (21, 42, 85) for i in [j for j in range(len(tr)) if tr[j] == T][:8]]
    errs = {}
    if args.precision != "fp64":
        f64 = lw.Ensemble([tr[i] for i in sub], [seeds[i] for i in sub], [heights[i] for i in sub], [omegas[i] for i in sub], **prec["fp64"])
        red = lw.Ensemble([tr[i] for i in sub], [seeds[i] for i in sub], [heights[i] for i in sub], [omegas[i] for i in sub],
                          **prec[args.precision])
        f64.run(seconds)
        red.run(seconds)
        hl2, phi = [], []
        for k, i in enumerate(sub):
            T = tr[i]
            nl = 4
            while nl < 3 * T + 1:
                nl *= 2
            a, b_ = np.zeros((nl // 2, nl)), np.zeros((nl // 2, nl))
            lw._check(lib.lmw_ensemble_member_grid(f64._h, k, 0, lw._dp(a), a.size))
            lw._check(lib.lmw_ensemble_member_grid(red._h, k, 0, lw._dp(b_), b_.size))
            hl2.append(float(np.sqrt(((b_ - a) ** 2).mean() / (a ** 2).mean())))
            p64, pr = f64.member_state(k)[2], red.member_state(k)[2]
            phi.append(float(np.abs(pr - p64).max() / np.abs(p64).max()))
        errs = {"vs": "FP64 runs of the same 24 members (8 per truncation), 2 model days", "height_rel_l2_max": max(hl2),
                "height_rel_l2_median": statistics.median(hl2), "phi_normrel_max": max(phi)}
        f64.close()
        red.close()

    # --- the three truncation groups run one after another (an ensemble engine per truncation, each run to the
    # end before the next starts) against the same 1024 members run together, the groups' kernels interleaving
    # on their own streams: what the concurrent form gains over back-to-back launches of each group. Wall time
    # around each synchronised 2-day run, the faster of two, the same way for both forms.
    # (N = 1 only, like the other configurations below: at N > 1 the other ranks would hold their GPUs idle while
    # rank 0 runs them, and the N = 1 line reports them)
    ragged = None
    if rank == 0 and world == 1:
        def wall_run(e, z):
            best = 1e30
            for _ in range(2):
                e.set_states(*z)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                e.run(seconds)
                torch.cuda.synchronize()
                best = min(best, time.perf_counter() - t0)
            return best * 1e3

        per = {}
        for T in (21, 42, 85):
            idx = [i for i in range(len(tr)) if tr[i] == T]
            e1 = lw.Ensemble([tr[i] for i in idx], [seeds[i] for i in idx], [heights[i] for i in idx], [omegas[i] for i in idx],
                             **prec[args.precision])
            z1 = e1.get_states()
            e1.run(seconds)
            per[str(T)] = wall_run(e1, z1)
            e1.close()
        together = wall_run(ens, z0)
        ragged = {"together_ms": together, "back_to_back_ms": sum(per.values()), "per_group_ms": per,
                  "gain": sum(per.values()) / together,
                  "what": "one 2-day run of the 1024 members: the three truncation groups together (one ensemble, the groups' "
                          "launches interleaved on three streams) against each group alone, one after another (wall time, "
                          "synchronised, L2 not flushed)"}

    # --- the other configurations (rank 0, N = 1)
    workloads = []
    if rank == 0 and world == 1:
        workloads = other_workloads(lw, lib, args, ens)

    # --- CPU baseline (rank 0, N = 1): the oracle on every host core, a timed pass of whole member-steps
    cpu = None
    if cpu_pool is not None:
        r = cpu_pool.run(args.ref_seconds)
        cpu_pool.close()
        cpu = {"value": r["value"], "unit": "member-sim-days/s", "cores": cpu_pool.cores, "kind": "port",
               "sample": f"one timed pass of {r['wall_s']:.1f} s on {cpu_pool.cores} cores (oracle port, one process per core): "
                         f"{r['member_steps'][21]} T21, {r['member_steps'][42]} T42 and {r['member_steps'][85]} T85 member-steps executed "
                         f"({r['member_days']:.3f} member-days), in the workload's proportions of member-steps per truncation",
               "member_steps": {str(k): v for k, v in r["member_steps"].items()}}

    # the like-for-like figure: the same ensemble in FP64 on the GPU against the FP64 CPU arm
    like = None
    fp64_value = next((w["value"] for w in workloads if w.get("config") == "3: ensemble in fp64"), None)
    if args.precision == "fp64":
        fp64_value = value
    if cpu is not None and fp64_value:
        like = {"gpu_fp64": fp64_value, "cpu_fp64": cpu["value"], "ratio": fp64_value / cpu["value"], "unit": "member-sim-days/s",
                "what": "the same 1024-member ensemble in FP64 on the GPU (one 2-day run) against the CPU baseline above"}

    clocks = clk.summary()
    if rank == 0:
        cfg = dict(WORKLOAD)
        cfg["precision"] = args.precision
        cfg["groups"] = groups
        cfg["l2"] = "flushed (512 MB write) between timed steps; the working set of a step is L2-resident by design"
        cfg["parallelism"] = f"replicas x{world} (independent ensembles, no collective)" if world > 1 else "single GPU"
        line = {"metric": METRIC, "value": value, "unit": "member-sim-days/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "bf16x%d->f32 Legendre, f32 FFT, f64 state" % (3 if args.precision == "split3" else 6)
                if args.precision.startswith("split") else args.precision,
                "data": "synthetic (seeded balanced turbulence)", "config": cfg,
                "e2e": {"value": e2e, "unit": "member-sim-days/s", "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes},
                "gpu_launches": int(launches), "error": errs, "roofline": roofline, "cpu_baseline": cpu, "like_for_like": like, "clocks": clocks,
                "groups_together_vs_back_to_back": ragged, "workloads": workloads}
        print(json.dumps(line), flush=True)
    ens.close()
    dist.close()
    return 0


def other_workloads(lw, lib, args, ens):
    """Configs 0, 1 and 2 and the ensemble in the other precisions (device-timed with synchronisation)."""
    import numpy as np

    out = []
    if args.quick:
        return out
    # config 0: T42 plain FP64, 480 steps of 900 s (the parity configuration)
    s = lw.Sphere(42, diffusion=nu4(42))
    s.turbulence(1, 8000.0, 30.0, 21)
    st = s.get_state()
    s.run(480 * 900.0, 900.0)
    ts = []
    for _ in range(3):
        s.set_state(*st)
        t0 = time.perf_counter()
        s.run(480 * 900.0, 900.0)
        ts.append(time.perf_counter() - t0)
    out.append({"config": "0: sphere T42 plain FP64, 480 x 900 s", "value": 5.0 / min(ts), "unit": "sim-days/s",
                "parity": "within 1e-12 norm-relative of the reference's own run (tests/test_sphere_gpu.py)",
                "cpu_1core": cpu_single_rate("t42")})
    s.close()
    # config 1: beta-plane 1024 x 512, dt 60 s
    p = lw.Plane(1024, 512, 1024 * 5000.0, 512 * 5000.0, f0=1e-4, beta=1.6e-11, gravity=9.81, depth=100.0)
    p.jet(20.0, 1.0e5, 0.1, 1)
    p.run(64 * 60.0, 60.0)
    p.jet(20.0, 1.0e5, 0.1, 1)
    t0 = time.perf_counter()
    p.run(5000 * 60.0, 60.0)
    el = time.perf_counter() - t0
    out.append({"config": "1: beta-plane 1024 x 512 C-grid FP64, dt 60 s, 5000 steps", "value": 5000 * 60.0 / 86400.0 / el, "unit": "sim-days/s",
                "parity": "bitwise identical to the reference's own 5000-step run (tests/test_plane_gpu.py, SHA-256 of h, u, v)",
                "cpu_1core": cpu_single_rate("plane")})
    p.close()
    # config 2: T170 precision study, 2 model days
    step_note = ("the configuration names 450 s (T170) and 225 s (T341); both exceed the reference's own RK4 limit for this "
                 "state (316 s and 159 s; Sphere::run refuses them, cpp/sphere.cpp:463), so the study steps at 240 s and 150 s")
    res = precision_study(170, 2.0)
    out.append({"config": "2: sphere T170 precision study, 2 model days at 240 s", **res, "deviation": step_note,
                "cpu_1core_fp64": cpu_single_rate("t170", 3.0)})
    res = precision_study(341, 2.0, modes=("fp64", "fp32", "split3", "split6"))
    out.append({"config": "2: sphere T341 precision study, 2 model days at 150 s", **res, "deviation": step_note})
    # config 4: the learned surrogate at T42 (bounded: see surrogate_workload)
    out.append(surrogate_workload(lw))
    # the ensemble in the other precisions (one 2-day run each)
    tr, seeds, heights, omegas = ensemble_specs(0)
    for name, kw in (("fp64", dict(precision=lw.FP64)), ("fp32", dict(precision=lw.FP32)),
                     ("split6", dict(precision=lw.SPLIT_BF16, split_terms=6)), ("split3", dict(precision=lw.SPLIT_BF16, split_terms=3))):
        if name == args.precision:
            continue
        e = lw.Ensemble(tr, seeds, heights, omegas, **kw)
        e.run(3600.0)
        t0 = time.perf_counter()
        e.run(DAYS * 86400.0)
        el = time.perf_counter() - t0
        out.append({"config": f"3: ensemble in {name}", "value": 1024 * DAYS / el, "unit": "member-sim-days/s"})
        e.close()
    return out


def surrogate_workload(lw, trajectories=2560, windows=80, epochs=200, members=1024, rollout_windows=80, member_windows=16,
                       kinetic_weight=0.25, maps=16, averaging=0.9998, drift_trajectories=768, drift_windows=8, drift_epochs=100):
    """Config 4 inside the benchmark: the T42 residual MLP (5676 -> 4096 x 3 -> 5676, GELU, BF16 on tcgen05) trained
    on the configured 204,800 solver pairs (`trajectories` x `windows`; split-precision RK4 data, FP64 state; 6-hour
    windows of 900 s steps, mean height 8000 m) for `epochs` epochs with symmetry-augmented batches, averaged
    weights and the kinetic-energy part of the loss weighted by `kinetic_weight`; then `drift_trajectories` more
    RK4 trajectories that start from states the trained network advanced `drift_windows` windows, and a continued
    fit of `drift_epochs` epochs on all training trajectories (the held-out ones stay held out). Then hybrid
    rollouts of `members` held-out members (the `maps`-map averaged network; split-precision RK4 checking every 4th
    window against the 1e-3 threshold): over the configured 20 days (`rollout_windows`) with FP64 RK4 replacing
    each failed window (the network keeps the member), and over `member_windows` windows with FP64 RK4 taking
    failed members over for good."""
    t0 = time.perf_counter()
    sur = lw.Surrogate(42, hidden=4096, seed=1)
    sur.set_kinetic_weight(kinetic_weight)
    sur.set_averaging(averaging)
    sur.set_symmetry_average(maps)
    gen_s = sur.generate(trajectories, windows, seed0=1_000_000, hmin=8000.0, hmax=8000.0, precision=lw.SPLIT_BF16)
    fit0 = sur.fit(epochs, batch=512, lr=3e-4, lr_min=3e-5, val_fraction=0.1, seed=1, loss="energy")
    gen2_s = sur.generate_drifted(drift_trajectories, drift_windows, seed0=3_000_000, hmin=8000.0, hmax=8000.0, precision=lw.SPLIT_BF16)
    fit = sur.fit(drift_epochs, batch=512, lr=3e-4, lr_min=3e-5, val_fraction=0.1, seed=2, loss="energy")
    fit["seconds"] += fit0["seconds"]
    train_ms, fwd_ms = sur.time(512, 10)
    _, fwd1024 = sur.time(1024, 10)
    sur.set_takeover("window")
    r = sur.rollout(members, seed0=9_000_001, windows=rollout_windows, check_every=4, threshold=1e-3, check_precision=lw.SPLIT_BF16,
                    ref_windows=4, hmin=8000.0, hmax=8000.0)
    sur.set_takeover("member")
    rm = sur.rollout(members, seed0=9_000_001, windows=member_windows, check_every=4, threshold=1e-3, check_precision=lw.SPLIT_BF16,
                     ref_windows=4, hmin=8000.0, hmax=8000.0)
    sur.close()
    fl = 2 * (5676 * 4096 * 2 + 4096 * 4096 * 2)
    return {"config": "4: learned surrogate T42, 6-hour windows (configured training, 20-day rollout)",
            "unit": "member-sim-days/s",
            "network_only": members * 0.25 / (maps * fwd1024 * 1e-3), "network_in_rollout": r["network_rate"],
            "hybrid": r["hybrid_rate"], "plain_rk4_fp64": r["rk4_rate"],
            "speedup_network_vs_rk4": members * 0.25 / (maps * fwd1024 * 1e-3) / r["rk4_rate"],
            "speedup_hybrid_vs_rk4": r["hybrid_rate"] / r["rk4_rate"],
            "takeover": "window: FP64 RK4 replaces each checked window over the threshold, the network keeps the member",
            "window_height_error": {"validation_mean": fit["val_err_mean"], "validation_p90": fit["val_err_p90"],
                                    "persistence_mean": fit["val_persist_mean"], "untrained_mean": fit["val_untrained_mean"],
                                    "rollout_checks_median": r["err_median"], "rollout_checks_p90": r["err_p90"],
                                    "rollout_checks_max": r["err_max"], "rollout_checks_over_threshold": r["frac_over"]},
            "windows_replaced": r["taken_over"], "checks": r["checks"],
            "member_takeover": {"rollout_windows": member_windows, "taken_over": rm["taken_over"], "hybrid": rm["hybrid_rate"],
                                "speedup_hybrid_vs_rk4": rm["hybrid_rate"] / rm["rk4_rate"],
                                "rollout_checks_over_threshold": rm["frac_over"]},
            "threshold": 1e-3, "members": members, "rollout_windows": rollout_windows, "kinetic_weight": kinetic_weight,
            "symmetry_maps_averaged": maps, "weight_averaging": averaging,
            "drift": {"trajectories": drift_trajectories, "network_windows": drift_windows, "epochs": drift_epochs, "generate_s": gen2_s,
                      "validation_mean_before": fit0["val_err_mean"], "validation_p90_before": fit0["val_err_p90"]},
            "pairs": trajectories * windows, "epochs": epochs, "generate_s": gen_s, "train_s": fit["seconds"],
            "train_step_ms_batch512": train_ms, "forward_ms_batch1024": fwd1024,
            "forward_tflops_batch1024": fl * 1024 / (fwd1024 * 1e-3) / 1e12, "wall_s": time.perf_counter() - t0}


# ----------------------------------------------------------------------------------------------- studies and cases
# Step sizes inside the reference's RK4 limit for an 8000 m layer over two days (a 450 s step at T170 exceeds the
# reference's own limit of 316 s for this state, and at 300 s the limit falls below the step on day 2).
STUDY_STEP = {42: 900.0, 85: 450.0, 170: 240.0, 341: 150.0}


def weighted_l2(a, b, w):
    import numpy as np

    wt = w[:, None]
    return float(np.sqrt((wt * (a - b) ** 2).sum() / (wt * b ** 2).sum()))


def precision_study(T: int, days: float, seed: int = 1, modes=("fp64", "fp32", "split3", "split6", "split3_plain", "split6_plain")) -> dict:
    """The same seeded state run in FP64, FP32 and split-BF16 (3 and 6 products per term; the default form adds the
    linear terms of the tendencies in spectral space, outside the BF16 products; the "_plain" form sends every term
    through the BF16 products) for `days`;
    errors against the FP64 run (relative L2 of the height, area-weighted with the Gauss weights; L-infinity;
    relative drift of energy and potential enstrophy) and speeds."""
    import lmweather_gb300 as lw
    import numpy as np

    dt = STUDY_STEP.get(T, 300.0 * 170 / T)
    cfg = {"fp64": dict(precision=lw.FP64), "fp32": dict(precision=lw.FP32),
           "split3": dict(precision=lw.SPLIT_BF16, split_terms=3), "split6": dict(precision=lw.SPLIT_BF16, split_terms=6),
           "split3_plain": dict(precision=lw.SPLIT_BF16, split_terms=3), "split6_plain": dict(precision=lw.SPLIT_BF16, split_terms=6)}
    seconds = days * 86400.0
    out = {"truncation": T, "dt_s": dt, "days": days, "steps": int(round(seconds / dt)), "runs": {}}
    ref = None
    for name in modes:
        s = lw.Sphere(T, diffusion=nu4(T), max_truncation=max(T, 170), **cfg[name])
        if name.endswith("_plain"):
            s.set_split_form(False)
        s.turbulence(seed, 8000.0, 30.0, T // 2)
        mu, w = s.gauss()
        st = s.get_state()
        s.run(64 * dt, dt)  # warm the graphs; the studied span starts from the same state after it
        s.set_state(*st)
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


def run_case(args) -> int:
    """One named workload for a fixed number of RK4 steps (the command that profiler captures wrap): t42 (config-0
    sphere), t85, t170, t341, plane (1024 x 512 beta-plane jet, dt 60 s), ens (an ensemble of --members spheres at
    --truncation, the groups of the benchmark ensemble; --plan forces split plan entries, e.g.
    analysis_stages=1,analysis_ctas_per_sm=3), mlp (training steps of the surrogate's network). One untimed warm-up
    step runs first; the stepped region is bracketed by cudaProfilerStart/Stop, so a profiler run with
    --profile-from-start off captures only its launches."""
    import lmweather_gb300 as lw
    from lmweather_gb300 import build

    build.build()
    if args.case == "plane":
        p = lw.Plane(1024, 512, 1024 * 5000.0, 512 * 5000.0, f0=1e-4, beta=1.6e-11, gravity=9.81, depth=100.0)
        p.jet(20.0, 1.0e5, 0.1, 1)
        p.step(60.0)
        lw.profiler_range(True)
        t0 = time.perf_counter()
        for _ in range(args.case_steps):
            p.step(60.0)
        lw.profiler_range(False)
        print(f"plane 1024x512: {args.case_steps} steps in {time.perf_counter() - t0:.4f} s")
        return 0
    if args.case == "mlp":
        import numpy as np

        rng = np.random.default_rng(1)
        net = lw.Mlp(5676, 4096, 5676, max_batch=args.batch, seed=1, last_layer_scale=0.1)
        x = rng.standard_normal((args.batch, 5676)).astype(np.float32)
        t = 0.1 * rng.standard_normal((args.batch, 5676)).astype(np.float32)
        net.backward(x, t)
        lw.profiler_range(True)
        t0 = time.perf_counter()
        for _ in range(args.case_steps):
            net.backward(x, t)
            net.adam(1e-4)
        lw.profiler_range(False)
        print(f"mlp 5676-4096x3-5676 batch {args.batch}: {args.case_steps} training steps in {time.perf_counter() - t0:.4f} s")
        return 0
    prec = {"fp64": lw.FP64, "fp32": lw.FP32, "split3": lw.SPLIT_BF16, "split6": lw.SPLIT_BF16}[args.precision]
    terms = 6 if args.precision == "split6" else 3
    if args.case == "ens":
        T, B = args.truncation, args.members
        s = lw.Sphere(T, diffusion=nu4(T), precision=prec, members=B, split_terms=terms)
        for b in range(B):
            s.turbulence(b + 1, 5000.0 + 5000.0 * b / B, 30.0, T // 2, member=b)
        if args.plan:
            s.set_split_plan(**{k: int(v) for k, v in (kv.split("=") for kv in args.plan.split(","))})
        if prec == lw.SPLIT_BF16:
            print("plan", s.split_plan())
        dt = 0.9 * min(s.stable_dt(1.5, member=b) for b in range(B))
        s.step(dt)
        lw.profiler_range(True)
        t0 = time.perf_counter()
        for _ in range(args.case_steps):
            s.step(dt)
        lw.profiler_range(False)
        print(f"ensemble T{T} x {B}: {args.case_steps} steps in {time.perf_counter() - t0:.4f} s")
        return 0
    T = {"t42": 42, "t85": 85, "t170": 170, "t341": 341}[args.case]
    dt = STUDY_STEP[T]
    s = lw.Sphere(T, diffusion=nu4(T), precision=prec, max_truncation=max(T, 170), split_terms=terms)
    s.turbulence(1, 8000.0, 30.0, T // 2)
    s.step(dt)
    lw.profiler_range(True)
    t0 = time.perf_counter()
    for _ in range(args.case_steps):
        s.step(dt)
    lw.profiler_range(False)
    print(f"sphere T{T}: {args.case_steps} steps in {time.perf_counter() - t0:.4f} s")
    return 0


def surrogate_study(truncation=42, hidden=4096, trajectories=2560, windows=80, epochs=100, batch=512, lr=3e-4, lr_min=3e-5,
                    hmin=8000.0, hmax=8000.0, members=1024, rollout_windows=80, check_every=4, threshold=1e-3, ref_windows=4, seed=1,
                    check_precision=None, loss="energy", thresholds=(), clip=2.0, data_precision=0, augment=True, averaging=0.9995,
                    sym_average=8, kinetic_weight=1.0, takeovers=("member",), drift_trajectories=0, drift_windows=8, drift_epochs=50) -> dict:
    """The learned surrogate end to end: solver trajectories (balanced turbulence on training seeds, RK4 at 900 s,
    del^4 with a 1-day e-folding at n = T; pairs (state, state + 6 h) from every window; the last tenth of the
    trajectories held out) -> training on the GPU -> validation errors per 6-hour window -> a hybrid rollout of
    held-out members in which RK4 checks every `check_every`-th window and takes members over, timed against plain
    FP64 RK4 on the same members. Errors: relative L2 of the height grid over one window (area-weighted, from the
    Phi coefficients) against RK4 from the same start state."""
    import lmweather_gb300 as lw

    if check_precision is None:
        check_precision = lw.SPLIT_BF16
    sur = lw.Surrogate(truncation, hidden=hidden, seed=seed)
    sur.set_clip(clip)
    sur.set_augment(augment)
    sur.set_averaging(averaging)
    sur.set_symmetry_average(sym_average)
    sur.set_kinetic_weight(kinetic_weight)
    gen_s = sur.generate(trajectories, windows, seed0=1_000_000 * seed, hmin=hmin, hmax=hmax, precision=data_precision)
    fit = sur.fit(epochs, batch=batch, lr=lr, lr_min=lr_min, val_fraction=0.1, seed=seed, loss=loss)
    drift = None
    if drift_trajectories > 0:
        # more training trajectories from states the trained network advanced drift_windows windows, then a
        # continued fit on all training trajectories (the held-out validation trajectories stay the same)
        gen2 = sur.generate_drifted(drift_trajectories, drift_windows, seed0=3_000_000 * seed, hmin=hmin, hmax=hmax, precision=data_precision)
        fit2 = sur.fit(drift_epochs, batch=batch, lr=lr, lr_min=lr_min, val_fraction=0.1, seed=seed + 1, loss=loss)
        drift = {"trajectories": drift_trajectories, "network_windows": drift_windows, "epochs": drift_epochs, "generate_s": gen2,
                 "fit_before": fit}
        fit = fit2
    hist_loss, _ = sur.history()
    train_ms, fwd_ms = sur.time(batch, 10)
    out = {"truncation": truncation, "features": sur.features, "hidden": hidden, "pairs": trajectories * windows,
           "trajectories": trajectories, "windows_per_trajectory": windows, "mean_height_range_m": [hmin, hmax],
           "data_precision": ["fp64", "fp32", "split3"][data_precision], "generate_s": gen_s, "loss": loss, "clip_ratio": clip,
           "epochs": epochs, "lr": [lr, lr_min], "fit": fit, "loss_by_epoch": [round(v, 4) for v in hist_loss.tolist()],
           "train_step_ms": train_ms, "forward_ms_batch": fwd_ms, "batch": batch, "augment": augment, "averaging": averaging,
           "symmetry_maps_averaged": sym_average, "kinetic_weight": kinetic_weight, "drift": drift,
           "check_precision": ["fp64", "fp32", "split3"][check_precision]}
    if members > 0 and rollout_windows > 0:
        for tk in takeovers:
            # "member": RK4 takes a failed member over for good; "window": RK4 replaces the failed window only
            sur.set_takeover(tk)
            key = "rollout" if tk == takeovers[0] else f"rollout_{tk}"
            r = sur.rollout(members, seed0=9_000_000 + seed, windows=rollout_windows, check_every=check_every, threshold=threshold,
                            check_precision=check_precision, ref_windows=ref_windows, hmin=hmin, hmax=hmax)
            r["speedup_hybrid_vs_rk4"] = r["hybrid_rate"] / r["rk4_rate"]
            r["speedup_network_vs_rk4"] = r["network_rate"] / r["rk4_rate"]
            out[key] = dict(takeover=tk, members=members, windows=rollout_windows, check_every=check_every, threshold=threshold, **r)
            sweep = []
            for th in thresholds:
                q = sur.rollout(members, seed0=9_000_000 + seed, windows=rollout_windows, check_every=check_every, threshold=th,
                                check_precision=check_precision, ref_windows=ref_windows, hmin=hmin, hmax=hmax)
                sweep.append({"threshold": th, "taken_over": q["taken_over"], "err_mean": q["err_mean"], "err_max": q["err_max"],
                              "speedup_hybrid_vs_rk4": q["hybrid_rate"] / q["rk4_rate"]})
            if sweep:
                out["threshold_sweep" if tk == takeovers[0] else f"threshold_sweep_{tk}"] = sweep
    sur.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="split3", choices=["split3", "split6", "fp32", "fp64"])
    ap.add_argument("--quick", action="store_true", help="skip the other configurations")
    ap.add_argument("--ref-seconds", type=float, default=12.0, help="wall seconds of one timed CPU pass")
    # a named workload for profiler captures, instead of the benchmark
    ap.add_argument("--case", choices=["t42", "t85", "t170", "t341", "plane", "ens", "mlp"])
    ap.add_argument("--case-steps", type=int, default=4)
    ap.add_argument("--truncation", type=int, default=85)
    ap.add_argument("--members", type=int, default=128)
    ap.add_argument("--batch", type=int, default=512)
    ap.add_argument("--plan", default="", help="split plan entries to force in the ens case")
    # a study, instead of the benchmark: the precision study (--truncation, --days) or the surrogate end to end
    ap.add_argument("--study", choices=["precision", "surrogate"])
    ap.add_argument("--days", type=float, default=2.0)
    ap.add_argument("--trajectories", type=int, default=2560)
    ap.add_argument("--windows", type=int, default=80)
    ap.add_argument("--epochs", type=int, default=300)
    ap.add_argument("--rollout-windows", type=int, default=80)
    ap.add_argument("--rollout-members", type=int, default=1024)
    ap.add_argument("--threshold", type=float, default=1e-3)
    ap.add_argument("--check-precision", default="split3", choices=["fp64", "split3"])
    ap.add_argument("--sweep", default="", help="comma-separated extra take-over thresholds")
    ap.add_argument("--augment", type=int, default=1, help="symmetry augmentation of the training pairs (1/0)")
    ap.add_argument("--averaging", type=float, default=0.9998, help="weight averaging decay (0: last weights)")
    ap.add_argument("--sym-average", type=int, default=16, help="symmetry maps averaged at inference (1: plain network)")
    ap.add_argument("--kinetic-weight", type=float, default=0.25, help="weight of the kinetic-energy part of the loss")
    ap.add_argument("--takeover", default="window,member", help="rollout takeover modes to run (window: RK4 replaces a failed window; "
                    "member: RK4 keeps a failed member)")
    ap.add_argument("--lr-min", type=float, default=3e-5)
    ap.add_argument("--drift-trajectories", type=int, default=768, help="training trajectories added from network-advanced states")
    ap.add_argument("--drift-windows", type=int, default=8, help="network windows before those trajectories start")
    ap.add_argument("--drift-epochs", type=int, default=100, help="epochs of the continued fit after adding them")
    ap.add_argument("--data-precision", default="split3", choices=["fp64", "split3"])
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.case:
        return run_case(args)
    if args.study:
        from lmweather_gb300 import build

        build.build()
        if args.study == "precision":
            print(json.dumps(precision_study(args.truncation, args.days)))
        else:
            import lmweather_gb300 as lw

            print(json.dumps(surrogate_study(42, trajectories=args.trajectories, windows=args.windows, epochs=args.epochs, batch=args.batch,
                                             lr_min=args.lr_min, members=args.rollout_members, rollout_windows=args.rollout_windows,
                                             threshold=args.threshold, check_precision=lw.SPLIT_BF16 if args.check_precision == "split3" else lw.FP64,
                                             thresholds=tuple(float(v) for v in args.sweep.split(",") if v), augment=bool(args.augment),
                                             averaging=args.averaging, data_precision=2 if args.data_precision == "split3" else 0,
                                             sym_average=args.sym_average, kinetic_weight=args.kinetic_weight,
                                             takeovers=tuple(args.takeover.split(",")), drift_trajectories=args.drift_trajectories,
                                             drift_windows=args.drift_windows, drift_epochs=args.drift_epochs)))
        return 0
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_ours(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
