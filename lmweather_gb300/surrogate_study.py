"""The learned surrogate end to end (T42 by default): solver trajectories -> training on the GPU -> validation
errors per 6-hour window -> a hybrid rollout of held-out members in which plain RK4 checks every 4th window and
takes members over, timed against plain RK4 on the same members.

    python -m lmweather_gb300.surrogate_study --trajectories 2560 --windows 80 --epochs 40

Training data: balanced turbulence (nforce = T/2, 30 m/s, n^-3 kinetic-energy spectrum) on training seeds, run by
FP64 RK4 at dt = 900 s with del^4 diffusion of a 1-day e-folding at n = T; pairs (state, state + 6 h) from every
window of every trajectory; the last tenth of the trajectories is held out for validation. The rollout members
use seeds no trajectory used. Errors: relative L2 of the height grid over one window (area-weighted, from the Phi
coefficients), against RK4 from the same start state.
"""
from __future__ import annotations

import argparse
import json

import numpy as np


def study(truncation=42, hidden=4096, trajectories=2560, windows=80, epochs=100, batch=512, lr=3e-4, lr_min=3e-5, hmin=8000.0,
          hmax=8000.0, members=1024, rollout_windows=80, check_every=4, threshold=1e-3, ref_windows=4, seed=1,
          check_precision=0, loss="energy", thresholds=(), clip=2.0, data_precision=0) -> dict:
    import lmweather_gb300 as lw

    sur = lw.Surrogate(truncation, hidden=hidden, seed=seed)
    sur.set_clip(clip)
    gen_s = sur.generate(trajectories, windows, seed0=1_000_000 * seed, hmin=hmin, hmax=hmax, precision=data_precision)
    fit = sur.fit(epochs, batch=batch, lr=lr, lr_min=lr_min, val_fraction=0.1, seed=seed, loss=loss)
    hist_loss, _ = sur.history()
    train_ms, fwd_ms = sur.time(batch, 10)
    out = {"truncation": truncation, "features": sur.features, "hidden": hidden, "pairs": trajectories * windows,
           "trajectories": trajectories, "windows_per_trajectory": windows, "mean_height_range_m": [hmin, hmax],
           "data_precision": ["fp64", "fp32", "split3"][data_precision], "generate_s": gen_s, "loss": loss, "clip_ratio": clip,
           "epochs": epochs, "lr": [lr, lr_min], "fit": fit, "loss_by_epoch": [round(v, 4) for v in hist_loss.tolist()], "train_step_ms": train_ms, "forward_ms_batch": fwd_ms, "batch": batch}
    if members > 0 and rollout_windows > 0:
        r = sur.rollout(members, seed0=9_000_000 + seed, windows=rollout_windows, check_every=check_every, threshold=threshold,
                        check_precision=check_precision, ref_windows=ref_windows, hmin=hmin, hmax=hmax)
        r["speedup_hybrid_vs_rk4"] = r["hybrid_rate"] / r["rk4_rate"]
        r["speedup_network_vs_rk4"] = r["network_rate"] / r["rk4_rate"]
        out["rollout"] = dict(members=members, windows=rollout_windows, check_every=check_every, threshold=threshold, **r)
        sweep = []
        for th in thresholds:
            try:
                q = sur.rollout(members, seed0=9_000_000 + seed, windows=rollout_windows, check_every=check_every, threshold=th,
                                check_precision=check_precision, ref_windows=ref_windows, hmin=hmin, hmax=hmax)
                sweep.append({"threshold": th, "taken_over": q["taken_over"], "err_mean": q["err_mean"], "err_max": q["err_max"],
                              "speedup_hybrid_vs_rk4": q["hybrid_rate"] / q["rk4_rate"]})
            except (RuntimeError, ValueError) as e:
                sweep.append({"threshold": th, "failed": str(e)})
        if sweep:
            out["threshold_sweep"] = sweep
    sur.close()
    return out


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--truncation", type=int, default=42)
    ap.add_argument("--hidden", type=int, default=4096)
    ap.add_argument("--trajectories", type=int, default=2560)
    ap.add_argument("--windows", type=int, default=80)
    ap.add_argument("--epochs", type=int, default=100)
    ap.add_argument("--batch", type=int, default=512)
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--lr-min", type=float, default=3e-5)
    ap.add_argument("--hmin", type=float, default=8000.0)
    ap.add_argument("--hmax", type=float, default=8000.0)
    ap.add_argument("--members", type=int, default=1024)
    ap.add_argument("--rollout-windows", type=int, default=80)
    ap.add_argument("--check-every", type=int, default=4)
    ap.add_argument("--threshold", type=float, default=1e-3)
    ap.add_argument("--check-precision", type=int, default=0)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--loss", default="energy", choices=["energy", "normalised"])
    ap.add_argument("--sweep", default="", help="comma-separated extra thresholds for rollouts")
    ap.add_argument("--clip", type=float, default=2.0)
    ap.add_argument("--data-precision", type=int, default=0)
    args = ap.parse_args()
    from lmweather_gb300 import build

    build.build()
    print(json.dumps(study(args.truncation, args.hidden, args.trajectories, args.windows, args.epochs, args.batch, args.lr, args.lr_min,
                           args.hmin, args.hmax, args.members, args.rollout_windows, args.check_every, args.threshold, seed=args.seed,
                           check_precision=args.check_precision, loss=args.loss, clip=args.clip, data_precision=args.data_precision,
                           thresholds=tuple(float(v) for v in args.sweep.split(",") if v))))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
