"""The multi-GPU path is replicas only (members are independent): each rank steps its own 1024-member ensemble and
the benchmark takes the max over ranks of the device time. These tests cover that host logic on CPU with two gloo
ranks: the barrier and max-over-ranks reduction, the per-rank member specs, and the reference arm's rank rule."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench

    d = bench.Dist(world, "gloo")
    d.barrier()
    out[rank] = d.max(10.0 + rank)
    d.close()


def test_max_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    port = _free_port()
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        assert out[0] == 11.0 and out[1] == 11.0


def test_replica_specs_differ_by_rank_only_in_seeds_and_heights():
    import bench

    t0, s0, h0, o0 = bench.ensemble_specs(0)
    t1, s1, h1, o1 = bench.ensemble_specs(1)
    assert t0 == t1 and o0 == o1 and len(t0) == 1024
    assert sorted(t0).count(21) == 512 and t0.count(42) == 384 and t0.count(85) == 128
    assert not set(s0) & set(s1)
    assert h0 != h1 and all(5000.0 <= h <= 10000.0 for h in h0 + h1)


def test_reference_arm_runs_on_rank_zero_only():
    import argparse

    import bench

    args = argparse.Namespace(steps=1, warmup=0)
    assert bench.run_reference(args, rank=1, world=2) == 0


@pytest.mark.parametrize("config", ["t42", "plane"])
def test_single_config_cpu_timing(config):
    """The 1-core CPU figure beside configs 0 and 1: the oracle port stepping the seeded state, a bounded sample."""
    import bench

    bench.build_oracle()
    r = bench.cpu_single_rate(config, budget_s=0.05)
    assert r["cores"] == 1 and r["kind"] == "port" and r["unit"] == "sim-days/s"
    assert r["value"] > 0 and "RK4 steps" in r["sample"]


def test_reference_arm_line_keeps_the_contract():
    """`bench.py --impl reference` times the oracle port on the host's cores and prints one JSON line with the
    benchmark's keys: the metric and unit of the GPU arm, a timed cpu_baseline and an e2e figure without copies."""
    import json
    import subprocess

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0",
                          "--ref-seconds", "0.5"], capture_output=True, text=True, timeout=600, cwd=root)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads([l for l in out.stdout.splitlines() if l.startswith("{")][-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling", "dtype", "config"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1 and line["cpu_baseline"]["sample"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
