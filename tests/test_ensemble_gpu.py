"""Mixed-truncation ensembles: every member equals the same sphere stepped on its own (same step size), and a
member's guard failure stops the run with the reference's message."""
import numpy as np
import pytest

from oracle_lib import OracleSphere

pytestmark = pytest.mark.gpu

A = 6.37122e6


def nu4(T):
    return A ** 4 / (86400.0 * (T * (T + 1.0)) ** 2)


def test_ensemble_members_match_single_runs(engine):
    tr = [21, 10, 21, 42, 21, 42]
    seeds = [11, 12, 13, 14, 15, 16]
    heights = [6000.0, 7000.0, 9000.0, 8000.0, 5500.0, 9500.0]
    omegas = [7.292e-5 * f for f in (0.5, 1.0, 2.0, 1.0, 0.5, 2.0)]
    ens = engine.Ensemble(tr, seeds, heights, omegas)
    ens.run(6 * 3600.0)
    groups = {g["truncation"]: g for g in ens.groups()}
    assert sorted(groups) == [10, 21, 42] and groups[21]["members"] == 3
    for i, T in enumerate(tr):
        s = engine.Sphere(T, omega=omegas[i], diffusion=nu4(T))
        s.turbulence(seeds[i], heights[i], 30.0, T // 2)
        s.run(6 * 3600.0, groups[T]["dt"])
        for a, b in zip(ens.member_state(i), s.get_state()):
            scale = np.abs(b).max()
            assert np.abs(a - b).max() <= 1e-13 * scale
        assert ens.member_diagnostics(i)["mean_height"] == pytest.approx(heights[i], rel=1e-12)  # the recipe's mean


def test_ensemble_members_against_oracle(engine, oracle_built):
    # one member of each truncation of the benchmark ensemble, with the rotation rate scaled by 0.5 or 2 and mean
    # heights other than 8000 m, against the oracle (the reference's algorithm in C, bitwise equal to it) from the
    # member's initial state at the group's own step, for at least 64 steps of every group
    tr = [85, 21, 42]
    seeds = [7001, 7002, 7003]
    heights = [6300.0, 9400.0, 5200.0]
    omegas = [7.292e-5 * 2.0, 7.292e-5 * 0.5, 7.292e-5 * 2.0]
    ens = engine.Ensemble(tr, seeds, heights, omegas, precision=engine.FP64)
    start = [ens.member_state(i) for i in range(3)]
    whole = ens.get_states()
    ens.run(86400.0)  # a day at the groups' stable steps (each run takes them from the current states)
    seconds = 65 * {g["truncation"]: g for g in ens.groups()}[21]["dt"]
    ens.set_states(*whole)
    ens.run(seconds)
    groups = {g["truncation"]: g for g in ens.groups()}
    assert all(g["steps"] >= 64 for g in groups.values()), groups
    for i, T in enumerate(tr):
        o = OracleSphere(T, omega=omegas[i], diffusion=nu4(T))
        o.set_state(*start[i])
        o.run(seconds, groups[T]["dt"])
        got, ref = ens.member_state(i), o.get_state()
        wind = max(np.abs(ref[0]).max(), np.abs(ref[1]).max())
        ez, ed = np.abs(got[0] - ref[0]).max() / wind, np.abs(got[1] - ref[1]).max() / wind
        ef = np.abs(got[2] - ref[2]).max() / np.abs(ref[2]).max()
        print(f"T{T} member vs oracle after {groups[T]['steps']} steps: zeta {ez:.2e} delta {ed:.2e} Phi {ef:.2e}")
        assert ez <= 1e-12 and ed <= 1e-12 and ef <= 1e-12, (T, ez, ed, ef)
        assert ens.member_diagnostics(i)["energy"] == pytest.approx(o.diagnostics()["energy"], rel=1e-12)


def test_ensemble_split_precision_close_to_fp64(engine):
    tr = [42] * 20 + [21] * 5
    rng = np.random.default_rng(3)
    seeds = list(range(100, 125))
    heights = list(rng.uniform(5000.0, 10000.0, 25))
    omegas = [7.292e-5 * (0.5, 1.0, 2.0)[i % 3] for i in range(25)]
    ref = engine.Ensemble(tr, seeds, heights, omegas, precision=engine.FP64)
    spl = engine.Ensemble(tr, seeds, heights, omegas, precision=engine.SPLIT_BF16, split_terms=6)
    ref.run(6 * 3600.0)
    spl.run(6 * 3600.0)
    worst = 0.0
    for i in range(25):
        f64, fsp = ref.member_state(i)[2], spl.member_state(i)[2]
        worst = max(worst, np.abs(fsp - f64).max() / np.abs(f64).max())
    print(f"ensemble split (6 terms) vs FP64 after 6 h: worst Phi norm-relative {worst:.2e}")
    assert worst < 1e-6


@pytest.mark.parametrize("precision", ["fp64", "split3"])
def test_whole_ensemble_state_io(engine, precision):
    """get_states / set_states (one copy per run of members of one truncation, layout conversion on the device)
    equal the per-member calls bit for bit, with members of different truncations interleaved; a restart from
    get_states continues exactly like the uninterrupted run."""
    kw = dict(precision=engine.FP64) if precision == "fp64" else dict(precision=engine.SPLIT_BF16, split_terms=3)
    tr = [21, 42, 21, 21, 10, 42, 42, 21]
    seeds = [31 + i for i in range(len(tr))]
    heights = [5000.0 + 600.0 * i for i in range(len(tr))]
    omegas = [7.292e-5 * (0.5, 1.0, 2.0)[i % 3] for i in range(len(tr))]
    ens = engine.Ensemble(tr, seeds, heights, omegas, **kw)
    ens.run(3 * 3600.0)
    z, d, f = ens.get_states()
    off = 0
    for i, T in enumerate(tr):
        mm = (T + 1) ** 2
        for a, b in zip(ens.member_state(i), (z[off:off + mm], d[off:off + mm], f[off:off + mm])):
            assert np.array_equal(a, b)
        off += mm
    assert off == ens.state_size()
    # restart: a second ensemble given these states continues exactly like the first
    other = engine.Ensemble(tr, [s + 1000 for s in seeds], heights, omegas, **kw)
    other.set_states(z, d, f)
    for i in range(len(tr)):
        for a, b in zip(ens.member_state(i), other.member_state(i)):
            assert np.array_equal(a, b)
    ens.run(3 * 3600.0)
    other.run(3 * 3600.0)
    for a, b in zip(ens.get_states(), other.get_states()):
        assert np.array_equal(a, b)
    with pytest.raises(ValueError, match="state_size"):
        ens.set_states(z[:-1], d, f)
