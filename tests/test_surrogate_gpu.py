"""Learned surrogate on the GPU: the tcgen05 BF16 GEMM, the network's forward and backward passes and Adam against
the CPU oracle (oracle/mlp_oracle.py), training on solver trajectories and the hybrid rollout's RK4 checks and
takeovers."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import mlp_oracle as mo  # noqa: E402

pytestmark = pytest.mark.gpu


def normrel(a, b):
    return float(np.abs(np.asarray(a, np.float64) - b).max() / max(1e-300, np.abs(b).max()))


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 384, 320), (1280, 4096, 128)])
def test_gemm_bf16_against_fp64(engine, M, N, K):
    rng = np.random.default_rng(M + N + K)
    a = rng.standard_normal((M, K)).astype(np.float32)
    b = rng.standard_normal((N, K)).astype(np.float32)
    c = engine.gemm_bf16(a, b)
    want = mo.bf16(a).astype(np.float64) @ mo.bf16(b).astype(np.float64).T
    # FP32 accumulation of K products of BF16 values
    assert np.abs(c - want).max() <= 1e-5 * np.sqrt(K) * np.abs(want).max()


def small_net(engine, din=200, hidden=256, dout=150, seed=3):
    rng = np.random.default_rng(seed)
    shapes = [(hidden, din), (hidden, hidden), (hidden, hidden), (dout, hidden)]
    W = [(rng.standard_normal(s) / np.sqrt(s[1])).astype(np.float32) for s in shapes]
    b = [(0.1 * rng.standard_normal(s[0])).astype(np.float32) for s in shapes]
    net = engine.Mlp(din, hidden, dout, max_batch=256, seed=seed)
    for l in range(4):
        net.set_layer(l, W[l], b[l])
    return net, W, b, rng


def test_forward_backward_against_oracle(engine):
    net, W, b, rng = small_net(engine)
    x = rng.standard_normal((128, 200)).astype(np.float32)
    t = rng.standard_normal((128, 150)).astype(np.float32)
    mask = ((rng.random(150) > 0.2) * rng.uniform(0.5, 2.0, 150)).astype(np.float32)
    y = net.forward(x)
    loss_o, y_o, grads_o = mo.loss_and_backward(W, b, x, t, mask)
    # BF16 activations: a rounding flip moves one activation by one BF16 ulp (2^-8 relative)
    assert normrel(y, y_o) < 2e-3
    loss = net.backward(x, t, mask)
    assert abs(loss - loss_o) < 2e-3 * loss_o
    for l in range(4):
        gw, gb = net.grad(l)
        assert normrel(gw, grads_o[l][0]) < 2e-2, l
        assert normrel(gb, grads_o[l][1]) < 2e-2, l
    # gradients of masked outputs are exactly zero
    gw3, gb3 = net.grad(3)
    assert np.all(gw3[mask == 0] == 0) and np.all(gb3[mask == 0] == 0)


def test_adam_against_oracle(engine):
    net, W, b, rng = small_net(engine, seed=4)
    x = rng.standard_normal((256, 200)).astype(np.float32)
    t = rng.standard_normal((256, 150)).astype(np.float32)
    net.backward(x, t)
    grads = [net.grad(l) for l in range(4)]
    net.adam(lr=1e-3)
    for l in range(4):
        w1, b1 = net.get_layer(l)
        wo, _, _ = mo.adam_step(W[l], np.zeros_like(W[l]), np.zeros_like(W[l]), grads[l][0], 1, 1e-3)
        bo, _, _ = mo.adam_step(b[l], np.zeros_like(b[l]), np.zeros_like(b[l]), grads[l][1], 1, 1e-3)
        assert np.abs(w1 - wo).max() < 1e-6
        assert np.abs(b1 - bo).max() < 1e-6


def test_training_fits_a_smooth_map(engine):
    rng = np.random.default_rng(11)
    A = (rng.standard_normal((64, 96)) / np.sqrt(96)).astype(np.float32)
    x = rng.standard_normal((1024, 96)).astype(np.float32)
    t = np.tanh(x @ A.T).astype(np.float32)
    net = engine.Mlp(96, 256, 64, max_batch=256, seed=2, last_layer_scale=0.1)
    first = None
    for it in range(400):
        s = (it % 4) * 256
        loss = net.backward(x[s:s + 256], t[s:s + 256])
        first = loss if first is None else first
        net.adam(lr=1e-3)
    assert loss < first / 10


@pytest.fixture(scope="module")
def trained(engine):
    sur = engine.Surrogate(21, hidden=512, seed=7)
    sur.generate(256, 16, seed0=100, hmin=8000.0, hmax=8000.0)
    stats = sur.fit(20, batch=128, lr=1e-3, lr_min=1e-4, val_fraction=0.125, seed=3)
    return sur, stats


def test_surrogate_gains_over_persistence_and_untrained(trained):
    sur, st = trained
    assert sur.features == 6 * 22 * 23 // 2
    # the trained network is far closer to RK4 over one window than the state left unchanged, and than the
    # network before training
    assert st["val_err_mean"] < 0.75 * st["val_persist_mean"]
    assert st["val_err_mean"] < 0.75 * st["val_untrained_mean"]


def test_advance_keeps_mass_and_is_per_member(trained, engine):
    sur, _ = trained
    # members advanced through the public entry point keep their mass (the Phi (0,0) coefficient) exactly
    s = engine.Sphere(21, diffusion=6.37122e6 ** 4 / (86400.0 * (21 * 22) ** 2))
    s.turbulence(seed=5, mean_height=7000.0, max_wind=30.0, nforce=10)
    z, d, f = s.get_state()
    T = 21
    packed = []
    for fld in (z, d, f):
        for m in range(T + 1):
            for n in range(m, T + 1):
                c = fld[m * (T + 1) + n]
                packed += [c.real, c.imag]
    st = np.array([packed, packed])
    out = sur.advance(st)
    phi00 = 2 * 2 * (T + 1) * (T + 2) // 2
    assert out[0, phi00] == st[0, phi00]
    assert np.array_equal(out[0], out[1])
    assert not np.array_equal(out[0], st[0])


def _packed_map(st, T, quarter_turns, reflect):
    """The symmetry map of packed states [member][6 ntri] (zeta, delta, Phi; (m, n) in triangle order, re/im):
    rotation by quarter_turns x 90 degrees about the polar axis (coefficient times i^(m quarter_turns)), then the
    equatorial reflection (Phi, delta times (-1)^(n-m), zeta times -(-1)^(n-m))."""
    out = st.copy()
    ntri = (T + 1) * (T + 2) // 2
    for q in range(3):
        tri = 0
        for m in range(T + 1):
            for n in range(m, T + 1):
                f = (q * ntri + tri) * 2
                c = (st[:, f] + 1j * st[:, f + 1]) * (1j ** ((m * quarter_turns) % 4))
                if reflect:
                    c = c * ((-1.0) ** (n - m)) * (-1.0 if q == 0 else 1.0)
                out[:, f], out[:, f + 1] = c.real, c.imag
                tri += 1
    return out


def test_symmetry_averaged_network_is_equivariant(trained, engine):
    # with the increments averaged over the eight maps {0, 90, 180, 270 degrees} x {no reflection, reflection},
    # advancing a mapped state gives the mapped advance of the state (up to the order of the FP32 sums), as the
    # exact dynamics do; the plain network (one map) is not equivariant
    sur, _ = trained
    T = 21
    s = engine.Sphere(T, diffusion=6.37122e6 ** 4 / (86400.0 * (T * (T + 1)) ** 2), members=2)
    for b in range(2):
        s.turbulence(seed=11 + b, mean_height=8000.0, max_wind=30.0, nforce=10, member=b)
    rows = []
    for b in range(2):
        z, d, f = s.get_state(member=b)
        packed = []
        for fld in (z, d, f):
            for m in range(T + 1):
                for n in range(m, T + 1):
                    c = fld[m * (T + 1) + n]
                    packed += [c.real, c.imag]
        rows.append(packed)
    st = np.array(rows)
    for maps, tol in ((8, 1e-5), (1, None)):
        sur.set_symmetry_average(maps)
        base = sur.advance(st)
        inc = base - st
        for qt, rf in ((1, False), (2, True), (3, True)):
            got = sur.advance(_packed_map(st, T, qt, rf)) - _packed_map(st, T, qt, rf)
            want = _packed_map(inc, T, qt, rf)
            rel = np.abs(got - want).max() / np.abs(want).max()
            if tol is not None:
                assert rel < tol, (qt, rf, rel)
            else:
                assert rel > 1e-4, (qt, rf, rel)
    sur.set_symmetry_average(8)


@pytest.mark.parametrize("check,takeover", [("fp64", "member"), ("split3", "member"), ("split3", "window")])
def test_rollout_takeover_semantics(trained, engine, check, takeover):
    sur, _ = trained
    # threshold 0 and a check every window: every member is taken over at the first check (member mode), or every
    # window of every member is replaced (window mode), so the hybrid is plain FP64 RK4 (a split-precision check is
    # only decides: the window of a member it takes over is recomputed in FP64)
    cp = engine.FP64 if check == "fp64" else engine.SPLIT_BF16
    sur.set_takeover(takeover)
    r0 = sur.rollout(8, seed0=900, windows=3, check_every=1, threshold=0.0, ref_windows=1, hmin=7000.0, hmax=7000.0, with_states=True,
                     check_precision=cp)
    assert r0["taken_over"] == (8 if takeover == "member" else 24) and r0["checks"] == 3 and r0["frac_over"] == 1.0
    # a plain RK4 run of the same members ends in the same states bit for bit
    T = 21
    ref = engine.Sphere(T, diffusion=6.37122e6 ** 4 / (86400.0 * (T * (T + 1)) ** 2), members=8)
    for j in range(8):
        ref.turbulence(seed=900 + j, mean_height=7000.0, max_wind=30.0, nforce=T // 2, member=j)
    ref.run(3 * 21600.0, 900.0)
    for j in range(8):
        z, d, f = ref.get_state(member=j)
        packed = []
        for fld in (z, d, f):
            for m in range(T + 1):
                for n in range(m, T + 1):
                    c = fld[m * (T + 1) + n]
                    packed += [c.real, c.imag]
        assert np.array_equal(r0["final_states"][j], np.array(packed))
    # an unreachable threshold takes nobody over and the per-window errors are recorded
    r1 = sur.rollout(8, seed0=900, windows=4, check_every=2, threshold=1e9, ref_windows=1, with_errors=True)
    assert r1["taken_over"] == 0 and r1["checks"] == 2
    assert r1["window_errors"].shape == (2, 8) and np.all(r1["window_errors"] > 0)
    assert r1["hybrid_rate"] > 0 and r1["rk4_rate"] > 0
    sur.set_takeover("member")
    with pytest.raises(ValueError):
        sur.set_takeover("never")


def test_drifted_trajectories_keep_the_held_out_set(engine):
    # trajectories started from network-advanced states go before the existing ones: the held-out validation
    # trajectories of the first fit stay the same, so the same network scores the same validation error
    sur = engine.Surrogate(21, hidden=256, seed=5)
    sur.generate(40, 4, seed0=300, hmin=8000.0, hmax=8000.0)
    st = sur.fit(2, batch=128, lr=1e-3, lr_min=1e-4, val_fraction=0.1, seed=2)
    sur.generate_drifted(24, 2, seed0=700, hmin=8000.0, hmax=8000.0)
    again = sur.fit(0, batch=128, val_fraction=0.1, seed=3)
    assert again["val_err_mean"] == pytest.approx(st["val_err_mean"], rel=1e-9)
    # and a continued fit trains on the larger set
    more = sur.fit(2, batch=128, lr=1e-3, lr_min=1e-4, val_fraction=0.1, seed=4)
    assert np.isfinite(more["val_err_mean"]) and more["val_err_mean"] > 0
    with pytest.raises(ValueError):
        engine.Surrogate(21, hidden=256, seed=6).generate_drifted(8, 1)
    sur.close()


def test_member_takeovers_at_several_checks(trained, engine):
    # members taken over at different checks join one FP64 engine; each member is taken over at its first check
    # above the threshold (the network members' window errors do not depend on who was taken over before)
    sur, _ = trained
    sur.set_takeover("member")
    kw = dict(seed0=1300, windows=4, check_every=1, ref_windows=1, hmin=7000.0, hmax=7000.0, check_precision=engine.SPLIT_BF16)
    r1 = sur.rollout(8, threshold=1e9, with_errors=True, **kw)
    err = r1["window_errors"]
    assert np.all(err > 0)
    # a threshold between the members' errors, so that members are taken over at different checks
    th = float(np.median(err))
    over = err > th
    when = [int(np.argmax(over[:, b])) if over[:, b].any() else -1 for b in range(8)]
    r2 = sur.rollout(8, threshold=th, with_states=True, **kw)
    assert r2["taken_over"] == sum(w >= 0 for w in when)
    assert np.all(np.isfinite(r2["final_states"]))
