"""The surrogate network's CPU oracle pinned on its own terms (the reference has no learned component): the analytic
backward pass against central finite differences of the forward pass in float64, BF16 rounding against known
values, Adam against its closed form on a scalar, and the host-side argument checks of the network entry points."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import mlp_oracle as mo  # noqa: E402


def test_backward_matches_finite_differences():
    for seed in range(3):
        assert mo.finite_difference_check(np.random.default_rng(seed), probes=40) < 1e-6


def test_bf16_rounding_known_values():
    x = np.array([1.0, 1.00390625, 1.005859375, 1.01171875, -2.0, 3.0e-39, 65280.0, 65408.0], np.float32)
    want = np.array([1.0, 1.0, 1.0078125, 1.015625, -2.0, 2.9842e-39, 65280.0, 65536.0], np.float32)
    got = mo.bf16(x)
    assert np.allclose(got[:5], want[:5], rtol=0, atol=0)
    assert got[6] == 65280.0 and got[7] == 65536.0
    # every result is a BF16 value: the low 16 bits are zero
    assert not np.any(got.view(np.uint32) & 0xFFFF)


def test_adam_scalar_closed_form():
    # first step of Adam moves every weight by lr * sign(g) (up to eps)
    w, m, v = np.ones(3, np.float32), np.zeros(3, np.float32), np.zeros(3, np.float32)
    g = np.array([0.5, -2.0, 1e-3], np.float32)
    w1, m1, v1 = mo.adam_step(w, m, v, g, 1, 1e-2)
    assert np.allclose(w1, 1.0 - 1e-2 * np.sign(g), rtol=0, atol=1e-6)
    assert np.allclose(m1, 0.1 * g) and np.allclose(v1, 0.001 * g * g)


def test_rounded_and_exact_modes_agree_to_bf16_precision():
    rng = np.random.default_rng(5)
    W = [rng.standard_normal(s).astype(np.float32) / np.sqrt(s[1]) for s in [(64, 40), (64, 64), (64, 64), (30, 64)]]
    b = [np.zeros(s.shape[0], np.float32) for s in W]
    x = rng.standard_normal((16, 40)).astype(np.float32)
    ye, _ = mo.forward(W, b, x, exact=True)
    yr, _ = mo.forward(W, b, x, exact=False)
    rel = np.abs(ye - yr).max() / np.abs(ye).max()
    assert 1e-4 < rel < 5e-2


def test_network_entry_points_check_arguments(engine):
    lib = engine.load_library()
    assert lib.lmw_mlp_forward(None, None, 128, None) == 1
    assert "null network" in lib.lmw_last_error().decode()
    assert lib.lmw_surrogate_fit(None, 1, 128, 1e-3, 1e-4, 0.1, 1, 1, None) == 1
    assert "null surrogate" in lib.lmw_last_error().decode()
    with pytest.raises((ValueError, RuntimeError)):
        engine.Mlp(10, 100, 10)  # hidden width not a multiple of 128 (or no device)
