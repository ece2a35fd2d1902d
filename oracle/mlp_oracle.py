"""CPU oracle of the learned surrogate's network (test infrastructure: imported only by tests/).

The reference has no learned component; the surrogate's network is this project's own. This module restates its
arithmetic in numpy so the GPU kernels can be checked against it:

* four fully connected layers in -> h -> h -> h -> out, GELU(z) = z * (1 + erf(z / sqrt 2)) / 2 after the first
  three, the output layer linear;
* BF16 rounding (round to nearest even) exactly where the GPU rounds: the input, the weights, every
  pre-activation Z and activation GELU(Z) (both computed from the FP32 sum), the output gradient and every
  hidden gradient; products and sums in (at least) FP32;
* loss 1/(2 B) sum_b sum_f w_f (y - t)^2 with per-output weights w (0 masks an output), output gradient
  w (y - t) / B;
* Adam (Kingma & Ba 2015) in FP32 with bias corrections 1/(1 - beta^t).

With `exact=True` nothing is rounded and everything is float64: `finite_difference_check` uses that mode to pin
the analytic backward pass to central differences of the forward pass.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

SQRT1_2 = 0.70710678118654752
INV_SQRT_2PI = 0.39894228040143268


def bf16(x) -> np.ndarray:
    """Round float32 values to the nearest BF16 value (ties to even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z * SQRT1_2))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z * SQRT1_2)) + z * INV_SQRT_2PI * np.exp(-0.5 * z * z)


def _r(x, exact):
    return np.asarray(x, np.float64) if exact else bf16(x)


def _mm(a, b):
    """a @ b accumulated in float64 (at least as precise as the tensor cores' FP32 accumulation)."""
    return np.asarray(a, np.float64) @ np.asarray(b, np.float64)


def forward(weights, biases, x, exact=False):
    """weights[l]: [nout][nin]; returns (y, cache)."""
    cast = (lambda v: np.asarray(v, np.float64)) if exact else (lambda v: np.asarray(v, np.float32))
    X = _r(x, exact)
    acts, zs = [X], []
    for l in range(3):
        z = cast(_mm(X, _r(weights[l], exact).T) + biases[l])
        zs.append(_r(z, exact))
        X = _r(cast(gelu(z)), exact)
        acts.append(X)
    y = cast(_mm(X, _r(weights[3], exact).T) + biases[3])
    return y, (acts, zs)


def loss_and_backward(weights, biases, x, target, mask=None, exact=False):
    """Returns (loss, y, [(gW_l, gb_l) for l = 0..3])."""
    cast = (lambda v: np.asarray(v, np.float64)) if exact else (lambda v: np.asarray(v, np.float32))
    y, (acts, zs) = forward(weights, biases, x, exact)
    B = y.shape[0]
    m = np.ones(y.shape[1]) if mask is None else np.asarray(mask, np.float64)
    e = np.asarray(y, np.float64) - np.asarray(target, np.float64)
    loss = 0.5 * float((m * e * e).sum()) / B
    g = _r(cast(m * e / B), exact)
    grads = [None] * 4
    for l in range(3, -1, -1):
        gw = cast(_mm(g.T, acts[l]))
        gb = cast(np.asarray(g, np.float64).sum(axis=0))
        grads[l] = (gw, gb)
        if l == 0:
            break
        da = _mm(g, _r(weights[l], exact))
        g = _r(cast(da * gelu_grad(np.asarray(zs[l - 1], np.float64))), exact)
    return loss, y, grads


def adam_step(w, m, v, g, t, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam step in float32 (t = step number starting at 1). Returns (w, m, v)."""
    f = np.float32
    w, m, v, g = (np.asarray(a, np.float32) for a in (w, m, v, g))
    c1 = f(1.0 / (1.0 - beta1 ** t))
    c2 = f(1.0 / (1.0 - beta2 ** t))
    m = f(beta1) * m + f(1.0 - beta1) * g
    v = f(beta2) * v + f(1.0 - beta2) * g * g
    w = w - f(lr) * (m * c1) / (np.sqrt(v * c2) + f(eps))
    return w, m, v


def finite_difference_check(rng, din=5, hidden=6, dout=4, batch=3, probes=20, h=1e-6):
    """Largest relative difference between the exact-mode analytic gradients and central differences of the loss
    for `probes` randomly chosen weights and biases."""
    dims = [(hidden, din), (hidden, hidden), (hidden, hidden), (dout, hidden)]
    W = [rng.standard_normal(s) / np.sqrt(s[1]) for s in dims]
    b = [rng.standard_normal(s[0]) * 0.1 for s in dims]
    x = rng.standard_normal((batch, din))
    t = rng.standard_normal((batch, dout))
    mask = (rng.random(dout) > 0.25) * rng.uniform(0.5, 2.0, dout)
    _, _, grads = loss_and_backward(W, b, x, t, mask, exact=True)
    worst = 0.0
    for _ in range(probes):
        l = int(rng.integers(4))
        use_bias = bool(rng.integers(2))
        P = b[l] if use_bias else W[l]
        idx = tuple(int(rng.integers(n)) for n in P.shape)
        old = P[idx]
        P[idx] = old + h
        lp, _, _ = loss_and_backward(W, b, x, t, mask, exact=True)
        P[idx] = old - h
        lm, _, _ = loss_and_backward(W, b, x, t, mask, exact=True)
        P[idx] = old
        fd = (lp - lm) / (2 * h)
        an = grads[l][1][idx] if use_bias else grads[l][0][idx]
        worst = max(worst, abs(fd - an) / max(1e-8, abs(fd) + abs(an)))
    return worst
