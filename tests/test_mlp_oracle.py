"""The FP64 surrogate oracle (oracle/mlp_oracle.py) checked against itself:
hand-written backpropagation against central finite differences, the mixture
is a normalised density, and Adam reduces the loss on a fixed batch."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import mlp_oracle as M

BOX = np.array([-1.0, -0.5, -2.0, 3.0, 1.5, 2.0])


def batch(rng, n):
    pos = BOX[:3] + (BOX[3:] - BOX[:3]) * rng.random((n, 3))
    d = rng.normal(size=(n, 3)) + np.array([0.0, 0.0, 2.0])
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    w = rng.lognormal(0.0, 1.0, n)
    return pos, d, w


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    theta = M.init_params(1).astype(np.float64)
    theta += 0.05 * rng.normal(size=theta.shape) * (theta != 0)
    pos, d, w = batch(rng, 24)
    _, g = M.loss_and_grad(theta, pos, d, w, BOX)
    idx = rng.choice(np.where(g != 0)[0], size=60, replace=False)
    eps = 1e-6
    for i in idx:
        tp, tm = theta.copy(), theta.copy()
        tp[i] += eps
        tm[i] -= eps
        fd = (M.loss_and_grad(tp, pos, d, w, BOX)[0] - M.loss_and_grad(tm, pos, d, w, BOX)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(fd)) + 1e-7, (i, fd, g[i])


def test_mixture_is_normalised():
    rng = np.random.default_rng(1)
    theta = M.init_params(2).astype(np.float64)
    pos, _, _ = batch(rng, 3)
    mx = M.mixture(M.forward(theta, M.encode(pos, BOX))["o"])
    # Monte Carlo integral over the sphere of q
    u = rng.normal(size=(200000, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    for n in range(3):
        lf = M.log_vmf(np.repeat(mx["mu"][n:n + 1], u.shape[0], 0), np.repeat(mx["kappa"][n:n + 1], u.shape[0], 0), u)
        q = (mx["pi"][n] * np.exp(lf)).sum(1)
        assert abs(q.mean() * 4 * np.pi - 1.0) < 0.02


def test_adam_reduces_loss():
    rng = np.random.default_rng(3)
    theta = M.init_params(4).astype(np.float64)
    pos, d, w = batch(rng, 256)
    l0, _ = M.loss_and_grad(theta, pos, d, w, BOX)
    m = np.zeros_like(theta)
    v = np.zeros_like(theta)
    for t in range(1, 101):
        _, g = M.loss_and_grad(theta, pos, d, w, BOX)
        theta, m, v = M.adam(theta, g, m, v, t, lr=3e-3)
    l1, _ = M.loss_and_grad(theta, pos, d, w, BOX)
    assert l1 < l0 - 0.5, (l0, l1)


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.0e38, 1e-40])
    r = M.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -7  # ties to even
    assert r[3] == -2.5
