"""The MLP oracle (oracle/mlp_oracle.py) against finite differences: the
reference point for the GPU rank-predictor kernels' gradient checks."""

import numpy as np

from oracle import mlp_oracle as mo


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    dims = (5, 7, 6, 1)
    p = mo.init_params(dims, rng)
    X = rng.normal(size=(9, 5))
    y = rng.normal(size=9)
    yhat, cache = mo.forward(p, dims, X)
    loss, dy = mo.mse(yhat, y)
    g = mo.backward(p, dims, X, cache, dy)
    h = 1e-6
    num = np.empty_like(p)
    for i in range(p.size):
        q = p.copy()
        q[i] += h
        lp, _ = mo.mse(mo.forward(q, dims, X)[0], y)
        q[i] -= 2 * h
        lm, _ = mo.mse(mo.forward(q, dims, X)[0], y)
        num[i] = (lp - lm) / (2 * h)
    assert np.max(np.abs(num - g)) <= 1e-7 * max(1.0, np.abs(g).max())


def test_gelu_grad_matches_finite_differences():
    z = np.linspace(-6, 6, 101)
    h = 1e-6
    num = (mo.gelu(z + h) - mo.gelu(z - h)) / (2 * h)
    assert np.max(np.abs(num - mo.gelu_grad(z))) < 1e-8


def test_adam_first_step_moves_by_lr():
    p = np.array([1.0, -2.0, 3.0])
    g = np.array([0.5, -0.1, 0.0])
    m, v = np.zeros(3), np.zeros(3)
    mo.adam_step(p, g, m, v, 1e-2, 0.9, 0.999, 1e-8, 1)
    # bias-corrected first step: -lr * sign(g) where g != 0
    assert np.allclose(p, [1.0 - 1e-2, -2.0 + 1e-2, 3.0], atol=1e-8)
