"""CPU oracle for the rank predictor's MLP (test infrastructure only).

The reference has no learned component, so there is no reference file to
follow here: this is a float64 NumPy restatement of the published building
blocks the GPU kernels implement (seemps2_gb300/csrc/mlp.cu), used by the tests
to check the GPU forward pass, gradients and optimiser step:

  * layer k: Z = X W_k^T + b_k; hidden layers then A = gelu(Z) with the tanh
    approximation gelu(z) = 0.5 z (1 + tanh(c (z + 0.044715 z^3))),
    c = sqrt(2 / pi) (Hendrycks & Gimpel, "Gaussian Error Linear Units", 2016);
  * loss: mean squared error over the batch;
  * optimiser: Adam (Kingma & Ba, 2015) with bias-corrected moments.

Parameters are one flat array, layer by layer: W_k (dims[k+1] x dims[k],
row-major) then b_k (dims[k+1]) -- the layout of the C ABI.
"""

from __future__ import annotations

import numpy as np

C_GELU = np.sqrt(2.0 / np.pi)


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(C_GELU * (z + 0.044715 * z**3)))


def gelu_grad(z):
    t = np.tanh(C_GELU * (z + 0.044715 * z**3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * C_GELU * (1.0 + 3.0 * 0.044715 * z * z)


def unpack(params, dims):
    """List of (W, b) views of the flat parameter array."""
    out, o = [], 0
    for k in range(len(dims) - 1):
        n_in, n_out = dims[k], dims[k + 1]
        W = params[o:o + n_out * n_in].reshape(n_out, n_in)
        o += n_out * n_in
        b = params[o:o + n_out]
        o += n_out
        out.append((W, b))
    assert o == params.size
    return out


def init_params(dims, rng):
    """Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights and biases."""
    parts = []
    for k in range(len(dims) - 1):
        bound = 1.0 / np.sqrt(dims[k])
        parts.append(rng.uniform(-bound, bound, size=dims[k + 1] * dims[k]))
        parts.append(rng.uniform(-bound, bound, size=dims[k + 1]))
    return np.concatenate(parts)


def forward(params, dims, X):
    """Output (batch x dims[-1]) and the (Z, A) cache of every layer."""
    cache, a = [], X
    layers = unpack(params, dims)
    for k, (W, b) in enumerate(layers):
        z = a @ W.T + b
        a = gelu(z) if k + 1 < len(layers) else z
        cache.append((z, a))
    return a, cache


def mse(yhat, y):
    """Mean squared error and its gradient with respect to yhat."""
    r = yhat.reshape(-1) - y.reshape(-1)
    return float(np.mean(r * r)), (2.0 * r / r.size).reshape(yhat.shape)


def backward(params, dims, X, cache, dY):
    """Gradient of a scalar loss with dL/dY = dY, in the flat parameter layout."""
    layers = unpack(params, dims)
    grads = []
    g = dY
    for k in range(len(layers) - 1, -1, -1):
        W, b = layers[k]
        a_in = X if k == 0 else cache[k - 1][1]
        grads.append((g.T @ a_in, g.sum(axis=0)))
        if k > 0:
            g = (g @ W) * gelu_grad(cache[k - 1][0])
    flat = []
    for gW, gb in reversed(grads):
        flat += [gW.reshape(-1), gb]
    return np.concatenate(flat)


def adam_step(p, g, m, v, lr, b1, b2, eps, t):
    """One Adam update in place; returns (p, m, v)."""
    m[:] = b1 * m + (1 - b1) * g
    v[:] = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1**t)
    vh = v / (1 - b2**t)
    p[:] = p - lr * mh / (np.sqrt(vh) + eps)
    return p, m, v
