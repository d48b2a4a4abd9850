"""The MLP oracle (float64 NumPy) against central finite differences: it is
the reference the GPU training kernels' gradients are checked against."""
from __future__ import annotations

import numpy as np

import mlp_oracle as M


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    nin, width, nout, hidden = 7, 9, 3, 3
    n = sum(o * i + o for (o, i) in M.shapes(nin, width, nout, hidden))
    p = rng.standard_normal(n) * 0.5
    X = rng.standard_normal((11, nin))
    T = rng.standard_normal((11, nout))
    loss, g = M.loss_grad(p, X, T, nin, width, nout, hidden)
    h = 1e-6
    fd = np.zeros(n)
    for k in range(n):
        e = np.zeros(n)
        e[k] = h
        fd[k] = (M.loss_grad(p + e, X, T, nin, width, nout, hidden)[0] -
                 M.loss_grad(p - e, X, T, nin, width, nout, hidden)[0]) / (2 * h)
    assert np.allclose(g, fd, rtol=1e-6, atol=1e-9)
    assert loss > 0


def test_gelu_derivative():
    x = np.linspace(-6, 6, 1001)
    h = 1e-6
    fd = (M.gelu(x + h) - M.gelu(x - h)) / (2 * h)
    assert np.allclose(M.gelu_grad(x), fd, atol=1e-8)
