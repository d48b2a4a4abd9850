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


def test_bf16_rounding_known_answers():
    """Round to nearest, ties to even, on 8 significant bits."""
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, 1.0 + 2 ** -7 + 2 ** -8, -np.pi, 0.0, 65504.0], np.float32)
    want = [1.0, 1.0, 1.0 + 2 ** -7, 1.0 + 2 ** -6, -3.140625, 0.0, 65536.0]
    assert np.array_equal(M.bf16(x), np.array(want))
