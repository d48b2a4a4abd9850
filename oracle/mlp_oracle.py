"""TEST INFRASTRUCTURE ONLY - CPU oracle of the learned coarse propagator's
network (the reference has no counterpart: DGFEM-Acoustic has no learned
part).  Restates, in float64 NumPy, what the product's MLP kernels compute:

  layers l = 0..L-1 with W_l [out][in] row-major then b_l [out] packed in one
  parameter vector; hidden layers z = a W^T + b, a' = gelu(z) with the tanh
  form gelu(x) = x/2 (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))); last layer
  linear; loss = mean over rows x outputs of (y - t)^2.

Only the tests may import this module.
"""
from __future__ import annotations

import numpy as np

_C = np.sqrt(2.0 / np.pi)


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(_C * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    t = np.tanh(_C * (x + 0.044715 * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * _C * (1.0 + 3 * 0.044715 * x * x)


def shapes(nin: int, width: int, nout: int, hidden: int):
    dims = [nin] + [width] * hidden + [nout]
    return [(dims[l + 1], dims[l]) for l in range(hidden + 1)]


def unpack(p: np.ndarray, nin: int, width: int, nout: int, hidden: int):
    out, off = [], 0
    for (o, i) in shapes(nin, width, nout, hidden):
        W = p[off:off + o * i].reshape(o, i)
        off += o * i
        b = p[off:off + o]
        off += o
        out.append((W, b))
    assert off == p.size
    return out


def forward(p, X, nin, width, nout, hidden):
    layers = unpack(np.asarray(p, np.float64), nin, width, nout, hidden)
    a = np.asarray(X, np.float64)
    acts, zs = [a], []
    for l, (W, b) in enumerate(layers):
        z = a @ W.T + b
        if l + 1 < len(layers):
            zs.append(z)
            a = gelu(z)
            acts.append(a)
        else:
            return z, acts, zs


def loss_grad(p, X, T, nin, width, nout, hidden):
    """(loss, gradient packed like p) of the mean squared error."""
    layers = unpack(np.asarray(p, np.float64), nin, width, nout, hidden)
    Y, acts, zs = forward(p, X, nin, width, nout, hidden)
    T = np.asarray(T, np.float64)
    n = Y.size
    loss = float(np.sum((Y - T) ** 2) / n)
    dz = 2.0 * (Y - T) / n
    grads = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        W, _ = layers[l]
        grads[l] = (dz.T @ acts[l], dz.sum(axis=0))
        if l > 0:
            dz = (dz @ W) * gelu_grad(zs[l - 1])
    g = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
    return loss, g


def bf16(x):
    """Round to BF16 (round to nearest, ties to even) and back to float64."""
    b = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def forward_bf16(p, X, nin, width, nout, hidden):
    """What the tensor-core inference computes: inputs, weights and hidden
    activations rounded to BF16, products and sums exact here (FP32
    accumulation on the device), biases and GELU unrounded."""
    layers = unpack(np.asarray(p, np.float64), nin, width, nout, hidden)
    a = bf16(np.asarray(X, np.float32))
    for l, (W, b) in enumerate(layers):
        z = a @ bf16(W.astype(np.float32)).T + b.astype(np.float32)
        if l + 1 < len(layers):
            a = bf16(gelu(z).astype(np.float32))
        else:
            return z
