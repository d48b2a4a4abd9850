"""Host-side check of the mixed kernel's operand slicing arithmetic (no GPU:
FP32 arithmetic in NumPy rounds as the device does)."""
from __future__ import annotations

import numpy as np


def test_slicing_by_magic_constants_equals_rounding_of_scaled_values():
    """The mixed kernel cuts y (|y| < 256) into s0 + s1 + s2 + s3, s_k on the
    grid 2^-8k, by adding and subtracting 1.5 * 2^(23-8k) in FP32.  That must
    give exactly the slices of rounding the scaled remainders to integers
    (round half to even), ties included, and leave a remainder below 2^-25."""
    rng = np.random.default_rng(0)
    f = np.float32

    def by_rint(y):
        m0 = np.rint(y)
        y1 = (y - m0) * f(256)
        m1 = np.rint(y1)
        y2 = (y1 - m1) * f(256)
        m2 = np.rint(y2)
        m3 = np.rint((y2 - m2) * f(256))
        return m0, m1 * f(2.0 ** -8), m2 * f(2.0 ** -16), m3 * f(2.0 ** -24)

    def by_constants(y):
        m0 = (y + f(12582912.0)) - f(12582912.0)
        r1 = y - m0
        m1 = (r1 + f(49152.0)) - f(49152.0)
        r2 = r1 - m1
        m2 = (r2 + f(192.0)) - f(192.0)
        m3 = ((r2 - m2) + f(0.75)) - f(0.75)
        return m0, m1, m2, m3

    ys = [rng.uniform(-256, 256, 50_000).astype(f),
          (rng.standard_normal(50_000) * 2.0 ** rng.integers(-30, 8, 50_000)).astype(f),
          (rng.integers(-511, 511, 20_000) * 0.5).astype(f)]
    for k in (1, 2, 3):
        g = rng.integers(-2 ** 20, 2 ** 20, 20_000) * 2.0 ** (-8 * k) + 0.5 * 2.0 ** (-8 * k)
        ys.append(g.astype(f))
    for y in ys:
        y = y[np.abs(y) < 256]
        a, b = by_rint(y), by_constants(y)
        for i in range(4):
            assert np.array_equal(a[i], b[i])
        total = b[0].astype(np.float64) + b[1] + b[2] + b[3]
        assert np.all(np.abs(total - y) <= 2.0 ** -25 * 1.0001)
