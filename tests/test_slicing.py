"""Host-side check of the mixed kernel's operand slicing arithmetic (no GPU:
FP32 arithmetic in NumPy rounds as the device does)."""
from __future__ import annotations

import numpy as np

import ozaki_model as OZ


def _bf16_exact(x: np.ndarray) -> bool:
    bits = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    return bool(np.all((bits & np.uint32(0xFFFF)) == 0))


def test_slicing_by_magic_constants_equals_rounding_of_scaled_values():
    """The mixed kernel cuts y (|y| < 256) into s0 + s1 + s2 + s3, s_k on the
    grid 2^-9k, by adding and subtracting 1.5 * 2^(23-9k) in FP32.  That must
    give exactly the slices of rounding the scaled remainders to integers
    (round half to even), ties included; every slice is an integer of
    magnitude at most 256 times 2^-9k (exact in BF16) and the remainder is
    below 2^-28 (2^-19 after three slices)."""
    rng = np.random.default_rng(0)
    f = np.float32

    def by_rint(y):
        m0 = np.rint(y)
        y1 = (y - m0) * f(512)
        m1 = np.rint(y1)
        y2 = (y1 - m1) * f(512)
        m2 = np.rint(y2)
        m3 = np.rint((y2 - m2) * f(512))
        return m0, m1 * f(2.0 ** -9), m2 * f(2.0 ** -18), m3 * f(2.0 ** -27)

    ys = [rng.uniform(-256, 256, 50_000).astype(f),
          (rng.standard_normal(50_000) * 2.0 ** rng.integers(-30, 8, 50_000)).astype(f),
          (rng.integers(-511, 511, 20_000) * 0.5).astype(f)]
    for k in (1, 2, 3):
        g = rng.integers(-2 ** 13, 2 ** 13, 20_000) * 2.0 ** (-9 * k) + 0.5 * 2.0 ** (-9 * k)
        ys.append(g[np.abs(g) < 256].astype(f))
    for y in ys:
        y = y[np.abs(y) < 256]
        a, b = by_rint(y), OZ.slice_fp32(y, 4)
        for i in range(4):
            assert np.array_equal(a[i], b[i])
            digits = b[i].astype(np.float64) * 2.0 ** (9 * i)
            assert np.all(digits == np.rint(digits)) and np.all(np.abs(digits) <= 256)
            assert _bf16_exact(b[i])
        three = b[0].astype(np.float64) + b[1] + b[2]
        assert np.all(np.abs(three - y) <= 2.0 ** -19 * 1.0001)
        assert np.all(np.abs(three + b[3] - y) <= 2.0 ** -28 * 1.0001)


def test_level_zero_sums_stay_exact_in_fp32():
    """Products of top slices are at most 2^16 in magnitude, so a level-0 sum
    over K <= 256 terms stays within 2^24 (exact in the FP32 accumulator)."""
    rng = np.random.default_rng(1)
    A = (rng.standard_normal((64, 252)) * 10.0 ** rng.uniform(-3, 3, (64, 1))).astype(np.float32)
    ea = OZ.row_exponent(A)
    m0 = OZ.slice_fp32(A * np.exp2(8 - ea).astype(np.float32)[:, None])[0]
    assert np.max(np.abs(m0)) <= 256
    assert 252 * 256 * 256 <= 2 ** 24


def test_contraction_model_is_accurate_to_the_row_scales():
    """Four (three) A slices against four operator slices (36 bits), pairs
    i + j <= 3: the error stays below 2^-34 (2^-26) of |a|_max |b|_max K per
    entry."""
    rng = np.random.default_rng(2)
    K = 100
    A = (rng.standard_normal((128, K)) * 10.0 ** rng.uniform(-2, 2, (128, 1))).astype(np.float32)
    B = rng.standard_normal((20, K)) * 10.0 ** rng.uniform(-1, 1, (20, 1))
    exact = A.astype(np.float64) @ B.T
    scale = np.max(np.abs(A), 1)[:, None] * np.max(np.abs(B), 1)[None, :] * K
    for na, bits in ((4, 34), (3, 26)):
        C = OZ.contract(A, B, na)
        assert np.all(np.abs(C - exact) <= 2.0 ** -bits * scale)
