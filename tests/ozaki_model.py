"""NumPy model of the exact-accumulation tensor-core contraction.

Each GEMM row a (one element-field row of the stage's A operand: contravariant
fluxes and scaled face-flux jumps, FP32) is written as fixed-point slices with
a common per-row exponent: a = 2^ea * sum_s m_s 2^(-8(s+1)), |m_s| <= 256
(integers of at most 8 significant bits, exact in BF16).  Each row of the
operator B (one output node) is sliced the same way with exponent eb.  Slice
products are integers < 2^16; a K-sum of up to 104 of them stays below 2^24,
so the FP32 accumulator of the tensor core adds them exactly.  Pairs (i, j)
with i + j = 0 and i + j = 1 go to exact accumulators, all pairs with
2 <= i + j <= 4 to a third one (its rounding sits 2^-40 below the result).
The epilogue combines the three accumulators in extended precision.
"""
from __future__ import annotations

import numpy as np

SLICE_BITS = 8


def slice_rows(x: np.ndarray, nslices: int):
    """Fixed-point slices of each row: returns (exponents[rows], [m_0, m_1, ...])
    with x[r] ~= 2^e[r] * sum_s m_s[r] * 2^(-8(s+1))."""
    x = np.asarray(x, dtype=np.float64)
    amax = np.max(np.abs(x), axis=1)
    e = np.where(amax > 0, np.floor(np.log2(np.where(amax > 0, amax, 1.0))) + 1, 0).astype(np.int64)
    r = x * np.exp2(-e)[:, None]                 # |r| < 1
    out = []
    for s in range(nslices):
        scale = 2.0 ** (SLICE_BITS * (s + 1))
        m = np.round(r * scale)
        out.append(m)
        r = r - m / scale
    return e, out


PAIRS = [(i, j) for i in range(3) for j in range(4) if i + j <= 4]


def contract(A: np.ndarray, B: np.ndarray, a_slices: int = 3, b_slices: int = 4) -> np.ndarray:
    """C = A @ B.T with the tensor-core slice arithmetic (FP32 accumulators)."""
    ea, am = slice_rows(A, a_slices)
    eb, bm = slice_rows(B, b_slices)
    acc = [np.zeros((A.shape[0], B.shape[0]), dtype=np.float32) for _ in range(3)]
    for i, j in PAIRS:
        if i >= a_slices or j >= b_slices:
            continue
        s = i + j
        prod = am[i] @ bm[j].T                  # exact integers (< 2^24 per pair)
        slot = min(s, 2)
        unit = 2.0 ** (-SLICE_BITS * (s - slot)) if slot == 2 else 1.0
        acc[slot] = (acc[slot].astype(np.float64) + prod * unit).astype(np.float32)
    C = (acc[0].astype(np.float64) * 2.0 ** (-2 * SLICE_BITS)
         + acc[1].astype(np.float64) * 2.0 ** (-3 * SLICE_BITS)
         + acc[2].astype(np.float64) * 2.0 ** (-4 * SLICE_BITS))
    return C * np.exp2(ea)[:, None] * np.exp2(eb)[None, :]
