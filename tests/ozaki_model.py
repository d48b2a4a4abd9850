"""NumPy model of the exact-accumulation tensor-core contraction of the
mixed stage kernel (DG_PREC_MIXED).

Each GEMM row a (one element-field row of the stage's A operand: contravariant
fluxes and scaled face values, FP32) is written as fixed-point slices with a
common per-row exponent and radix 2^9:
    a = 2^(ea-8) * (m_0 + m_1 2^-9 + m_2 2^-18 + m_3 2^-27),  |m_s| <= 256,
four slices (three where tensor memory is short: 3D order 4), each an integer
of at most 8 significant bits (exact in BF16).  Each row of
the FP64 operator B (one output node) is sliced the same way with exponent eb
into four slices.  Slice products are integers times 2^-9(i+j); the pairs with
i + j <= 3 are formed and summed per level L = i + j in FP32 accumulators
(level 0 exact for K <= 256: |sum| <= K 2^16 <= 2^24).  The epilogue combines
the four levels in extended precision.
"""
from __future__ import annotations

import numpy as np

RADIX_BITS = 9
B_SLICES, MAX_LEVEL = 4, 3
MAGIC = (12582912.0, 24576.0, 48.0, 0.09375)  # 1.5 * 2^(23 - 9k): rounding to 2^-9k


def row_exponent(x: np.ndarray) -> np.ndarray:
    """e with |x| < 2^e for the largest |x| of each row (frexp convention)."""
    amax = np.max(np.abs(np.asarray(x, dtype=np.float64)), axis=1)
    return np.where(amax > 0, np.floor(np.log2(np.where(amax > 0, amax, 1.0))) + 1, 0).astype(np.int64)


def slice_fp32(y: np.ndarray, n: int = 4) -> list[np.ndarray]:
    """The kernel's FP32 slicing of y = x * 2^(8-ea) (|y| < 256) into n
    slices: adding and subtracting 1.5 * 2^(23-9k) rounds to the grid 2^-9k;
    remainders exact."""
    f = np.float32
    r = np.asarray(y, dtype=f)
    out = []
    for k in range(n):
        m = (r + f(MAGIC[k])) - f(MAGIC[k])
        out.append(m)
        r = r - m
    return out


def slice_fp64(x: np.ndarray, e: np.ndarray, n: int) -> list[np.ndarray]:
    """Host slicing of the FP64 operator rows: n radix-2^9 slices, each the
    nearest multiple of 2^-9k of the remainder (as values of the scaled row)."""
    r = np.asarray(x, dtype=np.float64) * np.exp2(8 - e)[:, None]
    out = []
    for s in range(n):
        unit = 2.0 ** (-RADIX_BITS * s)
        m = np.round(r / unit) * unit
        out.append(m)
        r = r - m
    return out


def contract(A: np.ndarray, B: np.ndarray, a_slices: int = 4) -> np.ndarray:
    """C = A @ B.T with the tensor-core slice arithmetic (FP32 accumulators)."""
    A = np.asarray(A, dtype=np.float32)
    ea, eb = row_exponent(A), row_exponent(B)
    am = slice_fp32(A * np.exp2(8 - ea).astype(np.float32)[:, None], a_slices)
    bm = slice_fp64(B, eb, B_SLICES)
    levels = [np.zeros((A.shape[0], B.shape[0]), dtype=np.float32) for _ in range(MAX_LEVEL + 1)]
    for i in range(a_slices):
        for j in range(B_SLICES):
            if i + j <= MAX_LEVEL:
                prod = am[i].astype(np.float64) @ bm[j].T   # exact: integers times 2^-9(i+j)
                levels[i + j] = (levels[i + j].astype(np.float64) + prod).astype(np.float32)
    C = sum(lv.astype(np.float64) for lv in levels)
    return C * np.exp2(ea - 8)[:, None] * np.exp2(eb - 8)[None, :]
