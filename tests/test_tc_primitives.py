"""Tensor-core primitives of the mixed form (tcgen05 MMA with A in tensor
memory, B through a shared-memory descriptor, commit/mbarrier completion):
an exact integer GEMM must come back bit for bit."""
from __future__ import annotations

import ctypes

import pytest

import dgcuda as D

pytestmark = pytest.mark.gpu


def test_tcgen05_bf16_gemm_is_exact():
    err = ctypes.c_double(-1)
    code = D.lib().dg_tc_selftest(0, ctypes.byref(err))
    assert code == 0, D.lib().dg_last_error().decode()
    assert err.value == 0.0


def test_tcgen05_tf32_gemm_is_exact():
    """kind::tf32 with A in tensor memory (one 32-bit value per column) and B
    through the same no-swizzle K-major descriptor: the building block of the
    3xTF32 stage kernel."""
    err = ctypes.c_double(-1)
    code = D.lib().dg_tc_selftest_tf32(0, ctypes.byref(err))
    assert code == 0, D.lib().dg_last_error().decode()
    assert err.value == 0.0
