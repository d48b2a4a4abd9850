"""The Python mirror of the C ABI checks what it hands the library: shapes
of states, output buffers the library writes into, per-mesh arrays and
source weights are validated before any call (objects built without a
device, so no GPU is needed)."""
from __future__ import annotations

import numpy as np
import pytest

import dgcuda as D


def test_output_buffers():
    D._check_out(np.empty((4, 10)), (4, 10))
    D._check_out(np.empty((8, 10))[::2], (4, 10))  # strided rows, each contiguous
    bad = {
        "dtype": np.empty((4, 10), dtype=np.float32),
        "shape": np.empty((4, 9)),
        "rows": np.empty((4, 20))[:, ::2],
        "list": [[0.0] * 10] * 4,
    }
    ro = np.empty((4, 10))
    ro.flags["WRITEABLE"] = False
    bad["readonly"] = ro
    for name, out in bad.items():
        with pytest.raises(ValueError):
            D._check_out(out, (4, 10))


def _solver(ndof):
    s = object.__new__(D.Solver)
    s._h, s.ndof = None, ndof
    return s


def _multi(ndofs):
    class P:
        def __init__(self, n):
            self.ndof = n

    m = object.__new__(D.MultiSolver)
    m._h, m.pres = None, [P(n) for n in ndofs]
    return m


def test_solver_state_and_sources():
    s = _solver(10)
    with pytest.raises(ValueError):
        s.set_state(np.zeros((4, 9)))
    with pytest.raises(ValueError):
        s.set_state(np.zeros((3, 10)))
    with pytest.raises(ValueError):
        s.get_state(out=np.zeros((4, 10), dtype=np.float32))
    with pytest.raises(ValueError):
        s.set_batch_sources([(0, [1, 2, 3], [0.5, 0.5], 1.0, 900.0, 0.0, 1.0)])


def test_multi_solver_arrays():
    m = _multi([10, 20, 30])
    for bad in (np.zeros(2), np.zeros(4), 0.0):
        with pytest.raises(ValueError):
            m.rk4_steps(np.zeros(3), bad, 1)
        with pytest.raises(ValueError):
            m.rk4_steps_timed(bad, np.ones(3), 1)
    with pytest.raises(ValueError):
        m.autotune(np.ones(2))
    with pytest.raises(ValueError):
        m.set_state(1, np.zeros((4, 10)))
    with pytest.raises(ValueError):
        m.set_state(3, np.zeros((4, 10)))
    with pytest.raises(ValueError):
        m.get_state(-1)
    with pytest.raises(ValueError):
        m.set_sources([(0, [1, 2], [1.0], 1.0, 900.0, 0.0, 1.0)])
