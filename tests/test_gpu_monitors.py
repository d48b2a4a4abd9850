"""Monitors and failure detection on the GPU, with no GPU fault involved.

* dg_error_vs: the FP64 relative L2 error between two contexts' states,
  reduced on the device, equals the NumPy figure from their host copies,
  for every pair of precisions and for batch members.
* dg_monitors reads the mixed form's state as the FP64 sum of its FP32 pair.
* A NaN written into the host state before upload is reported by
  dg_monitors and dg_error_vs as DG_ERR_NONFINITE with its count (the
  reference has no check: its config errors terminate and its mesh
  constructor asserts, configParser.cpp:145-147, Mesh.cpp:74-78).
* A bounded tensor-core mbarrier wait forced to run out returns the kernel's
  error flag after draining its MMAs; the context stays usable.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import dgcuda as D

pytestmark = pytest.mark.gpu

C0, RHO0 = 340.0, 1.225


def rel_l2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def case():
    mesh = D.Mesh.box_tet(3, 3, 2, order=3, side_names=("Absorbing", "Reflecting") * 3)
    pre = D.Precomp(mesh)
    v0 = (60.0, 0.0, 0.0)
    dt = D.cfl_dt(pre, C0, v0)
    u0 = pre.initial_state([(0, 0.45, 0.5, 0.4, 0.02, 1.0)])
    u0[1:4] += 1e-3 * np.random.default_rng(3).standard_normal((3, pre.ndof))
    return pre, v0, dt, u0


def run(pre, v0, dt, u0, precision, nsteps=25, nbatch=1):
    s = D.Solver(pre, C0, RHO0, v0, precision=precision, flux="upwind", nbatch=nbatch)
    s.set_state(u0)
    if nbatch > 1:
        for m in range(1, nbatch):
            s.set_state(u0 * (1.0 + 0.5 * m), member=m)
    s.rk4_steps(0.0, dt, nsteps)
    return s


@pytest.mark.parametrize("prec", ["fp64", "fp32", "mixed"])
def test_error_monitor_equals_host_figure(case, prec):
    pre, v0, dt, u0 = case
    ref = run(pre, v0, dt, u0, "fp64")
    s = run(pre, v0, dt, u0, prec)
    rel, bad = s.error_vs(ref)
    assert bad == 0
    a, b = s.get_state(), ref.get_state()
    for q in range(4):
        want = rel_l2(a[q], b[q])
        if prec == "fp64":
            assert rel[q] == 0.0
        else:
            assert want > 0 and abs(rel[q] - want) <= 1e-9 * want, (q, rel[q], want)
    # symmetric call with the roles swapped, and a context against itself
    rel2, _ = ref.error_vs(s)
    for q in range(4):
        want = rel_l2(b[q], a[q])
        assert abs(rel2[q] - want) <= 1e-9 * max(want, 1e-300)
    assert s.error_vs(s)[0] == [0.0] * 4


def test_error_monitor_batch_members(case):
    pre, v0, dt, u0 = case
    ref = run(pre, v0, dt, u0, "fp64", nsteps=10, nbatch=3)
    s = run(pre, v0, dt, u0, "mixed", nsteps=10, nbatch=3)
    for m in range(3):
        rel, _ = s.error_vs(ref, member=m, ref_member=m)
        a, b = s.get_state(member=m), ref.get_state(member=m)
        for q in range(4):
            want = rel_l2(a[q], b[q])
            assert abs(rel[q] - want) <= 1e-9 * want
    # member 2 started at twice member 0's state; scaling by 2 commutes with
    # every FP64 rounding of the linear step, so it is still exactly twice it
    rel, _ = ref.error_vs(ref, member=2, ref_member=0)
    assert all(abs(r - 1.0) < 1e-12 for r in rel)


def test_error_monitor_rejects_other_meshes(case):
    pre, v0, dt, u0 = case
    s = run(pre, v0, dt, u0, "fp64", nsteps=1)
    other = D.Precomp(D.Mesh.box_tet(2, 2, 2, order=3))
    o = D.Solver(other, C0, RHO0, precision="fp64")
    with pytest.raises(D.DGError) as ei:
        s.error_vs(o)
    assert ei.value.code == -1
    with pytest.raises(D.DGError):
        s.error_vs(s, member=1)


def test_mixed_monitors_read_the_state_pair(case):
    """The mixed form keeps its state as an FP32 pair (~48 bits): its FP64
    energy and L2 monitors equal the FP64 context's on the same state to far
    better than FP32 rounding (reading the high word alone gives ~1e-8)."""
    pre, v0, dt, u0 = case
    a = D.Solver(pre, C0, RHO0, v0, precision="fp64")
    b = D.Solver(pre, C0, RHO0, v0, precision="mixed")
    a.set_state(u0)
    b.set_state(u0)
    ea, la, _ = a.monitors()
    eb, lb, _ = b.monitors()
    assert abs(eb - ea) <= 1e-12 * ea
    for q in range(4):
        assert abs(lb[q] - la[q]) <= 1e-12 * la[q]


@pytest.mark.parametrize("prec", ["fp64", "fp32", "mixed"])
def test_nan_in_host_state_is_reported(case, prec):
    pre, v0, dt, u0 = case
    s = D.Solver(pre, C0, RHO0, v0, precision=prec)
    bad_u = u0.copy()
    bad_u[2, 17] = np.nan
    bad_u[0, 3] = np.inf
    s.set_state(bad_u)
    code = D.lib().dg_monitors(s._h, None, None, None)
    assert code == -4
    _, _, nbad = s.monitors()
    assert nbad == 2
    ref = D.Solver(pre, C0, RHO0, v0, precision="fp64")
    ref.set_state(u0)
    rel, nbad = s.error_vs(ref)
    assert nbad == 2
    # a clean state clears the report
    s.set_state(u0)
    assert s.monitors()[2] == 0


def test_bounded_tensor_core_wait_runs_out_and_returns_its_flag():
    flags = ctypes.c_int(-1)
    code = D.lib().dg_tc_wait_selftest(0, ctypes.byref(flags))
    assert code == 0, D.lib().dg_last_error().decode()
    assert flags.value == 1  # timed out, MMAs drained, tensor memory freed
    err = ctypes.c_double(-1)
    assert D.lib().dg_tc_selftest(0, ctypes.byref(err)) == 0 and err.value == 0.0
