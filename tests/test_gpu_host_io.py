"""State transfer through the C ABI: from pinned host memory the conversion
kernels read and write the host arrays directly (no staging copy); the
result must be bit-identical to the staged path taken for pageable arrays,
in every precision and for batch members."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import dgcuda as D

pytestmark = pytest.mark.gpu


class Pinned:
    def __init__(self, shape):
        n = int(np.prod(shape))
        self.ptr = D.lib().dg_host_alloc(8 * n)
        assert self.ptr
        self.a = np.ctypeslib.as_array((C.c_double * n).from_address(self.ptr)).reshape(shape)

    def free(self):
        D.lib().dg_host_free(self.ptr)


@pytest.mark.parametrize("precision", ["fp64", "fp32", "mixed"])
def test_pinned_and_pageable_transfers_agree(precision):
    mesh = D.Mesh.box_tet(3, 3, 2, order=3, side_names=("Reflecting", "Absorbing") * 3)
    pre = D.Precomp(mesh)
    dt = D.cfl_dt(pre, 340.0)
    rng = np.random.default_rng(7)
    u0, u1 = rng.standard_normal((2, 4, pre.ndof))
    bufs = [Pinned((4, pre.ndof)) for _ in range(4)]
    try:
        bufs[0].a[:] = u0
        bufs[1].a[:] = u1
        out = []
        for ins, outs in (((u0, u1), (np.empty((4, pre.ndof)), np.empty((4, pre.ndof)))),
                          ((bufs[0].a, bufs[1].a), (bufs[2].a, bufs[3].a))):
            s = D.Solver(pre, 340.0, 1.225, precision=precision, flux="upwind", nbatch=2)
            s.set_state(ins[0], member=0)
            s.set_state(ins[1], member=1)
            s.rk4_steps(0.0, dt, 3)
            s.get_state(outs[0], member=0)
            s.get_state(outs[1], member=1)
            out.append((outs[0].copy(), outs[1].copy()))
            s.close()
        assert np.array_equal(out[0][0], out[1][0])
        assert np.array_equal(out[0][1], out[1][1])
        # round trip without steps
        s = D.Solver(pre, 340.0, 1.225, precision=precision, flux="upwind")
        s.set_state(bufs[0].a)
        s.get_state(bufs[2].a)
        got = bufs[2].a
        if precision == "fp64":
            assert np.array_equal(got, u0)
        elif precision == "fp32":
            assert np.array_equal(got, u0.astype(np.float32).astype(np.float64))
        else:  # FP32 pair: 48 significant bits
            assert np.abs(got - u0).max() <= 2.0 ** -46 * np.abs(u0).max()
        s.close()
    finally:
        for b in bufs:
            b.free()


@pytest.mark.parametrize("prec", ["fp64", "fp32", "mixed"])
def test_async_copy_out_frames_equal_blocking_copies(prec):
    """dg_get_state_async snapshots the state after the work already
    enqueued and copies it out on a side stream while later steps run: three
    frames (two in pinned memory, one pageable; the third call reuses the
    first slot) equal the blocking dg_get_state of a second context taken at
    the same steps, bit for bit."""
    mesh = D.Mesh.box_tet(3, 2, 2, order=3, side_names=("Absorbing", "Reflecting") * 3)
    pre = D.Precomp(mesh)
    v0 = (50.0, 0.0, 0.0)
    dt = D.cfl_dt(pre, 340.0, v0)
    u0 = pre.initial_state([(0, 0.5, 0.5, 0.5, 0.02, 1.0)])
    a = D.Solver(pre, 340.0, 1.225, v0, precision=prec, flux="upwind")
    b = D.Solver(pre, 340.0, 1.225, v0, precision=prec, flux="upwind")
    a.set_state(u0)
    b.set_state(u0)
    outs = [D.pinned_array((4, pre.ndof)), D.pinned_array((4, pre.ndof)), np.empty((4, pre.ndof))]
    tickets, want = [], []
    t = tb = 0.0
    for k in range(3):
        t = a.rk4_steps(t, dt, 5)
        tickets.append(a.get_state_async(outs[k]))
        tb = b.rk4_steps(tb, dt, 5)
        want.append(b.get_state().copy())
    a.rk4_steps(t, dt, 7)  # more work after the last save
    for tk in reversed(tickets):
        a.wait_state(tk)
    for k in range(3):
        assert np.array_equal(outs[k], want[k]), k
    with pytest.raises(D.DGError):
        a.wait_state(99)


@pytest.mark.parametrize("prec", ["fp64", "fp32", "mixed"])
def test_staged_state_uploads_equal_blocking_uploads(prec):
    """dg_stage_state copies a state to the device on a side stream and
    dg_commit_state makes it the state in stream order: each step sequence
    fed through stage/commit (the next input staged before the current step
    runs, one input pageable, a third stage reusing the first slot) equals,
    bit for bit, the same sequence fed through the blocking dg_set_state;
    committing an overwritten or unknown ticket is an error."""
    mesh = D.Mesh.box_tet(3, 2, 2, order=3, side_names=("Absorbing", "Reflecting") * 3)
    pre = D.Precomp(mesh)
    v0 = (50.0, 0.0, 0.0)
    dt = D.cfl_dt(pre, 340.0, v0)
    rng = np.random.default_rng(11)
    ins = [D.pinned_array((4, pre.ndof)), D.pinned_array((4, pre.ndof)), np.empty((4, pre.ndof))]
    for k, u in enumerate(ins):
        u[:] = pre.initial_state([(0, 0.3 + 0.2 * k, 0.5, 0.5, 0.02, 1.0)]) + 1e-3 * rng.standard_normal((4, pre.ndof))
    a = D.Solver(pre, 340.0, 1.225, v0, precision=prec, flux="upwind")
    b = D.Solver(pre, 340.0, 1.225, v0, precision=prec, flux="upwind")
    got, want = [], []
    tk = a.stage_state(ins[0])
    t = tb = 0.0
    for k in range(3):
        a.commit_state(tk)
        if k + 1 < 3:
            tk = a.stage_state(ins[k + 1])  # crosses the host link while step k runs
        t = a.rk4_steps(t, dt, 4)
        got.append(a.get_state().copy())
        b.set_state(ins[k])
        tb = b.rk4_steps(tb, dt, 4)
        want.append(b.get_state().copy())
    for k in range(3):
        assert np.array_equal(got[k], want[k]), k
    old = a.stage_state(ins[0])
    a.stage_state(ins[1])
    a.stage_state(ins[2])  # the third stage reuses the slot of the first
    with pytest.raises(D.DGError):
        a.commit_state(old)
    with pytest.raises(D.DGError):
        a.commit_state(99)
