"""Batched contexts: several independent states (sources, initial
conditions) on one mesh stepped by one launch per stage.  Every member must
match its own oracle run: FP64 to 1e-10 relative L2 per field, the mixed
form to 1e-6, FP32 to 1e-5.  Receivers must record exactly the pressure the
state holds after each step."""
from __future__ import annotations

import numpy as np
import pytest

import dgcuda as D
import oracle_py as O

pytestmark = pytest.mark.gpu

C0, RHO0 = 340.0, 1.225
TOL = {"fp64": 1e-10, "fp32": 1e-5, "mixed": 1e-6}


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / nb if nb > 0 else np.linalg.norm(a - b)


def box3d(order):
    return D.Mesh.box_tet(3, 3, 2, (0.0, 0.0, 0.0), (1.0, 1.0, 0.7), order=order,
                          side_names=("Absorbing", "Reflecting") * 3)


def member_inputs(pre, nb, seed):
    """Per member: an initial pulse and one source (reference type for even
    members, Gaussian-weighted for odd ones) at seeded positions."""
    rng = np.random.default_rng(seed)
    lo, hi = pre.dof_coords().min(axis=0), pre.dof_coords().max(axis=0)
    out = []
    for m in range(nb):
        x = lo + (hi - lo) * rng.uniform(0.25, 0.75, 3)
        u0 = pre.initial_state([(0, *x, 0.03, 1.0 + m)])
        xs = lo + (hi - lo) * rng.uniform(0.2, 0.8, 3)
        gaussian = m % 2 == 1
        size = 0.12 if gaussian else 0.2
        freq, amp, dur = rng.uniform(800.0, 2000.0), rng.uniform(0.5, 2.0), 1.0
        out.append((u0, gaussian, xs, size, amp, freq, dur))
    return out


def oracle_member(mesh, dt, inp, nsteps, method="Runge-Kutta", upwind=False, v0=(0.0, 0.0, 0.0)):
    u0, gaussian, xs, size, amp, freq, dur = inp
    src = np.array([[1.0 if gaussian else 0.0, *xs, size, amp, freq, 0.0, dur]])
    orc = O.Oracle(mesh.raw(), dt, C0, RHO0, v0=v0, bcs=mesh.bcs(), upwind=upwind, sources=src)
    orc.set_method(method)
    orc.set_state(u0)
    t, _ = orc.run(0.0, nsteps)
    return t, orc.get_state()


def batch_sources(pre, inputs):
    srcs = []
    for m, (u0, gaussian, xs, size, amp, freq, dur) in enumerate(inputs):
        if gaussian:
            dofs, w = pre.gaussian_source(*xs, size)
        else:
            dofs, w = pre.source_dofs(*xs, size), None
        srcs.append((m, dofs, w, amp, freq, 0.0, dur))
    return srcs


@pytest.mark.parametrize("precision,flux", [("fp64", "reference"), ("fp32", "upwind"), ("mixed", "upwind")])
@pytest.mark.parametrize("order", [2, 3])
def test_batch_members_match_their_oracle_runs(precision, flux, order):
    mesh = box3d(order)
    pre = D.Precomp(mesh)
    v0 = (30.0, 0.0, -10.0)
    dt = D.cfl_dt(pre, C0, v0)
    nb, nsteps = 4, 37
    inputs = member_inputs(pre, nb, seed=order)
    sol = D.Solver(pre, C0, RHO0, v0, precision=precision, flux=flux, nbatch=nb)
    for m, inp in enumerate(inputs):
        sol.set_state(inp[0], member=m)
    sol.set_batch_sources(batch_sources(pre, inputs))
    t = sol.rk4_steps(0.0, dt, nsteps)
    for m, inp in enumerate(inputs):
        got = sol.get_state(member=m)
        tr, ref = oracle_member(mesh, dt, inp, nsteps, upwind=(flux == "upwind"), v0=v0)
        assert t == tr
        for q in range(4):
            assert rel_l2(got[q], ref[q]) <= TOL[precision], (m, q, rel_l2(got[q], ref[q]))


def test_batch_forward_euler_2d():
    mesh = D.Mesh.box_tri(5, 4, (-1.0, -1.0), (1.0, 0.8), order=3,
                          side_names=("Reflecting", "Absorbing", "Reflecting", "Absorbing"))
    pre = D.Precomp(mesh)
    dt = 0.2 * D.cfl_dt(pre, C0)
    inputs = member_inputs(pre, 3, seed=11)
    inputs = [(u0 * np.array([[1], [1], [1], [0]]), g, xs * np.array([1, 1, 0]), s, a, f, d)
              for (u0, g, xs, s, a, f, d) in inputs]
    sol = D.Solver(pre, C0, RHO0, precision="fp64", nbatch=3)
    for m, inp in enumerate(inputs):
        sol.set_state(inp[0], member=m)
    sol.set_batch_sources(batch_sources(pre, inputs))
    t = sol.euler_steps(0.0, dt, 21)
    for m, inp in enumerate(inputs):
        tr, ref = oracle_member(mesh, dt, inp, 21, method="Euler1")
        got = sol.get_state(member=m)
        assert t == tr
        for q in range(3):
            assert rel_l2(got[q], ref[q]) <= TOL["fp64"]


def test_common_state_and_sources_reach_every_member():
    mesh = box3d(2)
    pre = D.Precomp(mesh)
    dt = D.cfl_dt(pre, C0)
    u0 = pre.initial_state([(0, 0.4, 0.5, 0.3, 0.02, 1.0)])
    sol = D.Solver(pre, C0, RHO0, precision="fp64", nbatch=3)
    sol.set_state(u0)
    sol.set_sources([(pre.source_dofs(0.6, 0.4, 0.35, 0.2), 1.0, 1500.0, 0.0, 1.0)])
    sol.rk4_steps(0.0, dt, 9)
    a = sol.get_state(member=0)
    for m in (1, 2):
        assert np.array_equal(sol.get_state(member=m), a)
    with pytest.raises(RuntimeError):
        sol.get_state(member=3)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_receivers_record_the_state_after_each_step(precision):
    mesh = box3d(2)
    pre = D.Precomp(mesh)
    dt = D.cfl_dt(pre, C0)
    inputs = member_inputs(pre, 2, seed=5)
    rec = np.random.default_rng(9).choice(pre.ndof, 6, replace=False).astype(np.int32)
    nsteps = 40

    def make():
        s = D.Solver(pre, C0, RHO0, precision=precision, flux="upwind", nbatch=2)
        for m, inp in enumerate(inputs):
            s.set_state(inp[0], member=m)
        s.set_batch_sources(batch_sources(pre, inputs))
        return s

    sol = make()
    sol.set_receivers(rec, max_steps=nsteps)
    sol.rk4_steps(0.0, dt, nsteps)
    tr = sol.traces()
    assert tr.shape == (2, 6, nsteps)
    step = make()
    t = 0.0
    for k in range(nsteps):
        t = step.rk4_steps(t, dt, 1)
        for m in range(2):
            p = step.get_state(member=m)[0, rec]
            assert np.array_equal(tr[m, :, k], p), (k, m)
