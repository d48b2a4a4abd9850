"""Known-answer checks of the CPU oracle (the reference publishes no golden
data for this path, so the oracle is pinned to analytic properties of the
discretisation instead)."""
from __future__ import annotations

import numpy as np
import pytest

import dgcuda as D
import oracle_py as O

C0, RHO0 = 340.0, 1.225


def oracle_for(mesh, dt, v0=(0.0, 0.0, 0.0), upwind=False, sources=None, num_threads=0):
    return O.Oracle(mesh.raw(), dt, C0, RHO0, v0=v0, bcs=mesh.bcs(), upwind=upwind, sources=sources,
                    num_threads=num_threads)


def energy(pre, lay, u):
    K, np_ = pre.num_el, pre.np
    detj = pre.arrays()["el_jacobian_dets"]
    M = lay["mass"]
    e = 0.0
    for q in range(pre.dim + 1):
        Q = u[q].reshape(K, np_)
        w = np.einsum("ei,ij,ej->e", Q, M, Q) * detj
        e += w.sum() / (RHO0 * C0 * C0) if q == 0 else RHO0 * w.sum()
    return 0.5 * e


@pytest.mark.parametrize("dim,order", [(2, 1), (2, 3), (3, 2), (3, 3)])
def test_constant_pressure_is_steady(dim, order):
    m = (D.Mesh.box_tri(4, 3, order=order, side_names=("Reflecting",) * 4) if dim == 2 else
         D.Mesh.box_tet(2, 2, 2, order=order, side_names=("Reflecting",) * 6))
    pre = D.Precomp(m)
    orc = oracle_for(m, 1e-5)
    u = np.zeros((4, pre.ndof))
    u[0] = 3.0
    r = orc.rhs(u)
    assert np.abs(r).max() < 1e-12 * 3.0 * C0 * C0 * RHO0 * 1e-5 * 1e3


@pytest.mark.parametrize("dim,order", [(2, 2), (2, 3), (3, 3)])
def test_linear_pressure_gives_exact_acceleration(dim, order):
    m = (D.Mesh.box_tri(3, 3, order=order, side_names=("Reflecting",) * 4) if dim == 2 else
         D.Mesh.box_tet(2, 2, 1, order=order, side_names=("Reflecting",) * 6))
    pre = D.Precomp(m)
    dt = 1e-5
    orc = oracle_for(m, dt)
    x = pre.dof_coords()
    a = np.array([0.7, -1.3, 0.4])[:dim]
    u = np.zeros((4, pre.ndof))
    u[0] = x[:, :dim] @ a + 2.0
    r = orc.rhs(u)
    for d in range(dim):
        assert np.allclose(r[1 + d], -dt * a[d] / RHO0, rtol=1e-10, atol=1e-14)
    assert np.abs(r[0]).max() < 1e-9


def standing_mode_error(n, order):
    m = D.Mesh.box_tri(n, n, (-1, -1), (1, 1), order=order, side_names=("Reflecting",) * 4)
    pre = D.Precomp(m)
    x = pre.dof_coords()
    k = np.pi / 2
    w = C0 * k
    T = 0.25 * 2 * np.pi / w
    steps = 40 * n // 4
    dt = T / steps
    orc = oracle_for(m, dt, upwind=True)
    u = np.zeros((4, pre.ndof))
    u[0] = np.cos(k * (x[:, 0] + 1))
    orc.set_state(u)
    orc.run(0.0, steps)
    got = orc.get_state()
    p_ex = np.cos(k * (x[:, 0] + 1)) * np.cos(w * T)
    v_ex = k / (RHO0 * w) * np.sin(k * (x[:, 0] + 1)) * np.sin(w * T)
    return np.abs(got[0] - p_ex).max() + RHO0 * C0 * np.abs(got[1] - v_ex).max()


@pytest.mark.parametrize("order", [1, 2])
def test_standing_mode_converges_at_high_order(order):
    e1, e2 = standing_mode_error(4, order), standing_mode_error(8, order)
    rate = np.log2(e1 / e2)
    assert rate > order + 0.5, (e1, e2, rate)


def standing_mode_error_3d(n, order):
    """The same x-standing mode in a reflecting cube [-1,1]^3 of n^3 x 6 tets;
    vy and vz stay zero."""
    m = D.Mesh.box_tet(n, n, n, (-1, -1, -1), (1, 1, 1), order=order, side_names=("Reflecting",) * 6)
    pre = D.Precomp(m)
    x = pre.dof_coords()
    k = np.pi / 2
    w = C0 * k
    T = 0.25 * 2 * np.pi / w
    steps = 10 * n
    orc = oracle_for(m, T / steps, upwind=True)
    u = np.zeros((4, pre.ndof))
    u[0] = np.cos(k * (x[:, 0] + 1))
    orc.set_state(u)
    orc.run(0.0, steps)
    got = orc.get_state()
    p_ex = np.cos(k * (x[:, 0] + 1)) * np.cos(w * T)
    v_ex = k / (RHO0 * w) * np.sin(k * (x[:, 0] + 1)) * np.sin(w * T)
    return np.abs(got[0] - p_ex).max() + RHO0 * C0 * (np.abs(got[1] - v_ex).max() + np.abs(got[2:]).max())


@pytest.mark.parametrize("order", [1, 2, 3])
def test_standing_mode_converges_at_high_order_3d(order):
    # measured rates on 3^3 -> 6^3 cubes: 1.79, 2.80, 3.90 (p + 1 asymptotically)
    e1, e2 = standing_mode_error_3d(3, order), standing_mode_error_3d(6, order)
    rate = np.log2(e1 / e2)
    assert rate > order + 0.5, (e1, e2, rate)


@pytest.mark.parametrize("dim,order", [(2, 2), (2, 3), (2, 4), (3, 2), (3, 3)])
def test_constant_state_is_steady_on_curved_elements(dim, order):
    # every element curved (per-point form), reflecting walls: the Gauss(2p)
    # volume and face integrals of a constant flux cancel to rounding
    from curved_model import boundary_fixed_mesh

    m = boundary_fixed_mesh(D, dim, order)
    pre = D.Precomp(m)
    assert pre.num_curved == pre.num_el
    orc = oracle_for(m, 1e-5, upwind=True)
    u = np.zeros((4, pre.ndof))
    u[0] = 1.0
    orc.set_state(u)
    orc.run(0.0, 5)
    got = orc.get_state()
    assert np.abs(got[0] - 1.0).max() < 1e-12
    assert np.abs(got[1:]).max() < 1e-14


def test_right_hand_side_is_the_same_for_every_thread_count():
    # numThreads = 1 is read as 0 (configParser.cpp:57-58): with a one-thread
    # outer team the nested face loop would share its scratch vectors
    m = D.Mesh.box_tet(2, 2, 2, order=2, side_names=("Reflecting", "Absorbing") * 3)
    pre = D.Precomp(m)
    u0 = pre.initial_state([(0, 0.4, 0.5, 0.6, 0.02, 1.0)])
    ref = oracle_for(m, 1e-5, upwind=True, num_threads=0).rhs(u0)
    for nt in (1, 2, 3):
        o = oracle_for(m, 1e-5, upwind=True, num_threads=nt)
        for _ in range(3):
            assert np.array_equal(o.rhs(u0), ref), nt


def test_upwind_energy_decays_and_reference_sign_3d_p3_grows():
    m = D.Mesh.box_tet(2, 2, 2, order=3, side_names=("Reflecting",) * 6)
    pre = D.Precomp(m)
    lay = pre.layout()
    dt = D.cfl_dt(pre, C0)
    rng = np.random.default_rng(1)
    u0 = np.zeros((4, pre.ndof))
    u0[0] = pre.initial_state([(0, 0.5, 0.5, 0.5, 0.05, 1.0)])[0] + 1e-3 * rng.standard_normal(pre.ndof)
    e0 = energy(pre, lay, u0)
    up = oracle_for(m, dt, upwind=True)
    up.set_state(u0)
    energies = []
    for _ in range(5):
        up.run(0.0, 4)
        energies.append(energy(pre, lay, up.get_state()))
    assert all(b <= a * (1 + 1e-12) for a, b in zip([e0] + energies, energies)), energies
    # the reference's jump sign for 3D order 3 (fc = -1 with the first-point
    # normal pointing out of the first neighbour) is anti-dissipative
    ref = oracle_for(m, dt, upwind=False)
    assert ref.mesh()["fc"] == -1
    ref.set_state(u0)
    ref.run(0.0, 20)
    assert energy(pre, lay, ref.get_state()) > e0


def test_centred_pulse_keeps_point_symmetry():
    m = D.Mesh.box_tri(6, 6, (-1, -1), (1, 1), order=3, side_names=("Reflecting",) * 4)
    pre = D.Precomp(m)
    x = pre.dof_coords().reshape(pre.num_el, pre.np, 3)
    cent = x.mean(axis=1)
    key = {tuple(np.round(c[:2], 9)): e for e, c in enumerate(cent)}
    perm = np.empty((pre.num_el, pre.np), dtype=int)
    for e in range(pre.num_el):
        e2 = key[tuple(np.round(-cent[e, :2], 9))]
        for i in range(pre.np):
            d = np.abs(x[e2, :, :2] + x[e, i, :2]).sum(axis=1)
            perm[e, i] = e2 * pre.np + int(np.argmin(d))
    dt = D.cfl_dt(pre, C0)
    orc = oracle_for(m, dt)
    orc.set_state(pre.initial_state([(0, 0.0, 0.0, 0.0, 0.05, 1.0)]))
    orc.run(0.0, 30)
    u = orc.get_state()
    flat = perm.reshape(-1)
    scale = np.abs(u[0]).max()
    assert np.abs(u[0] - u[0][flat]).max() < 1e-12 * scale
    vs = np.abs(u[1]).max()
    assert np.abs(u[1] + u[1][flat]).max() < 1e-11 * vs


def test_reference_time_loop_step_count():
    m = D.Mesh.box_tri(2, 2, order=1, side_names=("Reflecting",) * 4)
    pre = D.Precomp(m)
    dt = 1e-4
    orc = oracle_for(m, dt)
    n, _ = orc.run_until(0.0, (7 - 0.5) * dt)
    assert n == 7


def test_nested_and_deduplicated_face_loops_agree():
    m = D.Mesh.box_tri(5, 5, order=2, side_names=("Reflecting", "Absorbing") * 2)
    pre = D.Precomp(m)
    u0 = pre.initial_state([(0, 0.1, 0.2, 0.0, 0.1, 1.0)])
    a = oracle_for(m, 1e-5, num_threads=3)
    a.set_state(u0)
    a.run(0.0, 5, dedup=False)
    b = oracle_for(m, 1e-5, num_threads=3)
    b.set_state(u0)
    b.run(0.0, 5, dedup=True)
    assert np.array_equal(a.get_state(), b.get_state())


def test_forward_euler_step_is_state_plus_rhs():
    """timeIntMethod = Euler1 (solver.cpp:152-153): one step from u gives
    u + dt M^-1 (S - F) evaluated at u, which oracle_rhs returns."""
    mesh = D.Mesh.box_tri(4, 3, (-1.0, -1.0), (1.0, 1.0), order=3,
                          side_names=("Reflecting", "Absorbing", "Reflecting", "Absorbing"))
    pre = D.Precomp(mesh)
    dt = 0.2 * D.cfl_dt(pre, 340.0, (0.0, 0.0, 0.0))
    u0 = pre.initial_state([(0, 0.1, 0.2, 0.0, 0.05, 1.0)])
    u0[1:3] += 1e-3 * np.random.default_rng(3).standard_normal((2, pre.ndof))
    orc = O.Oracle(mesh.raw(), dt, 340.0, 1.225, bcs=mesh.bcs())
    rhs = orc.rhs(u0)
    orc.set_state(u0)
    orc.set_method("Euler1")
    t, _ = orc.run(0.0, 1)
    got = orc.get_state()
    assert t == dt
    assert np.allclose(got, u0 + rhs, rtol=0, atol=1e-13 * np.abs(u0).max())
