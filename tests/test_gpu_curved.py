"""Curved (isoparametric, non-affine) elements on the GPU: the per-point
kernel together with the affine kernels must reproduce the oracle, which
evaluates every element and face at the points of its Gauss(2p) rule as the
reference does (Mesh.cpp:31-78, 135-194, 440-557).  FP64 is held to 1e-10
relative L2 per field at every order 2-5, FP32 to 1e-5."""
from __future__ import annotations

import numpy as np
import pytest

import dgcuda as D
import oracle_py as O
from curved_model import bump3, curved_mesh as _curved_mesh

pytestmark = pytest.mark.gpu

C0, RHO0 = 340.0, 1.225


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / nb if nb > 0 else np.linalg.norm(a - b)


def curved_mesh(dim, order, warp=None):
    return _curved_mesh(D, dim, order, warp)


def initial(pre, seed=3):
    rng = np.random.default_rng(seed)
    c = pre.dof_coords().mean(axis=0)
    u0 = pre.initial_state([(0, *c, 0.05, 1.0)])
    u0[1:pre.dim + 1] += 1e-3 * rng.standard_normal((pre.dim, pre.ndof))
    return u0


def run_pair(m, pre, nsteps, precision="fp64", flux="reference", v0=(0.0, 0.0, 0.0), method="rk4", nbatch=1):
    dt = 0.5 * D.cfl_dt(pre, C0, v0)
    u0 = initial(pre)
    s = D.Solver(pre, C0, RHO0, v0, precision=precision, flux=flux, nbatch=nbatch)
    s.set_state(u0)
    if method == "rk4":
        s.rk4_steps(0.0, dt, nsteps)
    else:
        s.euler_steps(0.0, dt, nsteps)
    orc = O.Oracle(m.raw(), dt, C0, RHO0, v0=v0, bcs=m.bcs(), upwind=(flux == "upwind"))
    if method != "rk4":
        orc.set_method("Euler1")
    orc.set_state(u0)
    orc.run(0.0, nsteps)
    return s, orc.get_state()


@pytest.mark.parametrize("dim,order", [(2, 2), (2, 3), (2, 4), (2, 5), (3, 2), (3, 3), (3, 4), (3, 5)])
def test_fully_curved_mesh_matches_oracle(dim, order):
    m, pre = curved_mesh(dim, order)
    assert pre.num_curved == pre.num_el
    v0 = (30.0, -20.0, 10.0 if dim == 3 else 0.0)
    s, ref = run_pair(m, pre, 15, v0=v0)
    info = s.info()
    assert info["curved"] == pre.num_el
    got = s.get_state()
    tol = 1e-10
    for q in range(dim + 1):
        assert rel(got[q], ref[q]) <= tol, (q, rel(got[q], ref[q]))


@pytest.mark.parametrize("flux", ["reference", "upwind"])
def test_partly_curved_mesh_matches_oracle(flux):
    m, pre = curved_mesh(3, 3, warp=bump3)
    assert 0 < pre.num_curved < pre.num_el
    s, ref = run_pair(m, pre, 20, flux=flux)
    assert s.info()["curved"] == pre.num_curved
    got = s.get_state()
    for q in range(4):
        assert rel(got[q], ref[q]) <= 1e-10, (q, rel(got[q], ref[q]))


def test_curved_forward_euler_matches_oracle():
    m, pre = curved_mesh(2, 3)
    s, ref = run_pair(m, pre, 9, method="euler")
    got = s.get_state()
    for q in range(3):
        assert rel(got[q], ref[q]) <= 1e-10


def test_curved_fp32_matches_oracle():
    m, pre = curved_mesh(3, 3)
    s, ref = run_pair(m, pre, 15, precision="fp32", flux="upwind")
    got = s.get_state()
    for q in range(4):
        assert rel(got[q], ref[q]) <= 1e-5, (q, rel(got[q], ref[q]))


def test_curved_batch_members_are_independent_runs():
    m, pre = curved_mesh(3, 2, warp=bump3)
    dt = 0.5 * D.cfl_dt(pre, C0)
    us = [initial(pre, seed=k) for k in range(3)]
    b = D.Solver(pre, C0, RHO0, nbatch=3)
    for k, u in enumerate(us):
        b.set_state(u, member=k)
    b.rk4_steps(0.0, dt, 8)
    for k, u in enumerate(us):
        s = D.Solver(pre, C0, RHO0)
        s.set_state(u)
        s.rk4_steps(0.0, dt, 8)
        assert np.array_equal(b.get_state(member=k), s.get_state())


def test_curved_energy_monitor_uses_element_mass():
    m, pre = curved_mesh(3, 3)
    u = initial(pre)
    s = D.Solver(pre, C0, RHO0)
    s.set_state(u)
    energy, l2, status = s.monitors()
    ca = pre.curved_arrays()
    w = ca["el_qp"][:, 3]
    q = u.reshape(4, pre.num_el, pre.np)
    tot = np.zeros(4)
    for e in range(pre.num_el):
        M = np.einsum("gi,gj,g->ij", ca["el_phi"], ca["el_phi"], w * ca["el_detj"][e])
        for f in range(4):
            tot[f] += q[f, e] @ M @ q[f, e]
    assert status == 0
    assert abs(energy - 0.5 * (tot[0] / (RHO0 * C0 ** 2) + RHO0 * tot[1:].sum())) <= 1e-12 * energy
    assert np.allclose(l2, np.sqrt(tot), rtol=1e-12)


def test_curved_msh_round_trip_runs(tmp_path):
    m, pre = curved_mesh(3, 2)
    path = tmp_path / "curved.msh"
    m.write_msh(path)
    m2 = D.Mesh.read_msh(path)
    pre2 = D.Precomp(m2)
    assert pre2.num_curved == pre.num_curved
    s, ref = run_pair(m2, pre2, 10)
    got = s.get_state()
    for q in range(4):
        assert rel(got[q], ref[q]) <= 1e-10


@pytest.mark.parametrize("dim,order,warp", [(3, 3, "bump"), (3, 2, "full"), (2, 3, "full")])
def test_mixed_form_on_curved_meshes(dim, order, warp):
    """Mixed form on curved meshes: straight elements on the tensor-core
    kernel, curved ones on the per-point kernel in FP32 with the same FP32-pair
    state update; 1e-6 relative L2 against the oracle over a short run, as
    for straight meshes."""
    m, pre = curved_mesh(dim, order, warp=bump3 if warp == "bump" else None)
    v0 = (30.0, -20.0, 10.0 if dim == 3 else 0.0)
    s, ref = run_pair(m, pre, 15, precision="mixed", flux="upwind", v0=v0)
    assert s.info()["curved"] == pre.num_curved
    got = s.get_state()
    for q in range(dim + 1):
        assert rel(got[q], ref[q]) <= 1e-6, (q, rel(got[q], ref[q]))


def test_mixed_form_on_curved_mesh_batch_euler_and_long_run():
    """Forward Euler and a batch in the mixed form on a partly curved mesh,
    and 400 RK4 steps against the FP64 form (1e-5)."""
    m, pre = curved_mesh(3, 3, warp=bump3)
    s, ref = run_pair(m, pre, 9, precision="mixed", flux="upwind", method="euler")
    got = s.get_state()
    for q in range(4):
        assert rel(got[q], ref[q]) <= 1e-6, (q, rel(got[q], ref[q]))
    dt = 0.5 * D.cfl_dt(pre, C0)
    us = [initial(pre, seed=k) for k in range(2)]
    mx = D.Solver(pre, C0, RHO0, precision="mixed", flux="upwind", nbatch=2)
    f64 = D.Solver(pre, C0, RHO0, precision="fp64", flux="upwind", nbatch=2)
    for k, u in enumerate(us):
        mx.set_state(u, member=k)
        f64.set_state(u, member=k)
    mx.rk4_steps(0.0, dt, 400)
    f64.rk4_steps(0.0, dt, 400)
    for k in range(2):
        a, b = mx.get_state(member=k), f64.get_state(member=k)
        for q in range(4):
            assert rel(a[q], b[q]) <= 1e-5, (k, q, rel(a[q], b[q]))


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-5)])
def test_curved_batch_sources_and_receivers(precision, tol):
    """Members of a batch on a partly curved mesh, each with its own pulse
    and source (reference type or Gaussian-weighted), against their own
    oracle runs; receivers record the pressure after every step."""
    from test_gpu_batch import batch_sources, member_inputs, oracle_member

    m, pre = curved_mesh(3, 2, warp=bump3)
    assert 0 < pre.num_curved < pre.num_el
    dt = 0.5 * D.cfl_dt(pre, C0)
    inputs = member_inputs(pre, 3, seed=21)
    rec = np.random.default_rng(2).choice(pre.ndof, 5, replace=False).astype(np.int32)
    nsteps = 17
    sol = D.Solver(pre, C0, RHO0, precision=precision, flux="upwind", nbatch=3)
    for k, inp in enumerate(inputs):
        sol.set_state(inp[0], member=k)
    sol.set_batch_sources(batch_sources(pre, inputs))
    sol.set_receivers(rec, max_steps=nsteps)
    t = sol.rk4_steps(0.0, dt, nsteps)
    tr = sol.traces()
    for k, inp in enumerate(inputs):
        got = sol.get_state(member=k)
        t_ref, ref = oracle_member(m, dt, inp, nsteps, upwind=True)
        assert t == t_ref
        for q in range(4):
            assert rel(got[q], ref[q]) <= tol, (k, q, rel(got[q], ref[q]))
        assert np.array_equal(tr[k, :, -1], got[0][rec])
