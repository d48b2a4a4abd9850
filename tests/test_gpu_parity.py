"""GPU parity: the product's CUDA path (through the C ABI) against the CPU
oracle on the same seeded inputs.  FP64 tolerance: 1e-10 relative L2 per
field (the factored operators differ from the oracle's quadrature only by
rounding); FP32: 1e-5 relative L2."""
from __future__ import annotations

import numpy as np
import pytest

import dgcuda as D
import oracle_py as O

pytestmark = pytest.mark.gpu

C0, RHO0 = 340.0, 1.225
FP64_TOL = 1e-10
FP32_TOL = 1e-5


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / nb if nb > 0 else np.linalg.norm(a - b)


def make_mesh(dim, order, bc):
    if dim == 2:
        names = {"refl": ("Reflecting",) * 4, "abs": ("Absorbing",) * 4,
                 "mixed": ("Reflecting", "Absorbing", "Reflecting", "Absorbing")}[bc]
        return D.Mesh.box_tri(5, 4, (-1.0, -1.0), (1.0, 0.8), order=order, side_names=names)
    names = {"refl": ("Reflecting",) * 6, "abs": ("Absorbing",) * 6,
             "mixed": ("Absorbing", "Reflecting") * 3}[bc]
    return D.Mesh.box_tet(3, 2, 2, (0.0, 0.0, 0.0), (1.0, 0.7, 0.6), order=order, side_names=names)


def run_pair(dim, order, bc, v0=(0.0, 0.0, 0.0), flux="reference", nsteps=12, precision="fp64",
             sources=None, seed=0, use_graph=True, method="Runge-Kutta", dt_scale=1.0):
    mesh = make_mesh(dim, order, bc)
    pre = D.Precomp(mesh)
    dt = dt_scale * D.cfl_dt(pre, C0, v0)
    rng = np.random.default_rng(seed)
    centre = pre.dof_coords().mean(axis=0)
    u0 = pre.initial_state([(0, *centre, 0.02, 1.0)])
    u0[1:dim + 1] += 1e-3 * rng.standard_normal((dim, pre.ndof))
    sol = D.Solver(pre, C0, RHO0, v0, precision=precision, flux=flux, use_graph=use_graph)
    sol.set_state(u0)
    src_cfg = None
    if sources:
        lst = []
        for (x, y, z, size, amp, f, ph, dur) in sources:
            lst.append((pre.source_dofs(x, y, z, size), amp, f, ph, dur))
        sol.set_sources(lst)
        src_cfg = np.array([[0, x, y, z, size, amp, f, ph, dur] for (x, y, z, size, amp, f, ph, dur) in sources])
    steps = sol.euler_steps if method == "Euler1" else sol.rk4_steps
    t = steps(0.0, dt, nsteps)
    got = sol.get_state()
    orc = O.Oracle(mesh.raw(), dt, C0, RHO0, v0=v0, bcs=mesh.bcs(), upwind=(flux == "upwind"), sources=src_cfg)
    orc.set_method(method)
    orc.set_state(u0)
    t_ref, _ = orc.run(0.0, nsteps)
    ref = orc.get_state()
    assert t == t_ref
    return got, ref, dim


@pytest.mark.parametrize("dim,order", [(2, 1), (2, 2), (2, 3), (2, 4), (2, 5), (3, 1), (3, 2), (3, 3), (3, 4),
                                       (3, 5)])
@pytest.mark.parametrize("bc", ["refl", "mixed"])
def test_fp64_matches_oracle(dim, order, bc):
    got, ref, dim = run_pair(dim, order, bc)
    for q in range(dim + 1):
        assert rel_l2(got[q], ref[q]) <= FP64_TOL, (q, rel_l2(got[q], ref[q]))
    assert np.all(got[3] == 0) if dim == 2 else True


@pytest.mark.parametrize("dim,order,v0", [(2, 3, (60.0, -30.0, 0.0)), (3, 3, (102.0, 0.0, 0.0)),
                                          (3, 2, (20.0, 10.0, -15.0))])
def test_fp64_mean_flow(dim, order, v0):
    got, ref, dim = run_pair(dim, order, "abs", v0=v0)
    for q in range(dim + 1):
        assert rel_l2(got[q], ref[q]) <= FP64_TOL


@pytest.mark.parametrize("dim,order", [(2, 3), (3, 3), (3, 2)])
def test_fp64_upwind_mode(dim, order):
    got, ref, dim = run_pair(dim, order, "mixed", flux="upwind")
    for q in range(dim + 1):
        assert rel_l2(got[q], ref[q]) <= FP64_TOL


def test_fp64_sources():
    srcs = [(0.2, 0.1, 0.0, 0.3, 2.0, 1500.0, 0.0, 1e-3), (-0.3, 0.2, 0.0, 0.25, 1.0, 900.0, 0.5, 2e-5)]
    got, ref, dim = run_pair(2, 3, "refl", sources=srcs, nsteps=40)
    for q in range(3):
        assert rel_l2(got[q], ref[q]) <= FP64_TOL


def test_graph_and_direct_launches_agree():
    a, _, _ = run_pair(2, 3, "mixed", nsteps=70, use_graph=True)
    b, _, _ = run_pair(2, 3, "mixed", nsteps=70, use_graph=False)
    assert np.array_equal(a, b)


def test_config1_fp64_1000_steps_matches_oracle():
    """The reference's CPU-runnable case in full: [-1,1]^2 as 64x64 cells x 2
    triangles (8192 elements), order 3, reflecting walls, Gaussian pulse at
    the origin (size 0.02), dt from CFL 0.5, 1000 RK4 steps.  The oracle runs
    its de-duplicated face loop (bit-identical to the reference's nested
    loop, tests/test_oracle.py) on every host core."""
    import os

    mesh = D.Mesh.box_tri(64, 64, (-1.0, -1.0), (1.0, 1.0), order=3, side_names=("Reflecting",) * 4)
    pre = D.Precomp(mesh)
    assert pre.num_el == 8192
    dt = D.cfl_dt(pre, C0)
    u0 = pre.initial_state([(0, 0.0, 0.0, 0.0, 0.02, 1.0)])
    sol = D.Solver(pre, C0, RHO0)
    sol.set_state(u0)
    t = sol.rk4_steps(0.0, dt, 1000)
    got = sol.get_state()
    orc = O.Oracle(mesh.raw(), dt, C0, RHO0, bcs=mesh.bcs(), num_threads=os.cpu_count() or 1)
    orc.set_state(u0)
    t_ref, _ = orc.run(0.0, 1000, dedup=True)
    ref = orc.get_state()
    assert t == t_ref
    for q in range(3):
        assert rel_l2(got[q], ref[q]) <= FP64_TOL, (q, rel_l2(got[q], ref[q]))
    assert np.all(got[3] == 0)


@pytest.mark.parametrize("dim,order", [(2, 3), (3, 3)])
def test_fp32_close_to_oracle(dim, order):
    got, ref, dim = run_pair(dim, order, "mixed", precision="fp32", flux="upwind")
    for q in range(dim + 1):
        assert rel_l2(got[q], ref[q]) <= FP32_TOL


MIXED_TOL = 1e-6


@pytest.mark.parametrize("dim,order", [(2, 1), (2, 2), (2, 3), (2, 4), (2, 5), (3, 1), (3, 2), (3, 3), (3, 4)])
@pytest.mark.parametrize("bc", ["refl", "mixed"])
def test_mixed_form_matches_oracle(dim, order, bc):
    """Tensor-core form: FP32 stage data, exact contraction, state as an FP32
    pair -- close to FP64 over a short run (tolerance 1e-6 relative L2: the
    stage inputs are rounded to FP32)."""
    got, ref, dim = run_pair(dim, order, bc, precision="mixed", flux="upwind", v0=(30.0, -20.0, 10.0))
    for q in range(dim + 1):
        assert rel_l2(got[q], ref[q]) <= MIXED_TOL, (q, rel_l2(got[q], ref[q]))


def test_mixed_form_with_sources_and_partial_tiles():
    srcs = [(0.2, 0.1, 0.0, 0.3, 2.0, 1500.0, 0.0, 1e-3)]
    got, ref, dim = run_pair(2, 3, "refl", sources=srcs, nsteps=40, precision="mixed")
    for q in range(3):
        assert rel_l2(got[q], ref[q]) <= MIXED_TOL


def test_mixed_form_long_run_against_fp64():
    """1000 steps of a 3D order-3 box with Mach 0.3 mean flow and absorbing
    walls (a growing, boundary-driven solution): the mixed form stays within
    1e-5 relative L2 of the FP64 form."""
    mesh = D.Mesh.box_tet(6, 6, 6, order=3, side_names=("Absorbing",) * 6)
    pre = D.Precomp(mesh)
    v0 = (0.3 * C0, 0.0, 0.0)
    dt = D.cfl_dt(pre, C0, v0)
    u0 = pre.initial_state([(0, 0.45, 0.55, 0.5, 2 * 0.05 ** 2, 1.0)])
    out = {}
    for prec in ("fp64", "mixed"):
        s = D.Solver(pre, C0, RHO0, v0, precision=prec, flux="upwind")
        s.set_state(u0)
        s.rk4_steps(0.0, dt, 1000)
        out[prec] = s.get_state()
    for q in range(4):
        assert rel_l2(out["mixed"][q], out["fp64"][q]) <= 1e-5


# Forward Euler ("Euler1", the reference's default integrator).  37 steps =
# one captured 32-step graph chunk plus an odd remainder, which exercises the
# state buffer swap; dt at a fifth of the RK4 CFL value keeps Euler bounded.
@pytest.mark.parametrize("dim,order,bc", [(2, 3, "mixed"), (3, 2, "mixed"), (3, 3, "abs")])
def test_fp64_euler_matches_oracle(dim, order, bc):
    got, ref, dim = run_pair(dim, order, bc, nsteps=37, method="Euler1", dt_scale=0.2, v0=(20.0, 10.0, 0.0))
    for q in range(dim + 1):
        assert rel_l2(got[q], ref[q]) <= FP64_TOL, (q, rel_l2(got[q], ref[q]))


def test_fp64_euler_with_sources_direct_launches():
    srcs = [(0.2, 0.1, 0.0, 0.3, 2.0, 1500.0, 0.0, 1e-3)]
    got, ref, dim = run_pair(2, 3, "refl", sources=srcs, nsteps=21, method="Euler1", dt_scale=0.2,
                             use_graph=False)
    for q in range(3):
        assert rel_l2(got[q], ref[q]) <= FP64_TOL


@pytest.mark.parametrize("precision,tol", [("fp32", FP32_TOL), ("mixed", MIXED_TOL)])
@pytest.mark.parametrize("dim,order", [(2, 3), (3, 3)])
def test_reduced_precision_euler(precision, tol, dim, order):
    got, ref, dim = run_pair(dim, order, "mixed", precision=precision, flux="upwind", nsteps=37,
                             method="Euler1", dt_scale=0.2)
    for q in range(dim + 1):
        assert rel_l2(got[q], ref[q]) <= tol, (q, rel_l2(got[q], ref[q]))


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
def test_euler_then_rk4_in_one_context(precision, tol):
    """An odd number of Euler steps followed by RK4 steps on the same context
    (the state must be back in its own buffers between calls)."""
    mesh = make_mesh(2, 3, "mixed")
    pre = D.Precomp(mesh)
    dt = 0.2 * D.cfl_dt(pre, C0, (0.0, 0.0, 0.0))
    u0 = pre.initial_state([(0, 0.1, -0.2, 0.0, 0.02, 1.0)])
    sol = D.Solver(pre, C0, RHO0, (0.0, 0.0, 0.0), precision=precision, flux="upwind")
    sol.set_state(u0)
    t = sol.euler_steps(0.0, dt, 5)
    t = sol.rk4_steps(t, dt, 33)
    got = sol.get_state()
    orc = O.Oracle(mesh.raw(), dt, C0, RHO0, bcs=mesh.bcs(), upwind=True)
    orc.set_state(u0)
    orc.set_method("Euler1")
    tr, _ = orc.run(0.0, 5)
    orc.set_method("Runge-Kutta")
    tr, _ = orc.run(tr, 33)
    ref = orc.get_state()
    assert t == tr
    for q in range(3):
        assert rel_l2(got[q], ref[q]) <= tol


@pytest.mark.parametrize("dim,order,nbatch", [(3, 2, 3), (2, 3, 1), (2, 5, 2), (3, 1, 1)])
def test_mixed_form_one_and_two_tile_pipelines_agree(dim, order, nbatch):
    """The tensor-core kernels run one tile pipeline per CTA or two (each with
    half of the warps and of the tensor memory, where that fits).  Both do
    the same exact sums on every tile, so the states are bit-identical."""
    mesh = make_mesh(dim, order, "mixed")
    pre = D.Precomp(mesh)
    v0 = (30.0, -20.0, 10.0 if dim == 3 else 0.0)
    dt = D.cfl_dt(pre, C0, v0)
    u0 = pre.initial_state([(0, *pre.dof_coords().mean(axis=0), 0.02, 1.0)])
    out = {}
    for pipes in (1, 2):
        s = D.Solver(pre, C0, RHO0, v0, precision="mixed", flux="upwind", nbatch=nbatch, tc_pipelines=pipes)
        assert s.info()["tc_pipelines"] == pipes
        for m in range(nbatch):
            s.set_state(u0 * (1.0 + m), member=m)
        s.rk4_steps(0.0, dt, 9)
        out[pipes] = [s.get_state(member=m) for m in range(nbatch)]
        s.close()
    for m in range(nbatch):
        assert np.array_equal(out[1][m], out[2][m]), m
