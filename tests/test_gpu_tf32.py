"""The 3xTF32 tensor-core form (DG_PREC_TF32X3) against the oracle.

Same pipeline as the exact tensor-core form (FP32 stage data, state kept as an
FP32 pair), but the volume + lift contraction is a_hi b_hi + a_hi b_lo +
a_lo b_hi with TF32 parts on kind::tf32 MMAs and FP32 accumulation.  A CPU
emulation of this arithmetic with round-to-nearest sums (tests/tc_model.py,
two A and two B parts) gives 0.5e-7 to 4.1e-7 relative L2 against FP64 after
these 12-step runs; on the GB300 the tensor cores' own FP32 accumulation
measured up to 2.8e-6 (3D order 4, 165 K-columns), so the tolerance is 5e-6.
Over long runs of a growing solution those sums are amplified (see the
long-run test)."""
from __future__ import annotations

import numpy as np
import pytest

import dgcuda as D
from test_gpu_parity import C0, RHO0, make_mesh, rel_l2, run_pair

pytestmark = pytest.mark.gpu

TF32_TOL = 5e-6


@pytest.mark.parametrize("dim,order", [(2, 1), (2, 2), (2, 3), (2, 4), (2, 5), (3, 1), (3, 2), (3, 3), (3, 4)])
@pytest.mark.parametrize("bc", ["refl", "mixed"])
def test_tf32x3_form_matches_oracle(dim, order, bc):
    got, ref, dim = run_pair(dim, order, bc, precision="tf32x3", flux="upwind", v0=(30.0, -20.0, 10.0))
    for q in range(dim + 1):
        assert rel_l2(got[q], ref[q]) <= TF32_TOL, (q, rel_l2(got[q], ref[q]))


def test_tf32x3_with_sources_and_partial_tiles():
    srcs = [(0.2, 0.1, 0.0, 0.3, 2.0, 1500.0, 0.0, 1e-3)]
    got, ref, dim = run_pair(2, 3, "refl", sources=srcs, nsteps=40, precision="tf32x3")
    for q in range(3):
        assert rel_l2(got[q], ref[q]) <= TF32_TOL


@pytest.mark.parametrize("dim,order", [(2, 3), (3, 3)])
def test_tf32x3_euler(dim, order):
    got, ref, dim = run_pair(dim, order, "mixed", precision="tf32x3", flux="upwind", nsteps=37,
                             method="Euler1", dt_scale=0.2)
    for q in range(dim + 1):
        assert rel_l2(got[q], ref[q]) <= TF32_TOL, (q, rel_l2(got[q], ref[q]))


def test_tf32x3_batch_members_against_fp64_batch():
    mesh = make_mesh(3, 3, "mixed")
    pre = D.Precomp(mesh)
    v0 = (40.0, 0.0, 0.0)
    dt = D.cfl_dt(pre, C0, v0)
    u0 = pre.initial_state([(0, 0.5, 0.35, 0.3, 0.02, 1.0)])
    sols = {}
    for prec in ("fp64", "tf32x3"):
        s = D.Solver(pre, C0, RHO0, v0, precision=prec, flux="upwind", nbatch=3)
        for m in range(3):
            s.set_state(u0 * (1.0 + m), member=m)
        s.rk4_steps(0.0, dt, 15)
        sols[prec] = s
    for m in range(3):
        rel, bad = sols["tf32x3"].error_vs(sols["fp64"], member=m, ref_member=m)
        assert bad == 0 and max(rel) <= TF32_TOL, (m, rel)


def test_tf32x3_long_run_against_fp64():
    """The growing Mach-0.3 case of the exact form's long-run test (1000
    steps, 3D order 3, absorbing walls): 3xTF32 stays finite and within 1e-2
    of FP64.  It does not meet the exact form's 1e-5 here: measured 1.9e-3 on
    the GB300 (the benchmark reports 1.4e-3 after config 2's 2000 steps);
    the tensor cores' FP32 sums of every K-step are rounded, and the growing
    solution amplifies that error."""
    mesh = D.Mesh.box_tet(6, 6, 6, order=3, side_names=("Absorbing",) * 6)
    pre = D.Precomp(mesh)
    v0 = (0.3 * C0, 0.0, 0.0)
    dt = D.cfl_dt(pre, C0, v0)
    u0 = pre.initial_state([(0, 0.45, 0.55, 0.5, 2 * 0.05 ** 2, 1.0)])
    sols = {}
    for prec in ("fp64", "tf32x3"):
        s = D.Solver(pre, C0, RHO0, v0, precision=prec, flux="upwind")
        s.set_state(u0)
        s.rk4_steps(0.0, dt, 1000)
        sols[prec] = s
    rel, bad = sols["tf32x3"].error_vs(sols["fp64"])
    assert bad == 0 and max(rel) <= 1e-2, rel
    print(f"3xTF32 after 1000 steps: rel-L2 vs FP64 {max(rel):.3e}")
