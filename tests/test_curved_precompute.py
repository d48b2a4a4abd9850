"""Curved elements on the CPU: the product's quadrature tables, its per-point
precompute against the oracle's (which restates gmsh's getJacobians and the
reference's normal construction, Mesh.cpp:31-78, 135-194), the affine/curved
classification, and the per-point algebra of the curved stage kernel (NumPy
model) against the oracle's right-hand side."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import dgcuda as D
import oracle_py as O
from curved_model import boundary_fixed_mesh, bump3, curved_mesh, model_rhs

ROOT = Path(__file__).resolve().parent.parent


def _tables(path, prefix):
    out = {}
    for m in re.finditer(r"static const double (\w+)\[\] = \{(.*?)\};", path.read_text(), re.S):
        vals = np.array([float(v) for v in re.findall(r"[-+0-9.eE]+", m.group(2))])
        out[m.group(1).replace(prefix, "")] = vals.reshape(-1, 4)
    return out


def test_product_rules_equal_the_oracle_rules():
    a = _tables(ROOT / "dgfem-acoustic_gb300/csrc/host/rules.inc", "kRule")
    b = _tables(ROOT / "oracle/quadrature_tables.inc", "k")
    assert sorted(a) == sorted(b) and len(a) == 15
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def _oracle_points(m):
    orc = O.Oracle(m.raw(), 1e-6, 340.0, 1.225, bcs=m.bcs())
    v = O.MeshView()
    O.lib().oracle_mesh(orc._h, C.byref(v))
    K, F, ng, ngf = v.num_el, v.f_num, v.n_el_qp, v.n_f_qp
    return (orc.mesh(), O._arr(v.el_jac_dets, K * ng, np.float64).reshape(K, ng),
            O._arr(v.f_jac_dets, F * ngf, np.float64).reshape(F, ngf),
            O._arr(v.f_normals, F * ngf * 3, np.float64).reshape(F, ngf, 3))


@pytest.mark.parametrize("dim,order", [(2, 2), (2, 3), (2, 5), (3, 2), (3, 3), (3, 4), (3, 5)])
def test_per_point_arrays_match_the_oracle(dim, order):
    m, pre = curved_mesh(D, dim, order)
    assert pre.num_curved == pre.num_el
    ca, ar = pre.curved_arrays(), pre.arrays()
    om, edet, fdet, fnrm = _oracle_points(m)
    # the oracle builds its monomial basis in extended precision, so every
    # order agrees to a few 1e-14
    tol = 1e-12
    assert np.abs(ca["el_detj"] - edet).max() <= tol * np.abs(edet).max()
    assert np.abs(ca["f_detj"] - fdet).max() <= tol * np.abs(fdet).max()
    assert np.abs(ca["f_normal"] - fnrm).max() <= tol
    assert np.array_equal(ar["el_f_orientation"], om["el_f_orientation"])
    assert np.array_equal(ar["f_node_tags"], om["f_node_tags"])
    # first-point arrays are the per-point arrays at point 0
    assert np.array_equal(ar["f_normals"], ca["f_normal"][:, 0, :])
    assert np.array_equal(ar["el_jacobian_dets"], ca["el_detj"][:, 0])


def test_affine_and_curved_classification():
    m = D.Mesh.box_tet(2, 2, 2, order=3)
    pre = D.Precomp(m)
    assert pre.num_curved == 0 and pre.curved_arrays() == {}
    m, pre = curved_mesh(D, 3, 3, warp=bump3)
    flags = pre.curved_arrays()["curved"]
    assert 0 < pre.num_curved == flags.sum() < pre.num_el
    # elements entirely in x < 0.5 are left straight
    xyz = pre.dof_coords().reshape(pre.num_el, pre.np, 3)
    assert not flags[(xyz[:, :, 0] < 0.5 - 1e-12).all(axis=1)].any()
    # order 1 elements are always affine
    m1 = D.Mesh.box_tet(2, 2, 2, order=1)
    m1.warp(lambda x: x + 0.03 * np.sin(3 * x))
    assert D.Precomp(m1).num_curved == 0


def test_layout_view_rejects_curved_meshes():
    m, pre = curved_mesh(D, 2, 2)
    with pytest.raises(D.DGError) as ei:
        pre.layout()
    assert ei.value.code == -3


def test_curved_msh_round_trip(tmp_path):
    m, pre = curved_mesh(D, 3, 3, warp=bump3)
    m.write_msh(tmp_path / "c.msh")
    pre2 = D.Precomp(D.Mesh.read_msh(tmp_path / "c.msh"))
    assert pre2.num_curved == pre.num_curved
    a, b = pre.curved_arrays(), pre2.curved_arrays()
    assert np.allclose(a["el_detj"], b["el_detj"], rtol=1e-14, atol=0)


@pytest.mark.parametrize("dim,order,v0,upwind", [(2, 3, (40.0, 10.0, 0.0), False), (3, 2, (30.0, -20.0, 10.0), False),
                                                 (3, 2, (0.0, 0.0, 0.0), True)])
def test_per_point_algebra_matches_the_oracle_rhs(dim, order, v0, upwind):
    m, pre = curved_mesh(D, dim, order)
    rng = np.random.default_rng(1)
    u = rng.standard_normal((4, pre.ndof))
    if dim == 2:
        u[3] = 0
    dt = 1e-6
    orc = O.Oracle(m.raw(), dt, 340.0, 1.225, v0=v0, bcs=m.bcs(), upwind=upwind)
    ref = orc.rhs(u)
    got = dt * model_rhs(pre, u, 340.0, 1.225, v0, upwind=upwind)
    for q in range(dim + 1):
        assert np.linalg.norm(got[q] - ref[q]) <= 1e-12 * np.linalg.norm(ref[q])



@pytest.mark.parametrize("dim,order", [(2, 2), (2, 3), (2, 5), (3, 2), (3, 3), (3, 4)])
def test_per_point_geometry_keeps_volume_surface_and_normals(dim, order):
    # detJ of a degree-p map has degree dim*(p-1) <= 2p: the Gauss(2p) rules
    # integrate it exactly, so the curved elements fill the unit domain exactly
    pre = D.Precomp(boundary_fixed_mesh(D, dim, order))
    c = pre.curved_arrays()
    a = pre.arrays()
    assert c["curved"].all()
    w, wf = c["el_qp"][:, 3], c["f_qp"][:, 3]
    assert abs((c["el_detj"] * w).sum() - 1.0) < 1e-13
    bnd = a["f_is_boundary"] != 0
    assert abs((np.abs(c["f_detj"][bnd]) * wf).sum() - 2.0 * dim) < 1e-13
    # per-point normals are unit vectors; on the (planar) boundary faces they
    # are coordinate axes
    assert np.abs(np.linalg.norm(c["f_normal"], axis=2) - 1.0).max() < 1e-13
    assert np.abs(np.abs(c["f_normal"][bnd]).max(axis=2) - 1.0).max() < 1e-13
