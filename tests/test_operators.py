"""Known answers of the reference-element operators and the geometry that
dg_create uploads (host side, no GPU): the reference mass matrix sums to the
reference element's measure and is symmetric positive definite; the weak
derivative operators D_u = M^-1 Dn_u^T M annihilate constants after
weighting (1^T M D_u = 0) and give back a strong derivative that is exact on
polynomials of degree <= p; the face lifts weight to the reference face
measure; element and boundary-face Jacobian determinants add up to the
domain's volume and surface."""
from __future__ import annotations

import itertools

import numpy as np
import pytest

import dgcuda as D

REF_MEASURE = {2: 0.5, 3: 1.0 / 6.0}       # gmsh reference triangle / tetrahedron
REF_FACE_MEASURE = {2: 2.0, 3: 0.5}        # gmsh reference line [-1, 1] / triangle


def operators(dim, order):
    m = D.Mesh.box_tri(1, 1, order=order) if dim == 2 else D.Mesh.box_tet(1, 1, 1, order=order)
    pre = D.Precomp(m)
    L = pre.layout()
    NP, nf, nfp = L["np"], L["nf"], L["nfp"]
    ops = L["ops"]
    Du = [ops[u * NP * NP:(u + 1) * NP * NP].reshape(NP, NP).T for u in range(dim)]  # stored [u][j][i]
    lift = ops[dim * NP * NP:dim * NP * NP + nf * nfp * NP].reshape(nf * nfp, NP).T  # stored [slot][i]
    # reference coordinates of element 0's nodes (vertices first, gmsh order)
    x = pre.dof_coords()[:NP, :dim]
    A = np.stack([x[k + 1] - x[0] for k in range(dim)], axis=1)
    xi = np.linalg.solve(A, (x - x[0]).T).T
    return L["mass"], Du, lift, xi, nf, nfp


CASES = [(d, p) for d in (2, 3) for p in range(1, 6)]


@pytest.mark.parametrize("dim,order", CASES)
def test_mass_matrix(dim, order):
    M = operators(dim, order)[0]
    assert abs(M.sum() - REF_MEASURE[dim]) < 1e-13
    assert np.abs(M - M.T).max() < 1e-15
    assert np.linalg.eigvalsh(M).min() > 0


@pytest.mark.parametrize("dim,order", CASES)
def test_weak_derivative_operators(dim, order):
    M, Du, _, xi, _, _ = operators(dim, order)
    Minv = np.linalg.inv(M)
    for u in range(dim):
        # integral of d(1)/du times any polynomial vanishes
        assert np.abs((M @ Du[u]).sum(axis=0)).max() < 1e-14
        # strong derivative Dn_u = M^-1 D_u^T M, exact on degree <= p
        Dn = Minv @ Du[u].T @ M
        for a in itertools.product(range(order + 1), repeat=dim):
            if sum(a) > order:
                continue
            f = np.prod([xi[:, k] ** a[k] for k in range(dim)], axis=0)
            b = list(a)
            if b[u] == 0:
                want = np.zeros(len(f))
            else:
                c = b[u]
                b[u] -= 1
                want = c * np.prod([xi[:, k] ** b[k] for k in range(dim)], axis=0)
            assert np.abs(Dn @ f - want).max() < 1e-11, (u, a)


@pytest.mark.parametrize("dim,order", CASES)
def test_face_lifts_weigh_the_reference_face(dim, order):
    M, _, lift, _, nf, nfp = operators(dim, order)
    ML = M @ lift  # = E_f M_f per face: the face mass scattered to the element's face nodes
    for f in range(nf):
        assert abs(ML[:, f * nfp:(f + 1) * nfp].sum() - REF_FACE_MEASURE[dim]) < 1e-13


@pytest.mark.parametrize("dim,order", [(2, 1), (2, 4), (3, 2), (3, 3)])
def test_jacobians_add_up_to_volume_and_surface(dim, order):
    if dim == 2:
        m = D.Mesh.box_tri(3, 5, (-1.0, 0.0), (2.0, 0.5), order=order)
        vol, surf = 3.0 * 0.5, 2 * (3.0 + 0.5)
    else:
        m = D.Mesh.box_tet(2, 3, 2, (0.0, 0.0, 0.0), (1.0, 2.0, 0.5), order=order)
        vol, surf = 1.0, 2 * (1.0 * 2.0 + 1.0 * 0.5 + 2.0 * 0.5)
    a = D.Precomp(m).arrays()
    assert abs(a["el_jacobian_dets"].sum() * REF_MEASURE[dim] - vol) < 1e-12 * vol
    bnd = a["f_is_boundary"] != 0
    assert abs(np.abs(a["f_jacobian_dets"][bnd]).sum() * REF_FACE_MEASURE[dim] - surf) < 1e-12 * surf
