"""Pins the oracle's restatement of gmsh's reference elements with exact
rational arithmetic (CPU only).

The reference takes its Lagrange bases, node lattices and "Gauss<2p>" rules
from the gmsh SDK (Mesh.cpp:25-38, 124-142), which is not in the reference
checkout; the oracle restates them (oracle/dg_oracle.cpp: Basis, get_rule).
These tests recompute, in exact fractions:
  * the integral of every monomial of degree <= 2p over the reference simplex
    and compare the oracle's rules against it;
  * the Lagrange basis on the oracle's lattice (exact inverse of the monomial
    Vandermonde), compared with the oracle's basis values and gradients at
    its rule points, and from it the exact reference mass and stiffness
    matrices, compared entry by entry with what the oracle's rule and basis
    give;
  * the node order of two elements against the node diagrams of the gmsh
    file-format documentation.
"""
from __future__ import annotations

import math
from fractions import Fraction as Fr
from functools import lru_cache

import numpy as np
import pytest

import oracle_py as O


def monomials(dim: int, p: int) -> list[tuple[int, int, int]]:
    out = []
    for a in range(p + 1):
        for b in range(p + 1 - a if dim >= 2 else 1):
            for c in range(p + 1 - a - b if dim == 3 else 1):
                out.append((a, b, c))
    return out


@lru_cache(maxsize=None)
def mono_integral(dim: int, a: int, b: int, c: int) -> Fr:
    """Exact integral of x^a y^b z^c over gmsh's reference element: the line
    [-1, 1], the triangle (0,0),(1,0),(0,1), the tetrahedron with vertices
    at the origin and the unit points."""
    if dim == 1:
        return Fr(2, a + 1) if a % 2 == 0 else Fr(0)
    k = a + b + c
    return Fr(math.factorial(a) * math.factorial(b) * math.factorial(c), math.factorial(k + dim))


def exact_nodes(nodes: np.ndarray, p: int) -> list[tuple[Fr, Fr, Fr]]:
    out = []
    for x in nodes:
        r = tuple(Fr(round(v * p), p) for v in x)
        assert max(abs(float(q) - v) for q, v in zip(r, x)) < 1e-15
        out.append(r)
    return out


def inverse(A: list[list[Fr]]) -> list[list[Fr]]:
    n = len(A)
    M = [row[:] + [Fr(int(i == j)) for j in range(n)] for i, row in enumerate(A)]
    for k in range(n):
        piv = next(r for r in range(k, n) if M[r][k] != 0)
        M[k], M[piv] = M[piv], M[k]
        d = M[k][k]
        M[k] = [v / d for v in M[k]]
        for r in range(n):
            if r != k and M[r][k] != 0:
                f = M[r][k]
                M[r] = [a - f * b for a, b in zip(M[r], M[k])]
    return [row[n:] for row in M]


def exact_matrices(dim: int, p: int, nodes: list[tuple[Fr, Fr, Fr]]):
    mono = monomials(dim, p)
    n = len(mono)
    assert n == len(nodes)
    V = [[x ** m[0] * y ** m[1] * z ** m[2] for m in mono] for (x, y, z) in nodes]
    Cinv = inverse(V)  # phi_k = sum_m Cinv[m][k] mono_m
    # Gram matrices of the monomials
    G = [[mono_integral(dim, a[0] + b[0], a[1] + b[1], a[2] + b[2]) for b in mono] for a in mono]
    Gu = []
    for u in range(dim):
        rows = []
        for a in mono:
            if a[u] == 0:
                rows.append([Fr(0)] * n)
                continue
            d = list(a)
            d[u] -= 1
            rows.append([a[u] * mono_integral(dim, d[0] + b[0], d[1] + b[1], d[2] + b[2]) for b in mono])
        Gu.append(rows)

    def congruence(Gm):
        # C^T Gm C
        T = [[sum(Gm[m][mm] * Cinv[mm][j] for mm in range(n) if Cinv[mm][j] != 0) for j in range(n)]
             for m in range(n)]
        return [[sum(Cinv[m][i] * T[m][j] for m in range(n) if Cinv[m][i] != 0) for j in range(n)]
                for i in range(n)]

    return congruence(G), [congruence(g) for g in Gu]


CASES = [(1, p) for p in range(1, 6)] + [(2, p) for p in range(1, 6)] + [(3, 1), (3, 2), (3, 3), (3, 4)]


@pytest.mark.parametrize("dim,order", CASES + [(3, 5)])
def test_rules_integrate_every_monomial_of_degree_2p(dim, order):
    ref = O.reference_element(dim, order)
    rule = ref["rule"]
    w = rule[:, 3]
    for (a, b, c) in monomials(dim, 2 * order):
        got = float(np.sum(w * rule[:, 0] ** a * rule[:, 1] ** b * rule[:, 2] ** c))
        want = float(mono_integral(dim, a, b, c))
        if want == 0.0:
            assert abs(got) <= 1e-15, (a, b, c, got)
        else:
            assert abs(got - want) <= 5e-14 * abs(want), (a, b, c, got, want)
    if dim >= 2:
        # interior points of the simplex (gmsh's rules have no points outside)
        x = rule[:, :dim]
        assert np.all(x >= -1e-15) and np.all(x.sum(axis=1) <= 1 + 1e-15)


@pytest.mark.parametrize("dim,order", CASES)
def test_lattice_is_the_order_p_simplex_lattice(dim, order):
    nodes = exact_nodes(O.reference_element(dim, order)["nodes"], order)
    assert len(set(nodes)) == len(nodes) == len(monomials(dim, order))
    if dim == 1:
        assert nodes[0][0] == -1 and nodes[1][0] == 1
    else:
        verts = [(Fr(0), Fr(0), Fr(0)), (Fr(1), Fr(0), Fr(0)), (Fr(0), Fr(1), Fr(0)), (Fr(0), Fr(0), Fr(1))]
        assert nodes[:dim + 1] == verts[:dim + 1]
        for x in nodes:
            assert all(v >= 0 for v in x) and sum(x) <= 1


@pytest.mark.parametrize("dim,order", CASES + [(3, 5)])
def test_basis_at_rule_points_equals_the_exact_lagrange_basis(dim, order):
    """The oracle's basis values and gradients at its rule points against the
    exact Lagrange basis of its lattice (rational inverse Vandermonde,
    evaluated at the same double rule points in 40-digit arithmetic)."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    ref = O.reference_element(dim, order)
    nodes = exact_nodes(ref["nodes"], order)
    mono = monomials(dim, order)
    n = len(mono)
    Ci = inverse([[x ** m[0] * y ** m[1] * z ** m[2] for m in mono] for (x, y, z) in nodes])
    Cm = [[mp.mpf(v.numerator) / v.denominator for v in row] for row in Ci]
    rule = ref["rule"]
    phi = np.empty((rule.shape[0], n))
    grad = np.zeros((rule.shape[0], n, 3))
    for g in range(rule.shape[0]):
        x = [mp.mpf(float(v)) for v in rule[g, :3]]
        mv = [x[0] ** a * x[1] ** b * x[2] ** c for (a, b, c) in mono]
        dmv = []
        for u in range(dim):
            row = []
            for (a, b, c) in mono:
                e = [a, b, c]
                if e[u] == 0:
                    row.append(mp.mpf(0))
                    continue
                k = e[u]
                e[u] -= 1
                row.append(k * x[0] ** e[0] * x[1] ** e[1] * x[2] ** e[2])
            dmv.append(row)
        for k in range(n):
            phi[g, k] = float(sum(Cm[m][k] * mv[m] for m in range(n)))
            for u in range(dim):
                grad[g, k, u] = float(sum(Cm[m][k] * dmv[u][m] for m in range(n)))
    # x86-64 long double carries 11 bits more than double: orders <= 4 agree
    # to double rounding, order 5 (monomial coefficients ~1e4) to ~10 ulp
    assert np.abs(ref["phi"] - phi).max() <= 1e-14 * np.abs(phi).max()
    assert np.abs(ref["grad"] - grad).max() <= 1e-14 * np.abs(grad).max()


@pytest.mark.parametrize("dim,order", CASES)
def test_mass_and_stiffness_equal_exact_rational_integrals(dim, order):
    """The rule-and-basis matrices equal the exact integrals.  At 2D order 5
    they agree to 4.6e-14 absolute (6e-13 of the largest entry): the same
    difference as the exact basis integrated with the double-rounded rule
    gives, i.e. the rule's own rounding amplified by the order-5 monomial
    coefficients; every other case agrees to 1e-13 of the largest entry."""
    ref = O.reference_element(dim, order)
    nodes = exact_nodes(ref["nodes"], order)
    M, S = exact_matrices(dim, order, nodes)
    tol = 5e-12 if (dim, order) == (2, 5) else 1e-13
    Mf = np.array([[float(v) for v in row] for row in M])
    scale = np.abs(Mf).max()
    assert np.abs(ref["mass"] - Mf).max() <= tol * scale
    # the exact mass matrix integrates 1 to the element measure
    assert sum(map(sum, M)) == mono_integral(dim, 0, 0, 0)
    for u in range(dim):
        Sf = np.array([[float(v) for v in row] for row in S[u]])
        assert np.abs(ref["stiff"][u] - Sf).max() <= tol * np.abs(Sf).max()
        # columns of S_u sum to zero: sum_i dphi_i/du = 0
        assert all(sum(S[u][i][j] for i in range(len(nodes))) == 0 for j in range(len(nodes)))


def test_node_order_follows_the_gmsh_diagrams():
    """Second-order tetrahedron and third-order triangle node positions as
    drawn in the gmsh file-format documentation (node ordering section)."""
    h, t = Fr(1, 2), Fr(1, 3)
    z = Fr(0)
    tet = exact_nodes(O.reference_element(3, 2)["nodes"], 2)
    assert tet[4:] == [(h, z, z), (h, h, z), (z, h, z), (z, z, h), (z, h, h), (h, z, h)]
    tri = exact_nodes(O.reference_element(2, 3)["nodes"], 3)
    assert tri[3:] == [(t, z, z), (2 * t, z, z), (2 * t, t, z), (t, 2 * t, z), (z, 2 * t, z), (z, t, z),
                       (t, t, z)]
