"""Generates oracle/quadrature_tables.inc: the "Gauss<2p>" integration rules the
oracle uses in place of gmsh's (gmsh 4.1.4, a dependency absent from the
reference checkout; called at Mesh.cpp:31-38 and 135-142).

TEST INFRASTRUCTURE ONLY (part of the oracle).

Rules, restated from the published tables and refined here to full double
precision by least squares on the moment equations (exactness of every
monomial up to the rule's degree is verified before writing):
  * lines: Gauss-Legendre, p+1 points, increasing abscissa;
  * triangles (reference (0,0),(1,0),(0,1)), Dunavant (1985): degree 2 (3 pts),
    4 (6), 6 (12), 8 (16), 10 (25);
  * tetrahedra (reference (0,0,0),(1,0,0),(0,1,0),(0,0,1)): degree 2 (4 pts),
    degree 4 (14 pts, positive weights), degree 6 (Keast 1986, 24 pts);
    degree 8 and 10 use the Stroud conical product of Gauss-Jacobi rules.
Within a symmetric orbit the first point is the one whose barycentric
coordinate lambda_0 is the orbit's distinct value; orbits are listed in the
order of the published tables.

Run: python oracle/gen_quadrature.py  (writes the .inc next to this file)
"""
from __future__ import annotations

import itertools
from fractions import Fraction
from math import factorial
from pathlib import Path

import numpy as np
from scipy.special import roots_jacobi, roots_legendre

HERE = Path(__file__).resolve().parent


# ---- orbit expansion -------------------------------------------------------
def tri_orbit(kind, params):
    if kind == "S3":
        return [(1 / 3, 1 / 3, 1 / 3)]
    if kind == "S21":
        a = params[0]
        b = 1 - 2 * a
        return [(b, a, a), (a, b, a), (a, a, b)]
    if kind == "S111":
        a, b = params
        c = 1 - a - b
        out = []
        for perm in [(c, a, b), (c, b, a), (a, c, b), (b, c, a), (a, b, c), (b, a, c)]:
            out.append(perm)
        return out
    raise ValueError(kind)


def tet_orbit(kind, params):
    if kind == "S4":
        return [(0.25, 0.25, 0.25, 0.25)]
    if kind == "S31":
        a = params[0]
        b = 1 - 3 * a
        return [(b, a, a, a), (a, b, a, a), (a, a, b, a), (a, a, a, b)]
    if kind == "S22":
        a = params[0]
        b = 0.5 - a
        pts = []
        for idx in [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]:
            lam = [b] * 4
            for i in idx:
                lam[i] = a
            pts.append(tuple(lam))
        return pts
    if kind == "S211":
        a, b = params
        c = 1 - 2 * a - b
        seen = []
        for perm in itertools.permutations([a, a, b, c]):
            if not any(np.allclose(perm, s) for s in seen):
                seen.append(perm)
        # put the orbit's "c" value first in lambda_0 for the first point
        seen.sort(key=lambda l: (-l[0], -l[1], -l[2]))
        return seen
    raise ValueError(kind)


NPARAM = {"S3": 0, "S4": 0, "S21": 1, "S31": 1, "S22": 1, "S111": 2, "S211": 2}


def expand(spec, x, dim):
    """spec: list of (kind, nparams); x: flat params then weights."""
    pts, wts = [], []
    off = 0
    nw = len(spec)
    weights = x[len(x) - nw:]
    for oi, kind in enumerate(spec):
        k = NPARAM[kind]
        params = x[off:off + k]
        off += k
        orb = tri_orbit(kind, params) if dim == 2 else tet_orbit(kind, params)
        for lam in orb:
            pts.append(lam[1:])  # reference coords = (lambda_1, lambda_2[, lambda_3])
            wts.append(weights[oi])
    return np.array(pts), np.array(wts)


def monomials(dim, deg):
    if dim == 2:
        return [(i, j) for i in range(deg + 1) for j in range(deg + 1 - i)]
    return [(i, j, k) for i in range(deg + 1) for j in range(deg + 1 - i) for k in range(deg + 1 - i - j)]


def exact_moment(m):
    # integral over the unit simplex of x^a y^b (z^c) = a! b! c! / (a+b+c+d)!
    d = len(m)
    num = 1
    for e in m:
        num *= factorial(e)
    return Fraction(num, factorial(sum(m) + d))


def residual(spec, x, dim, deg):
    pts, w = expand(spec, x, dim)
    res = []
    for m in monomials(dim, deg):
        v = np.prod([pts[:, i] ** m[i] for i in range(dim)], axis=0)
        res.append(np.dot(w, v) - float(exact_moment(m)))
    return np.array(res)


def refine(spec, x0, dim, deg):
    """Gauss-Newton on the moment equations (finite-difference Jacobian)."""
    x = np.array(x0, dtype=float)
    for _ in range(60):
        r = residual(spec, x, dim, deg)
        if np.max(np.abs(r)) < 1e-17:
            break
        J = np.empty((len(r), len(x)))
        for k in range(len(x)):
            h = 1e-7 * max(1.0, abs(x[k]))
            xp = x.copy()
            xp[k] += h
            J[:, k] = (residual(spec, xp, dim, deg) - r) / h
        x = x - np.linalg.lstsq(J, r, rcond=None)[0]
    err = np.max(np.abs(residual(spec, x, dim, deg)))
    if err > 5e-16:
        raise RuntimeError(f"rule did not converge: dim {dim} deg {deg} err {err}")
    return x


# (spec, initial params..., weights normalised to the reference simplex volume)
TRI = {
    2: (["S21"], [1 / 6, 1 / 6]),
    4: (["S21", "S21"], [0.445948490915965, 0.091576213509771, 0.223381589678011 / 2, 0.109951743655322 / 2]),
    6: (["S21", "S21", "S111"], [0.249286745170910, 0.063089014491502, 0.053145049844817, 0.310352451033784,
                                 0.116786275726379 / 2, 0.050844906370207 / 2, 0.082851075618374 / 2]),
    8: (["S3", "S21", "S21", "S21", "S111"],
        [0.459292588292723, 0.170569307751760, 0.050547228317031, 0.008394777409958, 0.263112829634638,
         0.144315607677787 / 2, 0.095091634267285 / 2, 0.103217370534718 / 2, 0.032458497623198 / 2,
         0.027230314174435 / 2]),
    10: (["S3", "S21", "S21", "S111", "S111", "S111"],
         [0.485577633383657, 0.109481575485037, 0.141707219414880, 0.307939838764121, 0.025003534762686,
          0.246672560639903, 0.009540815400299, 0.066803251012200,
          0.090817990382754 / 2, 0.036725957756467 / 2, 0.045321059435528 / 2, 0.072757916845420 / 2,
          0.028327242531057 / 2, 0.009421666963733 / 2]),
}
TET = {
    2: (["S31"], [0.1381966011250105, 1 / 24]),
    4: (["S31", "S31", "S22"], [0.0927352503108912, 0.3108859192633006, 0.0455037041256496,
                                0.01224884051939366, 0.01878132095300264, 0.007091003462846911]),
    6: (["S31", "S31", "S31", "S211"], [0.214602871259151, 0.040673958534611, 0.322337890142275,
                                        0.063661001875018, 0.269672331458316,
                                        0.006653791709695, 0.001679535175887, 0.009226196923942,
                                        0.008035714285714]),
}


def conical_tet(deg):
    n = deg // 2 + 1
    # collapsed coordinates: Gauss-Jacobi in each direction on [0,1]
    xa, wa = roots_jacobi(n, 0, 0)
    xb, wb = roots_jacobi(n, 1, 0)
    xc, wc = roots_jacobi(n, 2, 0)
    pts, wts = [], []
    for i in range(n):
        for j in range(n):
            for k in range(n):
                a = (1 + xa[i]) / 2
                b = (1 + xb[j]) / 2
                c = (1 + xc[k]) / 2
                z = c
                y = b * (1 - c)
                x = a * (1 - b) * (1 - c)
                w = wa[i] * wb[j] * wc[k] / 8 / 4 / 2
                pts.append((x, y, z))
                wts.append(w)
    pts, wts = np.array(pts), np.array(wts)
    # verify
    for m in monomials(3, deg):
        v = np.prod([pts[:, t] ** m[t] for t in range(3)], axis=0)
        assert abs(np.dot(wts, v) - float(exact_moment(m))) < 1e-15, m
    return pts, wts


def gauss_legendre(n):
    x, w = roots_legendre(n)
    order = np.argsort(x)
    return x[order], w[order]


def main():
    lines = ["// Generated by oracle/gen_quadrature.py - do not edit.",
             "// TEST INFRASTRUCTURE ONLY (oracle quadrature rules).", ""]

    def emit(name, pts, wts, dim):
        lines.append(f"static const double {name}[] = {{")
        for p, w in zip(pts, wts):
            coords = list(p) + [0.0] * (3 - len(p))
            lines.append("    " + ", ".join(f"{c:.17g}" for c in coords) + f", {w:.17g},")
        lines.append("};")
        lines.append(f"static const int {name}_n = {len(wts)};")
        lines.append("")

    for p in range(1, 6):
        x, w = gauss_legendre(p + 1)
        emit(f"kLine{2 * p}", [(xi,) for xi in x], w, 1)
    for deg, (spec, x0) in TRI.items():
        x = refine(spec, x0, 2, deg)
        pts, w = expand(spec, x, 2)
        emit(f"kTri{deg}", pts, w, 2)
    for deg in (2, 4, 6, 8, 10):
        if deg in TET:
            spec, x0 = TET[deg]
            x = refine(spec, x0, 3, deg)
            pts, w = expand(spec, x, 3)
        else:
            pts, w = conical_tet(deg)
        emit(f"kTet{deg}", pts, w, 3)
    (HERE / "quadrature_tables.inc").write_text("\n".join(lines) + "\n")
    print("wrote", HERE / "quadrature_tables.inc")


if __name__ == "__main__":
    main()
