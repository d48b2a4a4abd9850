"""Writes rules.inc: the "Gauss<2p>" integration rules that the curved-element
precompute evaluates its per-point geometry on.  The reference takes these
rules from gmsh 4.1.4 (Mesh.cpp:31-38, 135-142), which is not part of its
checkout; the published rules are restated here:

  * lines on [-1, 1]: Gauss-Legendre with p+1 points, increasing abscissa;
  * triangles (0,0),(1,0),(0,1): the fully symmetric rules of Dunavant (1985)
    of degree 2 (3 points), 4 (6), 6 (12), 8 (16) and 10 (25);
  * tetrahedra (0,0,0),(1,0,0),(0,1,0),(0,0,1): symmetric rules of degree 2
    (4 points), 4 (14, positive weights) and 6 (Keast 1986, 24 points); degree
    8 and 10 are Stroud conical products of Gauss-Jacobi rules.

The published orbit parameters (about 15 digits) are refined to full double
precision by Gauss-Newton on the moment equations; every monomial up to the
rule's degree is checked before the file is written.  Points of an orbit are
listed with the orbit's distinct barycentric value in lambda_0 first.

Run: python gen_rules.py  (writes rules.inc next to this file)
"""
from __future__ import annotations

import itertools
from fractions import Fraction
from math import factorial
from pathlib import Path

import numpy as np
from scipy.special import roots_jacobi, roots_legendre

OUT = Path(__file__).resolve().parent / "rules.inc"
NPARAM = {"S3": 0, "S21": 1, "S111": 2, "S4": 0, "S31": 1, "S22": 1, "S211": 2}


def orbit(kind, prm):
    """Barycentric points of a symmetric orbit."""
    if kind == "S3":
        return [(1 / 3, 1 / 3, 1 / 3)]
    if kind == "S21":
        a = prm[0]
        return [(1 - 2 * a, a, a), (a, 1 - 2 * a, a), (a, a, 1 - 2 * a)]
    if kind == "S111":
        a, b = prm
        c = 1 - a - b
        return [(c, a, b), (c, b, a), (a, c, b), (b, c, a), (a, b, c), (b, a, c)]
    if kind == "S4":
        return [(0.25,) * 4]
    if kind == "S31":
        a = prm[0]
        b = 1 - 3 * a
        return [tuple(b if i == j else a for i in range(4)) for j in range(4)]
    if kind == "S22":
        a = prm[0]
        b = 0.5 - a
        return [tuple(a if i in pair else b for i in range(4)) for pair in itertools.combinations(range(4), 2)]
    if kind == "S211":
        a, b = prm
        c = 1 - 2 * a - b
        pts = []
        for cand in itertools.permutations([a, a, b, c]):
            if not any(np.allclose(cand, q) for q in pts):
                pts.append(cand)
        pts.sort(key=lambda l: (-l[0], -l[1], -l[2]))
        return pts
    raise ValueError(kind)


def points(spec, x):
    """Reference coordinates (lambda_1.., the first barycentric dropped) and
    weights of the rule given by orbit kinds and parameters-then-weights x."""
    pts, wts = [], []
    weights = x[len(x) - len(spec):]
    off = 0
    for oi, kind in enumerate(spec):
        prm = x[off:off + NPARAM[kind]]
        off += NPARAM[kind]
        for lam in orbit(kind, prm):
            pts.append(lam[1:])
            wts.append(weights[oi])
    return np.array(pts), np.array(wts)


def monomials(dim, deg):
    return [m for m in itertools.product(range(deg + 1), repeat=dim) if sum(m) <= deg]


def moment(m):
    """Integral of prod x_i^m_i over the unit simplex: prod m_i! / (sum m + d)!."""
    num = 1
    for e in m:
        num *= factorial(e)
    return Fraction(num, factorial(sum(m) + len(m)))


def residual(spec, x, dim, deg):
    pts, w = points(spec, x)
    res = []
    for m in monomials(dim, deg):
        v = np.prod([pts[:, i] ** m[i] for i in range(dim)], axis=0)
        res.append(np.dot(w, v) - float(moment(m)))
    return np.array(res)


def refine(spec, x0, dim, deg):
    x = np.array(x0, dtype=float)
    for _ in range(60):
        r = residual(spec, x, dim, deg)
        if np.abs(r).max() < 1e-17:
            break
        J = np.empty((r.size, x.size))
        for k in range(x.size):
            h = 1e-7 * max(1.0, abs(x[k]))
            xp = x.copy()
            xp[k] += h
            J[:, k] = (residual(spec, xp, dim, deg) - r) / h
        x -= np.linalg.lstsq(J, r, rcond=None)[0]
    if np.abs(residual(spec, x, dim, deg)).max() > 5e-16:
        raise RuntimeError(f"rule dim {dim} degree {deg} did not converge")
    return x


# published parameters: orbit kinds, then orbit parameters, then weights
# (Dunavant's weights are for unit area and are halved to the reference triangle)
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
    """Stroud conical product on the collapsed cube, n = deg/2 + 1 points per
    direction (Gauss-Jacobi weights (0,0), (1,0), (2,0))."""
    n = deg // 2 + 1
    ra, wa = roots_jacobi(n, 0, 0)
    rb, wb = roots_jacobi(n, 1, 0)
    rc, wc = roots_jacobi(n, 2, 0)
    pts, wts = [], []
    for i, j, k in itertools.product(range(n), repeat=3):
        a, b, c = (1 + ra[i]) / 2, (1 + rb[j]) / 2, (1 + rc[k]) / 2
        pts.append((a * (1 - b) * (1 - c), b * (1 - c), c))
        wts.append(wa[i] * wb[j] * wc[k] / 64)
    return np.array(pts), np.array(wts)


def check(pts, w, dim, deg):
    for m in monomials(dim, deg):
        v = w @ np.prod(pts ** np.array(m), axis=1)
        if abs(v - float(moment(m))) > 1e-15:
            raise RuntimeError(f"dim {dim} degree {deg}: monomial {m} off by {v - float(moment(m))}")


def main():
    out = ["// Generated by gen_rules.py - do not edit.", "// Rows: u, v, w, weight.", ""]

    def emit(name, pts, w):
        out.append(f"static const double {name}[] = {{")
        for p, wt in zip(pts, w):
            c = list(p) + [0.0] * (3 - len(p))
            out.append("    " + ", ".join(f"{v:.17g}" for v in c) + f", {wt:.17g},")
        out.append("};")
        out.append(f"static const int {name}_n = {len(w)};")
        out.append("")

    for p in range(1, 6):
        x, w = roots_legendre(p + 1)
        o = np.argsort(x)
        emit(f"kRuleLine{2 * p}", [(v,) for v in x[o]], w[o])
    for deg, (spec, x0) in TRI.items():
        pts, w = points(spec, refine(spec, x0, 2, deg))
        check(pts, w, 2, deg)
        emit(f"kRuleTri{deg}", pts, w)
    for deg in (2, 4, 6, 8, 10):
        if deg in TET:
            spec, x0 = TET[deg]
            pts, w = points(spec, refine(spec, x0, 3, deg))
        else:
            pts, w = conical_tet(deg)
        check(pts, w, 3, deg)
        emit(f"kRuleTet{deg}", pts, w)
    OUT.write_text("\n".join(out) + "\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main()
