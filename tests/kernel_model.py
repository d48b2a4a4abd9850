"""NumPy model of the GPU stage kernel's arithmetic on the element-centric
layout that dg_create uploads (dg_layout_build).

Used on the CPU to check the layout and the factored algebra against the
oracle's element-by-element quadrature before any GPU run: one right-hand
side r = dt * (sum_u D_u Fhat_u - sum_f (detJf/detJe) LIFT_f Fn_f).
"""
from __future__ import annotations

import numpy as np


def rhs(layout: dict, u: np.ndarray, dt: float, c0: float, rho0: float, v0=(0.0, 0.0, 0.0)) -> np.ndarray:
    dim, np_, nf, nfp, nq, nperm = (layout[k] for k in ("dim", "np", "nf", "nfp", "nq", "nperm"))
    K = layout["geo"].shape[0]
    ops, tabs = layout["ops"], layout["tabs"]
    D = ops[:dim * np_ * np_].reshape(dim, np_, np_)          # [u][j][i]
    LIFT = ops[dim * np_ * np_:].reshape(nf * nfp, np_)       # [slot][i]
    fmask = tabs[:nf * nfp].reshape(nf, nfp)
    perm = tabs[nf * nfp:].reshape(nperm, nfp)
    Q = u[:nq].reshape(nq, K, np_)
    v0 = np.asarray(v0[:dim], float)
    rc2, inv_rho = rho0 * c0 * c0, 1.0 / rho0

    dq = np.einsum("uji,fej->fuei", D, Q)                      # reference derivatives
    B = layout["geo"]                                          # [e][x][u]
    g = np.einsum("exu,fuei->fxei", B, dq)                     # physical derivatives
    V = np.empty((nq, K, np_))
    V[0] = np.einsum("x,xei->ei", v0, g[0]) + rc2 * sum(g[1 + x, x] for x in range(dim))
    for d in range(dim):
        V[1 + d] = np.einsum("x,xei->ei", v0, g[1 + d]) + inv_rho * g[0, d]

    Fn = np.zeros((nq, K, nf * nfp))
    conn, fgeo = layout["conn"], layout["fgeo"]
    for lf in range(nf):
        nb, word = conn[:, lf, 0], conn[:, lf, 1]
        kind = (word >> 5) & 3
        nlf, pm = word & 3, (word >> 2) & 7
        tau = np.where(word & 128, -1.0, 1.0)
        n = fgeo[:, lf, :dim]
        scale = fgeo[:, lf, dim]
        vn0 = n @ v0
        for k in range(nfp):
            own = Q[:, :, fmask[lf, k]]                        # [nq][K]
            out = np.zeros((nq, K))
            inter = kind == 0
            if inter.any():
                e = np.nonzero(inter)[0]
                nvi = fmask[nlf[e], perm[pm[e], k]]
                o = Q[:, nb[e], nvi]
                ow = own[:, e]
                sp = ow[0] + o[0]
                svn = np.einsum("xe,ex->e", ow[1:] + o[1:], n[e])
                hj = 0.5 * c0 * tau[e]
                out[0, e] = hj * (ow[0] - o[0]) + 0.5 * (vn0[e] * sp + rc2 * svn)
                for d in range(dim):
                    out[1 + d, e] = hj * (ow[1 + d] - o[1 + d]) + 0.5 * (vn0[e] * (ow[1 + d] + o[1 + d])
                                                                        + inv_rho * sp * n[e, d])
            refl = kind == 1
            if refl.any():
                e = np.nonzero(refl)[0]
                ow = own[:, e]
                vn = np.einsum("xe,ex->e", ow[1:], n[e])
                vw = ow[1:] - vn * n[e].T
                vwn = np.einsum("xe,ex->e", vw, n[e])
                out[0, e] = vn0[e] * ow[0] + rc2 * vwn
                for d in range(dim):
                    out[1 + d, e] = vn0[e] * vw[d] + inv_rho * ow[0] * n[e, d]
            absb = kind == 2
            if absb.any():
                e = np.nonzero(absb)[0]
                ow = own[:, e]
                vn = np.einsum("xe,ex->e", ow[1:], n[e])
                out[0, e] = 0.25 * c0 * ow[0] + 0.25 * c0 * c0 * rho0 * vn
                for d in range(dim):
                    out[1 + d, e] = 0.25 * n[e, d] * inv_rho * ow[0] + 0.25 * c0 * n[e, d] * vn
            Fn[:, :, lf * nfp + k] = out * scale
    L = np.einsum("si,fes->fei", LIFT, Fn)
    r = np.zeros((4, K * np_))
    r[:nq] = (dt * (V - L)).reshape(nq, -1)
    return r
