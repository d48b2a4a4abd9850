"""NumPy model of the tensor-core form of the stage right-hand side.

Per tile the tensor-core kernel forms, for every (element, field) row,
  A = [Fhat_u(j) for u, j | -(detJf/detJe) Fn(slot)]     (FP32, split into
      two TF32 pieces),
  B = [D_u(i, j) | LIFT(i, slot)]                          (FP64 operators,
      split into three TF32 pieces),
and C = sum of the five TF32 products a1b1 + a1b2 + a2b1 + a1b3 + a2b2,
accumulated in FP32, is dt^-1 times the stage right-hand side.  The model
mirrors that arithmetic so its error against FP64 can be checked on the CPU.
"""
from __future__ import annotations

import numpy as np

import kernel_model as KM


def tf32(x: np.ndarray) -> np.ndarray:
    """Round FP32 to TF32 (10 explicit mantissa bits), nearest, ties away."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    b = (b + np.uint32(0x1000)) & np.uint32(0xFFFFE000)
    return b.view(np.float32)


def split(x: np.ndarray, pieces: int) -> list[np.ndarray]:
    out, r = [], np.asarray(x, dtype=np.float64)
    for _ in range(pieces):
        p = tf32(r.astype(np.float32))
        out.append(p)
        r = r - p.astype(np.float64)
    return out


def operator_matrix(layout: dict) -> np.ndarray:
    """B[i][k]: k < dim*np -> D_u[i][j] (k = u*np + j); then LIFT[slot][i]."""
    dim, np_, nf, nfp = (layout[k] for k in ("dim", "np", "nf", "nfp"))
    ops = layout["ops"]
    D = ops[:dim * np_ * np_].reshape(dim, np_, np_)      # [u][j][i]
    LIFT = ops[dim * np_ * np_:].reshape(nf * nfp, np_)   # [slot][i]
    B = np.concatenate([D.transpose(2, 0, 1).reshape(np_, dim * np_), LIFT.T], axis=1)
    return B


def rhs(layout, u, dt, c0, rho0, v0=(0.0, 0.0, 0.0), a_pieces=2, b_pieces=3) -> np.ndarray:
    """One right-hand side with the tensor-core arithmetic (FP32 inputs)."""
    dim, np_, nf, nfp, nq = (layout[k] for k in ("dim", "np", "nf", "nfp", "nq"))
    K = layout["geo"].shape[0]
    B = operator_matrix(layout)
    Q = u[:nq].astype(np.float32).astype(np.float64).reshape(nq, K, np_)
    geo = layout["geo"].astype(np.float32).astype(np.float64)          # [e][x][u]
    v0a = np.asarray(v0[:dim], dtype=np.float64)
    # contravariant fluxes Fhat[f][u][e][j] (FP32 rounded)
    a_u = np.einsum("exu,x->eu", geo, v0a)
    w = np.einsum("exu,xej->uej", geo, Q[1:])
    Fh = np.empty((nq, dim, K, np_))
    Fh[0] = a_u.T[:, :, None] * Q[0][None] + rho0 * c0 * c0 * w
    for d in range(dim):
        Fh[1 + d] = a_u.T[:, :, None] * Q[1 + d][None] + (Q[0][None] / rho0) * geo[:, d, :].T[:, :, None]
    Fh = Fh.astype(np.float32)
    # face values: reuse the SIMT model's face part via a zero-volume call
    lay0 = dict(layout)
    fn = face_values(layout, Q, c0, rho0, v0)                          # [f][e][slot], scaled
    A = np.concatenate([Fh.transpose(0, 2, 1, 3).reshape(nq, K, dim * np_), -fn], axis=2)
    A = A.astype(np.float32).reshape(nq * K, -1)
    ap, bp = split(A, a_pieces), split(B, b_pieces)
    terms = [(0, 0), (0, 1), (1, 0), (0, 2), (1, 1), (2, 0)]
    C = np.zeros((nq * K, np_), dtype=np.float32)
    for ia, ib in terms:
        if ia < a_pieces and ib < b_pieces:
            C = C + (ap[ia] @ bp[ib].T).astype(np.float32)
    r = np.zeros((4, K * np_))
    r[:nq] = (np.float32(dt) * C.reshape(nq, K, np_)).reshape(nq, -1)
    return r


def face_values(layout, Q, c0, rho0, v0):
    """Scaled face values (detJf/detJe) Fn[f][e][slot] as in the stage kernel."""
    dim, np_, nf, nfp, nq, nperm = (layout[k] for k in ("dim", "np", "nf", "nfp", "nq", "nperm"))
    K = Q.shape[1]
    tabs = layout["tabs"]
    fmask = tabs[:nf * nfp].reshape(nf, nfp)
    perm = tabs[nf * nfp:].reshape(nperm, nfp)
    conn = layout["conn"]
    fgeo = layout["fgeo"].astype(np.float32).astype(np.float64)
    v0 = np.asarray(v0[:dim], float)
    rc2, inv_rho = rho0 * c0 * c0, 1.0 / rho0
    Fn = np.zeros((nq, K, nf * nfp))
    for lf in range(nf):
        nb, word = conn[:, lf, 0], conn[:, lf, 1]
        kind = (word >> 5) & 3
        nlf, pm = word & 3, (word >> 2) & 7
        tau = np.where(word & 128, -1.0, 1.0)
        n = fgeo[:, lf, :dim]
        scale = fgeo[:, lf, dim]
        vn0 = n @ v0
        for k in range(nfp):
            own = Q[:, :, fmask[lf, k]]
            out = np.zeros((nq, K))
            e = np.nonzero(kind == 0)[0]
            if e.size:
                o = Q[:, nb[e], fmask[nlf[e], perm[pm[e], k]]]
                ow = own[:, e]
                sp = ow[0] + o[0]
                svn = np.einsum("xe,ex->e", ow[1:] + o[1:], n[e])
                hj = 0.5 * c0 * tau[e]
                out[0, e] = hj * (ow[0] - o[0]) + 0.5 * (vn0[e] * sp + rc2 * svn)
                for d in range(dim):
                    out[1 + d, e] = hj * (ow[1 + d] - o[1 + d]) + 0.5 * (vn0[e] * (ow[1 + d] + o[1 + d])
                                                                        + inv_rho * sp * n[e, d])
            e = np.nonzero(kind == 1)[0]
            if e.size:
                ow = own[:, e]
                vn = np.einsum("xe,ex->e", ow[1:], n[e])
                vw = ow[1:] - vn * n[e].T
                out[0, e] = vn0[e] * ow[0] + rc2 * np.einsum("xe,ex->e", vw, n[e])
                for d in range(dim):
                    out[1 + d, e] = vn0[e] * vw[d] + inv_rho * ow[0] * n[e, d]
            e = np.nonzero(kind == 2)[0]
            if e.size:
                ow = own[:, e]
                vn = np.einsum("xe,ex->e", ow[1:], n[e])
                out[0, e] = 0.25 * c0 * ow[0] + 0.25 * c0 * c0 * rho0 * vn
                for d in range(dim):
                    out[1 + d, e] = 0.25 * n[e, d] * inv_rho * ow[0] + 0.25 * c0 * n[e, d] * vn
            Fn[:, :, lf * nfp + k] = (out * scale).astype(np.float32)
    return Fn
