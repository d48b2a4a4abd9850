"""Curved test meshes and a NumPy model of the per-point right-hand side.

The warps move the nodes of generated boxes by smooth maps, which curves the
elements (the high-order nodes leave the affine image of the reference
lattice).  model_rhs restates, element by element, what the per-point stage
kernel computes, from the arrays dg_mesh_desc passes: the flux interpolated to
the element rule's points and contracted with w detJ J^-T and the reference
gradients, traces at the face rule's points with the per-point normal,
weighted by w detJf and projected on the face basis, then the element's own
inverse mass matrix."""
from __future__ import annotations

import numpy as np


def warp3(x, a=0.04):
    y = x.copy()
    y[:, 0] = x[:, 0] + a * np.sin(np.pi * x[:, 1]) * np.sin(np.pi * x[:, 2])
    y[:, 1] = x[:, 1] + a * np.sin(np.pi * x[:, 0]) * np.cos(np.pi * x[:, 2])
    y[:, 2] = x[:, 2] + a * np.sin(2 * x[:, 0] + x[:, 1])
    return y


def warp2(x, a=0.05):
    return np.stack([x[:, 0] + a * np.sin(np.pi * x[:, 1]), x[:, 1] + a * np.sin(np.pi * x[:, 0]) * np.cos(x[:, 1]),
                     x[:, 2]], 1)


def bump3(x, a=0.15):
    """Identity for x < 0.5 (those elements stay affine), a smooth bulge beyond."""
    y = x.copy()
    s = np.clip(x[:, 0] - 0.5, 0.0, None) ** 3
    y[:, 1] = x[:, 1] + a * s * np.sin(np.pi * x[:, 2])
    y[:, 2] = x[:, 2] + a * s * np.cos(np.pi * x[:, 1])
    return y


def boundary_fixed_mesh(D, dim, order, n=3, a=0.04):
    """Unit square / cube of n^dim cells (reflecting walls) whose nodes move
    by a map that vanishes on the boundary: every element is curved, yet the
    discrete domain is still exactly the unit square / cube."""
    if dim == 3:
        m = D.Mesh.box_tet(n, n, n, (0, 0, 0), (1, 1, 1), order=order, side_names=("Reflecting",) * 6)

        def fn(x):
            b = a * np.sin(np.pi * x[:, 0]) * np.sin(np.pi * x[:, 1]) * np.sin(np.pi * x[:, 2])
            y = x.copy()
            y[:, 0] += b
            y[:, 1] += 0.5 * b
            y[:, 2] -= 0.7 * b
            return y
    else:
        m = D.Mesh.box_tri(n, n, (0, 0), (1, 1), order=order, side_names=("Reflecting",) * 4)

        def fn(x):
            b = a * np.sin(np.pi * x[:, 0]) * np.sin(np.pi * x[:, 1])
            y = x.copy()
            y[:, 0] += b
            y[:, 1] -= 0.6 * b
            return y
    m.warp(fn)
    return m


def curved_mesh(D, dim, order, warp=None):
    if dim == 3:
        m = D.Mesh.box_tet(2, 2, 2, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), order=order,
                           side_names=("Reflecting", "Absorbing") * 3)
        m.warp(warp or warp3)
    else:
        m = D.Mesh.box_tri(4, 3, (-1.0, -1.0), (1.0, 1.0), order=order,
                           side_names=("Reflecting", "Absorbing", "Absorbing", "Reflecting"))
        m.warp(warp or warp2)
    return m, D.Precomp(m)


def model_rhs(pre, u, c0, rho, v0, upwind=False):
    """M_e^-1 (S - F) of every element, all elements taken as curved."""
    ar, ca = pre.arrays(), pre.curved_arrays()
    dim, K, np_, nf, nfp = pre.dim, pre.num_el, pre.np, pre.nf, pre.nfp
    nq = dim + 1
    w, wf = ca["el_qp"][:, 3], ca["f_qp"][:, 3]
    phi, dphi, fphi = ca["el_phi"], ca["el_dphi"], ca["f_phi"]
    v0 = np.asarray(v0, dtype=float)
    rc2, irho = rho * c0 * c0, 1.0 / rho
    q = u[:nq].reshape(nq, K, np_)
    out = np.zeros((nq, K * np_))
    for e in range(K):
        detj = ca["el_detj"][e]
        M = np.einsum("gi,gj,g->ij", phi, phi, w * detj)
        U = phi @ q[:, e, :].T                                   # [ng][nq]
        F = np.zeros((len(w), dim, nq))
        for x in range(dim):
            F[:, x, 0] = v0[x] * U[:, 0] + rc2 * U[:, 1 + x]
            for d in range(dim):
                F[:, x, 1 + d] = v0[x] * U[:, 1 + d] + (U[:, 0] * irho if x == d else 0.0)
        A = ca["el_jac"][e].reshape(-1, 3, 3)[:, :dim, :dim]     # A[g][u][x]
        B = np.linalg.inv(A)                                      # B[g][x][u] = J^-T
        Fc = np.einsum("g,gxu,gxq->guq", w * detj, B, F)
        S = np.einsum("giu,guq->qi", dphi[:, :, :dim], Fc)
        Fl = np.zeros((nq, np_))
        for lf in range(nf):
            f = ar["el_f_ids"][e, lf]
            side = 0 if ar["f_nbr_el_ids"][f, 0] == e else 1
            o = ar["el_f_orientation"][e, lf]
            own = ar["f_n_to_el_n_ids"][f, :, side]
            n = o * ca["f_normal"][f, :, :dim]                    # [ngf][dim]
            wj = wf * ca["f_detj"][f]
            qi = fphi @ q[:, e, own].T                            # [ngf][nq]
            vn0 = n @ v0[:dim]
            Fn = np.zeros_like(qi)
            if not ar["f_is_boundary"][f]:
                nb = ar["f_nbr_el_ids"][f, 1 - side]
                qo = fphi @ q[:, nb, ar["f_n_to_el_n_ids"][f, :, 1 - side]].T
                tau = 1.0 if upwind else (pre.fc * o if side == 0 else -pre.fc * o)
                sp = qi[:, 0] + qo[:, 0]
                svn = np.einsum("gx,gx->g", qi[:, 1:] + qo[:, 1:], n)
                Fn[:, 0] = 0.5 * (vn0 * sp + rc2 * svn) + 0.5 * c0 * tau * (qi[:, 0] - qo[:, 0])
                Fn[:, 1:] = (0.5 * (vn0[:, None] * (qi[:, 1:] + qo[:, 1:]) + irho * sp[:, None] * n)
                             + 0.5 * c0 * tau * (qi[:, 1:] - qo[:, 1:]))
            elif ar["f_bc"][f] == 1:
                vn = np.einsum("gx,gx->g", qi[:, 1:], n)
                vw = qi[:, 1:] - vn[:, None] * n
                Fn[:, 0] = vn0 * qi[:, 0] + rc2 * np.einsum("gx,gx->g", vw, n)
                Fn[:, 1:] = vn0[:, None] * vw + irho * qi[:, :1] * n
            else:
                vn = np.einsum("gx,gx->g", qi[:, 1:], n)
                Fn[:, 0] = 0.25 * c0 * qi[:, 0] + 0.25 * c0 * c0 * rho * vn
                Fn[:, 1:] = 0.25 * n * irho * qi[:, :1] + 0.25 * c0 * n * vn[:, None]
            Fl[:, own] += np.einsum("gk,g,gq->qk", fphi, wj, Fn)
        out[:, e * np_:(e + 1) * np_] = np.linalg.solve(M, (S - Fl).T).T
    return out
