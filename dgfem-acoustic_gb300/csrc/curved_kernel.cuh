// Stage kernel of curved (non-affine, isoparametric) elements: the per-point
// form of the reference's right-hand side, with geometry that varies inside
// an element.  One CTA per curved element (grid-stride), arithmetic and
// element data in the context's precision (FP64 or FP32).  Per element:
//
//   volume  U(g) = sum_j phi_j(g) q_j at the points g of the element rule,
//           Fc_u(g) = sum_x [w detJ J^-T]_(x,u)(g) Flux_x(U(g)),
//           S_i = sum_u sum_g dphi_i/du(g) Fc_u(g)
//           (Mesh::getElStiffVector, Mesh.cpp:476-489, with the flux
//           interpolated to the points first: the flux is linear in q);
//   faces   traces of the element and of its neighbour at the points of the
//           face rule (face node order of the reference's unique face),
//           numerical flux with the normal of that point
//           (Mesh::precomputeFlux, Mesh.cpp:500-539; boundary traces of
//           Mesh::updateFlux, Mesh.cpp:595-671), weighted by w detJf and
//           projected on the face basis: F_k = sum_g phi_k(g) w detJf Fn(g),
//           scattered to the element's nodes (Mesh::getElFlux, Mesh.cpp:548-557);
//   update  r = dt M_e^-1 (S - F) with the element's own inverse mass matrix
//           applied as the reference does (eigen::linEq, utils.cpp:118-123,
//           called at solver.cpp:46-48), then the RK4 / forward-Euler stage
//           combination of the affine kernels.
//
// The affine stage kernels run over the list of the other elements, and both
// kernels read only stage inputs and write only their own elements, so the two
// launches of a stage are independent.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "stage_kernel.cuh"

namespace dgk {

template <typename Real>
struct CurvedArgs {
    const Real *win;
    const Real *u;
    Real *acc;
    Real *wout;
    long long fstride, bstride;
    const int *el;         // [C] element ids
    const Real *minv;      // [C][np*np] row-major inverse mass (applied as its transpose, as linEq)
    const Real *wm;        // [C][ng][DIM*DIM] w detJ J^-T at x*DIM+u
    const Real *fw;        // [C][NF][ngf][4] outward normal, w detJf
    const int2 *fconn;     // [C][NF] neighbour (-1), word: kind bits 5-6, jump sign bit 7
    const uint8_t *fmap;   // [C][NF][2][nfp] own / neighbour element node of face node k
    const Real *phi;       // [ng][np]
    const Real *dphi;      // [DIM][ng][np]
    const Real *fphi;      // [ngf][nfp]
    int C, np, ng, ngf, nfp;
    int stage;             // 0-3 RK4 stages, 4 forward Euler
    Real dt, rc2, inv_rho, half_c0, c0, rho, v0[3];
};

// Shared memory for an element of np nodes (rsize = bytes of the arithmetic type).
__host__ __device__ inline size_t curved_smem_bytes(int dim, int np, int ng, int ngf, int rsize) {
    const int nq = dim + 1, nf = dim + 1;
    size_t d = (size_t)nq * np        // state
               + (size_t)ng * dim * nq  // contravariant flux at the points
               + (size_t)nf * ngf * nq  // weighted numerical flux at the face points
               + (size_t)nq * np;       // S - F
    return d * rsize + (size_t)nf * np * sizeof(int);
}

// Physical flux of the linearised Euler equations with uniform mean flow
// (Mesh.cpp:577-592): F[x][0] = v0_x p + rho c0^2 v_x, F[x][1+d] = v0_x v_d +
// delta_xd p / rho.
template <int DIM, typename Real>
__device__ __forceinline__ void lee_flux(const Real *q, const Real *v0, Real rc2, Real inv_rho,
                                         Real (&F)[DIM][DIM + 1]) {
#pragma unroll
    for (int x = 0; x < DIM; ++x) {
        F[x][0] = fma(v0[x], q[0], rc2 * q[1 + x]);
#pragma unroll
        for (int d = 0; d < DIM; ++d) F[x][1 + d] = v0[x] * q[1 + d] + (x == d ? q[0] * inv_rho : Real(0));
    }
}

// Normal numerical flux at one face point seen from the element (outward
// normal n): interior Lax-Friedrichs with jump sign tau, reflecting wall
// (normal velocity removed, flux projected), absorbing (R K R^-1 q).
template <int DIM, typename Real>
__device__ __forceinline__ void face_flux(int kind, Real tau, const Real *own, const Real *o, const Real *n,
                                          Real rc2, Real inv_rho, Real half_c0, Real c0, Real rho,
                                          const Real *v0, Real (&Fn)[DIM + 1]) {
    Real vn0 = Real(0);
#pragma unroll
    for (int x = 0; x < DIM; ++x) vn0 = fma(v0[x], n[x], vn0);
    if (kind == kKindInterior) {
        const Real sp = own[0] + o[0];
        Real svn = Real(0);
#pragma unroll
        for (int x = 0; x < DIM; ++x) svn = fma(own[1 + x] + o[1 + x], n[x], svn);
        const Real hj = half_c0 * tau;
        Fn[0] = fma(hj, own[0] - o[0], Real(0.5) * fma(vn0, sp, rc2 * svn));
#pragma unroll
        for (int d = 0; d < DIM; ++d)
            Fn[1 + d] = fma(hj, own[1 + d] - o[1 + d], Real(0.5) * fma(vn0, own[1 + d] + o[1 + d], inv_rho * sp * n[d]));
    } else if (kind == kKindReflecting) {
        Real vn = Real(0);
#pragma unroll
        for (int x = 0; x < DIM; ++x) vn = fma(own[1 + x], n[x], vn);
        Real vw[DIM], vwn = Real(0);
#pragma unroll
        for (int x = 0; x < DIM; ++x) {
            vw[x] = own[1 + x] - vn * n[x];
            vwn = fma(vw[x], n[x], vwn);
        }
        Fn[0] = fma(vn0, own[0], rc2 * vwn);
#pragma unroll
        for (int d = 0; d < DIM; ++d) Fn[1 + d] = fma(vn0, vw[d], inv_rho * own[0] * n[d]);
    } else {
        Real vn = Real(0);
#pragma unroll
        for (int x = 0; x < DIM; ++x) vn = fma(own[1 + x], n[x], vn);
        const Real q0 = Real(0.25) * c0;
        Fn[0] = fma(q0, own[0], Real(0.25) * c0 * c0 * rho * vn);
#pragma unroll
        for (int d = 0; d < DIM; ++d) Fn[1 + d] = fma(Real(0.25) * n[d] * inv_rho, own[0], q0 * n[d] * vn);
    }
}

template <int DIM, typename Real>
__global__ void __launch_bounds__(128) curved_stage_kernel(const CurvedArgs<Real> a) {
    constexpr int NQ = DIM + 1, NF = DIM + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int np = a.np, ng = a.ng, ngf = a.ngf, nfp = a.nfp;
    Real *sW = reinterpret_cast<Real *>(smem_raw);  // [NQ][np]
    Real *sFc = sW + NQ * np;                        // [ng][DIM][NQ]
    Real *sFn = sFc + ng * DIM * NQ;                 // [NF][ngf][NQ]
    Real *sR = sFn + NF * ngf * NQ;                  // [NQ][np]
    int *sK = reinterpret_cast<int *>(sR + NQ * np);     // [NF][np] face position of node i, or -1
    const int tid = threadIdx.x, nt = blockDim.x;
    const long long boff = (long long)blockIdx.y * a.bstride;
    const Real *win = a.win + boff;
    const Real v0[3] = {a.v0[0], a.v0[1], a.v0[2]};
    for (int c = blockIdx.x; c < a.C; c += gridDim.x) {
        const int e = a.el[c];
        const long long ebase = (long long)e * np;
        for (int t = tid; t < NQ * np; t += nt) {
            const int q = t / np, i = t - q * np;
            sW[t] = win[q * a.fstride + ebase + i];
        }
        for (int t = tid; t < NF * np; t += nt) sK[t] = -1;
        __syncthreads();
        const uint8_t *fmap = a.fmap + (size_t)c * NF * 2 * nfp;
        for (int t = tid; t < NF * nfp; t += nt) {
            const int lf = t / nfp, k = t - lf * nfp;
            sK[lf * np + fmap[(lf * 2) * nfp + k]] = k;
        }
        // volume points and face points
        const int nwork = ng + NF * ngf;
        for (int t = tid; t < nwork; t += nt) {
            if (t < ng) {
                const int g = t;
                Real U[NQ];
#pragma unroll
                for (int q = 0; q < NQ; ++q) U[q] = Real(0);
                const Real *ph = a.phi + (size_t)g * np;
                for (int j = 0; j < np; ++j) {
                    const Real p = __ldg(ph + j);
#pragma unroll
                    for (int q = 0; q < NQ; ++q) U[q] = fma(p, sW[q * np + j], U[q]);
                }
                Real F[DIM][DIM + 1];
                lee_flux<DIM, Real>(U, v0, a.rc2, a.inv_rho, F);
                const Real *w = a.wm + ((size_t)c * ng + g) * DIM * DIM;
#pragma unroll
                for (int u = 0; u < DIM; ++u)
#pragma unroll
                    for (int q = 0; q < NQ; ++q) {
                        Real s = Real(0);
#pragma unroll
                        for (int x = 0; x < DIM; ++x) s = fma(__ldg(w + x * DIM + u), F[x][q], s);
                        sFc[(g * DIM + u) * NQ + q] = s;
                    }
            } else {
                const int lf = (t - ng) / ngf, g = (t - ng) - lf * ngf;
                const int2 cn = a.fconn[(size_t)c * NF + lf];
                const int kind = (cn.y >> 5) & 3;
                const Real tau = (cn.y & 128) ? Real(-1) : Real(1);
                const uint8_t *own = fmap + (lf * 2) * nfp;
                const uint8_t *nbm = own + nfp;
                const Real *fp = a.fphi + (size_t)g * nfp;
                Real qi[NQ], qo[NQ];
#pragma unroll
                for (int q = 0; q < NQ; ++q) { qi[q] = Real(0); qo[q] = Real(0); }
                const long long nbase = (long long)(kind == kKindInterior ? cn.x : 0) * np;
                for (int k = 0; k < nfp; ++k) {
                    const Real p = __ldg(fp + k);
                    const int vi = own[k];
#pragma unroll
                    for (int q = 0; q < NQ; ++q) qi[q] = fma(p, sW[q * np + vi], qi[q]);
                    if (kind == kKindInterior) {
                        const long long at = nbase + nbm[k];
#pragma unroll
                        for (int q = 0; q < NQ; ++q) qo[q] = fma(p, __ldg(win + q * a.fstride + at), qo[q]);
                    }
                }
                const Real *fw = a.fw + (((size_t)c * NF + lf) * ngf + g) * 4;
                Real n[DIM];
#pragma unroll
                for (int x = 0; x < DIM; ++x) n[x] = __ldg(fw + x);
                const Real wj = __ldg(fw + 3);
                Real Fn[NQ];
                face_flux<DIM, Real>(kind, tau, qi, qo, n, a.rc2, a.inv_rho, a.half_c0, a.c0, a.rho, v0, Fn);
#pragma unroll
                for (int q = 0; q < NQ; ++q) sFn[(lf * ngf + g) * NQ + q] = wj * Fn[q];
            }
        }
        __syncthreads();
        // S - F at the nodes
        for (int t = tid; t < NQ * np; t += nt) {
            const int q = t / np, i = t - q * np;
            Real S = Real(0);
#pragma unroll
            for (int u = 0; u < DIM; ++u) {
                const Real *dp = a.dphi + (size_t)u * ng * np + i;
                for (int g = 0; g < ng; ++g) S = fma(__ldg(dp + (size_t)g * np), sFc[(g * DIM + u) * NQ + q], S);
            }
            Real Fl = Real(0);
#pragma unroll
            for (int lf = 0; lf < NF; ++lf) {
                const int k = sK[lf * np + i];
                if (k < 0) continue;
                Real s = Real(0);
                for (int g = 0; g < ngf; ++g) s = fma(__ldg(a.fphi + (size_t)g * nfp + k), sFn[(lf * ngf + g) * NQ + q], s);
                Fl += s;
            }
            sR[q * np + i] = S - Fl;
        }
        __syncthreads();
        // r = dt M^-1 (S - F) and the stage update
        const Real *mi = a.minv + (size_t)c * np * np;
        Real *acc = a.acc + boff;
        Real *wout = a.wout + boff;
        const Real *uu = a.u + boff;
        for (int t = tid; t < NQ * np; t += nt) {
            const int q = t / np, i = t - q * np;
            Real s = Real(0);
            for (int j = 0; j < np; ++j) s = fma(__ldg(mi + (size_t)j * np + i), sR[q * np + j], s);
            const Real r = a.dt * s;
            const Real qv = sW[q * np + i];
            const long long idx = q * a.fstride + ebase + i;
            if (a.stage == 0) {
                acc[idx] = r;
                wout[idx] = fma(Real(0.5), r, qv);
            } else if (a.stage == 1) {
                acc[idx] = fma(Real(2), r, acc[idx]);
                wout[idx] = fma(Real(0.5), r, uu[idx]);
            } else if (a.stage == 2) {
                acc[idx] = fma(Real(2), r, acc[idx]);
                wout[idx] = uu[idx] + r;
            } else if (a.stage == 3) {
                wout[idx] = uu[idx] + (acc[idx] + r) * (Real(1) / Real(6));
            } else {
                wout[idx] = qv + r;
            }
        }
        __syncthreads();
    }
}

}  // namespace dgk
