// Stage kernel of curved (non-affine, isoparametric) elements: the per-point
// form of the reference's right-hand side, with geometry that varies inside
// an element.  Arithmetic and element data in the context's precision (FP64
// or FP32).  A CTA takes a group of EPC curved elements at a time (grid-
// stride over the groups): it first copies the group's state and its
// neighbours' values at the shared face nodes into shared memory with
// asynchronous copies, so that all those scattered loads are in flight
// together; the per-element matrices (inverse mass, metric terms, face point
// data) are read through L1 where they are used, which keeps the shared
// memory per CTA small enough for 4-5 CTAs per SM.  Per element:
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
#include "tc_ptx.cuh"

namespace dgk {

template <typename Real>
struct CurvedArgs {
    const Real *win;
    const Real *u;
    Real *acc;
    Real *wout;
    long long fstride, bstride;
    const int *el;         // [C] element ids
    const int2 *fconn;     // [C][NF] neighbour (-1), word: kind bits 5-6, jump sign bit 7
    const Real *edata;     // [C][estride] inverse mass (row-major, applied as its transpose, as linEq),
                           // w detJ J^-T [ng][DIM*DIM] at x*DIM+u, [NF][ngf][4] outward normal and w detJf
                           // (layout: curved_edata)
    const uint8_t *fmap;   // [C][fstride_b] own / neighbour element node of face node k: [NF][2][nfp]
    const Real *phi;       // [ng][np]
    const Real *dphi;      // [DIM][ng][np]
    const Real *fphi;      // [ngf][nfp]
    int C, np, ng, ngf, nfp;
    int epc;               // elements per CTA group
    int estride;           // Reals per element in edata (curved_edata().stride)
    int mstride;           // bytes per element in fmap (a multiple of 16)
    int stage;             // 0-3 RK4 stages, 4 forward Euler
    Real dt, rc2, inv_rho, half_c0, c0, rho, v0[3];
    // state kept as an FP32 pair (mixed-form contexts): the low part of u and
    // where the new low part goes (u's for RK4, the Euler target's); null
    // otherwise
    const Real *ulo = nullptr;
    Real *olo = nullptr;
};

// Element data of one curved element, in Reals: inverse mass [np*np] at 0,
// metric terms [ng][DIM*DIM] at off_wm, face point data [NF][ngf][4] at
// off_fw, each block starting on a 16-byte boundary, total padded to 16 bytes.
struct CurvedEdata {
    int off_wm, off_fw, stride;
};

__host__ __device__ inline CurvedEdata curved_edata(int dim, int np, int ng, int ngf, int rsize) {
    CurvedEdata d;
    d.off_wm = (np * np + 3) / 4 * 4;
    d.off_fw = d.off_wm + (ng * dim * dim + 3) / 4 * 4;
    const int total = d.off_fw + (dim + 1) * ngf * 4;
    d.stride = (total * rsize + 15) / 16 * 16 / rsize;
    return d;
}

// Per-element shared-memory slot, in Reals.  Field values are stored four
// to a node or point (q innermost, padded to 4 in 2D) so that one 16-byte
// shared-memory load serves all fields.
struct CurvedSlot {
    int w, nb, fc, fn, r;  // state [np][4], neighbour face values [NF][nfp][4], Fc [ng][DIM][4],
                           // Fn [NF][ngf][4], S - F [np][4]
    int reals;
};

__host__ __device__ inline CurvedSlot curved_slot(int dim, int np, int ng, int ngf, int nfp) {
    const int nf = dim + 1;
    CurvedSlot s;
    s.w = 0;
    s.nb = s.w + 4 * np;
    s.fc = s.nb + 4 * nf * nfp;
    s.fn = s.fc + 4 * ng * dim;
    s.r = s.fn + 4 * nf * ngf;
    s.reals = s.r + 4 * np;
    return s;
}

// Shared memory of a CTA: epc slots of Reals, then per slot the face node
// maps (mstride bytes, 16-byte copies) and the face position table [NF][np]
// (int).
__host__ __device__ inline size_t curved_smem_bytes(int dim, int np, int ng, int ngf, int nfp, int mstride, int epc,
                                                    int rsize) {
    const CurvedSlot sl = curved_slot(dim, np, ng, ngf, nfp);
    const size_t ints = (size_t)(dim + 1) * np;
    return (size_t)epc * ((size_t)sl.reals * rsize + ints * sizeof(int) + mstride);
}

template <typename Real>
__device__ __forceinline__ void st4(Real *p, const Real (&v)[4]);
template <>
__device__ __forceinline__ void st4<float>(float *p, const float (&v)[4]) {
    *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
template <>
__device__ __forceinline__ void st4<double>(double *p, const double (&v)[4]) {
    *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]);
    *reinterpret_cast<double2 *>(p + 2) = make_double2(v[2], v[3]);
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
__global__ void __launch_bounds__(256) curved_stage_kernel(const CurvedArgs<Real> a) {
    constexpr int NQ = DIM + 1, NF = DIM + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int np = a.np, ng = a.ng, ngf = a.ngf, nfp = a.nfp, epc = a.epc;
    const CurvedSlot sl = curved_slot(DIM, np, ng, ngf, nfp);
    Real *sReal = reinterpret_cast<Real *>(smem_raw);
    uint8_t *sMall = reinterpret_cast<uint8_t *>(sReal + (size_t)epc * sl.reals);
    int *sKall = reinterpret_cast<int *>(sMall + (size_t)epc * a.mstride);
    const int tid = threadIdx.x, nt = blockDim.x;
    const long long boff = (long long)blockIdx.y * a.bstride;
    const Real *win = a.win + boff;
    const Real v0[3] = {a.v0[0], a.v0[1], a.v0[2]};
    const int ngroups = (a.C + epc - 1) / epc;
    const int edim = a.estride;
    const CurvedEdata eo = curved_edata(DIM, np, ng, ngf, (int)sizeof(Real));
    for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
        const int c0 = grp * epc;
        const int ne = min(epc, a.C - c0);
        // ---- copies: element data and face maps (16-byte chunks), state
        {
            const int mch = a.mstride / 16;
            for (int t = tid; t < ne * mch; t += nt) {
                const int s = t / mch, q = t - s * mch;
                dgtc::cp_async16(sMall + (size_t)s * a.mstride + q * 16, a.fmap + (size_t)(c0 + s) * a.mstride + q * 16,
                                 16);
            }
            const int nw = NQ * np;
            for (int t = tid; t < ne * nw; t += nt) {
                const int s = t / nw, r = t - s * nw;
                const int q = r / np, i = r - q * np;
                const long long at = q * a.fstride + (long long)__ldg(&a.el[c0 + s]) * np + i;
                Real *dst = sReal + (size_t)s * sl.reals + sl.w + i * 4 + q;
                if (sizeof(Real) == 8) dgtc::cp_async8(dst, win + at, 8);
                else dgtc::cp_async4(dst, win + at, 4);
            }
            for (int t = tid; t < ne * NF * np; t += nt) sKall[t] = -1;
        }
        dgtc::cp_async_commit();
        dgtc::cp_async_wait_all();
        __syncthreads();
        // neighbour values at the face nodes (the maps are in shared memory now)
        {
            const int nn = NF * nfp * NQ;
            for (int t = tid; t < ne * nn; t += nt) {
                const int s = t / nn, r = t - s * nn;
                const int lf = r / (nfp * NQ), kq = r - lf * nfp * NQ;
                const int q = kq / nfp, k = kq - q * nfp;
                const int2 cn = __ldg(&a.fconn[(size_t)(c0 + s) * NF + lf]);
                const uint8_t *nbm = sMall + (size_t)s * a.mstride + (lf * 2 + 1) * nfp;
                const bool interior = ((cn.y >> 5) & 3) == kKindInterior;
                const long long at = interior ? q * a.fstride + (long long)cn.x * np + nbm[k] : 0;
                Real *dst = sReal + (size_t)s * sl.reals + sl.nb + (lf * nfp + k) * 4 + q;
                if (sizeof(Real) == 8) dgtc::cp_async8(dst, win + at, interior ? 8 : 0);
                else dgtc::cp_async4(dst, win + at, interior ? 4 : 0);
            }
            for (int t = tid; t < ne * NF * nfp; t += nt) {
                const int s = t / (NF * nfp), r = t - s * NF * nfp;
                const int lf = r / nfp, k = r - lf * nfp;
                sKall[(s * NF + lf) * np + sMall[(size_t)s * a.mstride + (lf * 2) * nfp + k]] = k;
            }
        }
        dgtc::cp_async_commit();
        // volume points need only the own state: start them while the
        // neighbour values arrive
        for (int t = tid; t < ne * ng; t += nt) {
            const int s = t / ng, g = t - s * ng;
            const Real *base = sReal + (size_t)s * sl.reals;
            Real Ua[4] = {Real(0), Real(0), Real(0), Real(0)}, Ub[4] = {Real(0), Real(0), Real(0), Real(0)};
            const Real *ph = a.phi + (size_t)g * np;
            const int half = np / 2;
            for (int j = 0; j < half; ++j) {
                const Real p0 = __ldg(ph + j), p1 = __ldg(ph + j + half);
                Real w0[4], w1[4];
                load4<Real>(base + sl.w + j * 4, w0);
                load4<Real>(base + sl.w + (j + half) * 4, w1);
#pragma unroll
                for (int q = 0; q < NQ; ++q) {
                    Ua[q] = fma(p0, w0[q], Ua[q]);
                    Ub[q] = fma(p1, w1[q], Ub[q]);
                }
            }
            if (np & 1) {
                const Real p = __ldg(ph + np - 1);
                Real w4[4];
                load4<Real>(base + sl.w + (np - 1) * 4, w4);
#pragma unroll
                for (int q = 0; q < NQ; ++q) Ua[q] = fma(p, w4[q], Ua[q]);
            }
            Real U[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) U[q] = Ua[q] + Ub[q];
            Real F[DIM][DIM + 1];
            lee_flux<DIM, Real>(U, v0, a.rc2, a.inv_rho, F);
            const Real *w = a.edata + (size_t)(c0 + s) * edim + eo.off_wm + g * DIM * DIM;
            Real *fc = sReal + (size_t)s * sl.reals + sl.fc + g * DIM * 4;
#pragma unroll
            for (int u = 0; u < DIM; ++u) {
                Real o[4] = {Real(0), Real(0), Real(0), Real(0)};
#pragma unroll
                for (int q = 0; q < NQ; ++q)
#pragma unroll
                    for (int x = 0; x < DIM; ++x) o[q] = fma(__ldg(w + x * DIM + u), F[x][q], o[q]);
                st4<Real>(fc + u * 4, o);
            }
        }
        dgtc::cp_async_wait_all();
        __syncthreads();
        // face points
        for (int t = tid; t < ne * NF * ngf; t += nt) {
            const int s = t / (NF * ngf), r = t - s * NF * ngf;
            const int lf = r / ngf, g = r - lf * ngf;
            Real *base = sReal + (size_t)s * sl.reals;
            const int2 cn = __ldg(&a.fconn[(size_t)(c0 + s) * NF + lf]);
            const int kind = (cn.y >> 5) & 3;
            const Real tau = (cn.y & 128) ? Real(-1) : Real(1);
            const uint8_t *own = sMall + (size_t)s * a.mstride + (lf * 2) * nfp;
            const Real *fp = a.fphi + (size_t)g * nfp;
            const Real *nb = base + sl.nb + lf * nfp * 4;
            Real qi[4] = {Real(0), Real(0), Real(0), Real(0)}, qo[4] = {Real(0), Real(0), Real(0), Real(0)};
            for (int k = 0; k < nfp; ++k) {
                const Real p = __ldg(fp + k);
                Real a4[4], b4[4];
                load4<Real>(base + sl.w + own[k] * 4, a4);
                load4<Real>(nb + k * 4, b4);
#pragma unroll
                for (int q = 0; q < NQ; ++q) {
                    qi[q] = fma(p, a4[q], qi[q]);
                    qo[q] = fma(p, b4[q], qo[q]);
                }
            }
            Real w4[4];
            {
                const Real *fwp = a.edata + (size_t)(c0 + s) * edim + eo.off_fw + (lf * ngf + g) * 4;
#pragma unroll
                for (int x = 0; x < 4; ++x) w4[x] = __ldg(fwp + x);
            }
            Real n[DIM];
#pragma unroll
            for (int x = 0; x < DIM; ++x) n[x] = w4[x];
            Real Fn[NQ];
            face_flux<DIM, Real>(kind, tau, qi, qo, n, a.rc2, a.inv_rho, a.half_c0, a.c0, a.rho, v0, Fn);
            Real o[4] = {Real(0), Real(0), Real(0), Real(0)};
#pragma unroll
            for (int q = 0; q < NQ; ++q) o[q] = w4[3] * Fn[q];
            st4<Real>(base + sl.fn + (lf * ngf + g) * 4, o);
        }
        __syncthreads();
        // S - F at the nodes, all fields of a node in one thread
        for (int t = tid; t < ne * np; t += nt) {
            const int s = t / np, i = t - s * np;
            Real *base = sReal + (size_t)s * sl.reals;
            // one accumulator set per reference direction: DIM x NQ independent chains
            Real Su[DIM][4];
#pragma unroll
            for (int u = 0; u < DIM; ++u)
#pragma unroll
                for (int q = 0; q < 4; ++q) Su[u][q] = Real(0);
            const Real *dp = a.dphi + i;
            const Real *fc = base + sl.fc;
            for (int g = 0; g < ng; ++g) {
#pragma unroll
                for (int u = 0; u < DIM; ++u) {
                    const Real d = __ldg(dp + ((size_t)u * ng + g) * np);
                    Real f4[4];
                    load4<Real>(fc + (g * DIM + u) * 4, f4);
#pragma unroll
                    for (int q = 0; q < NQ; ++q) Su[u][q] = fma(d, f4[q], Su[u][q]);
                }
            }
            Real S[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                S[q] = Su[0][q];
#pragma unroll
                for (int u = 1; u < DIM; ++u) S[q] += Su[u][q];
            }
            const int *sK = sKall + (size_t)s * NF * np;
#pragma unroll
            for (int lf = 0; lf < NF; ++lf) {
                const int k = sK[lf * np + i];
                if (k < 0) continue;
                const Real *fn = base + sl.fn + lf * ngf * 4;
                for (int g = 0; g < ngf; ++g) {
                    const Real p = __ldg(a.fphi + (size_t)g * nfp + k);
                    Real f4[4];
                    load4<Real>(fn + g * 4, f4);
#pragma unroll
                    for (int q = 0; q < NQ; ++q) S[q] = fma(-p, f4[q], S[q]);
                }
            }
            st4<Real>(base + sl.r + i * 4, S);
        }
        __syncthreads();
        // r = dt M^-1 (S - F) and the stage update
        Real *acc = a.acc + boff;
        Real *wout = a.wout + boff;
        const Real *uu = a.u + boff;
        for (int t = tid; t < ne * np; t += nt) {
            const int s = t / np, i = t - s * np;
            const Real *base = sReal + (size_t)s * sl.reals;
            const Real *mi = a.edata + (size_t)(c0 + s) * edim;
            // two interleaved halves of the node sum: 2 x NQ independent chains
            Real sa[4] = {Real(0), Real(0), Real(0), Real(0)}, sb[4] = {Real(0), Real(0), Real(0), Real(0)};
            const int half = np / 2;
            for (int j = 0; j < half; ++j) {
                const Real m0 = __ldg(mi + j * np + i), m1 = __ldg(mi + (j + half) * np + i);
                Real r0[4], r1[4];
                load4<Real>(base + sl.r + j * 4, r0);
                load4<Real>(base + sl.r + (j + half) * 4, r1);
#pragma unroll
                for (int q = 0; q < NQ; ++q) {
                    sa[q] = fma(m0, r0[q], sa[q]);
                    sb[q] = fma(m1, r1[q], sb[q]);
                }
            }
            if (np & 1) {
                const int j = np - 1;
                const Real m = __ldg(mi + j * np + i);
                Real r4[4];
                load4<Real>(base + sl.r + j * 4, r4);
#pragma unroll
                for (int q = 0; q < NQ; ++q) sa[q] = fma(m, r4[q], sa[q]);
            }
            Real sum[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) sum[q] = sa[q] + sb[q];
            Real q4[4];
            load4<Real>(base + sl.w + i * 4, q4);
            const long long ebase = (long long)__ldg(&a.el[c0 + s]) * np + i;
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                const Real rv = a.dt * sum[q];
                const Real qv = q4[q];
                const long long idx = q * a.fstride + ebase;
                if (a.ulo) {
                    // the mixed form's update of a state kept as an FP32 pair
                    // (the same formulas as its tensor-core stage kernel)
                    const Real pu = uu[idx], pl = a.ulo[boff + idx];
                    if (a.stage == 0) {
                        acc[idx] = rv;
                        wout[idx] = pu + (pl + Real(0.5) * rv);
                    } else if (a.stage == 1) {
                        acc[idx] = fma(Real(2), rv, acc[idx]);
                        wout[idx] = pu + (pl + Real(0.5) * rv);
                    } else if (a.stage == 2) {
                        acc[idx] = fma(Real(2), rv, acc[idx]);
                        wout[idx] = pu + (pl + rv);
                    } else {
                        const Real dlt = a.stage == 4 ? rv : (acc[idx] + rv) * (Real(1) / Real(6));
                        const Real s = pu + dlt;
                        const Real bp = s - pu;
                        Real e = (pu - (s - bp)) + (dlt - bp);
                        e += pl;
                        const Real nh = s + e;
                        wout[idx] = nh;
                        a.olo[boff + idx] = e - (nh - s);
                    }
                    continue;
                }
                if (a.stage == 0) {
                    acc[idx] = rv;
                    wout[idx] = fma(Real(0.5), rv, qv);
                } else if (a.stage == 1) {
                    acc[idx] = fma(Real(2), rv, acc[idx]);
                    wout[idx] = fma(Real(0.5), rv, uu[idx]);
                } else if (a.stage == 2) {
                    acc[idx] = fma(Real(2), rv, acc[idx]);
                    wout[idx] = uu[idx] + rv;
                } else if (a.stage == 3) {
                    wout[idx] = uu[idx] + (acc[idx] + rv) * (Real(1) / Real(6));
                } else {
                    wout[idx] = qv + rv;
                }
            }
        }
        __syncthreads();
    }
}

}  // namespace dgk
