// Fused RK4 stage kernel: one launch computes, for a tile of elements,
//   r = dt * ( sum_u D_u Fhat_u  -  sum_f (detJf/detJe) LIFT_f Fn_f )
// and applies the classical RK4 stage update.  It replaces, per stage, the
// reference's Mesh::updateFlux (Mesh.cpp:569-674), Mesh::precomputeFlux
// (Mesh.cpp:500-539), Mesh::getElFlux (Mesh.cpp:548-557),
// Mesh::getElStiffVector (Mesh.cpp:476-489), eigen::minus / eigen::linEq
// (utils.cpp:118-136, called at solver.cpp:46-48) and the RK combination
// (solver.cpp:261-285).
//
// Algebra (affine elements, B = dx/du^-1, detJ constant):
//   M_e^-1 S_e = sum_u D_u Fhat_u,   Fhat_u = sum_x B[x][u] Flux[x],
//   D_u = Mhat^-1 Shat_u (weak derivative);  applied here to the primitive
//   fields first: grad_x q = sum_u B[x][u] (D_u q), then
//   V_p  = v0.grad p + rho0 c0^2 div v,   V_vd = v0.grad v_d + grad_d p / rho0.
//   M_e^-1 F_e = sum_f (detJf/detJe) Mhat^-1 E_f Mfhat Fn_f.
// Face values (element-centric: each interior face is evaluated from both
// sides; n_e is the element's outward normal, tau the jump sign):
//   interior   Fn = 1/2 n_e.(F(q) + F(q_o)) + 1/2 tau c0 (q - q_o)   (Mesh.cpp:519-527)
//   reflecting Fn = F(q_w).n_e, q_w = (p, v - (v.n)n)                (Mesh.cpp:616-647)
//   absorbing  Fn = R K R^-1 q                                        (Mesh.cpp:391-418, 649-668)
//
// Thread layout: a block holds EPB elements, one thread per element node;
// the state of the tile and the face values are staged in shared memory, the
// reference-element operators stay in shared memory for the whole (grid-
// stride, persistent) launch.  State is field-major, element-major inside a
// field: q[f * fstride + e * NP + i], the reference's u[f][el*Np+n] layout.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace dgk {

template <int DIM, int P>
struct Shape {
    static constexpr int NP = DIM == 2 ? (P + 1) * (P + 2) / 2 : (P + 1) * (P + 2) * (P + 3) / 6;
    static constexpr int NF = DIM + 1;
    static constexpr int NFP = DIM == 2 ? P + 1 : (P + 1) * (P + 2) / 2;
    static constexpr int NQ = DIM + 1;
    static constexpr int NPERM = DIM == 2 ? 2 : 6;
    static constexpr int NSLOT = NF * NFP;
    static constexpr int NOPS = DIM * NP * NP + NSLOT * NP;   // D then LIFT
    static constexpr int NOPS_PAD = (NOPS + 3) / 4 * 4;        // keeps the state tile 16-byte aligned
    static constexpr int NTAB = NF * NFP + NPERM * NFP;       // fmask then perm
};

// Connectivity word of an element face: bits 0-1 neighbour's local face,
// 2-4 face permutation, 5-6 kind (0 interior, 1 reflecting, 2 absorbing),
// 7 negative jump sign.
enum : int { kKindInterior = 0, kKindReflecting = 1, kKindAbsorbing = 2 };
enum : int { kStageEuler = 5 };

template <typename Real>
struct StageArgs {
    const Real *win;       // stage input
    const Real *u;         // state at the start of the step
    Real *acc;             // k1 + 2 k2 + 2 k3 accumulator
    Real *wout;            // next stage input (stage 4: the new state, == u)
    long long fstride;     // elements * NP (distance between fields)
    long long bstride;     // distance between batch members (sources)
    const Real *geo;       // [K][DIM*DIM]  B[x][u] at x*DIM+u (rounded once to Real)
    const Real *fgeo;      // [K][NF][4]    outward normal (DIM) and detJf/detJe
    const int2 *conn;      // [K][NF]       neighbour element, connectivity word
    const Real *ops;       // NOPS reference operators
    const uint8_t *tabs;   // NTAB tables
    const int *elist = nullptr;  // elements to run (the straight-sided ones of a mesh with curved elements), or null: all
    int K;                 // elements to run
    Real dt;
    Real rc2;      // rho0 c0^2
    Real inv_rho;  // 1 / rho0
    Real half_c0;  // c0 / 2
    Real c0;
    Real rho;
    Real v0[3];
};

template <int DIM, int P, typename Real, int EPB>
struct StageSmem {
    using S = Shape<DIM, P>;
    static constexpr size_t ops = sizeof(Real) * S::NOPS_PAD;
    static constexpr size_t q = sizeof(Real) * EPB * S::NP * 4;
    static constexpr size_t fn = sizeof(Real) * EPB * S::NSLOT * 4;
    static constexpr size_t tab = (S::NTAB + 15) / 16 * 16;
    static constexpr size_t total = ops + q + fn + tab;
};

template <typename Real>
__device__ __forceinline__ void load4(const Real *p, Real (&v)[4]);
template <>
__device__ __forceinline__ void load4<float>(const float *p, float (&v)[4]) {
    float4 t = *reinterpret_cast<const float4 *>(p);
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
template <>
__device__ __forceinline__ void load4<double>(const double *p, double (&v)[4]) {
    double2 a = *reinterpret_cast<const double2 *>(p);
    double2 b = *reinterpret_cast<const double2 *>(p + 2);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}

// One tile of EPB elements: stages the state, evaluates the right-hand side
// and applies the stage update.  sQ, sFn are the tile buffers; sOps, sTab
// hold the reference operators and the face tables of order P.  Threads
// with tid >= EPB*NP only take part in the barriers.
template <int DIM, int P, typename Real, int STAGE, int EPB>
__device__ __forceinline__ void stage_tile(const StageArgs<Real> &a, long long boff, int tile, Real *sQ, Real *sFn,
                                           const Real *sOps, const uint8_t *sTab, int tid) {
    using S = Shape<DIM, P>;
    constexpr int NP = S::NP, NF = S::NF, NFP = S::NFP, NQ = S::NQ, NSLOT = S::NSLOT;
    constexpr int NT = EPB * NP;
    const Real *sD = sOps;
    const Real *sL = sOps + DIM * NP * NP;
    const uint8_t *sFmask = sTab;
    const uint8_t *sPerm = sTab + NF * NFP;
    // threads past EPB*NP (a CTA larger than the tile) work on element 0,
    // node 0 but never write shared or global memory
    const bool active = tid < NT;
    const int le = active ? tid / NP : 0;
    const int i = active ? tid - le * NP : 0;
    const Real *win = a.win + boff;
    const int idx = tile * EPB + le;
    const bool valid = active && (idx < a.K);
    // meshes with curved elements: the tiles run over the list of the others
    const int e = (a.elist && valid) ? __ldg(&a.elist[idx]) : idx;
    const long long base = (long long)e * NP + i;
    Real q[NQ];
#pragma unroll
    for (int f = 0; f < NQ; ++f) {
        q[f] = valid ? win[f * a.fstride + base] : Real(0);
        if (active) sQ[(le * NP + i) * 4 + f] = q[f];
    }
    __syncthreads();

    // Reference-space derivatives of the primitive fields.
    Real dq[NQ][DIM];
#pragma unroll
    for (int f = 0; f < NQ; ++f)
#pragma unroll
        for (int u = 0; u < DIM; ++u) dq[f][u] = Real(0);
#pragma unroll 2
    for (int j = 0; j < NP; ++j) {
        Real qj[4];
        load4<Real>(&sQ[(le * NP + j) * 4], qj);
#pragma unroll
        for (int u = 0; u < DIM; ++u) {
            const Real d = sD[(u * NP + j) * NP + i];
#pragma unroll
            for (int f = 0; f < NQ; ++f) dq[f][u] = fma(d, qj[f], dq[f][u]);
        }
    }
    // Physical derivatives and the volume term.
    Real V[NQ];
    {
        Real B[DIM][DIM];
#pragma unroll
        for (int x = 0; x < DIM; ++x)
#pragma unroll
            for (int u = 0; u < DIM; ++u)
                B[x][u] = valid ? a.geo[(long long)e * DIM * DIM + x * DIM + u] : Real(0);
        Real g[NQ][DIM];
#pragma unroll
        for (int f = 0; f < NQ; ++f)
#pragma unroll
            for (int x = 0; x < DIM; ++x) {
                Real s = Real(0);
#pragma unroll
                for (int u = 0; u < DIM; ++u) s = fma(B[x][u], dq[f][u], s);
                g[f][x] = s;
            }
        Real div = Real(0), adv_p = Real(0);
#pragma unroll
        for (int x = 0; x < DIM; ++x) {
            div += g[1 + x][x];
            adv_p = fma(a.v0[x], g[0][x], adv_p);
        }
        V[0] = fma(a.rc2, div, adv_p);
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            Real adv = Real(0);
#pragma unroll
            for (int x = 0; x < DIM; ++x) adv = fma(a.v0[x], g[1 + d][x], adv);
            V[1 + d] = fma(a.inv_rho, g[0][d], adv);
        }
    }

    // Face values at the element's face nodes.
    for (int s = active ? i : NSLOT; s < NSLOT; s += NP) {
        const int lf = s / NFP;
        const int k = s - lf * NFP;
        const int vi = sFmask[lf * NFP + k];
        Real own[4];
        load4<Real>(&sQ[(le * NP + vi) * 4], own);
        Real Fn[NQ];
#pragma unroll
        for (int f = 0; f < NQ; ++f) Fn[f] = Real(0);
        Real scale = Real(0);
        if (valid) {
            const int2 cn = a.conn[(long long)e * NF + lf];
            Real g4[4];
            load4<Real>(&a.fgeo[((long long)e * NF + lf) * 4], g4);
            Real n[DIM];
#pragma unroll
            for (int x = 0; x < DIM; ++x) n[x] = g4[x];
            scale = g4[DIM];
            Real vn0 = Real(0);
#pragma unroll
            for (int x = 0; x < DIM; ++x) vn0 = fma(a.v0[x], n[x], vn0);
            const int kind = (cn.y >> 5) & 3;
            if (kind == kKindInterior) {
                const int nlf = cn.y & 3;
                const int pm = (cn.y >> 2) & 7;
                const Real tau = (cn.y & 128) ? Real(-1) : Real(1);
                const int nvi = sFmask[nlf * NFP + sPerm[pm * NFP + k]];
                const long long nb = (long long)cn.x * NP + nvi;
                Real o[NQ];
#pragma unroll
                for (int f = 0; f < NQ; ++f) o[f] = __ldg(&win[f * a.fstride + nb]);
                const Real sp = own[0] + o[0];
                Real svn = Real(0);
#pragma unroll
                for (int x = 0; x < DIM; ++x) svn = fma(own[1 + x] + o[1 + x], n[x], svn);
                const Real hj = a.half_c0 * tau;
                Fn[0] = fma(hj, own[0] - o[0], Real(0.5) * fma(vn0, sp, a.rc2 * svn));
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                    Fn[1 + d] = fma(hj, own[1 + d] - o[1 + d],
                                    Real(0.5) * fma(vn0, own[1 + d] + o[1 + d], a.inv_rho * sp * n[d]));
            } else if (kind == kKindReflecting) {
                Real vn = Real(0);
#pragma unroll
                for (int x = 0; x < DIM; ++x) vn = fma(own[1 + x], n[x], vn);
                Real vw[DIM];
                Real vwn = Real(0);
#pragma unroll
                for (int x = 0; x < DIM; ++x) {
                    vw[x] = own[1 + x] - vn * n[x];
                    vwn = fma(vw[x], n[x], vwn);
                }
                Fn[0] = fma(vn0, own[0], a.rc2 * vwn);
#pragma unroll
                for (int d = 0; d < DIM; ++d) Fn[1 + d] = fma(vn0, vw[d], a.inv_rho * own[0] * n[d]);
            } else {
                Real vn = Real(0);
#pragma unroll
                for (int x = 0; x < DIM; ++x) vn = fma(own[1 + x], n[x], vn);
                const Real q0 = Real(0.25) * a.c0;
                Fn[0] = fma(q0, own[0], Real(0.25) * a.c0 * a.c0 * a.rho * vn);
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                    Fn[1 + d] = fma(Real(0.25) * n[d] * a.inv_rho, own[0], q0 * n[d] * vn);
            }
        }
#pragma unroll
        for (int f = 0; f < NQ; ++f) sFn[(le * NSLOT + s) * 4 + f] = scale * Fn[f];
    }
    __syncthreads();

    // Lift and stage update.
    Real L[NQ];
#pragma unroll
    for (int f = 0; f < NQ; ++f) L[f] = Real(0);
#pragma unroll 4
    for (int s = 0; s < NSLOT; ++s) {
        const Real l = sL[s * NP + i];
        Real fn[4];
        load4<Real>(&sFn[(le * NSLOT + s) * 4], fn);
#pragma unroll
        for (int f = 0; f < NQ; ++f) L[f] = fma(l, fn[f], L[f]);
    }
    if (valid) {
        Real *acc = a.acc + boff;
        Real *wout = a.wout + boff;
        const Real *uu = a.u + boff;
#pragma unroll
        for (int f = 0; f < NQ; ++f) {
            const long long idx = f * a.fstride + base;
            const Real r = a.dt * (V[f] - L[f]);
            if (STAGE == 1) {
                acc[idx] = r;
                wout[idx] = fma(Real(0.5), r, q[f]);
            } else if (STAGE == 2) {
                acc[idx] = fma(Real(2), r, acc[idx]);
                wout[idx] = fma(Real(0.5), r, uu[idx]);
            } else if (STAGE == 3) {
                acc[idx] = fma(Real(2), r, acc[idx]);
                wout[idx] = uu[idx] + r;
            } else if (STAGE == kStageEuler) {
                wout[idx] = q[f] + r;
            } else {
                wout[idx] = uu[idx] + (acc[idx] + r) * (Real(1) / Real(6));
            }
        }
    }
    __syncthreads();
}

// STAGE 1-4: the classical RK4 stages; kStageEuler: one forward-Euler step
// wout = win + dt*RHS(win) (the reference's numStep with beta = 1).
template <int DIM, int P, typename Real, int STAGE, int EPB>
__global__ void __launch_bounds__(EPB *Shape<DIM, P>::NP)
    stage_kernel(const StageArgs<Real> a) {
    using S = Shape<DIM, P>;
    constexpr int NP = S::NP;
    constexpr int NT = EPB * NP;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Real *sOps = reinterpret_cast<Real *>(smem_raw);
    Real *sQ = sOps + S::NOPS_PAD;
    Real *sFn = sQ + EPB * NP * 4;
    uint8_t *sTab = reinterpret_cast<uint8_t *>(sFn + EPB * S::NSLOT * 4);
    const int tid = threadIdx.x;
    const long long boff = (long long)blockIdx.y * a.bstride;
    for (int k = tid; k < S::NOPS; k += NT) sOps[k] = a.ops[k];
    for (int k = tid; k < S::NTAB; k += NT) sTab[k] = a.tabs[k];
    __syncthreads();
    const int ntiles = (a.K + EPB - 1) / EPB;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x)
        stage_tile<DIM, P, Real, STAGE, EPB>(a, boff, tile, sQ, sFn, sOps, sTab, tid);
}

// Hard sources (solver.cpp:248-256): p = amp sin(2 pi f t + phase) while
// t < duration, scaled by a per-(source, node) weight (1 for the reference's
// sources).  Thread per source node; node j is the state value at offset
// at[j] (batch member and node folded in) and its sources are applied in
// order, so a later active source overwrites an earlier one (the reference's
// loop order).  t = t0 + kstep*dt by repeated addition, as the host loop.
template <typename Real>
__global__ void inject_kernel(Real *p, const long long *at, const int *node_src_off, const int *node_src,
                              const double *node_w, const double *params, const double *t0, int kstep, double dt,
                              int nnodes, Real *plo) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nnodes) return;
    double t = *t0;
    for (int k = 0; k < kstep; ++k) t += dt;
    bool set = false;
    double val = 0;
    for (int s = node_src_off[j]; s < node_src_off[j + 1]; ++s) {
        const double *pr = params + 4 * node_src[s];
        if (t < pr[3]) {
            val = node_w[s] * (pr[0] * sin(2 * M_PI * pr[1] * t + pr[2]));
            set = true;
        }
    }
    if (set) {
        p[at[j]] = Real(val);
        // state kept as a pair: low part of the injected value
        if (plo) plo[at[j]] = Real(val - double(Real(val)));
    }
}

// Receivers: the pressure of every batch member at nrec nodes after step
// (*step0 + kstep), into trace[member][rec][max_steps].
template <typename Real>
__global__ void record_kernel(const Real *p, const Real *plo, long long bstride, const int *rec_dof, int nrec,
                              int nbatch, double *trace, int max_steps, const long long *step0, int kstep) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nrec * nbatch) return;
    const long long step = *step0 + kstep;
    if (step >= max_steps) return;
    const int m = j / nrec, r = j - m * nrec;
    const long long at = m * bstride + rec_dof[r];
    double v = double(p[at]);
    if (plo) v += double(plo[at]);
    trace[(long long)j * max_steps + step] = v;
}

}  // namespace dgk
