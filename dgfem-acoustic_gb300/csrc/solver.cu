// C ABI of the GPU RK4 right-hand side (include/dgcuda.h): context creation
// (device layout of the reference Mesh arrays), state transfer, sources, the
// step loop (CUDA graphs of step chunks), per-kernel timing and monitors.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/dgcuda.h"
#include "host/capi_common.h"
#include "host/layout.h"
#include "host/refel.h"
#include "ctx.h"
#include "curved_kernel.cuh"
#include "kernels.h"
#include "stage_kernel.cuh"

using dg::fail;

namespace dgk {
bool get_kernels(int prec, int dim, int order, KernelSet *out) {
    if (prec == DG_PREC_FP64) return dim == 2 ? kernels_f64_2d(order, out) : kernels_f64_3d(order, out);
    return dim == 2 ? kernels_f32_2d(order, out) : kernels_f32_3d(order, out);
}
}  // namespace dgk

namespace {

const int kGraphChunk = 32;
// Time integrators ("Runge-Kutta" and "Euler1" in the reference's config) and
// the stage index of the forward-Euler kernel in launch_stage.
const int kMethodRK4 = 0, kMethodEuler = 1;
const int kEulerStage = 4;

template <typename Real>
__global__ void cast_kernel(const double *src, Real *dst, long long n) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    for (; i < n; i += (long long)gridDim.x * blockDim.x) dst[i] = Real(src[i]);
}
template <typename Real>
__global__ void uncast_kernel(const Real *src, double *dst, long long n) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    for (; i < n; i += (long long)gridDim.x * blockDim.x) dst[i] = double(src[i]);
}
// State kept as an FP32 pair (mixed form): x = hi + lo.
__global__ void split_kernel(const double *src, float *hi, float *lo, long long n) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    for (; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float h = float(src[i]);
        hi[i] = h;
        lo[i] = float(src[i] - double(h));
    }
}
__global__ void join_kernel(const float *hi, const float *lo, double *dst, long long n) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    for (; i < n; i += (long long)gridDim.x * blockDim.x) dst[i] = double(hi[i]) + double(lo[i]);
}
__global__ void copy_kernel(const double *src, double *dst, long long n) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    for (; i < n; i += (long long)gridDim.x * blockDim.x) dst[i] = src[i];
}

// Host arrays the GPU can address (pinned or registered host memory): the
// device-side address, else null.  The conversion kernels then read or write
// such an array themselves over the host link (NVLink-C2C on Grace), in one
// pass and without a staging copy per field.
const void *host_device_view(const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}
const int kHostIoBlocks = 2048;  // grid of the host-link kernels: many loads in flight

// Value i of a state kept in the context's precision, plus its low FP32 part
// when the state is an FP32 pair (mixed form): the FP64 value the form holds.
template <typename Real>
__device__ __forceinline__ double state_value(const Real *q, const float *lo, long long i) {
    return lo ? double(q[i]) + double(lo[i]) : double(q[i]);
}

// FP64 monitors: thread per element, u^T M u per field, non-finite count.
// Curved elements (cslot[e] >= 0) use their own mass matrix, applied as the
// rule it was summed on: u^T M u = sum_g w detJ(g) u(g)^2.  `ulo` (mixed form
// only, else null) is the low part of the state pair, same layout as u.
template <typename Real>
__global__ void monitor_kernel(const Real *u, const float *ulo, long long fstride, int K, int np, int nq,
                               const double *mass, const double *detj, double rho, double c0,
                               double *out /*[2+nq]*/, unsigned long long *bad, const int *cslot,
                               const double *cwdet, const double *cphi, int cng) {
    __shared__ double red[256][5];
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    double loc[5] = {0, 0, 0, 0, 0};
    unsigned long long nbad = 0;
    if (e < K) {
        const int cs = cslot ? cslot[e] : -1;
        for (int f = 0; f < nq; ++f) {
            const long long base = f * fstride + (long long)e * np;
            const Real *q = u + base;
            const float *ql = ulo ? ulo + base : nullptr;
            double s = 0;
            for (int i = 0; i < np; ++i)
                if (!isfinite(state_value(q, ql, i))) ++nbad;
            if (cs >= 0) {
                for (int g = 0; g < cng; ++g) {
                    double v = 0;
                    for (int j = 0; j < np; ++j) v += cphi[g * np + j] * state_value(q, ql, j);
                    s += cwdet[(long long)cs * cng + g] * v * v;
                }
                loc[1 + f] = s;
                continue;
            }
            for (int i = 0; i < np; ++i) {
                double qi = state_value(q, ql, i);
                double t = 0;
                for (int j = 0; j < np; ++j) t += mass[i * np + j] * state_value(q, ql, j);
                s += qi * t;
            }
            loc[1 + f] = s * detj[e];
        }
        double en = loc[1] / (rho * c0 * c0);
        for (int f = 1; f < nq; ++f) en += rho * loc[1 + f];
        loc[0] = 0.5 * en;
    }
    for (int k = 0; k < 5; ++k) red[threadIdx.x][k] = loc[k];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int k = 0; k < 5; ++k) red[threadIdx.x][k] += red[threadIdx.x + s][k];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 1 + nq; ++k) atomicAdd(&out[k], red[0][k]);
    if (nbad) atomicAdd(bad, nbad);
}

// FP64 error monitor: per field, sum (u - r)^2 and sum r^2 over the nodal
// values of two states of the same mesh (either precision, FP32 pairs joined),
// grid-stride, block reduction in shared memory, one atomic per block and
// quantity.  out[2f] = squared difference, out[2f+1] = squared reference;
// `bad` counts non-finite values of u.
template <typename RU, typename RR>
__global__ void error_kernel(const RU *u, const float *ulo, const RR *r, const float *rlo, long long n, int nq,
                             double *out /*[8]*/, unsigned long long *bad) {
    __shared__ double red[8][256];
    double loc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    unsigned long long nbad = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (int f = 0; f < nq; ++f)
        for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            const long long k = f * n + i;
            const double a = state_value(u, ulo, k), b = state_value(r, rlo, k);
            if (!isfinite(a)) ++nbad;
            loc[2 * f] += (a - b) * (a - b);
            loc[2 * f + 1] += b * b;
        }
    for (int k = 0; k < 8; ++k) red[k][threadIdx.x] = loc[k];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int k = 0; k < 8; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 2 * nq; ++k) atomicAdd(&out[k], red[k][0]);
    if (nbad) atomicAdd(bad, nbad);
}

template <typename RU, typename RR>
void launch_error(const void *u, const float *ulo, const void *r, const float *rlo, long long n, int nq,
                  double *out, unsigned long long *bad, cudaStream_t st) {
    const int blocks = (int)std::min<long long>((n + 255) / 256, 4 * 152);
    error_kernel<RU, RR><<<std::max(blocks, 1), 256, 0, st>>>(static_cast<const RU *>(u), ulo,
                                                             static_cast<const RR *>(r), rlo, n, nq, out, bad);
}

}  // namespace


namespace {

int cuda_fail(cudaError_t e, const char *what) {
    return fail(DG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(call)                                             \
    do {                                                     \
        cudaError_t _e = (call);                             \
        if (_e != cudaSuccess) return cuda_fail(_e, #call);  \
    } while (0)

void free_ctx(dg_ctx *c) {
    if (!c) return;
    if (c->device >= 0) cudaSetDevice(c->device);
    if (c->save_stream) {
        // copies to the caller's buffers may still be in flight
        cudaStreamSynchronize(c->save_stream);
        cudaStreamDestroy(c->save_stream);
    }
    if (c->load_stream) {
        // staged copies from the caller's buffers may still be in flight
        cudaStreamSynchronize(c->load_stream);
        cudaStreamDestroy(c->load_stream);
    }
    for (int k = 0; k < 2; ++k) {
        if (c->snap_ready[k]) cudaEventDestroy(c->snap_ready[k]);
        if (c->snap_done[k]) cudaEventDestroy(c->snap_done[k]);
        if (c->d_snap[k]) cudaFree(c->d_snap[k]);
        if (c->load_done[k]) cudaEventDestroy(c->load_done[k]);
        if (c->load_used[k]) cudaEventDestroy(c->load_used[k]);
        if (c->d_load[k]) cudaFree(c->d_load[k]);
    }
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    for (auto ev : c->events) cudaEventDestroy(ev);
    void *ptrs[] = {c->d_state, c->d_geo,     c->d_fgeo,    c->d_conn,    c->d_ops,     c->d_tabs,
                    c->d_t0,    c->d_stage64, c->d_mass,    c->d_detj,    c->d_mon,     c->d_bad,
                    c->d_src_at, c->d_src_off, c->d_src_list, c->d_src_w, c->d_src_params, c->d_ulo,
                    c->d_bimg,  c->d_beb,     c->d_err,     c->d_rec_dof, c->d_trace,   c->d_step0,
                    c->d_geo32, c->d_cel,     c->d_cslot,   c->d_cedata,  c->d_cwdet,   c->d_cphi,
                    c->d_cdphi, c->d_cfphi,   c->d_cfconn,  c->d_cfmap,   c->d_cphi64,  c->d_aff,
                    c->d_cmask, c->d_blist};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

template <typename Real>
void fill_args(dg_ctx *c, dgk::StageArgs<Real> &a, int stage, double dt) {
    a.fstride = c->ndof;
    a.bstride = c->bstride;
    if constexpr (sizeof(Real) == 8) a.geo = reinterpret_cast<const Real *>(c->d_geo);
    else a.geo = reinterpret_cast<const Real *>(c->d_geo32);
    a.fgeo = reinterpret_cast<const Real *>(c->d_fgeo);
    a.conn = c->d_conn;
    a.ops = reinterpret_cast<const Real *>(c->d_ops);
    a.tabs = c->d_tabs;
    a.elist = c->d_aff;
    a.K = c->naff;
    a.dt = Real(dt);
    a.rc2 = Real(c->rho0 * c->c0 * c->c0);
    a.inv_rho = Real(1.0 / c->rho0);
    a.half_c0 = Real(0.5 * c->c0);
    a.c0 = Real(c->c0);
    a.rho = Real(c->rho0);
    for (int k = 0; k < 3; ++k) a.v0[k] = Real(c->v0[k]);
    Real *u = (Real *)c->d_u, *acc = (Real *)c->d_acc, *wa = (Real *)c->d_wa, *wb = (Real *)c->d_wb;
    a.u = u;
    a.acc = acc;
    switch (stage) {
        case 0: a.win = u; a.wout = wa; break;
        case 1: a.win = wa; a.wout = wb; break;
        case 2: a.win = wb; a.wout = wa; break;
        case 3: a.win = wa; a.wout = u; break;
        default: a.win = u; a.wout = wa; break;  // forward Euler: u -> wa
    }
}

cudaError_t launch_affine_stage(dg_ctx *c, int stage, double dt);

template <typename Real>
cudaError_t launch_curved(dg_ctx *c, int stage, double dt) {
    dgk::StageArgs<Real> s;
    fill_args<Real>(c, s, stage, dt);
    dgk::CurvedArgs<Real> a;
    a.win = s.win;
    a.u = s.u;
    a.acc = s.acc;
    a.wout = s.wout;
    a.fstride = c->ndof;
    a.bstride = c->bstride;
    a.el = c->d_cel;
    a.edata = static_cast<const Real *>(c->d_cedata);
    a.fconn = c->d_cfconn;
    a.fmap = c->d_cfmap;
    a.phi = static_cast<const Real *>(c->d_cphi);
    a.dphi = static_cast<const Real *>(c->d_cdphi);
    a.fphi = static_cast<const Real *>(c->d_cfphi);
    a.C = c->curved;
    a.np = c->np;
    a.ng = c->cng;
    a.ngf = c->cngf;
    a.nfp = c->nfp;
    a.epc = c->cepc;
    a.estride = c->cestride;
    a.mstride = c->cmstride;
    a.stage = stage == kEulerStage ? 4 : stage;
    a.dt = s.dt;
    a.rc2 = s.rc2;
    a.inv_rho = s.inv_rho;
    a.half_c0 = s.half_c0;
    a.c0 = s.c0;
    a.rho = s.rho;
    for (int k = 0; k < 3; ++k) a.v0[k] = s.v0[k];
    if (c->mixed) {
        // the state is an FP32 pair: low part in, new low part out (RK4: u's;
        // forward Euler: the target buffer's, swapped in after the step)
        a.ulo = reinterpret_cast<const Real *>(c->d_ulo);
        a.olo = stage == kEulerStage ? static_cast<Real *>(c->d_acc) : reinterpret_cast<Real *>(c->d_ulo);
    }
    void *args[] = {&a};
    return cudaLaunchKernel(c->curved_fn, dim3(c->curved_grid, c->nbatch, 1), dim3(256, 1, 1), args,
                            c->curved_smem, c->stream);
}

cudaError_t launch_stage(dg_ctx *c, int stage, double dt) {
    // no straight element at all: nothing for the affine / tensor-core kernel
    const bool none = c->curved > 0 && (c->mixed ? c->nblk == 0 : c->naff == 0);
    cudaError_t e = none ? cudaSuccess : launch_affine_stage(c, stage, dt);
    if (e != cudaSuccess || c->curved == 0) return e;
    return c->prec == DG_PREC_FP64 ? launch_curved<double>(c, stage, dt) : launch_curved<float>(c, stage, dt);
}

cudaError_t launch_affine_stage(dg_ctx *c, int stage, double dt) {
    if (c->mixed) {
        dgk::MixedArgs a;
        dgk::StageArgs<float> s;
        fill_args<float>(c, s, stage, dt);
        a.win = s.win;
        a.u = s.u;
        a.ulo = c->d_ulo;
        a.acc = s.acc;
        a.wout = s.wout;
        a.wlo = stage == kEulerStage ? static_cast<float *>(c->d_acc) : nullptr;
        a.fstride = s.fstride;
        a.bstride = c->bstride;
        a.nbatch = c->nbatch;
        a.geo = c->d_geo32;
        a.fgeo = s.fgeo;
        a.conn = s.conn;
        a.bimg = c->d_bimg;
        a.beb = c->d_beb;
        a.tabs = s.tabs;
        a.K = c->K;  // element blocks of the whole mesh; curved elements are masked
        a.cmask = c->d_cmask;
        a.blist = c->d_blist;
        a.nblk = c->nblk;
        a.dt = s.dt;
        a.rc2 = s.rc2;
        a.inv_rho = s.inv_rho;
        a.half_c0 = s.half_c0;
        a.c0 = s.c0;
        a.rho = s.rho;
        for (int k = 0; k < 3; ++k) a.v0[k] = s.v0[k];
        a.err = c->d_err;
        void *args[] = {&a};
        const void *fn = stage == kEulerStage ? c->mks.euler : c->mks.stage[stage];
        return cudaLaunchKernel(fn, dim3(c->grid), dim3(c->mks.threads), args, c->mks.smem, c->stream);
    }
    dim3 grid(c->grid, c->nbatch, 1), block(c->ks.threads, 1, 1);
    const void *fn = stage == kEulerStage ? c->ks.euler : c->ks.stage[stage];
    if (c->prec == DG_PREC_FP64) {
        dgk::StageArgs<double> a;
        fill_args<double>(c, a, stage, dt);
        void *args[] = {&a};
        return cudaLaunchKernel(fn, grid, block, args, c->ks.smem, c->stream);
    } else {
        dgk::StageArgs<float> a;
        fill_args<float>(c, a, stage, dt);
        void *args[] = {&a};
        return cudaLaunchKernel(fn, grid, block, args, c->ks.smem, c->stream);
    }
}

cudaError_t launch_inject(dg_ctx *c, int kstep, double dt) {
    if (!c->src_nodes) return cudaSuccess;
    dim3 grid((c->src_nodes + 127) / 128, 1, 1), block(128, 1, 1);
    void *p = c->d_u;  // field 0 of member 0 of u
    int nn = c->src_nodes;
    void *plo = c->d_ulo;  // null unless the state is kept as a pair
    void *args[] = {&p, &c->d_src_at, &c->d_src_off, &c->d_src_list, &c->d_src_w, &c->d_src_params, &c->d_t0,
                    &kstep, &dt, &nn, &plo};
    return cudaLaunchKernel(c->ks.inject, grid, block, args, 0, c->stream);
}

cudaError_t launch_record(dg_ctx *c, int kstep) {
    if (!c->rec_n) return cudaSuccess;
    const int n = c->rec_n * c->nbatch;
    dim3 grid((n + 127) / 128, 1, 1), block(128, 1, 1);
    void *p = c->d_u;
    void *plo = c->d_ulo;
    void *args[] = {&p, &plo, &c->bstride, &c->d_rec_dof, &c->rec_n, &c->nbatch, &c->d_trace, &c->rec_max,
                    &c->d_step0, &kstep};
    return cudaLaunchKernel(c->ks.record, grid, block, args, 0, c->stream);
}

// Forward-Euler steps ping-pong between (u, ulo) and (wa, acc): after each
// step the host swaps the roles so that the next launch reads the new state.
void swap_euler_buffers(dg_ctx *c) {
    std::swap(c->d_u, c->d_wa);
    if (c->mixed) {
        void *lo = c->d_ulo;
        c->d_ulo = static_cast<float *>(c->d_acc);
        c->d_acc = lo;
    }
}

cudaError_t launch_step(dg_ctx *c, int kstep, double dt, int method) {
    cudaError_t e = launch_inject(c, kstep, dt);
    if (method == kMethodEuler) {
        if (e == cudaSuccess) e = launch_stage(c, kEulerStage, dt);
        swap_euler_buffers(c);
    } else {
        for (int s = 0; s < 4 && e == cudaSuccess; ++s) e = launch_stage(c, s, dt);
    }
    if (e == cudaSuccess) e = launch_record(c, kstep);
    return e;
}

bool any_source_active(dg_ctx *c, double t) {
    for (double d : c->src_duration)
        if (t < d) return true;
    return false;
}

}  // namespace

extern "C" {

void dg_default_opts(dg_opts *o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->precision = DG_PREC_FP64;
    o->flux_sign = DG_FLUX_REFERENCE;
    o->device = 0;
    o->use_graph = 1;
}

int dg_create(const dg_mesh_desc *m, const dg_phys_desc *ph, const dg_opts *opts_in, dg_ctx **out) {
    return dg_create_batch(m, ph, opts_in, 1, out);
}

static int dg_create_batch_impl(const dg_mesh_desc *m, const dg_phys_desc *ph, const dg_opts *opts_in, int nbatch,
                    dg_ctx **out) {
    if (!m || !ph || !out) return fail(DG_ERR_ARG, "null argument");
    if (nbatch < 1 || nbatch > 65535) return fail(DG_ERR_ARG, "batch size must be in 1..65535");
    *out = nullptr;
    dg_opts opts;
    if (opts_in) opts = *opts_in;
    else dg_default_opts(&opts);
    if (m->dim != 2 && m->dim != 3) return fail(DG_ERR_UNSUPPORTED, "dimension must be 2 or 3");
    if (m->order < 1 || m->order > 5) return fail(DG_ERR_UNSUPPORTED, "order must be in 1..5");
    if (opts.precision != DG_PREC_FP64 && opts.precision != DG_PREC_FP32 && opts.precision != DG_PREC_MIXED &&
        opts.precision != DG_PREC_TF32X3)
        return fail(DG_ERR_ARG, "unknown precision");
    if (opts.flux_sign != DG_FLUX_REFERENCE && opts.flux_sign != DG_FLUX_UPWIND)
        return fail(DG_ERR_ARG, "unknown flux sign mode");
    if (!(ph->c0 > 0) || !(ph->rho0 > 0)) return fail(DG_ERR_ARG, "c0 and rho0 must be positive");
    dg::Layout lay;
    {
        std::string err;
        try {
            err = dg::build_layout(*m, opts.flux_sign, lay);
        } catch (std::exception &e) {
            err = e.what();
        }
        if (!err.empty()) return fail(DG_ERR_MESH, err);
    }
    const int dim = lay.dim, np = lay.np, nf = lay.nf, nfp = lay.nfp, K = lay.K;
    (void)nf; (void)nfp;
    dg_ctx *c = new dg_ctx();
    c->dim = dim; c->order = m->order; c->np = np; c->nf = nf; c->nfp = nfp; c->nq = dim + 1; c->K = K;
    c->ndof = (long long)K * np;
    c->nbatch = nbatch;
    c->bstride = c->ndof * c->nq;
    c->prec = opts.precision; c->flux_sign = opts.flux_sign; c->device = opts.device; c->use_graph = opts.use_graph;
    c->rsize = c->prec == DG_PREC_FP64 ? 8 : 4;
    c->c0 = ph->c0; c->rho0 = ph->rho0;
    for (int k = 0; k < 3; ++k) c->v0[k] = ph->v0[k];
    // both tensor-core forms keep the state as an FP32 pair and share the
    // mixed form's kernels and buffers; they differ in the contraction
    c->mixed = c->prec == DG_PREC_MIXED || c->prec == DG_PREC_TF32X3;
    c->naff = lay.curved.C > 0 ? (int)lay.curved.affine.size() : K;

    // the mixed form keeps FP32 stage data and uses the FP32 helper kernels
    if (!dgk::get_kernels(c->mixed ? DG_PREC_FP32 : c->prec, dim, m->order, &c->ks)) {
        free_ctx(c);
        return fail(DG_ERR_UNSUPPORTED, "no kernel compiled for this order");
    }
    if (opts.tc_pipelines < 0 || opts.tc_pipelines > 2) {
        free_ctx(c);
        return fail(DG_ERR_ARG, "tc_pipelines must be 0, 1 or 2");
    }
    if (c->mixed && !dgk::get_mixed_kernels(dim, m->order, lay.curved.C > 0, c->prec == DG_PREC_TF32X3 ? 1 : 0,
                                            opts.tc_pipelines, &c->mks)) {
        free_ctx(c);
        return fail(DG_ERR_UNSUPPORTED, "the tensor-core forms support orders 1-4 in 3D and 1-5 in 2D");
    }
    int rc = DG_OK;
    auto fin = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess && rc == DG_OK) rc = cuda_fail(e, what);
        return e == cudaSuccess;
    };
    do {
        if (!fin(cudaSetDevice(c->device), "cudaSetDevice")) break;
        if (!fin(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate")) break;
        size_t field_bytes = (size_t)c->ndof * c->rsize;
        size_t state_bytes = field_bytes * c->nq * c->nbatch;  // every member
        if (!fin(cudaMalloc(&c->d_state, 4 * state_bytes), "cudaMalloc(state)")) break;
        c->d_u = c->d_state;
        c->d_acc = c->d_state + state_bytes;
        c->d_wa = c->d_state + 2 * state_bytes;
        c->d_wb = c->d_state + 3 * state_bytes;
        if (!fin(cudaMemsetAsync(c->d_state, 0, 4 * state_bytes, c->stream), "cudaMemset")) break;
        // inverse Jacobians in the stage precision (FP32 contexts round them
        // once here instead of converting them in every stage)
        if (c->prec == DG_PREC_FP64) {
            if (!fin(cudaMalloc(&c->d_geo, lay.geo.size() * 8), "cudaMalloc(geo)")) break;
            if (!fin(cudaMemcpy(c->d_geo, lay.geo.data(), lay.geo.size() * 8, cudaMemcpyHostToDevice), "copy geo"))
                break;
        } else {
            std::vector<float> g32(lay.geo.begin(), lay.geo.end());
            if (!fin(cudaMalloc(&c->d_geo32, std::max<size_t>(g32.size(), 1) * 4), "cudaMalloc(geo32)")) break;
            if (!fin(cudaMemcpy(c->d_geo32, g32.data(), g32.size() * 4, cudaMemcpyHostToDevice), "copy geo32"))
                break;
        }
        auto upload_real = [&](const std::vector<double> &v, void **dst) -> bool {
            if (!fin(cudaMalloc(dst, v.size() * c->rsize), "cudaMalloc")) return false;
            if (c->prec == DG_PREC_FP64)
                return fin(cudaMemcpy(*dst, v.data(), v.size() * 8, cudaMemcpyHostToDevice), "copy");
            std::vector<float> f(v.begin(), v.end());
            return fin(cudaMemcpy(*dst, f.data(), f.size() * 4, cudaMemcpyHostToDevice), "copy");
        };
        if (!upload_real(lay.fgeo, &c->d_fgeo)) break;
        if (!upload_real(lay.ops, &c->d_ops)) break;
        if (!fin(cudaMalloc(&c->d_conn, lay.conn.size() * sizeof(int)), "cudaMalloc(conn)")) break;
        if (!fin(cudaMemcpy(c->d_conn, lay.conn.data(), lay.conn.size() * sizeof(int), cudaMemcpyHostToDevice),
                 "copy conn"))
            break;
        if (!fin(cudaMalloc(&c->d_tabs, lay.tabs.size()), "cudaMalloc(tabs)")) break;
        if (!fin(cudaMemcpy(c->d_tabs, lay.tabs.data(), lay.tabs.size(), cudaMemcpyHostToDevice), "copy tabs"))
            break;
        if (!fin(cudaMalloc(&c->d_t0, 8), "cudaMalloc(t0)")) break;
        if (!fin(cudaMalloc(&c->d_mass, (size_t)np * np * 8), "cudaMalloc(mass)")) break;
        if (!fin(cudaMemcpy(c->d_mass, lay.mass.data(), (size_t)np * np * 8, cudaMemcpyHostToDevice), "copy mass"))
            break;
        if (!fin(cudaMalloc(&c->d_detj, (size_t)K * 8), "cudaMalloc(detj)")) break;
        if (!fin(cudaMemcpy(c->d_detj, lay.detj.data(), (size_t)K * 8, cudaMemcpyHostToDevice), "copy detj"))
            break;
        if (!fin(cudaMalloc(&c->d_mon, 8 * 8), "cudaMalloc(mon)")) break;
        if (!fin(cudaMalloc(&c->d_bad, 8), "cudaMalloc(bad)")) break;
        if (!fin(cudaMalloc(&c->d_step0, 8), "cudaMalloc(step0)")) break;
        if (c->prec != DG_PREC_FP64)
            if (!fin(cudaMalloc(&c->d_stage64, (size_t)c->ndof * 8), "cudaMalloc(staging)")) break;
        for (int s = 0; s < 5; ++s)
            if (!fin(cudaFuncSetAttribute(s < 4 ? c->ks.stage[s] : c->ks.euler,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c->ks.smem),
                     "cudaFuncSetAttribute"))
                break;
        if (rc != DG_OK) break;
        int per_sm = 0, nsm = 0;
        if (!fin(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, c->ks.stage[0], c->ks.threads, c->ks.smem),
                 "occupancy"))
            break;
        if (!fin(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device), "attribute")) break;
        int ntiles = std::max(1, (c->naff + c->ks.epb - 1) / c->ks.epb);
        // resident blocks spread over the members (grid.y = member)
        const int resident = std::max(per_sm, 1) * nsm;
        c->grid = std::max(1, std::min(ntiles, (resident + nbatch - 1) / nbatch));
        if (c->mixed) {
            if (!fin(cudaMalloc(&c->d_ulo, state_bytes), "cudaMalloc(ulo)")) break;
            if (!fin(cudaMemsetAsync(c->d_ulo, 0, state_bytes, c->stream), "cudaMemset")) break;
            std::vector<uint8_t> img;
            std::vector<int> eb;
            c->mks.b_image(lay.ops.data(), img, eb);
            if (!fin(cudaMalloc(&c->d_bimg, img.size()), "cudaMalloc(bimg)")) break;
            if (!fin(cudaMemcpy(c->d_bimg, img.data(), img.size(), cudaMemcpyHostToDevice), "copy bimg")) break;
            if (!fin(cudaMalloc(&c->d_beb, eb.size() * sizeof(int)), "cudaMalloc(beb)")) break;
            if (!fin(cudaMemcpy(c->d_beb, eb.data(), eb.size() * sizeof(int), cudaMemcpyHostToDevice), "copy beb"))
                break;
            if (!fin(cudaMalloc(&c->d_err, sizeof(int)), "cudaMalloc(err)")) break;
            if (!fin(cudaMemset(c->d_err, 0, sizeof(int)), "cudaMemset(err)")) break;
            for (int s = 0; s < 5; ++s)
                if (!fin(cudaFuncSetAttribute(s < 4 ? c->mks.stage[s] : c->mks.euler,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c->mks.smem),
                         "cudaFuncSetAttribute(mixed)"))
                    break;
            if (rc != DG_OK) break;
            // one CTA per SM: each owns the SM's tensor memory and runs
            // mks.pipes tile pipelines
            long long mtiles = (long long)((K + c->mks.elems_per_tile - 1) / c->mks.elems_per_tile) * nbatch;
            if (mtiles >= (1LL << 31)) {
                rc = fail(DG_ERR_UNSUPPORTED, "mesh x batch too large for the mixed form's tile index");
                break;
            }
            const long long ctas = (mtiles + c->mks.pipes - 1) / c->mks.pipes;
            c->grid = (int)std::max(1LL, std::min(ctas, (long long)nsm));
        }
        if (lay.curved.C > 0) {
            const dg::CurvedLayout &cv = lay.curved;
            c->curved = cv.C;
            c->cng = cv.ng;
            c->cngf = cv.ngf;
            if (!dgk::get_curved_kernel(c->prec == DG_PREC_FP64 ? 0 : 1, dim, &c->curved_fn)) {
                rc = fail(DG_ERR_UNSUPPORTED, "no curved-element kernel for this precision");
                break;
            }
            // element data packed per element (inverse mass, metric, face point data), padded to 16 bytes
            const int rs = (int)c->rsize;
            const int nmi = np * np, nwm = cv.ng * dim * dim, nfw = nf * cv.ngf * 4;
            const dgk::CurvedEdata eo = dgk::curved_edata(dim, np, cv.ng, cv.ngf, rs);
            c->cestride = eo.stride;
            c->cmstride = (nf * 2 * nfp + 15) / 16 * 16;
            // elements per CTA group: about one node per thread in the node phases,
            // within 48 KB of shared memory per CTA (4-5 CTAs per SM; 32 KB and
            // 100 KB measured slower)
            c->cepc = std::max(1, std::min(16, 256 / np));
            auto smem_for = [&](int epc) {
                return dgk::curved_smem_bytes(dim, np, cv.ng, cv.ngf, nfp, c->cmstride, epc, rs);
            };
            while (c->cepc > 1 && smem_for(c->cepc) > 48 * 1024) --c->cepc;
            c->curved_smem = smem_for(c->cepc);
            if (c->curved_smem > 227 * 1024) {
                rc = fail(DG_ERR_UNSUPPORTED, "curved element data too large for shared memory at this order");
                break;
            }
            if (!fin(cudaFuncSetAttribute(c->curved_fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)c->curved_smem),
                     "cudaFuncSetAttribute(curved)"))
                break;
            auto up = [&](const void *src, size_t bytes, void **dst) -> bool {
                if (!fin(cudaMalloc(dst, std::max<size_t>(bytes, 16)), "cudaMalloc(curved)")) return false;
                return fin(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice), "copy curved");
            };
            if (!up(cv.el.data(), cv.el.size() * 4, (void **)&c->d_cel)) break;
            if (!up(cv.slot.data(), cv.slot.size() * 4, (void **)&c->d_cslot)) break;
            {
                std::vector<double> ed((size_t)cv.C * c->cestride, 0.0);
                std::vector<uint8_t> mp((size_t)cv.C * c->cmstride, 0);
                for (int k = 0; k < cv.C; ++k) {
                    double *d = &ed[(size_t)k * c->cestride];
                    std::copy_n(&cv.minv[(size_t)k * nmi], nmi, d);
                    std::copy_n(&cv.wm[(size_t)k * nwm], nwm, d + eo.off_wm);
                    std::copy_n(&cv.fw[(size_t)k * nfw], nfw, d + eo.off_fw);
                    std::copy_n(&cv.fmap[(size_t)k * nf * 2 * nfp], nf * 2 * nfp, &mp[(size_t)k * c->cmstride]);
                }
                bool ok;
                if (c->prec == DG_PREC_FP64) {
                    ok = up(ed.data(), ed.size() * 8, &c->d_cedata);
                } else {
                    std::vector<float> f(ed.begin(), ed.end());
                    ok = up(f.data(), f.size() * 4, &c->d_cedata);
                }
                if (!ok) break;
                if (!up(mp.data(), mp.size(), (void **)&c->d_cfmap)) break;
            }
            // reference operators in the context's precision; FP64 copies for the monitors
            auto upr = [&](const std::vector<double> &v, void **dst) -> bool {
                if (c->prec == DG_PREC_FP64) return up(v.data(), v.size() * 8, dst);
                std::vector<float> f(v.begin(), v.end());
                return up(f.data(), f.size() * 4, dst);
            };
            if (!upr(cv.phi, &c->d_cphi)) break;
            if (!upr(cv.dphi, &c->d_cdphi)) break;
            if (!upr(cv.fphi, &c->d_cfphi)) break;
            if (!up(cv.wdet.data(), cv.wdet.size() * 8, (void **)&c->d_cwdet)) break;
            if (!up(cv.phi.data(), cv.phi.size() * 8, (void **)&c->d_cphi64)) break;
            if (!up(cv.affine.data(), cv.affine.size() * 4, (void **)&c->d_aff)) break;
            if (c->mixed) {
                // per element block of the tensor-core kernel: which elements are curved
                const int el = c->mks.elems_per_tile;
                std::vector<unsigned long long> msk((K + el - 1) / el, 0ull);
                for (int e : cv.el) msk[e / el] |= 1ull << (e % el);
                if (!up(msk.data(), msk.size() * 8, (void **)&c->d_cmask)) break;
                // blocks whose elements are all curved are left to the per-point kernel
                std::vector<int> bl;
                for (size_t b = 0; b < msk.size(); ++b) {
                    const int n = std::min(el, K - (int)b * el);
                    const unsigned long long full = n == 64 ? ~0ull : ((1ull << n) - 1ull);
                    if (msk[b] != full) bl.push_back((int)b);
                }
                c->nblk = (int)bl.size();
                if (!up(bl.data(), bl.size() * 4, (void **)&c->d_blist)) break;
                const long long mt = (long long)c->nblk * nbatch;
                c->grid = (int)std::max(1LL, std::min(mt, (long long)nsm));
            }
            if (!up(cv.fconn.data(), cv.fconn.size() * 4, (void **)&c->d_cfconn)) break;
            int cper = 0;
            if (!fin(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&cper, c->curved_fn, 256, c->curved_smem),
                     "occupancy(curved)"))
                break;
            const int cres = std::max(cper, 1) * nsm;
            const int ngroups = (cv.C + c->cepc - 1) / c->cepc;
            c->curved_grid = std::max(1, std::min(ngroups, (cres + nbatch - 1) / nbatch));
        }
        if (!fin(cudaStreamSynchronize(c->stream), "sync")) break;
    } while (0);
    if (rc != DG_OK) {
        free_ctx(c);
        return rc;
    }
    *out = c;
    return DG_OK;
}

int dg_create_batch(const dg_mesh_desc *m, const dg_phys_desc *ph, const dg_opts *opts_in, int nbatch,
                    dg_ctx **out) {
    return dg::guarded([&]() { return dg_create_batch_impl(m, ph, opts_in, nbatch, out); });
}

void dg_destroy(dg_ctx *c) { free_ctx(c); }

}  // extern "C"

namespace {
int set_member(dg_ctx *c, int member, const double *const u[4]) {
    if (!c || !u) return fail(DG_ERR_ARG, "null argument");
    if (member < 0 || member >= c->nbatch) return fail(DG_ERR_ARG, "batch member out of range");
    for (int f = 0; f < c->nq; ++f)
        if (!u[f]) return fail(DG_ERR_ARG, "null field");
    if (c->dim == 2 && u[3]) {
        for (long long i = 0; i < c->ndof; ++i)
            if (u[3][i] != 0.0) return fail(DG_ERR_UNSUPPORTED, "2D meshes carry vz == 0; got a nonzero vz");
    }
    CK(cudaSetDevice(c->device));
    const long long moff = (long long)member * c->bstride;  // values
    for (int f = 0; f < c->nq; ++f) {
        const long long off = moff + f * c->ndof;
        char *dst = (char *)c->d_u + off * c->rsize;
        if (const double *hv = static_cast<const double *>(host_device_view(u[f]))) {
            if (c->prec == DG_PREC_FP64)
                copy_kernel<<<kHostIoBlocks, 256, 0, c->stream>>>(hv, (double *)dst, c->ndof);
            else if (c->mixed)
                split_kernel<<<kHostIoBlocks, 256, 0, c->stream>>>(hv, (float *)dst, c->d_ulo + off, c->ndof);
            else
                cast_kernel<float><<<kHostIoBlocks, 256, 0, c->stream>>>(hv, (float *)dst, c->ndof);
            CK(cudaGetLastError());
            continue;
        }
        if (c->prec == DG_PREC_FP64) {
            CK(cudaMemcpyAsync(dst, u[f], (size_t)c->ndof * 8, cudaMemcpyHostToDevice, c->stream));
        } else {
            CK(cudaMemcpyAsync(c->d_stage64, u[f], (size_t)c->ndof * 8, cudaMemcpyHostToDevice, c->stream));
            if (c->mixed)
                split_kernel<<<1024, 256, 0, c->stream>>>(c->d_stage64, (float *)dst, c->d_ulo + off, c->ndof);
            else
                cast_kernel<float><<<1024, 256, 0, c->stream>>>(c->d_stage64, (float *)dst, c->ndof);
            CK(cudaGetLastError());
        }
    }
    CK(cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int get_member(dg_ctx *c, int member, double *const u[4]) {
    if (!c || !u) return fail(DG_ERR_ARG, "null argument");
    if (member < 0 || member >= c->nbatch) return fail(DG_ERR_ARG, "batch member out of range");
    CK(cudaSetDevice(c->device));
    const long long moff = (long long)member * c->bstride;
    for (int f = 0; f < c->nq; ++f) {
        if (!u[f]) continue;
        const long long off = moff + f * c->ndof;
        const char *src = (const char *)c->d_u + off * c->rsize;
        if (double *hv = static_cast<double *>(const_cast<void *>(host_device_view(u[f])))) {
            if (c->prec == DG_PREC_FP64)
                copy_kernel<<<kHostIoBlocks, 256, 0, c->stream>>>((const double *)src, hv, c->ndof);
            else if (c->mixed)
                join_kernel<<<kHostIoBlocks, 256, 0, c->stream>>>((const float *)src, c->d_ulo + off, hv, c->ndof);
            else
                uncast_kernel<float><<<kHostIoBlocks, 256, 0, c->stream>>>((const float *)src, hv, c->ndof);
            CK(cudaGetLastError());
            continue;
        }
        if (c->prec == DG_PREC_FP64) {
            CK(cudaMemcpyAsync(u[f], src, (size_t)c->ndof * 8, cudaMemcpyDeviceToHost, c->stream));
        } else {
            if (c->mixed)
                join_kernel<<<1024, 256, 0, c->stream>>>((const float *)src, c->d_ulo + off, c->d_stage64, c->ndof);
            else
                uncast_kernel<float><<<1024, 256, 0, c->stream>>>((const float *)src, c->d_stage64, c->ndof);
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(u[f], c->d_stage64, (size_t)c->ndof * 8, cudaMemcpyDeviceToHost, c->stream));
        }
    }
    if (c->dim == 2 && u[3]) std::memset(u[3], 0, (size_t)c->ndof * 8);
    CK(cudaStreamSynchronize(c->stream));
    return DG_OK;
}

// Asynchronous copy-out of member 0: an FP64 snapshot of the state on the
// solver stream (after the work already enqueued there), then its copy to
// `host` on the side stream while the solver stream goes on.
int get_state_async(dg_ctx *c, double *host, long long *ticket) {
    if (!c || !host || !ticket) return fail(DG_ERR_ARG, "null argument");
    CK(cudaSetDevice(c->device));
    if (!c->save_stream) {
        CK(cudaStreamCreateWithFlags(&c->save_stream, cudaStreamNonBlocking));
        for (int k = 0; k < 2; ++k) {
            CK(cudaEventCreateWithFlags(&c->snap_ready[k], cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&c->snap_done[k], cudaEventDisableTiming));
        }
    }
    const int slot = (int)(c->save_next % 2);
    // the slot's previous frame must have left the device buffer
    if (c->save_ticket[slot] >= 0) CK(cudaEventSynchronize(c->snap_done[slot]));
    const size_t bytes = (size_t)4 * c->ndof * 8;
    if (!c->d_snap[slot]) {
        cudaError_t e = cudaMalloc(&c->d_snap[slot], bytes);
        if (e != cudaSuccess) {
            c->d_snap[slot] = nullptr;
            return fail(DG_ERR_CUDA, std::string("cudaMalloc(snapshot): ") + cudaGetErrorString(e));
        }
    }
    double *snap = c->d_snap[slot];
    for (int f = 0; f < c->nq; ++f) {
        const long long off = f * c->ndof;
        const char *src = (const char *)c->d_u + off * c->rsize;
        if (c->prec == DG_PREC_FP64)
            CK(cudaMemcpyAsync(snap + off, src, (size_t)c->ndof * 8, cudaMemcpyDeviceToDevice, c->stream));
        else if (c->mixed)
            join_kernel<<<1024, 256, 0, c->stream>>>((const float *)src, c->d_ulo + off, snap + off, c->ndof);
        else
            uncast_kernel<float><<<1024, 256, 0, c->stream>>>((const float *)src, snap + off, c->ndof);
        CK(cudaGetLastError());
    }
    if (c->nq < 4) CK(cudaMemsetAsync(snap + 3 * c->ndof, 0, (size_t)c->ndof * 8, c->stream));
    CK(cudaEventRecord(c->snap_ready[slot], c->stream));
    CK(cudaStreamWaitEvent(c->save_stream, c->snap_ready[slot], 0));
    CK(cudaMemcpyAsync(host, snap, bytes, cudaMemcpyDeviceToHost, c->save_stream));
    CK(cudaEventRecord(c->snap_done[slot], c->save_stream));
    c->save_ticket[slot] = c->save_next;
    *ticket = c->save_next++;
    return DG_OK;
}

// Starts the host-to-device copy of a whole state (member 0, fields one after
// the other, FP64) into a staging slot on the load stream; dg_commit_state
// makes it the state.
int stage_state(dg_ctx *c, const double *host, long long *ticket) {
    if (!c || !host || !ticket) return fail(DG_ERR_ARG, "null argument");
    CK(cudaSetDevice(c->device));
    if (!c->load_stream) {
        CK(cudaStreamCreateWithFlags(&c->load_stream, cudaStreamNonBlocking));
        for (int k = 0; k < 2; ++k) {
            CK(cudaEventCreateWithFlags(&c->load_done[k], cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&c->load_used[k], cudaEventDisableTiming));
        }
    }
    const int slot = (int)(c->load_next % 2);
    const size_t bytes = (size_t)c->nq * c->ndof * 8;
    if (!c->d_load[slot]) {
        cudaError_t e = cudaMalloc(&c->d_load[slot], bytes);
        if (e != cudaSuccess) {
            c->d_load[slot] = nullptr;
            return fail(DG_ERR_NOMEM, std::string("cudaMalloc(staging): ") + cudaGetErrorString(e));
        }
    }
    // the commit that last read this slot must have run first
    if (c->load_used_set[slot]) CK(cudaStreamWaitEvent(c->load_stream, c->load_used[slot], 0));
    CK(cudaMemcpyAsync(c->d_load[slot], host, bytes, cudaMemcpyHostToDevice, c->load_stream));
    CK(cudaEventRecord(c->load_done[slot], c->load_stream));
    c->load_ticket[slot] = c->load_next;
    *ticket = c->load_next++;
    return DG_OK;
}

// Makes a staged state the state of member 0: on the solver stream, after
// the staged copy and after the work already enqueued there.
int commit_state(dg_ctx *c, long long ticket) {
    if (!c) return fail(DG_ERR_ARG, "null context");
    if (ticket < 0 || ticket >= c->load_next) return fail(DG_ERR_ARG, "unknown ticket");
    const int slot = (int)(ticket % 2);
    if (c->load_ticket[slot] != ticket) return fail(DG_ERR_ARG, "ticket overwritten by a later staged state");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamWaitEvent(c->stream, c->load_done[slot], 0));
    const double *src = c->d_load[slot];
    for (int f = 0; f < c->nq; ++f) {
        const long long off = f * c->ndof;
        char *dst = (char *)c->d_u + off * c->rsize;
        if (c->prec == DG_PREC_FP64)
            CK(cudaMemcpyAsync(dst, src + off, (size_t)c->ndof * 8, cudaMemcpyDeviceToDevice, c->stream));
        else if (c->mixed)
            split_kernel<<<1024, 256, 0, c->stream>>>(src + off, (float *)dst, c->d_ulo + off, c->ndof);
        else
            cast_kernel<float><<<1024, 256, 0, c->stream>>>(src + off, (float *)dst, c->ndof);
        CK(cudaGetLastError());
    }
    CK(cudaEventRecord(c->load_used[slot], c->stream));
    c->load_used_set[slot] = true;
    return DG_OK;
}

int wait_state(dg_ctx *c, long long ticket) {
    if (!c) return fail(DG_ERR_ARG, "null context");
    if (ticket < 0 || ticket >= c->save_next) return fail(DG_ERR_ARG, "unknown ticket");
    CK(cudaSetDevice(c->device));
    const int slot = (int)(ticket % 2);
    // a later ticket on the same slot waited for this one before reusing it
    if (c->save_ticket[slot] == ticket) CK(cudaEventSynchronize(c->snap_done[slot]));
    return DG_OK;
}

// Uploads a source set: entries (member, node, source, weight) grouped by
// state value, sources of a value kept in order.
int upload_sources(dg_ctx *c, int nsrc, const double *params, const std::vector<long long> &at_of_entry,
                   const std::vector<int> &src_of_entry, const std::vector<double> &w_of_entry) {
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    if (c->d_src_at) cudaFree(c->d_src_at);
    for (int *p : {c->d_src_off, c->d_src_list})
        if (p) cudaFree(p);
    for (double *p : {c->d_src_w, c->d_src_params})
        if (p) cudaFree(p);
    c->d_src_at = nullptr;
    c->d_src_off = c->d_src_list = nullptr;
    c->d_src_w = c->d_src_params = nullptr;
    c->src_nodes = 0;
    c->src_duration.clear();
    if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }
    for (int s = 0; s < nsrc; ++s) c->src_duration.push_back(params[s * 4 + 3]);
    std::map<long long, std::vector<size_t>> per_value;  // state offset -> entries in order
    for (size_t k = 0; k < at_of_entry.size(); ++k) per_value[at_of_entry[k]].push_back(k);
    std::vector<long long> at;
    std::vector<int> off(1, 0), lst;
    std::vector<double> w;
    for (auto &kv : per_value) {
        at.push_back(kv.first);
        for (size_t k : kv.second) {
            lst.push_back(src_of_entry[k]);
            w.push_back(w_of_entry[k]);
        }
        off.push_back((int)lst.size());
    }
    c->src_nodes = (int)at.size();
    if (!c->src_nodes) return DG_OK;
    CK(cudaMalloc(&c->d_src_at, at.size() * 8));
    CK(cudaMalloc(&c->d_src_off, off.size() * 4));
    CK(cudaMalloc(&c->d_src_list, lst.size() * 4));
    CK(cudaMalloc(&c->d_src_w, w.size() * 8));
    CK(cudaMalloc(&c->d_src_params, (size_t)nsrc * 4 * 8));
    CK(cudaMemcpy(c->d_src_at, at.data(), at.size() * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->d_src_off, off.data(), off.size() * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->d_src_list, lst.data(), lst.size() * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->d_src_w, w.data(), w.size() * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->d_src_params, params, (size_t)nsrc * 4 * 8, cudaMemcpyHostToDevice));
    return DG_OK;
}
}  // namespace

extern "C" {

int dg_set_state(dg_ctx *c, const double *const u[4]) {
    if (!c) return fail(DG_ERR_ARG, "null argument");
    for (int m = 0; m < c->nbatch; ++m) {
        int rc = set_member(c, m, u);
        if (rc != DG_OK) return rc;
    }
    return DG_OK;
}

int dg_get_state(dg_ctx *c, double *const u[4]) { return get_member(c, 0, u); }

int dg_get_state_async(dg_ctx *c, double *host, long long *ticket) { return get_state_async(c, host, ticket); }

int dg_wait_state(dg_ctx *c, long long ticket) { return wait_state(c, ticket); }
int dg_stage_state(dg_ctx *c, const double *host, long long *ticket) { return stage_state(c, host, ticket); }
int dg_commit_state(dg_ctx *c, long long ticket) { return commit_state(c, ticket); }

int dg_set_state_member(dg_ctx *c, int member, const double *const u[4]) { return set_member(c, member, u); }

int dg_get_state_member(dg_ctx *c, int member, double *const u[4]) { return get_member(c, member, u); }

static int dg_set_sources_impl(dg_ctx *c, int nsrc, const int *offsets, const int *dof_idx, const double *params) {
    if (!c || nsrc < 0 || (nsrc > 0 && (!offsets || !params))) return fail(DG_ERR_ARG, "bad source arguments");
    std::vector<long long> at;
    std::vector<int> src;
    std::vector<double> w;
    for (int m = 0; m < c->nbatch; ++m)
        for (int s = 0; s < nsrc; ++s) {
            if (offsets[s + 1] < offsets[s]) return fail(DG_ERR_ARG, "source offsets must be non-decreasing");
            for (int k = offsets[s]; k < offsets[s + 1]; ++k) {
                const int d = dof_idx[k];
                if (d < 0 || d >= c->ndof) return fail(DG_ERR_ARG, "source node index out of range");
                at.push_back((long long)m * c->bstride + d);
                src.push_back(s);
                w.push_back(1.0);
            }
        }
    return upload_sources(c, nsrc, params, at, src, w);
}

int dg_set_sources(dg_ctx *c, int nsrc, const int *offsets, const int *dof_idx, const double *params) {
    return dg::guarded([&]() { return dg_set_sources_impl(c, nsrc, offsets, dof_idx, params); });
}

static int dg_set_batch_sources_impl(dg_ctx *c, int nsrc, const int *member, const int *offsets, const int *dof_idx,
                         const double *weights, const double *params) {
    if (!c || nsrc < 0 || (nsrc > 0 && (!member || !offsets || !params)))
        return fail(DG_ERR_ARG, "bad source arguments");
    std::vector<long long> at;
    std::vector<int> src;
    std::vector<double> w;
    for (int s = 0; s < nsrc; ++s) {
        if (member[s] < 0 || member[s] >= c->nbatch) return fail(DG_ERR_ARG, "source member out of range");
        if (offsets[s + 1] < offsets[s]) return fail(DG_ERR_ARG, "source offsets must be non-decreasing");
        for (int k = offsets[s]; k < offsets[s + 1]; ++k) {
            const int d = dof_idx[k];
            if (d < 0 || d >= c->ndof) return fail(DG_ERR_ARG, "source node index out of range");
            at.push_back((long long)member[s] * c->bstride + d);
            src.push_back(s);
            w.push_back(weights ? weights[k] : 1.0);
        }
    }
    return upload_sources(c, nsrc, params, at, src, w);
}

int dg_set_batch_sources(dg_ctx *c, int nsrc, const int *member, const int *offsets, const int *dof_idx,
                         const double *weights, const double *params) {
    return dg::guarded([&]() { return dg_set_batch_sources_impl(c, nsrc, member, offsets, dof_idx, weights, params); });
}

int dg_set_receivers(dg_ctx *c, int nrec, const int *dof_idx, int max_steps) {
    if (!c || nrec < 0 || max_steps < 0 || (nrec > 0 && !dof_idx)) return fail(DG_ERR_ARG, "bad receiver arguments");
    for (int r = 0; r < nrec; ++r)
        if (dof_idx[r] < 0 || dof_idx[r] >= c->ndof) return fail(DG_ERR_ARG, "receiver node index out of range");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    if (c->d_rec_dof) cudaFree(c->d_rec_dof);
    if (c->d_trace) cudaFree(c->d_trace);
    c->d_rec_dof = nullptr;
    c->d_trace = nullptr;
    c->rec_n = 0;
    c->rec_max = 0;
    c->rec_done = 0;
    if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }
    if (nrec == 0 || max_steps == 0) return DG_OK;
    const size_t tb = (size_t)nrec * c->nbatch * max_steps * 8;
    CK(cudaMalloc(&c->d_rec_dof, (size_t)nrec * 4));
    CK(cudaMalloc(&c->d_trace, tb));
    CK(cudaMemcpy(c->d_rec_dof, dof_idx, (size_t)nrec * 4, cudaMemcpyHostToDevice));
    CK(cudaMemset(c->d_trace, 0, tb));
    c->rec_n = nrec;
    c->rec_max = max_steps;
    return DG_OK;
}

int dg_get_traces(dg_ctx *c, double *out, int *steps) {
    if (!c || !out) return fail(DG_ERR_ARG, "null argument");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    if (steps) *steps = (int)std::min<long long>(c->rec_done, c->rec_max);
    if (!c->rec_n) return DG_OK;
    CK(cudaMemcpy(out, c->d_trace, (size_t)c->rec_n * c->nbatch * c->rec_max * 8, cudaMemcpyDeviceToHost));
    return DG_OK;
}

}  // extern "C"

namespace {
// Enqueues nsteps steps on the context stream (graph chunks of kGraphChunk).
int enqueue_steps(dg_ctx *c, double *t, double dt, int nsteps, int method = kMethodRK4) {
    int done = 0;
    while (done < nsteps) {
        int m = std::min(kGraphChunk, nsteps - done);
        double t0 = *t;
        // the chunk's source activity decides whether injection is launched
        double tend = t0;
        for (int k = 0; k < m; ++k) tend += dt;
        int with_src = (c->src_nodes && any_source_active(c, t0)) ? 1 : 0;
        CK(cudaMemcpyAsync(c->d_t0, &t0, 8, cudaMemcpyHostToDevice, c->stream));
        if (c->rec_n) {
            // pageable copy of a host value: staged before cudaMemcpyAsync returns
            const long long s0 = c->rec_done;
            CK(cudaMemcpyAsync(c->d_step0, &s0, 8, cudaMemcpyHostToDevice, c->stream));
        }
        if (c->use_graph && m == kGraphChunk) {
            if (!c->gexec || c->graph_dt != dt || c->graph_src != with_src || c->graph_method != method) {
                if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }
                cudaGraph_t g;
                CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
                cudaError_t e = cudaSuccess;
                int saved = c->src_nodes;
                if (!with_src) c->src_nodes = 0;
                for (int k = 0; k < m; ++k) {
                    cudaError_t ek = launch_step(c, k, dt, method);
                    if (e == cudaSuccess) e = ek;
                }
                c->src_nodes = saved;
                cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
                if (e != cudaSuccess) return cuda_fail(e, "launch during capture");
                if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
                e = cudaGraphInstantiate(&c->gexec, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
                c->graph_dt = dt;
                c->graph_src = with_src;
                c->graph_method = method;
            }
            CK(cudaGraphLaunch(c->gexec, c->stream));
        } else {
            int saved = c->src_nodes;
            if (!with_src) c->src_nodes = 0;
            cudaError_t e = cudaSuccess;
            for (int k = 0; k < m; ++k) {
                cudaError_t ek = launch_step(c, k, dt, method);
                if (e == cudaSuccess) e = ek;
            }
            c->src_nodes = saved;
            if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
            if (method == kMethodEuler && (m & 1)) {
                // an odd number of Euler steps leaves the state in the other
                // buffer pair: copy it back so the state pointers stay fixed
                swap_euler_buffers(c);
                const size_t fb = (size_t)c->bstride * c->nbatch * c->rsize;
                CK(cudaMemcpyAsync(c->d_u, c->d_wa, fb, cudaMemcpyDeviceToDevice, c->stream));
                if (c->mixed)
                    CK(cudaMemcpyAsync(c->d_ulo, c->d_acc, (size_t)c->bstride * c->nbatch * 4,
                                       cudaMemcpyDeviceToDevice, c->stream));
            }
        }
        // t0 lives on the host stack: a pageable copy is staged before return
        *t = tend;
        done += m;
        c->rec_done += m;
    }
    return DG_OK;
}
}  // namespace

extern "C" {

}  // extern "C"

namespace {
// Device-side error flag of the mixed kernels (a bounded wait that ran out).
int check_device_error(dg_ctx *c) {
    if (!c->d_err) return DG_OK;
    int h = 0;
    CK(cudaMemcpy(&h, c->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) return fail(DG_ERR_CUDA, "tensor-core stage kernel: an MMA completion wait timed out");
    return DG_OK;
}
}  // namespace

extern "C" {

int dg_euler_steps(dg_ctx *c, double *t, double dt, int nsteps) {
    if (!c || !t || nsteps < 0) return fail(DG_ERR_ARG, "bad step arguments");
    if (!(dt > 0) || !std::isfinite(dt)) return fail(DG_ERR_ARG, "dt must be positive and finite");
    CK(cudaSetDevice(c->device));
    int rc = enqueue_steps(c, t, dt, nsteps, kMethodEuler);
    if (rc != DG_OK) return rc;
    CK(cudaStreamSynchronize(c->stream));
    return check_device_error(c);
}

int dg_rk4_steps(dg_ctx *c, double *t, double dt, int nsteps) {
    if (!c || !t || nsteps < 0) return fail(DG_ERR_ARG, "bad step arguments");
    if (!(dt > 0) || !std::isfinite(dt)) return fail(DG_ERR_ARG, "dt must be positive and finite");
    CK(cudaSetDevice(c->device));
    int rc = enqueue_steps(c, t, dt, nsteps);
    if (rc != DG_OK) return rc;
    CK(cudaStreamSynchronize(c->stream));
    return check_device_error(c);
}

int dg_rk4_steps_timed(dg_ctx *c, double *t, double dt, int nsteps, double *ms) {
    if (!c || !t || !ms || nsteps < 0) return fail(DG_ERR_ARG, "bad step arguments");
    if (!(dt > 0) || !std::isfinite(dt)) return fail(DG_ERR_ARG, "dt must be positive and finite");
    CK(cudaSetDevice(c->device));
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaEventRecord(a, c->stream));
    int rc = enqueue_steps(c, t, dt, nsteps);
    if (rc == DG_OK) {
        CK(cudaEventRecord(b, c->stream));
        CK(cudaEventSynchronize(b));
        float f = 0;
        CK(cudaEventElapsedTime(&f, a, b));
        *ms = f;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc != DG_OK) return rc;
    return check_device_error(c);
}

int dg_profile_steps(dg_ctx *c, double *t, double dt, int nsteps, dg_kernel_times *out) {
    if (!c || !t || !out || nsteps < 0) return fail(DG_ERR_ARG, "bad arguments");
    if (!(dt > 0) || !std::isfinite(dt)) return fail(DG_ERR_ARG, "dt must be positive and finite");
    CK(cudaSetDevice(c->device));
    std::memset(out, 0, sizeof(*out));
    if (nsteps == 0) return DG_OK;
    // a pair of events around every launch
    size_t need = (size_t)nsteps * 9 * 2;
    while (c->events.size() < need) {
        cudaEvent_t ev;
        CK(cudaEventCreate(&ev));
        c->events.push_back(ev);
    }
    std::vector<int> kind;  // 0..3 stage, 4 inject, 5 curved-element stage
    size_t ei = 0;
    double tt = *t;
    for (int k = 0; k < nsteps; ++k) {
        CK(cudaMemcpyAsync(c->d_t0, &tt, 8, cudaMemcpyHostToDevice, c->stream));
        if (c->src_nodes && any_source_active(c, tt)) {
            CK(cudaEventRecord(c->events[ei++], c->stream));
            CK(launch_inject(c, 0, dt));
            CK(cudaEventRecord(c->events[ei++], c->stream));
            kind.push_back(4);
        }
        for (int s = 0; s < 4; ++s) {
            CK(cudaEventRecord(c->events[ei++], c->stream));
            CK(launch_affine_stage(c, s, dt));
            CK(cudaEventRecord(c->events[ei++], c->stream));
            kind.push_back(s);
            if (c->curved) {
                CK(cudaEventRecord(c->events[ei++], c->stream));
                CK(c->prec == DG_PREC_FP64 ? launch_curved<double>(c, s, dt) : launch_curved<float>(c, s, dt));
                CK(cudaEventRecord(c->events[ei++], c->stream));
                kind.push_back(5);
            }
        }
        tt += dt;
    }
    CK(cudaStreamSynchronize(c->stream));
    for (size_t j = 0; j < kind.size(); ++j) {
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, c->events[2 * j], c->events[2 * j + 1]));
        if (kind[j] == 4) { out->inject_ms += ms; out->inject_launches++; }
        else if (kind[j] == 5) { out->curved_ms += ms; out->curved_launches++; }
        else { out->stage_ms[kind[j]] += ms; out->stage_launches[kind[j]]++; }
    }
    float tot = 0;
    CK(cudaEventElapsedTime(&tot, c->events[0], c->events[2 * kind.size() - 1]));
    out->total_ms = tot;
    *t = tt;
    return check_device_error(c);
}

int dg_monitors(dg_ctx *c, double *energy, double *l2, long long *status) {
    if (!c) return fail(DG_ERR_ARG, "null context");
    CK(cudaSetDevice(c->device));
    CK(cudaMemsetAsync(c->d_mon, 0, 8 * 8, c->stream));
    CK(cudaMemsetAsync(c->d_bad, 0, 8, c->stream));
    int blocks = (c->K + 255) / 256;
    if (c->prec == DG_PREC_FP64)
        monitor_kernel<double><<<blocks, 256, 0, c->stream>>>((const double *)c->d_u, nullptr, c->ndof, c->K, c->np,
                                                              c->nq, c->d_mass, c->d_detj, c->rho0, c->c0, c->d_mon,
                                                              c->d_bad, c->d_cslot, c->d_cwdet, c->d_cphi64, c->cng);
    else
        monitor_kernel<float><<<blocks, 256, 0, c->stream>>>((const float *)c->d_u, c->mixed ? c->d_ulo : nullptr,
                                                             c->ndof, c->K, c->np, c->nq, c->d_mass, c->d_detj,
                                                             c->rho0, c->c0, c->d_mon, c->d_bad, c->d_cslot,
                                                             c->d_cwdet, c->d_cphi64, c->cng);
    CK(cudaGetLastError());
    double h[8];
    unsigned long long bad = 0;
    CK(cudaMemcpyAsync(h, c->d_mon, 8 * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&bad, c->d_bad, 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (energy) *energy = h[0];
    if (l2)
        for (int f = 0; f < 4; ++f) l2[f] = f < c->nq ? std::sqrt(std::max(h[1 + f], 0.0)) : 0.0;
    if (status) *status = (long long)bad;
    return bad ? DG_ERR_NONFINITE : DG_OK;
}

int dg_error_vs(dg_ctx *c, int member, dg_ctx *ref, int ref_member, double *rel_l2, long long *status) {
    if (!c || !ref || !rel_l2) return fail(DG_ERR_ARG, "null argument");
    if (member < 0 || member >= c->nbatch || ref_member < 0 || ref_member >= ref->nbatch)
        return fail(DG_ERR_ARG, "member out of range");
    if (c->ndof != ref->ndof || c->nq != ref->nq || c->np != ref->np)
        return fail(DG_ERR_ARG, "the two contexts do not hold states of the same mesh");
    if (c->device != ref->device) return fail(DG_ERR_ARG, "the two contexts live on different devices");
    CK(cudaSetDevice(c->device));
    if (ref != c) CK(cudaStreamSynchronize(ref->stream));
    CK(cudaMemsetAsync(c->d_mon, 0, 8 * 8, c->stream));
    CK(cudaMemsetAsync(c->d_bad, 0, 8, c->stream));
    const long long ou = (long long)member * c->bstride, orf = (long long)ref_member * ref->bstride;
    const char *u = static_cast<const char *>(c->d_u) + ou * (long long)c->rsize;
    const char *r = static_cast<const char *>(ref->d_u) + orf * (long long)ref->rsize;
    const float *ulo = c->mixed ? c->d_ulo + ou : nullptr;
    const float *rlo = ref->mixed ? ref->d_ulo + orf : nullptr;
    const bool u64 = c->prec == DG_PREC_FP64, r64 = ref->prec == DG_PREC_FP64;
    if (u64 && r64) launch_error<double, double>(u, ulo, r, rlo, c->ndof, c->nq, c->d_mon, c->d_bad, c->stream);
    else if (u64) launch_error<double, float>(u, ulo, r, rlo, c->ndof, c->nq, c->d_mon, c->d_bad, c->stream);
    else if (r64) launch_error<float, double>(u, ulo, r, rlo, c->ndof, c->nq, c->d_mon, c->d_bad, c->stream);
    else launch_error<float, float>(u, ulo, r, rlo, c->ndof, c->nq, c->d_mon, c->d_bad, c->stream);
    CK(cudaGetLastError());
    double h[8];
    unsigned long long bad = 0;
    CK(cudaMemcpyAsync(h, c->d_mon, 8 * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&bad, c->d_bad, 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int f = 0; f < 4; ++f) {
        if (f >= c->nq) { rel_l2[f] = 0.0; continue; }
        const double d = std::sqrt(std::max(h[2 * f], 0.0)), n = std::sqrt(std::max(h[2 * f + 1], 0.0));
        rel_l2[f] = n > 0 ? d / n : d;
    }
    if (status) *status = (long long)bad;
    return bad ? DG_ERR_NONFINITE : DG_OK;
}

int dg_synchronize(dg_ctx *c) {
    if (!c) return fail(DG_ERR_ARG, "null context");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int dg_info(dg_ctx *c, long long *dofs, int *fields, long long *state_bytes) {
    if (!c) return fail(DG_ERR_ARG, "null context");
    if (dofs) *dofs = c->ndof;
    if (fields) *fields = c->nq;
    if (state_bytes) *state_bytes = c->bstride * c->nbatch * (long long)c->rsize * 4;
    return DG_OK;
}

int dg_tc_info(dg_ctx *c, int *pipelines, int *tile_elems) {
    if (!c) return fail(DG_ERR_ARG, "null context");
    if (pipelines) *pipelines = c->mixed ? c->mks.pipes : 0;
    if (tile_elems) *tile_elems = c->mixed ? c->mks.elems_per_tile : 0;
    return DG_OK;
}

int dg_curved_info(dg_ctx *c, int *ncurved, int *points, int *face_points) {
    if (!c) return fail(DG_ERR_ARG, "null context");
    if (ncurved) *ncurved = c->curved;
    if (points) *points = c->cng;
    if (face_points) *face_points = c->cngf;
    return DG_OK;
}

void *dg_host_alloc(unsigned long long bytes) {
    void *p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) {
        dg::set_error("cudaMallocHost failed");
        return nullptr;
    }
    return p;
}

void dg_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

}  // extern "C"
