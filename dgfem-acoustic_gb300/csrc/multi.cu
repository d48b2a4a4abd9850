// Uneven multi-mesh batches: many 3D meshes of different sizes and orders
// stepped together, one persistent launch per RK4 stage for all of them, or
// (configuration kMultiPerOrder) one per order present.
//
// Work is a list of items (mesh, tile of that mesh's elements), sorted by
// order, that the CTAs of a persistent grid take in turn; a CTA loads the
// reference operators of an order into shared memory when the order of its
// items changes (at most once per order for a sorted list).  Each mesh keeps
// its own geometry and connectivity arrays; the states of all meshes live in
// one arena, so that source injection is one kernel for the whole batch.
// Elements per CTA follow from the CTA size (block threads / element
// nodes); dg_multi_autotune times each compiled CTA size on the batch and
// keeps the fastest.  No counterpart in the reference, which runs one mesh
// per process.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/dgcuda.h"
#include "host/capi_common.h"
#include "host/layout.h"
#include "stage_kernel.cuh"

namespace dgk {

// Block sizes the one-launch kernel is compiled for; configuration
// kMultiPerOrder launches one persistent kernel per order present instead,
// each sized for its order (the autotuner's fourth candidate).
constexpr int kMultiBlocks[3] = {128, 256, 512};
constexpr int kMultiPerOrder = 3;
constexpr int kMultiCfgs = 4;

__host__ __device__ constexpr int multi_np(int p) { return (p + 1) * (p + 2) * (p + 3) / 6; }
__host__ __device__ constexpr int multi_epb(int bt, int p) { return bt / multi_np(p) > 0 ? bt / multi_np(p) : 1; }

template <typename Real>
struct MultiMesh {
    StageArgs<Real> st[4];  // arguments of the four stages
    int order;
    int pad;
};

// Copies mesh m's arguments of one stage into shared memory (the CTA's
// threads read them from there for every tile of that mesh instead of
// loading the ~150-byte record from global memory per tile).  Called by the
// whole CTA when its next item belongs to another mesh: the first barrier
// keeps the previous tile's readers, the second publishes the copy.
template <typename Real>
__device__ __forceinline__ void load_mesh_args(const MultiMesh<Real> *meshes, int m, int stage, StageArgs<Real> *dst,
                                               int tid) {
    static_assert(sizeof(StageArgs<Real>) % 8 == 0, "copied as 8-byte words");
    __syncthreads();
    constexpr int W = (int)(sizeof(StageArgs<Real>) / 8);
    if (tid < W)
        reinterpret_cast<unsigned long long *>(dst)[tid] =
            __ldg(reinterpret_cast<const unsigned long long *>(&meshes[m].st[stage - 1]) + tid);
    __syncthreads();
}

// Shared-memory regions (in Real units) chosen by the host from the orders
// present: operators, tile state, face values; tables follow in bytes.
struct MultiSmem {
    int ops, q, fn;
};

template <typename Real, int STAGE, int BT>
__global__ void __launch_bounds__(BT) multi_stage_kernel(const MultiMesh<Real> *meshes, const int2 *items, int nitems,
                                                         const Real *const *ops_by_order,
                                                         const uint8_t *const *tabs_by_order, MultiSmem sm) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Real *sOps = reinterpret_cast<Real *>(smem_raw);
    Real *sQ = sOps + sm.ops;
    Real *sFn = sQ + sm.q;
    uint8_t *sTab = reinterpret_cast<uint8_t *>(sFn + sm.fn);
    __shared__ StageArgs<Real> sArgs;
    const int tid = threadIdx.x;
    int cur = 0, curm = -1;
    int2 wn = blockIdx.x < nitems ? items[blockIdx.x] : make_int2(0, 0);
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const int2 w = wn;
        // the next item's load overlaps this tile
        if (it + (int)gridDim.x < nitems) wn = items[it + gridDim.x];
        const int order = meshes[w.x].order;
        if (order != cur) {
            // every thread has finished the previous item's tile
            __syncthreads();
            const int np = multi_np(order);
            const int nops = 3 * np * np + 4 * ((order + 1) * (order + 2) / 2) * np;
            const int ntab = 4 * ((order + 1) * (order + 2) / 2) + 6 * ((order + 1) * (order + 2) / 2);
            const Real *ops = ops_by_order[order];
            const uint8_t *tabs = tabs_by_order[order];
            for (int k = tid; k < nops; k += BT) sOps[k] = ops[k];
            for (int k = tid; k < ntab; k += BT) sTab[k] = tabs[k];
            __syncthreads();
            cur = order;
        }
        if (w.x != curm) {
            load_mesh_args(meshes, w.x, STAGE, &sArgs, tid);
            curm = w.x;
        }
        const StageArgs<Real> &a = sArgs;
        switch (order) {
            case 1: stage_tile<3, 1, Real, STAGE, multi_epb(BT, 1)>(a, 0, w.y, sQ, sFn, sOps, sTab, tid); break;
            case 2: stage_tile<3, 2, Real, STAGE, multi_epb(BT, 2)>(a, 0, w.y, sQ, sFn, sOps, sTab, tid); break;
            case 3: stage_tile<3, 3, Real, STAGE, multi_epb(BT, 3)>(a, 0, w.y, sQ, sFn, sOps, sTab, tid); break;
            case 4: stage_tile<3, 4, Real, STAGE, multi_epb(BT, 4)>(a, 0, w.y, sQ, sFn, sOps, sTab, tid); break;
            default: stage_tile<3, 5, Real, STAGE, multi_epb(BT, 5)>(a, 0, w.y, sQ, sFn, sOps, sTab, tid); break;
        }
    }
}

// Elements per CTA of the per-order launches: those of the single-mesh
// kernels (about 128-256 threads per CTA).
__host__ __device__ constexpr int order_epb(int p) {
    return multi_np(p) <= 4 ? 32 : multi_np(p) <= 10 ? 16 : multi_np(p) <= 21 ? 8 : 4;
}

// One order's items (a contiguous range of the sorted item list), with its
// operators loaded into shared memory once per CTA.
template <typename Real, int STAGE, int P>
__global__ void __launch_bounds__(order_epb(P) * multi_np(P))
    multi_order_kernel(const MultiMesh<Real> *meshes, const int2 *items, int nitems, const Real *ops,
                       const uint8_t *tabs) {
    using S = Shape<3, P>;
    constexpr int EPB = order_epb(P);
    constexpr int NT = EPB * S::NP;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Real *sOps = reinterpret_cast<Real *>(smem_raw);
    Real *sQ = sOps + S::NOPS_PAD;
    Real *sFn = sQ + EPB * S::NP * 4;
    uint8_t *sTab = reinterpret_cast<uint8_t *>(sFn + EPB * S::NSLOT * 4);
    const int tid = threadIdx.x;
    __shared__ StageArgs<Real> sArgs;
    for (int k = tid; k < S::NOPS; k += NT) sOps[k] = ops[k];
    for (int k = tid; k < S::NTAB; k += NT) sTab[k] = tabs[k];
    __syncthreads();
    int curm = -1;
    int2 wn = blockIdx.x < nitems ? items[blockIdx.x] : make_int2(0, 0);
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const int2 w = wn;
        // the next item's load overlaps this tile
        if (it + (int)gridDim.x < nitems) wn = items[it + gridDim.x];
        if (w.x != curm) {
            load_mesh_args(meshes, w.x, STAGE, &sArgs, tid);
            curm = w.x;
        }
        stage_tile<3, P, Real, STAGE, EPB>(sArgs, 0, w.y, sQ, sFn, sOps, sTab, tid);
    }
}

// Hard sources of a multi-mesh batch: node j is the arena value at[j] of
// mesh node_mesh[j], whose time is t0[mesh] + kstep*dt[mesh] (repeated
// additions, as the reference loop).
template <typename Real>
__global__ void multi_inject_kernel(Real *p, const long long *at, const int *node_mesh, const int *node_src_off,
                                    const int *node_src, const double *node_w, const double *params,
                                    const double *t0, const double *dtm, int kstep, int nnodes) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nnodes) return;
    const int m = node_mesh[j];
    double t = t0[m];
    const double dt = dtm[m];
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
    if (set) p[at[j]] = Real(val);
}

template <typename Real>
struct MultiKernels {
    const void *stage[kMultiCfgs][4];   // one-launch configurations (the per-order slot is unused)
    const void *order[6][4];            // per-order kernels by order and stage
    const void *inject;
};

template <typename Real, int P>
void fill_order(MultiKernels<Real> &k) {
    k.order[P][0] = (const void *)&multi_order_kernel<Real, 1, P>;
    k.order[P][1] = (const void *)&multi_order_kernel<Real, 2, P>;
    k.order[P][2] = (const void *)&multi_order_kernel<Real, 3, P>;
    k.order[P][3] = (const void *)&multi_order_kernel<Real, 4, P>;
}

template <typename Real, int C>
void fill_cfg(MultiKernels<Real> &k) {
    k.stage[C][0] = (const void *)&multi_stage_kernel<Real, 1, kMultiBlocks[C]>;
    k.stage[C][1] = (const void *)&multi_stage_kernel<Real, 2, kMultiBlocks[C]>;
    k.stage[C][2] = (const void *)&multi_stage_kernel<Real, 3, kMultiBlocks[C]>;
    k.stage[C][3] = (const void *)&multi_stage_kernel<Real, 4, kMultiBlocks[C]>;
}

template <typename Real>
MultiKernels<Real> multi_kernels() {
    MultiKernels<Real> k;
    std::memset(&k, 0, sizeof(k));
    fill_cfg<Real, 0>(k);
    fill_cfg<Real, 1>(k);
    fill_cfg<Real, 2>(k);
    fill_order<Real, 1>(k);
    fill_order<Real, 2>(k);
    fill_order<Real, 3>(k);
    fill_order<Real, 4>(k);
    fill_order<Real, 5>(k);
    k.inject = (const void *)&multi_inject_kernel<Real>;
    return k;
}

}  // namespace dgk

struct dg_multi {
    int nmesh = 0, prec = DG_PREC_FP32, device = 0, use_graph = 1;
    size_t rsize = 4;
    cudaStream_t stream = nullptr;
    struct Mesh {
        int order = 0, np = 0, K = 0;
        long long ndof = 0, off = 0;  // values per field; arena offset of field 0
        double c0 = 1, rho0 = 1, v0[3] = {0, 0, 0};
        void *geo = nullptr, *fgeo = nullptr, *conn = nullptr;
    };
    std::vector<Mesh> m;
    long long total = 0;  // arena values (4 fields of every mesh)
    char *d_state = nullptr;  // u, acc, wa, wb arenas
    double *d_stage64 = nullptr;
    void *d_ops[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    uint8_t *d_tabs[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    void *d_ops_tab = nullptr;   // device array of the ops pointers by order
    void *d_tabs_tab = nullptr;  // device array of the table pointers by order
    void *d_meshes = nullptr;    // MultiMesh<Real>[nmesh]
    int2 *d_items[dgk::kMultiCfgs] = {nullptr, nullptr, nullptr, nullptr};
    int nitems[dgk::kMultiCfgs] = {0, 0, 0, 0};
    dgk::MultiSmem sm[dgk::kMultiCfgs];
    size_t smem[dgk::kMultiCfgs] = {0, 0, 0, 0};
    int grid[dgk::kMultiCfgs] = {0, 0, 0, 0};
    // per-order configuration: item range, grid and shared memory of each order
    int ord_start[6] = {0, 0, 0, 0, 0, 0}, ord_n[6] = {0, 0, 0, 0, 0, 0}, ord_grid[6] = {0, 0, 0, 0, 0, 0};
    size_t ord_smem[6] = {0, 0, 0, 0, 0, 0};
    int cfg = 1;
    std::vector<double> cur_dt;  // dt per mesh baked into the device stage arguments
    // sources
    int src_nodes = 0;
    long long *d_src_at = nullptr;
    int *d_src_mesh = nullptr, *d_src_off = nullptr, *d_src_list = nullptr;
    double *d_src_w = nullptr, *d_src_params = nullptr;
    std::vector<double> src_duration;
    std::vector<int> src_mesh;
    double *d_t0 = nullptr, *d_dt = nullptr;
    // graph cache
    cudaGraphExec_t gexec = nullptr;
    int graph_cfg = -1, graph_src = -1;
};

namespace {

using dg::fail;

int cuda_fail(cudaError_t e, const char *what) {
    return fail(DG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(call)                                             \
    do {                                                     \
        cudaError_t _e = (call);                             \
        if (_e != cudaSuccess) return cuda_fail(_e, #call);  \
    } while (0)

const int kChunk = 32;

template <typename Real>
__global__ void m_cast(const double *s, Real *d, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        d[i] = Real(s[i]);
}
template <typename Real>
__global__ void m_uncast(const Real *s, double *d, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        d[i] = double(s[i]);
}

void free_multi(dg_multi *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    std::vector<void *> ptrs = {c->d_state, c->d_stage64, c->d_ops_tab, c->d_tabs_tab, c->d_meshes, c->d_src_at,
                                c->d_src_mesh, c->d_src_off, c->d_src_list, c->d_src_w, c->d_src_params, c->d_t0,
                                c->d_dt};
    for (int o = 0; o < 6; ++o) {
        ptrs.push_back(c->d_ops[o]);
        ptrs.push_back(c->d_tabs[o]);
    }
    for (int k = 0; k < dgk::kMultiCfgs; ++k) ptrs.push_back(c->d_items[k]);
    for (auto &mm : c->m) {
        ptrs.push_back(mm.geo);
        ptrs.push_back(mm.fgeo);
        ptrs.push_back(mm.conn);
    }
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

template <typename Real>
int upload_mesh_args(dg_multi *c, const std::vector<double> &dt) {
    const size_t ab = (size_t)c->total * c->rsize;
    char *u = c->d_state, *acc = c->d_state + ab, *wa = c->d_state + 2 * ab, *wb = c->d_state + 3 * ab;
    std::vector<dgk::MultiMesh<Real>> mm(c->nmesh);
    for (int i = 0; i < c->nmesh; ++i) {
        const auto &g = c->m[i];
        const size_t off = (size_t)g.off * c->rsize;
        for (int s = 0; s < 4; ++s) {
            dgk::StageArgs<Real> &a = mm[i].st[s];
            std::memset(&a, 0, sizeof(a));
            Real *U = (Real *)(u + off), *A = (Real *)(acc + off), *WA = (Real *)(wa + off), *WB = (Real *)(wb + off);
            a.u = U;
            a.acc = A;
            switch (s) {
                case 0: a.win = U; a.wout = WA; break;
                case 1: a.win = WA; a.wout = WB; break;
                case 2: a.win = WB; a.wout = WA; break;
                default: a.win = WA; a.wout = U; break;
            }
            a.fstride = g.ndof;
            a.bstride = 0;
            a.geo = (const Real *)g.geo;
            a.fgeo = (const Real *)g.fgeo;
            a.conn = (const int2 *)g.conn;
            a.ops = (const Real *)c->d_ops[g.order];
            a.tabs = c->d_tabs[g.order];
            a.K = g.K;
            a.dt = Real(dt[i]);
            a.rc2 = Real(g.rho0 * g.c0 * g.c0);
            a.inv_rho = Real(1.0 / g.rho0);
            a.half_c0 = Real(0.5 * g.c0);
            a.c0 = Real(g.c0);
            a.rho = Real(g.rho0);
            for (int k = 0; k < 3; ++k) a.v0[k] = Real(g.v0[k]);
        }
        mm[i].order = g.order;
        mm[i].pad = 0;
    }
    CK(cudaMemcpy(c->d_meshes, mm.data(), mm.size() * sizeof(mm[0]), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->d_dt, dt.data(), dt.size() * 8, cudaMemcpyHostToDevice));
    c->cur_dt = dt;
    return DG_OK;
}

template <typename Real>
cudaError_t launch_multi_stage(dg_multi *c, int stage) {
    static const dgk::MultiKernels<Real> ks = dgk::multi_kernels<Real>();
    const int k = c->cfg;
    if (k == dgk::kMultiPerOrder) {
        // one launch per order, highest first (running the orders on
        // concurrent streams measured slower: the persistent grids compete)
        const dgk::MultiMesh<Real> *meshes = (const dgk::MultiMesh<Real> *)c->d_meshes;
        for (int p = 5; p >= 1; --p) {
            if (!c->ord_n[p]) continue;
            const int2 *items = c->d_items[k] + c->ord_start[p];
            int n = c->ord_n[p];
            const Real *ops = (const Real *)c->d_ops[p];
            const uint8_t *tabs = c->d_tabs[p];
            void *args[] = {&meshes, &items, &n, &ops, &tabs};
            const int threads = dgk::order_epb(p) * dgk::multi_np(p);
            cudaError_t e = cudaLaunchKernel(ks.order[p][stage], dim3(c->ord_grid[p]), dim3(threads), args,
                                             c->ord_smem[p], c->stream);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
    const dgk::MultiMesh<Real> *meshes = (const dgk::MultiMesh<Real> *)c->d_meshes;
    const int2 *items = c->d_items[k];
    int n = c->nitems[k];
    const Real *const *ops = (const Real *const *)c->d_ops_tab;
    const uint8_t *const *tabs = (const uint8_t *const *)c->d_tabs_tab;
    dgk::MultiSmem sm = c->sm[k];
    void *args[] = {&meshes, &items, &n, &ops, &tabs, &sm};
    return cudaLaunchKernel(ks.stage[k][stage], dim3(c->grid[k]), dim3(dgk::kMultiBlocks[k]), args, c->smem[k],
                            c->stream);
}

template <typename Real>
cudaError_t launch_multi_inject(dg_multi *c, int kstep) {
    static const dgk::MultiKernels<Real> ks = dgk::multi_kernels<Real>();
    if (!c->src_nodes) return cudaSuccess;
    void *p = c->d_state;
    int nn = c->src_nodes;
    void *args[] = {&p, &c->d_src_at, &c->d_src_mesh, &c->d_src_off, &c->d_src_list, &c->d_src_w,
                    &c->d_src_params, &c->d_t0, &c->d_dt, &kstep, &nn};
    return cudaLaunchKernel(ks.inject, dim3((nn + 127) / 128), dim3(128), args, 0, c->stream);
}

cudaError_t launch_multi_step(dg_multi *c, int kstep) {
    cudaError_t e = c->prec == DG_PREC_FP64 ? launch_multi_inject<double>(c, kstep) : launch_multi_inject<float>(c, kstep);
    for (int s = 0; s < 4 && e == cudaSuccess; ++s)
        e = c->prec == DG_PREC_FP64 ? launch_multi_stage<double>(c, s) : launch_multi_stage<float>(c, s);
    return e;
}

template <typename Real>
int setup_cfgs(dg_multi *c) {
    static const dgk::MultiKernels<Real> ks = dgk::multi_kernels<Real>();
    bool has[6] = {false, false, false, false, false, false};
    for (auto &g : c->m) has[g.order] = true;
    int nsm = 0;
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device));
    for (int k = 0; k < dgk::kMultiCfgs; ++k) {
        if (k == dgk::kMultiPerOrder) {
            // items grouped by order, tiles of the single-mesh kernels' size
            std::vector<int2> items;
            for (int p = 5; p >= 1; --p) {
                c->ord_start[p] = (int)items.size();
                for (int i = 0; i < c->nmesh; ++i) {
                    if (c->m[i].order != p) continue;
                    const int epb = dgk::order_epb(p);
                    const int nt = (c->m[i].K + epb - 1) / epb;
                    for (int t = 0; t < nt; ++t) items.push_back(make_int2(i, t));
                }
                c->ord_n[p] = (int)items.size() - c->ord_start[p];
                if (!c->ord_n[p]) continue;
                const int np = dgk::multi_np(p), nfp = (p + 1) * (p + 2) / 2, epb = dgk::order_epb(p);
                const int nops_pad = (3 * np * np + 4 * nfp * np + 3) / 4 * 4;
                c->ord_smem[p] = (size_t)(nops_pad + epb * np * 4 + epb * 4 * nfp * 4) * c->rsize +
                                 (4 * nfp + 6 * nfp + 15) / 16 * 16;
                int per_sm = 0;
                for (int s = 0; s < 4; ++s)
                    CK(cudaFuncSetAttribute(ks.order[p][s], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)c->ord_smem[p]));
                CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ks.order[p][0], epb * np, c->ord_smem[p]));
                if (per_sm < 1) return fail(DG_ERR_UNSUPPORTED, "per-order multi-mesh kernel does not fit on an SM");
                c->ord_grid[p] = std::max(1, std::min(c->ord_n[p], per_sm * nsm));
            }
            c->nitems[k] = (int)items.size();
            CK(cudaMalloc(&c->d_items[k], std::max<size_t>(items.size(), 1) * sizeof(int2)));
            CK(cudaMemcpy(c->d_items[k], items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice));
            continue;
        }
        const int bt = dgk::kMultiBlocks[k];
        dgk::MultiSmem sm = {0, 0, 0};
        int tab = 0;
        for (int p = 1; p <= 5; ++p) {
            if (!has[p]) continue;
            const int np = dgk::multi_np(p), nfp = (p + 1) * (p + 2) / 2, epb = dgk::multi_epb(bt, p);
            sm.ops = std::max(sm.ops, (3 * np * np + 4 * nfp * np + 3) / 4 * 4);
            sm.q = std::max(sm.q, epb * np * 4);
            sm.fn = std::max(sm.fn, epb * 4 * nfp * 4);
            tab = std::max(tab, 4 * nfp + 6 * nfp);
        }
        c->sm[k] = sm;
        c->smem[k] = (size_t)(sm.ops + sm.q + sm.fn) * c->rsize + (tab + 15) / 16 * 16;
        // items: (mesh, tile), higher orders first (the heavier tiles are dealt first)
        std::vector<int2> items;
        for (int p = 5; p >= 1; --p)
            for (int i = 0; i < c->nmesh; ++i) {
                if (c->m[i].order != p) continue;
                const int epb = dgk::multi_epb(bt, p);
                const int nt = (c->m[i].K + epb - 1) / epb;
                for (int t = 0; t < nt; ++t) items.push_back(make_int2(i, t));
            }
        c->nitems[k] = (int)items.size();
        CK(cudaMalloc(&c->d_items[k], std::max<size_t>(items.size(), 1) * sizeof(int2)));
        CK(cudaMemcpy(c->d_items[k], items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice));
        int per_sm = 0;
        for (int s = 0; s < 4; ++s)
            CK(cudaFuncSetAttribute(ks.stage[k][s], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c->smem[k]));
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ks.stage[k][0], bt, c->smem[k]));
        if (per_sm < 1) return fail(DG_ERR_UNSUPPORTED, "multi-mesh kernel does not fit on an SM");
        c->grid[k] = std::max(1, std::min(c->nitems[k], per_sm * nsm));
    }
    return DG_OK;
}

int enqueue_multi(dg_multi *c, double *t, const double *dt, int nsteps) {
    std::vector<double> dtv(dt, dt + c->nmesh);
    if (dtv != c->cur_dt) {
        int rc = c->prec == DG_PREC_FP64 ? upload_mesh_args<double>(c, dtv) : upload_mesh_args<float>(c, dtv);
        if (rc != DG_OK) return rc;
        if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }
    }
    int done = 0;
    std::vector<double> t0(t, t + c->nmesh);
    while (done < nsteps) {
        const int m = std::min(kChunk, nsteps - done);
        // a source stays in the chunk's launches while its mesh's time is below its duration
        bool active = false;
        for (size_t s = 0; s < c->src_duration.size(); ++s)
            if (t0[c->src_mesh[s]] < c->src_duration[s]) active = true;
        const int with_src = (c->src_nodes && active) ? 1 : 0;
        CK(cudaMemcpyAsync(c->d_t0, t0.data(), t0.size() * 8, cudaMemcpyHostToDevice, c->stream));
        // t0 is reused below: wait for the copy out of pageable memory
        CK(cudaStreamSynchronize(c->stream));
        const int saved = c->src_nodes;
        if (!with_src) c->src_nodes = 0;
        if (c->use_graph && m == kChunk) {
            if (!c->gexec || c->graph_cfg != c->cfg || c->graph_src != with_src) {
                if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }
                cudaGraph_t g;
                CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
                cudaError_t e = cudaSuccess;
                for (int k = 0; k < m; ++k) {
                    cudaError_t ek = launch_multi_step(c, k);
                    if (e == cudaSuccess) e = ek;
                }
                cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
                c->src_nodes = saved;
                if (e != cudaSuccess) return cuda_fail(e, "launch during capture");
                if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
                e = cudaGraphInstantiate(&c->gexec, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
                c->graph_cfg = c->cfg;
                c->graph_src = with_src;
            }
            c->src_nodes = saved;
            CK(cudaGraphLaunch(c->gexec, c->stream));
        } else {
            cudaError_t e = cudaSuccess;
            for (int k = 0; k < m; ++k) {
                cudaError_t ek = launch_multi_step(c, k);
                if (e == cudaSuccess) e = ek;
            }
            c->src_nodes = saved;
            if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
        }
        for (int i = 0; i < c->nmesh; ++i)
            for (int k = 0; k < m; ++k) t0[i] += dtv[i];
        done += m;
    }
    std::copy(t0.begin(), t0.end(), t);
    return DG_OK;
}

}  // namespace

extern "C" {

static int dg_multi_create_impl(int nmesh, const dg_mesh_desc *meshes, const dg_phys_desc *phys, const dg_opts *opts_in,
                    dg_multi **out) {
    if (!out || nmesh < 1 || !meshes || !phys) return fail(DG_ERR_ARG, "null argument or empty batch");
    *out = nullptr;
    dg_opts opts;
    if (opts_in) opts = *opts_in;
    else dg_default_opts(&opts);
    if (opts.precision != DG_PREC_FP64 && opts.precision != DG_PREC_FP32)
        return fail(DG_ERR_UNSUPPORTED, "multi-mesh batches run in FP64 or FP32");
    for (int i = 0; i < nmesh; ++i) {
        if (meshes[i].dim != 3) return fail(DG_ERR_UNSUPPORTED, "multi-mesh batches are 3D");
        if (meshes[i].order < 1 || meshes[i].order > 5) return fail(DG_ERR_UNSUPPORTED, "order must be in 1..5");
        if (!(phys[i].c0 > 0) || !(phys[i].rho0 > 0)) return fail(DG_ERR_ARG, "c0 and rho0 must be positive");
    }
    dg_multi *c = new dg_multi();
    c->nmesh = nmesh;
    c->prec = opts.precision;
    c->device = opts.device;
    c->use_graph = opts.use_graph;
    c->rsize = c->prec == DG_PREC_FP64 ? 8 : 4;
    int rc = DG_OK;
    auto fin = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess && rc == DG_OK) rc = cuda_fail(e, what);
        return e == cudaSuccess;
    };
    auto upload_real = [&](const std::vector<double> &v, void **dst) -> bool {
        if (!fin(cudaMalloc(dst, std::max<size_t>(v.size(), 1) * c->rsize), "cudaMalloc")) return false;
        if (c->prec == DG_PREC_FP64) return fin(cudaMemcpy(*dst, v.data(), v.size() * 8, cudaMemcpyHostToDevice), "copy");
        std::vector<float> f(v.begin(), v.end());
        return fin(cudaMemcpy(*dst, f.data(), f.size() * 4, cudaMemcpyHostToDevice), "copy");
    };
    do {
        if (!fin(cudaSetDevice(c->device), "cudaSetDevice")) break;
        if (!fin(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate")) break;
        long long off = 0;
        long long maxdof = 0;
        for (int i = 0; i < nmesh && rc == DG_OK; ++i) {
            dg::Layout lay;
            std::string err;
            try {
                err = dg::build_layout(meshes[i], opts.flux_sign, lay);
            } catch (std::exception &e) {
                err = e.what();
            }
            if (!err.empty()) {
                rc = fail(DG_ERR_MESH, "mesh " + std::to_string(i) + ": " + err);
                break;
            }
            if (lay.curved.C > 0) {
                rc = fail(DG_ERR_UNSUPPORTED, "mesh " + std::to_string(i) +
                                                  ": curved elements run in single-mesh contexts (dg_create)");
                break;
            }
            dg_multi::Mesh g;
            g.order = meshes[i].order;
            g.np = lay.np;
            g.K = lay.K;
            g.ndof = (long long)lay.K * lay.np;
            g.off = off;
            off += 4 * g.ndof;
            maxdof = std::max(maxdof, g.ndof);
            g.c0 = phys[i].c0;
            g.rho0 = phys[i].rho0;
            for (int k = 0; k < 3; ++k) g.v0[k] = phys[i].v0[k];
            // registered before its uploads, so that a failed upload's
            // buffers are released with the context
            c->m.push_back(g);
            dg_multi::Mesh &gm = c->m.back();
            if (!upload_real(lay.geo, &gm.geo)) break;
            if (!upload_real(lay.fgeo, &gm.fgeo)) break;
            if (!fin(cudaMalloc(&gm.conn, lay.conn.size() * 4), "cudaMalloc(conn)")) break;
            if (!fin(cudaMemcpy(gm.conn, lay.conn.data(), lay.conn.size() * 4, cudaMemcpyHostToDevice), "copy conn"))
                break;
            if (!c->d_ops[g.order]) {
                if (!upload_real(lay.ops, &c->d_ops[g.order])) break;
                if (!fin(cudaMalloc(&c->d_tabs[g.order], lay.tabs.size()), "cudaMalloc(tabs)")) break;
                if (!fin(cudaMemcpy(c->d_tabs[g.order], lay.tabs.data(), lay.tabs.size(), cudaMemcpyHostToDevice),
                         "copy tabs"))
                    break;
            }
        }
        if (rc != DG_OK) break;
        c->total = off;
        const size_t ab = (size_t)c->total * c->rsize;
        if (!fin(cudaMalloc(&c->d_state, 4 * ab), "cudaMalloc(state)")) break;
        if (!fin(cudaMemset(c->d_state, 0, 4 * ab), "cudaMemset")) break;
        if (c->prec != DG_PREC_FP64 && !fin(cudaMalloc(&c->d_stage64, (size_t)maxdof * 8), "cudaMalloc(staging)"))
            break;
        if (!fin(cudaMalloc(&c->d_ops_tab, 6 * sizeof(void *)), "cudaMalloc")) break;
        if (!fin(cudaMemcpy(c->d_ops_tab, c->d_ops, 6 * sizeof(void *), cudaMemcpyHostToDevice), "copy")) break;
        if (!fin(cudaMalloc(&c->d_tabs_tab, 6 * sizeof(void *)), "cudaMalloc")) break;
        if (!fin(cudaMemcpy(c->d_tabs_tab, c->d_tabs, 6 * sizeof(void *), cudaMemcpyHostToDevice), "copy")) break;
        size_t mesh_bytes = c->prec == DG_PREC_FP64 ? sizeof(dgk::MultiMesh<double>) : sizeof(dgk::MultiMesh<float>);
        if (!fin(cudaMalloc(&c->d_meshes, mesh_bytes * nmesh), "cudaMalloc(meshes)")) break;
        if (!fin(cudaMalloc(&c->d_t0, 8 * nmesh), "cudaMalloc(t0)")) break;
        if (!fin(cudaMalloc(&c->d_dt, 8 * nmesh), "cudaMalloc(dt)")) break;
        std::vector<double> dt0(nmesh, 0.0);
        rc = c->prec == DG_PREC_FP64 ? upload_mesh_args<double>(c, dt0) : upload_mesh_args<float>(c, dt0);
        if (rc != DG_OK) break;
        rc = c->prec == DG_PREC_FP64 ? setup_cfgs<double>(c) : setup_cfgs<float>(c);
    } while (0);
    if (rc != DG_OK) {
        free_multi(c);
        return rc;
    }
    *out = c;
    return DG_OK;
}

int dg_multi_create(int nmesh, const dg_mesh_desc *meshes, const dg_phys_desc *phys, const dg_opts *opts_in,
                    dg_multi **out) {
    return dg::guarded([&]() { return dg_multi_create_impl(nmesh, meshes, phys, opts_in, out); });
}

void dg_multi_destroy(dg_multi *c) { free_multi(c); }

int dg_multi_set_state(dg_multi *c, int mesh, const double *const u[4]) {
    if (!c || !u || mesh < 0 || mesh >= c->nmesh) return fail(DG_ERR_ARG, "bad argument");
    CK(cudaSetDevice(c->device));
    const auto &g = c->m[mesh];
    for (int f = 0; f < 4; ++f) {
        if (!u[f]) return fail(DG_ERR_ARG, "null field");
        char *dst = c->d_state + (size_t)(g.off + f * g.ndof) * c->rsize;
        if (c->prec == DG_PREC_FP64) {
            CK(cudaMemcpyAsync(dst, u[f], (size_t)g.ndof * 8, cudaMemcpyHostToDevice, c->stream));
        } else {
            CK(cudaMemcpyAsync(c->d_stage64, u[f], (size_t)g.ndof * 8, cudaMemcpyHostToDevice, c->stream));
            m_cast<float><<<512, 256, 0, c->stream>>>(c->d_stage64, (float *)dst, g.ndof);
            CK(cudaGetLastError());
        }
    }
    CK(cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int dg_multi_get_state(dg_multi *c, int mesh, double *const u[4]) {
    if (!c || !u || mesh < 0 || mesh >= c->nmesh) return fail(DG_ERR_ARG, "bad argument");
    CK(cudaSetDevice(c->device));
    const auto &g = c->m[mesh];
    for (int f = 0; f < 4; ++f) {
        if (!u[f]) continue;
        const char *src = c->d_state + (size_t)(g.off + f * g.ndof) * c->rsize;
        if (c->prec == DG_PREC_FP64) {
            CK(cudaMemcpyAsync(u[f], src, (size_t)g.ndof * 8, cudaMemcpyDeviceToHost, c->stream));
        } else {
            m_uncast<float><<<512, 256, 0, c->stream>>>((const float *)src, c->d_stage64, g.ndof);
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(u[f], c->d_stage64, (size_t)g.ndof * 8, cudaMemcpyDeviceToHost, c->stream));
            CK(cudaStreamSynchronize(c->stream));
        }
    }
    CK(cudaStreamSynchronize(c->stream));
    return DG_OK;
}

static int dg_multi_set_sources_impl(dg_multi *c, int nsrc, const int *mesh, const int *offsets, const int *dof_idx,
                         const double *weights, const double *params) {
    if (!c || nsrc < 0 || (nsrc > 0 && (!mesh || !offsets || !params))) return fail(DG_ERR_ARG, "bad source arguments");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    for (void *p : {(void *)c->d_src_at, (void *)c->d_src_mesh, (void *)c->d_src_off, (void *)c->d_src_list,
                    (void *)c->d_src_w, (void *)c->d_src_params})
        if (p) cudaFree(p);
    c->d_src_at = nullptr;
    c->d_src_mesh = c->d_src_off = c->d_src_list = nullptr;
    c->d_src_w = c->d_src_params = nullptr;
    c->src_nodes = 0;
    c->src_duration.clear();
    c->src_mesh.clear();
    if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }
    std::map<long long, std::vector<std::pair<int, double>>> per_value;
    std::map<long long, int> mesh_of;
    for (int s = 0; s < nsrc; ++s) {
        if (mesh[s] < 0 || mesh[s] >= c->nmesh) return fail(DG_ERR_ARG, "source mesh out of range");
        if (offsets[s + 1] < offsets[s]) return fail(DG_ERR_ARG, "source offsets must be non-decreasing");
        const auto &g = c->m[mesh[s]];
        for (int k = offsets[s]; k < offsets[s + 1]; ++k) {
            if (dof_idx[k] < 0 || dof_idx[k] >= g.ndof) return fail(DG_ERR_ARG, "source node index out of range");
            const long long at = g.off + dof_idx[k];
            per_value[at].push_back({s, weights ? weights[k] : 1.0});
            mesh_of[at] = mesh[s];
        }
        c->src_duration.push_back(params[4 * s + 3]);
        c->src_mesh.push_back(mesh[s]);
    }
    std::vector<long long> at;
    std::vector<int> nm, off(1, 0), lst;
    std::vector<double> w;
    for (auto &kv : per_value) {
        at.push_back(kv.first);
        nm.push_back(mesh_of[kv.first]);
        for (auto &e : kv.second) {
            lst.push_back(e.first);
            w.push_back(e.second);
        }
        off.push_back((int)lst.size());
    }
    c->src_nodes = (int)at.size();
    if (!c->src_nodes) return DG_OK;
    CK(cudaMalloc(&c->d_src_at, at.size() * 8));
    CK(cudaMalloc(&c->d_src_mesh, nm.size() * 4));
    CK(cudaMalloc(&c->d_src_off, off.size() * 4));
    CK(cudaMalloc(&c->d_src_list, lst.size() * 4));
    CK(cudaMalloc(&c->d_src_w, w.size() * 8));
    CK(cudaMalloc(&c->d_src_params, (size_t)nsrc * 32));
    CK(cudaMemcpy(c->d_src_at, at.data(), at.size() * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->d_src_mesh, nm.data(), nm.size() * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->d_src_off, off.data(), off.size() * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->d_src_list, lst.data(), lst.size() * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->d_src_w, w.data(), w.size() * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->d_src_params, params, (size_t)nsrc * 32, cudaMemcpyHostToDevice));
    return DG_OK;
}

int dg_multi_set_sources(dg_multi *c, int nsrc, const int *mesh, const int *offsets, const int *dof_idx,
                         const double *weights, const double *params) {
    return dg::guarded([&]() { return dg_multi_set_sources_impl(c, nsrc, mesh, offsets, dof_idx, weights, params); });
}

int dg_multi_rk4_steps(dg_multi *c, double *t, const double *dt, int nsteps) {
    if (!c || !t || !dt || nsteps < 0) return fail(DG_ERR_ARG, "bad step arguments");
    for (int i = 0; i < c->nmesh; ++i)
        if (!(dt[i] > 0) || !std::isfinite(dt[i])) return fail(DG_ERR_ARG, "dt must be positive and finite");
    CK(cudaSetDevice(c->device));
    int rc = enqueue_multi(c, t, dt, nsteps);
    if (rc != DG_OK) return rc;
    CK(cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int dg_multi_rk4_steps_timed(dg_multi *c, double *t, const double *dt, int nsteps, double *ms) {
    if (!c || !ms) return fail(DG_ERR_ARG, "null argument");
    CK(cudaSetDevice(c->device));
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaEventRecord(a, c->stream));
    int rc = enqueue_multi(c, t, dt, nsteps);
    if (rc == DG_OK) {
        CK(cudaEventRecord(b, c->stream));
        CK(cudaEventSynchronize(b));
        float f = 0;
        CK(cudaEventElapsedTime(&f, a, b));
        *ms = f;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return rc;
}

int dg_multi_set_config(dg_multi *c, int cfg) {
    if (!c || cfg < 0 || cfg >= dgk::kMultiCfgs) return fail(DG_ERR_ARG, "unknown tile configuration");
    c->cfg = cfg;
    return DG_OK;
}

int dg_multi_autotune(dg_multi *c, const double *dt, int trial_steps, int *chosen, double *ms_per_step) {
    if (!c || !dt || trial_steps < 1) return fail(DG_ERR_ARG, "bad autotune arguments");
    CK(cudaSetDevice(c->device));
    // time each candidate on a copy of the state, then put the state back
    const size_t ab = (size_t)c->total * c->rsize;
    void *saved = nullptr;
    CK(cudaMalloc(&saved, 4 * ab));
    CK(cudaMemcpyAsync(saved, c->d_state, 4 * ab, cudaMemcpyDeviceToDevice, c->stream));
    int best = c->cfg;
    double best_ms = 1e300;
    int rc = DG_OK;
    for (int k = 0; k < dgk::kMultiCfgs && rc == DG_OK; ++k) {
        c->cfg = k;
        std::vector<double> t(c->nmesh, 0.0);
        double ms = 0;
        rc = dg_multi_rk4_steps_timed(c, t.data(), dt, 1, &ms);  // warm-up
        if (rc == DG_OK) rc = dg_multi_rk4_steps_timed(c, t.data(), dt, trial_steps, &ms);
        if (rc != DG_OK) break;
        if (ms_per_step) ms_per_step[k] = ms / trial_steps;
        if (ms < best_ms) {
            best_ms = ms;
            best = k;
        }
    }
    cudaMemcpyAsync(c->d_state, saved, 4 * ab, cudaMemcpyDeviceToDevice, c->stream);
    cudaStreamSynchronize(c->stream);
    cudaFree(saved);
    if (rc != DG_OK) return rc;
    c->cfg = best;
    if (chosen) *chosen = best;
    return DG_OK;
}

int dg_multi_info(dg_multi *c, long long *dofs_per_field, int *ncfg, int *cfg, int *block_threads) {
    if (!c) return fail(DG_ERR_ARG, "null context");
    if (dofs_per_field) {
        long long s = 0;
        for (auto &g : c->m) s += g.ndof;
        *dofs_per_field = s;
    }
    if (ncfg) *ncfg = dgk::kMultiCfgs;
    if (cfg) *cfg = c->cfg;
    if (block_threads)
        for (int k = 0; k < dgk::kMultiCfgs; ++k) block_threads[k] = k == dgk::kMultiPerOrder ? 0 : dgk::kMultiBlocks[k];
    return DG_OK;
}

}  // extern "C"
