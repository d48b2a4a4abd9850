// The solver context behind the dg_ctx handle of the C ABI, shared by the
// translation units that work on a context's device buffers (the step loop,
// the learned coarse propagator and parareal).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "kernels.h"

struct dg_ctx {
    int dim = 0, order = 0, np = 0, nf = 0, nfp = 0, nq = 0, K = 0;
    long long ndof = 0;  // K * np
    int nbatch = 1;       // independent states (sources) on the mesh
    long long bstride = 0;  // values per batch member: nq * ndof
    int prec = 0, flux_sign = 0, device = 0, use_graph = 1;
    size_t rsize = 8;
    double c0 = 1, rho0 = 1, v0[3] = {0, 0, 0};
    cudaStream_t stream = nullptr;
    char *d_state = nullptr;  // u, acc, wa, wb
    void *d_u = nullptr, *d_acc = nullptr, *d_wa = nullptr, *d_wb = nullptr;
    double *d_geo = nullptr;
    void *d_fgeo = nullptr;
    int2 *d_conn = nullptr;
    void *d_ops = nullptr;
    uint8_t *d_tabs = nullptr;
    double *d_t0 = nullptr;
    double *d_stage64 = nullptr;  // FP64 staging (FP32 contexts)
    double *d_mass = nullptr, *d_detj = nullptr, *d_mon = nullptr;
    unsigned long long *d_bad = nullptr;
    // sources: node j is the field-0 value at d_src_at[j] (member folded in)
    int src_nodes = 0;
    long long *d_src_at = nullptr;
    int *d_src_off = nullptr, *d_src_list = nullptr;
    double *d_src_w = nullptr, *d_src_params = nullptr;
    std::vector<double> src_duration;
    // receivers
    int rec_n = 0, rec_max = 0;
    long long rec_done = 0;  // steps recorded so far
    int *d_rec_dof = nullptr;
    double *d_trace = nullptr;
    long long *d_step0 = nullptr;
    dgk::KernelSet ks;
    int grid = 0;
    // mixed form
    bool mixed = false;
    dgk::MixedKernelSet mks;
    float *d_ulo = nullptr;      // low part of the state pair
    float *d_geo32 = nullptr;    // inverse Jacobians rounded to FP32 (what the kernels use)
    uint8_t *d_bimg = nullptr;   // sliced operator image
    int *d_beb = nullptr;        // operator row exponents
    int *d_err = nullptr;        // device-side error flag (wait timeouts)
    // curved elements (per-point form)
    int curved = 0, cng = 0, cngf = 0;
    const void *curved_fn = nullptr;
    size_t curved_smem = 0;
    int curved_grid = 0;
    int naff = 0;                 // elements the affine kernels run (all when no element is curved)
    int *d_aff = nullptr;         // their ids when some element is curved
    int cepc = 1, cestride = 0, cmstride = 0;  // elements per CTA group, element data / map strides
    int *d_cel = nullptr, *d_cslot = nullptr;
    void *d_cedata = nullptr;                                        // context precision
    void *d_cphi = nullptr, *d_cdphi = nullptr, *d_cfphi = nullptr;
    double *d_cwdet = nullptr, *d_cphi64 = nullptr;                // FP64, for the monitors
    unsigned long long *d_cmask = nullptr;  // mixed form: curved elements per tensor-core tile
    int *d_blist = nullptr;                 // mixed form: element blocks with a straight element
    int nblk = 0;
    int2 *d_cfconn = nullptr;
    uint8_t *d_cfmap = nullptr;
    // graph cache
    cudaGraphExec_t gexec = nullptr;
    double graph_dt = 0;
    int graph_src = -1;
    int graph_method = -1;
    // events for profiling
    std::vector<cudaEvent_t> events;
    // asynchronous copy-out (dg_get_state_async): FP64 snapshots taken on the
    // solver stream into a two-slot ring, device-to-host copies on a side
    // stream; save_ticket[s] = last ticket issued on slot s (-1: none)
    cudaStream_t save_stream = nullptr;
    double *d_snap[2] = {nullptr, nullptr};
    cudaEvent_t snap_ready[2] = {nullptr, nullptr}, snap_done[2] = {nullptr, nullptr};
    long long save_ticket[2] = {-1, -1};
    long long save_next = 0;
    // staged state uploads (dg_stage_state / dg_commit_state): host-to-device
    // copies into a two-slot ring of FP64 device buffers on a side stream;
    // the commit converts a slot into the state on the solver stream.
    // load_ticket[s] = last ticket staged on slot s (-1: none); load_used[s]
    // is recorded by the commit that reads slot s (load_used_set[s])
    cudaStream_t load_stream = nullptr;
    double *d_load[2] = {nullptr, nullptr};
    cudaEvent_t load_done[2] = {nullptr, nullptr}, load_used[2] = {nullptr, nullptr};
    bool load_used_set[2] = {false, false};
    long long load_ticket[2] = {-1, -1};
    long long load_next = 0;
};
