// RK4 steps that allocate no device memory.
//
// dg_rk4_steps_noalloc runs the FP64 fused stage kernels on state and layout
// arrays that the caller owns on the device.  The three RK4 stage buffers
// (accumulator and the two stage inputs) live in one file-scope device array
// of fixed size, so the call makes no cudaMalloc/cudaFree and no allocating
// library call.  The array belongs to the library module: every GPU that
// loads the library holds it until the process exits.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>

#include "../../include/dgcuda.h"
#include "host/capi_common.h"
#include "kernels.h"
#include "stage_kernel.cuh"

namespace {

// Capacity of each of the three stage buffers, in FP64 values (fields times
// element nodes): 1,048,576 values, 24 MiB in total.
constexpr long long kNoAllocMaxValues = 1LL << 20;

static __device__ __align__(256) double g_stage_scratch[3 * kNoAllocMaxValues];

// Device address of the scratch array in the current device's context.  The
// host-side symbol is only a stand-in, never a device address, so the address
// is looked up with cudaGetSymbolAddress, on every call: the lookup is cheap,
// and a context that the application reset (cudaDeviceReset) and recreated
// gets the array's new address instead of a stale one.
int scratch_address(double **out) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_stage_scratch);
    if (e != cudaSuccess)
        return dg::fail(DG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    *out = static_cast<double *>(p);
    return DG_OK;
}

bool aligned(const void *p, uintptr_t n) { return (reinterpret_cast<uintptr_t>(p) % n) == 0; }

}  // namespace

extern "C" int dg_rk4_steps_noalloc(const dg_device_layout *lay, double *u, double *t, double dt, int nsteps,
                                    void *stream) {
    if (!lay || !u || !t || nsteps < 0) return dg::fail(DG_ERR_ARG, "null argument or negative step count");
    if (!(dt > 0)) return dg::fail(DG_ERR_ARG, "dt must be positive");
    if (lay->dim != 2 && lay->dim != 3) return dg::fail(DG_ERR_UNSUPPORTED, "dimension must be 2 or 3");
    if (lay->num_el < 1) return dg::fail(DG_ERR_ARG, "empty mesh");
    if (!lay->geo || !lay->fgeo || !lay->conn || !lay->ops || !lay->tabs)
        return dg::fail(DG_ERR_ARG, "null layout array");
    // the stage kernels read fgeo as 16-byte double2 vectors, conn as 8-byte
    // int2 pairs and geo, ops and u as doubles: a misaligned pointer would
    // fault on the device, so it is refused here, before any launch
    if (!aligned(lay->fgeo, 16)) return dg::fail(DG_ERR_ARG, "fgeo must be 16-byte aligned");
    if (!aligned(lay->conn, 8)) return dg::fail(DG_ERR_ARG, "conn must be 8-byte aligned");
    if (!aligned(lay->geo, 8) || !aligned(lay->ops, 8) || !aligned(u, 8))
        return dg::fail(DG_ERR_ARG, "geo, ops and u must be 8-byte aligned");
    dgk::KernelSet ks;
    if (!dgk::get_kernels(DG_PREC_FP64, lay->dim, lay->order, &ks))
        return dg::fail(DG_ERR_UNSUPPORTED, "order must be in 1..5");
    const int np = lay->dim == 2 ? (lay->order + 1) * (lay->order + 2) / 2
                                 : (lay->order + 1) * (lay->order + 2) * (lay->order + 3) / 6;
    const int nq = lay->dim + 1;
    const long long ndof = (long long)lay->num_el * np;
    if (ndof * nq > kNoAllocMaxValues)
        return dg::fail(DG_ERR_UNSUPPORTED, "state of " + std::to_string(ndof * nq) +
                                                " values exceeds the fixed scratch capacity of " +
                                                std::to_string(kNoAllocMaxValues) + " values per stage buffer");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return dg::fail(DG_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    double *scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc != DG_OK) return rc;
    for (int s = 0; s < 4; ++s) {
        e = cudaFuncSetAttribute(ks.stage[s], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ks.smem);
        if (e != cudaSuccess) return dg::fail(DG_ERR_CUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
    }
    int per_sm = 0, nsm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ks.stage[0], ks.threads, ks.smem);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return dg::fail(DG_ERR_CUDA, std::string("occupancy query: ") + cudaGetErrorString(e));
    const int ntiles = (lay->num_el + ks.epb - 1) / ks.epb;
    const int grid = std::max(1, std::min(ntiles, std::max(per_sm, 1) * nsm));

    dgk::StageArgs<double> a;
    a.fstride = ndof;
    a.bstride = 0;
    a.geo = lay->geo;
    a.fgeo = lay->fgeo;
    a.conn = reinterpret_cast<const int2 *>(lay->conn);
    a.ops = lay->ops;
    a.tabs = lay->tabs;
    a.K = lay->num_el;
    a.dt = dt;
    a.rc2 = lay->rho0 * lay->c0 * lay->c0;
    a.inv_rho = 1.0 / lay->rho0;
    a.half_c0 = 0.5 * lay->c0;
    a.c0 = lay->c0;
    a.rho = lay->rho0;
    for (int k = 0; k < 3; ++k) a.v0[k] = lay->v0[k];
    double *acc = scratch, *wa = scratch + kNoAllocMaxValues, *wb = scratch + 2 * kNoAllocMaxValues;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    for (int step = 0; step < nsteps; ++step) {
        for (int s = 0; s < 4; ++s) {
            a.u = u;
            a.acc = acc;
            switch (s) {
                case 0: a.win = u; a.wout = wa; break;
                case 1: a.win = wa; a.wout = wb; break;
                case 2: a.win = wb; a.wout = wa; break;
                default: a.win = wa; a.wout = u; break;
            }
            void *args[] = {&a};
            e = cudaLaunchKernel(ks.stage[s], dim3(grid), dim3(ks.threads), args, ks.smem, st);
            if (e != cudaSuccess) return dg::fail(DG_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
        }
        *t += dt;
    }
    return DG_OK;
}
