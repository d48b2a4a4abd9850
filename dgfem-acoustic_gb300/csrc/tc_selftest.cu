// Self-test of the tensor-core primitives used by the mixed-precision stage
// kernel: a 128x32x112 BF16 GEMM with A in tensor memory and B in shared
// memory (no-swizzle K-major descriptor), two accumulators, commit/mbarrier
// completion with a bounded wait.  Inputs are small integers, so the FP32
// result is exact and compared bit for bit on the host.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/dgcuda.h"
#include "host/capi_common.h"
#include "tc_ptx.cuh"

namespace {

constexpr int kM = 128, kN = 32, kK = 112, kSteps = kK / 16;

__host__ __device__ inline int a_val(int r, int k) { return ((r * 7 + k * 3) % 17) - 8; }
__host__ __device__ inline int b_val(int n, int k) { return ((n * 5 + k * 11) % 13) - 6; }

// Byte offset of B[n][k] in the no-swizzle K-major layout: per K-step of 16,
// four 8-row groups (SBO = 256 B), two 8-column halves (LBO = 128 B), rows of
// 16 B inside a core matrix.
__host__ __device__ inline uint32_t b_offset(int n, int k) {
    return (uint32_t)((k / 16) * 1024 + (n / 8) * 256 + ((k % 16) / 8) * 128 + (n % 8) * 16 + (k % 8) * 2);
}

// mode 0: the GEMM, result in out.  mode 1: the same MMAs are issued and
// committed, but the kernel first waits, with a 1 ms limit, on a second
// mbarrier that nothing arrives on; the wait runs out, the kernel records
// err bit 1, then drains its own MMAs with the normal bounded wait on the
// commit barrier (err bit 2 if that too ran out) and frees its tensor
// memory before returning -- the error path of the mixed stage kernel.
__global__ void __launch_bounds__(128, 1) tc_selftest_kernel(float *out, int *err, int mode) {
    __shared__ __align__(1024) unsigned char sB[kSteps * 1024];
    __shared__ __align__(8) uint64_t bar;
    __shared__ __align__(8) uint64_t bar_never;
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) {
        dgtc::tmem_alloc(&tbase, 256);
        dgtc::tmem_relinquish();
    }
    if (tid == 0) {
        dgtc::mbar_init(&bar, 1);
        dgtc::mbar_init(&bar_never, 1);
        dgtc::fence_mbar_init();
    }
    for (int idx = tid; idx < kN * kK; idx += blockDim.x) {
        int n = idx / kK, k = idx % kK;
        float v = (float)b_val(n, k);
        uint16_t h = (uint16_t)(__float_as_uint(v) >> 16);
        *reinterpret_cast<uint16_t *>(sB + b_offset(n, k)) = h;
    }
    dgtc::fence_proxy_async_smem();
    dgtc::fence_before_sync();
    __syncthreads();
    dgtc::fence_after_sync();
    const uint32_t base = tbase;
    // A row r = thread's row, K packed two per column, columns [0, 56)
    const int r = tid;
    for (int c0 = 0; c0 < kK / 2; c0 += 8) {
        uint32_t v[8];
        for (int c = 0; c < 8; ++c)
            v[c] = dgtc::pack_bf16((float)a_val(r, 2 * (c0 + c)), (float)a_val(r, 2 * (c0 + c) + 1));
        dgtc::tmem_st8(dgtc::tmem_lane_addr(base, warp, c0), v);
    }
    dgtc::tmem_st_wait();
    dgtc::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
        dgtc::fence_after_sync();
        const uint32_t idesc = dgtc::idesc_bf16_f32(kM, kN);
        const uint32_t sb = dgtc::smem_u32(sB);
        for (int t = 0; t < kSteps; ++t)
            dgtc::mma_bf16_ts(base + 128, base + t * 8, dgtc::desc_kmajor(sb + t * 1024, 128, 256), idesc, t > 0);
        for (int t = 0; t < 3; ++t)
            dgtc::mma_bf16_ts(base + 160, base + t * 8, dgtc::desc_kmajor(sb + t * 1024, 128, 256), idesc, t > 0);
        dgtc::mma_commit(&bar);
    }
    __syncwarp();
    if (mode == 1) {
        const bool got = dgtc::mbar_wait_bounded(&bar_never, 0, 1u << 20, 1000000ull);
        if (!__any_sync(0xffffffffu, got) && tid == 0) atomicOr(err, 1);
        // drain the MMAs in flight before the tensor memory is freed
        const bool drained = __all_sync(0xffffffffu, dgtc::mbar_wait_bounded(&bar, 0, 1u << 22));
        if (!drained && (tid & 31) == 0) atomicOr(err, 2);
        dgtc::fence_before_sync();
        __syncthreads();
        if (warp == 0) dgtc::tmem_dealloc(base, 256);
        return;
    }
    bool ok = dgtc::mbar_wait_bounded(&bar, 0, 1u << 22);
    ok = __all_sync(0xffffffffu, ok);
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
    } else {
        dgtc::fence_after_sync();
        uint32_t d0[16], d1[16], e0[16], e1[16];
        dgtc::tmem_ld16(dgtc::tmem_lane_addr(base, warp, 128), d0);
        dgtc::tmem_ld16(dgtc::tmem_lane_addr(base, warp, 144), d1);
        dgtc::tmem_ld16(dgtc::tmem_lane_addr(base, warp, 160), e0);
        dgtc::tmem_ld16(dgtc::tmem_lane_addr(base, warp, 176), e1);
        dgtc::tmem_ld_wait();
        for (int c = 0; c < 16; ++c) {
            out[r * 64 + c] = __uint_as_float(d0[c]);
            out[r * 64 + 16 + c] = __uint_as_float(d1[c]);
            out[r * 64 + 32 + c] = __uint_as_float(e0[c]);
            out[r * 64 + 48 + c] = __uint_as_float(e1[c]);
        }
    }
    dgtc::fence_before_sync();
    __syncthreads();
    if (warp == 0) dgtc::tmem_dealloc(base, 256);
}

}  // namespace

extern "C" int dg_tc_selftest(int device, double *max_abs_err) {
    if (!max_abs_err) return dg::fail(DG_ERR_ARG, "null argument");
    if (cudaSetDevice(device) != cudaSuccess) return dg::fail(DG_ERR_CUDA, "cudaSetDevice failed");
    float *d_out = nullptr;
    int *d_err = nullptr;
    if (cudaMalloc(&d_out, kM * 64 * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&d_err, sizeof(int)) != cudaSuccess) {
        cudaFree(d_out);
        return dg::fail(DG_ERR_CUDA, "cudaMalloc failed");
    }
    cudaMemset(d_out, 0, kM * 64 * sizeof(float));
    cudaMemset(d_err, 0, sizeof(int));
    tc_selftest_kernel<<<1, 128>>>(d_out, d_err, 0);
    cudaError_t e = cudaDeviceSynchronize();
    std::vector<float> h(kM * 64);
    int herr = 0;
    if (e == cudaSuccess) e = cudaMemcpy(h.data(), d_out, h.size() * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d_out);
    cudaFree(d_err);
    if (e != cudaSuccess) return dg::fail(DG_ERR_CUDA, std::string("tensor-core self-test: ") + cudaGetErrorString(e));
    if (herr) return dg::fail(DG_ERR_CUDA, "tensor-core self-test: MMA completion wait timed out");
    double worst = 0;
    for (int r = 0; r < kM; ++r)
        for (int n = 0; n < kN; ++n) {
            double full = 0, part = 0;
            for (int k = 0; k < kK; ++k) {
                full += (double)a_val(r, k) * b_val(n, k);
                if (k < 48) part += (double)a_val(r, k) * b_val(n, k);
            }
            worst = std::fmax(worst, std::fabs(full - h[r * 64 + n]));
            worst = std::fmax(worst, std::fabs(part - h[r * 64 + 32 + n]));
        }
    *max_abs_err = worst;
    return worst == 0 ? DG_OK : dg::fail(DG_ERR_CUDA, "tensor-core self-test: wrong GEMM result");
}

extern "C" int dg_tc_wait_selftest(int device, int *flags) {
    if (!flags) return dg::fail(DG_ERR_ARG, "null argument");
    if (cudaSetDevice(device) != cudaSuccess) return dg::fail(DG_ERR_CUDA, "cudaSetDevice failed");
    float *d_out = nullptr;
    int *d_err = nullptr;
    if (cudaMalloc(&d_out, kM * 64 * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&d_err, sizeof(int)) != cudaSuccess) {
        cudaFree(d_out);
        return dg::fail(DG_ERR_CUDA, "cudaMalloc failed");
    }
    cudaMemset(d_err, 0, sizeof(int));
    tc_selftest_kernel<<<1, 128>>>(d_out, d_err, 1);
    cudaError_t e = cudaDeviceSynchronize();
    int herr = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d_out);
    cudaFree(d_err);
    if (e != cudaSuccess) return dg::fail(DG_ERR_CUDA, std::string("tensor-core wait self-test: ") + cudaGetErrorString(e));
    *flags = herr;
    return DG_OK;
}

namespace {

// Byte offset of B[n][k] (32-bit elements) in the no-swizzle K-major layout:
// per K-step of 8, four 8-row groups (SBO = 256 B), two 4-column halves
// (LBO = 128 B), rows of 16 B inside a core matrix.
__host__ __device__ inline uint32_t b_offset_tf32(int n, int k) {
    return (uint32_t)((k / 8) * 1024 + (n / 8) * 256 + ((k % 8) / 4) * 128 + (n % 8) * 16 + (k % 4) * 4);
}

// The same 128x32x112 product with kind::tf32 MMAs: A (TF32 values in
// 32-bit tensor-memory columns, one K value per column), B in shared memory,
// 14 K-steps of 8 into one accumulator.  Small integers: exact.
__global__ void __launch_bounds__(128, 1) tc_selftest_tf32_kernel(float *out, int *err) {
    constexpr int kStepsT = kK / 8;
    __shared__ __align__(1024) unsigned char sB[kStepsT * 1024];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) {
        dgtc::tmem_alloc(&tbase, 256);
        dgtc::tmem_relinquish();
    }
    if (tid == 0) {
        dgtc::mbar_init(&bar, 1);
        dgtc::fence_mbar_init();
    }
    for (int idx = tid; idx < kN * kK; idx += blockDim.x) {
        const int n = idx / kK, k = idx % kK;
        *reinterpret_cast<float *>(sB + b_offset_tf32(n, k)) = (float)b_val(n, k);
    }
    dgtc::fence_proxy_async_smem();
    dgtc::fence_before_sync();
    __syncthreads();
    dgtc::fence_after_sync();
    const uint32_t base = tbase;
    const int r = tid;
    for (int c0 = 0; c0 < kK; c0 += 8) {
        uint32_t v[8];
        for (int c = 0; c < 8; ++c) v[c] = __float_as_uint((float)a_val(r, c0 + c));
        dgtc::tmem_st8(dgtc::tmem_lane_addr(base, warp, c0), v);
    }
    dgtc::tmem_st_wait();
    dgtc::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
        dgtc::fence_after_sync();
        const uint32_t idesc = dgtc::idesc_tf32_f32(kM, kN);
        const uint32_t sb = dgtc::smem_u32(sB);
        for (int t = 0; t < kStepsT; ++t)
            dgtc::mma_tf32_ts(base + 128, base + t * 8, dgtc::desc_kmajor(sb + t * 1024, 128, 256), idesc, t > 0);
        dgtc::mma_commit(&bar);
    }
    __syncwarp();
    bool ok = __all_sync(0xffffffffu, dgtc::mbar_wait_bounded(&bar, 0, 1u << 22));
    if (!ok) {
        if ((tid & 31) == 0) atomicOr(err, 1);
    } else {
        dgtc::fence_after_sync();
        uint32_t d0[16], d1[16];
        dgtc::tmem_ld16(dgtc::tmem_lane_addr(base, warp, 128), d0);
        dgtc::tmem_ld16(dgtc::tmem_lane_addr(base, warp, 144), d1);
        dgtc::tmem_ld_wait();
        for (int c = 0; c < 16; ++c) {
            out[r * 32 + c] = __uint_as_float(d0[c]);
            out[r * 32 + 16 + c] = __uint_as_float(d1[c]);
        }
    }
    dgtc::fence_before_sync();
    __syncthreads();
    if (warp == 0) dgtc::tmem_dealloc(base, 256);
}

}  // namespace

extern "C" int dg_tc_selftest_tf32(int device, double *max_abs_err) {
    if (!max_abs_err) return dg::fail(DG_ERR_ARG, "null argument");
    if (cudaSetDevice(device) != cudaSuccess) return dg::fail(DG_ERR_CUDA, "cudaSetDevice failed");
    float *d_out = nullptr;
    int *d_err = nullptr;
    if (cudaMalloc(&d_out, kM * 32 * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&d_err, sizeof(int)) != cudaSuccess) {
        cudaFree(d_out);
        return dg::fail(DG_ERR_CUDA, "cudaMalloc failed");
    }
    cudaMemset(d_out, 0, kM * 32 * sizeof(float));
    cudaMemset(d_err, 0, sizeof(int));
    tc_selftest_tf32_kernel<<<1, 128>>>(d_out, d_err);
    cudaError_t e = cudaDeviceSynchronize();
    std::vector<float> h(kM * 32);
    int herr = 0;
    if (e == cudaSuccess) e = cudaMemcpy(h.data(), d_out, h.size() * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d_out);
    cudaFree(d_err);
    if (e != cudaSuccess) return dg::fail(DG_ERR_CUDA, std::string("TF32 self-test: ") + cudaGetErrorString(e));
    if (herr) return dg::fail(DG_ERR_CUDA, "TF32 self-test: MMA completion wait timed out");
    double worst = 0;
    for (int r = 0; r < kM; ++r)
        for (int n = 0; n < kN; ++n) {
            double full = 0;
            for (int k = 0; k < kK; ++k) full += (double)a_val(r, k) * b_val(n, k);
            worst = std::fmax(worst, std::fabs(full - h[r * 32 + n]));
        }
    *max_abs_err = worst;
    return worst == 0 ? DG_OK : dg::fail(DG_ERR_CUDA, "TF32 self-test: wrong GEMM result");
}
