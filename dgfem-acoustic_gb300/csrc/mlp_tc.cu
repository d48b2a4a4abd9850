// BF16 tensor-core inference of the MLP's linear layers (tcgen05).
//
// One CTA of 128 threads computes 128 rows x up to 128 output columns of one
// layer (grid.y splits wider layers): the K dimension goes in chunks of 64
// through two shared-memory
// buffers (X rows and W rows, copied with cp.async in the canonical K-major
// no-swizzle layout of 8-row x 16-byte core matrices), thread 0 issues four
// kind::f16 MMAs (M = 128, N = np, K = 16) per chunk into an FP32 accumulator
// in tensor memory and commits them to the chunk buffer's mbarrier; the next
// chunk is copied while they run.  The epilogue reads the accumulator rows
// (one row per thread), adds the bias, applies GELU and stores BF16 (hidden
// layers) or FP32 (output layer), 16 columns per thread as 16-byte vectors.
// Every wait is bounded; a wait that gives
// up sets the error flag, and the CTA still waits (bounded) for its MMAs
// before it releases tensor memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>

#include "mlp_common.cuh"
#include "tc_ptx.cuh"

namespace dgk {

namespace {

constexpr int kRows = 128;   // rows per CTA (the MMA's M)
constexpr int kChunk = 64;   // K per chunk (four MMAs of K = 16)
constexpr int kStepA = kRows * 32;  // bytes of one K = 16 step of the X tile
constexpr int kMaxCols = 128;       // output columns per CTA
constexpr int kMaxDevices = 64;

// Byte offset of the 16-byte unit (row r, K unit u of 8 values) inside a
// chunk tile of R rows: K step u/2, then 8-row group, K half, row in group.
__device__ __forceinline__ uint32_t unit_off(int r, int u, int R) {
    return (uint32_t)((u >> 1) * R * 32 + (r >> 3) * 256 + (u & 1) * 128 + (r & 7) * 16);
}

__global__ void __launch_bounds__(128) tc_linear_kernel(int M, int N, int np_all, int kp, const __nv_bfloat16 *X,
                                                        const __nv_bfloat16 *Wall, const float *bias, int gelu,
                                                        __nv_bfloat16 *ybf, float *yf32, int ldy, uint32_t tcols,
                                                        int *err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // this CTA's output columns [n0, n0 + np)
    const int n0 = blockIdx.y * kMaxCols;
    const int np = min(kMaxCols, np_all - n0);
    const __nv_bfloat16 *W = Wall + (size_t)n0 * kp;
    const int stepB = np * 32;                      // bytes of one K step of the W tile
    const int bufBytes = kStepA * 4 + stepB * 4;    // one chunk: X tile then W tile
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + 2 * bufBytes);
    uint32_t *sTmem = reinterpret_cast<uint32_t *>(smem + 2 * bufBytes + 16);
    int *sFail = reinterpret_cast<int *>(smem + 2 * bufBytes + 20);
    if (warp == 0) {
        dgtc::tmem_alloc(sTmem, tcols);
        dgtc::tmem_relinquish();
    }
    if (tid == 0) {
        dgtc::mbar_init(&bar[0], 1);
        dgtc::mbar_init(&bar[1], 1);
        dgtc::fence_mbar_init();
        *sFail = 0;
    }
    dgtc::fence_before_sync();
    __syncthreads();
    dgtc::fence_after_sync();
    const uint32_t tbase = *sTmem;
    const int m0 = blockIdx.x * kRows;
    const int nchunks = kp / kChunk;
    const uint32_t idesc = dgtc::idesc_bf16_f32(kRows, np);

    auto issue_copies = [&](int c, int b) {
        unsigned char *sa = smem + b * bufBytes;
        unsigned char *sb = sa + kStepA * 4;
        const int k0 = c * kChunk;
        // X: 128 rows x 8 units; rows past M are zero-filled
        for (int t = tid; t < kRows * 8; t += 128) {
            const int r = t >> 3, u = t & 7;
            const int m = m0 + r;
            const bool ok = m < M;
            const __nv_bfloat16 *src = X + (size_t)(ok ? m : 0) * kp + k0 + u * 8;
            dgtc::cp_async16(sa + unit_off(r, u, kRows), src, ok ? 16u : 0u);
        }
        // W: np rows x 8 units
        for (int t = tid; t < np * 8; t += 128) {
            const int r = t >> 3, u = t & 7;
            dgtc::cp_async16(sb + unit_off(r, u, np), W + (size_t)r * kp + k0 + u * 8, 16u);
        }
        dgtc::cp_async_commit();
    };

    bool ok = true;
    issue_copies(0, 0);
    for (int c = 0; c < nchunks; ++c) {
        const int b = c & 1;
        if (c + 1 < nchunks) {
            // the other buffer was last read by chunk c-1's MMAs
            if (c >= 1 && !dgtc::mbar_wait_bounded(&bar[b ^ 1], ((c - 1) >> 1) & 1, 1u << 30)) {
                ok = false;
                *sFail = 1;
            }
            issue_copies(c + 1, b ^ 1);
            dgtc::cp_async_wait_group<1>();
        } else {
            dgtc::cp_async_wait_all();
        }
        dgtc::fence_proxy_async_smem();
        dgtc::fence_before_sync();
        __syncthreads();
        if (tid == 0 && !*sFail) {
            dgtc::fence_after_sync();
            const uint32_t sa = dgtc::smem_u32(smem + b * bufBytes);
            const uint32_t sb = sa + kStepA * 4;
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const uint64_t ad = dgtc::desc_kmajor(sa + t * kStepA, 128, 256);
                const uint64_t bd = dgtc::desc_kmajor(sb + t * stepB, 128, 256);
                dgtc::mma_bf16_ss(tbase, ad, bd, idesc, (c > 0 || t > 0) ? 1u : 0u);
            }
            dgtc::mma_commit(&bar[b]);
        }
    }
    // the last chunk's MMAs (which complete after all earlier ones)
    const int last = nchunks - 1;
    if (!dgtc::mbar_wait_bounded(&bar[last & 1], (last >> 1) & 1, 1u << 30)) ok = false;
    dgtc::fence_after_sync();
    __syncthreads();
    if (!ok) *sFail = 1;
    __syncthreads();
    if (!*sFail) {
        // epilogue: row m0 + 32*warp + lane, 16 columns at a time; columns
        // N..np-1 (zero weights, no bias) come out as act(0) = 0, which is
        // the next layer's zero K padding
        const int m = m0 + warp * 32 + lane;
        const bool vec32 = (N == np_all) && (ldy % 4 == 0);
        for (int c0 = 0; c0 < np; c0 += 16) {
            uint32_t v[16];
            dgtc::tmem_ld16(dgtc::tmem_lane_addr(tbase, warp, (uint32_t)c0), v);
            dgtc::tmem_ld_wait();
            if (m >= M) continue;
            float x[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int n = n0 + c0 + j;
                x[j] = __uint_as_float(v[j]) + (n < N ? bias[n] : 0.0f);
                if (gelu) x[j] = gelu_f(x[j]);
            }
            if (ybf) {
                // 16 BF16 = two 16-byte stores (ldy and n0 + c0 are multiples of 16)
                uint4 o[2];
                uint32_t *w = reinterpret_cast<uint32_t *>(o);
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const __nv_bfloat162 h = __floats2bfloat162_rn(x[2 * j], x[2 * j + 1]);
                    w[j] = *reinterpret_cast<const uint32_t *>(&h);
                }
                uint4 *dst = reinterpret_cast<uint4 *>(ybf + (size_t)m * ldy + n0 + c0);
                dst[0] = o[0];
                dst[1] = o[1];
            } else if (vec32) {
                float4 *dst = reinterpret_cast<float4 *>(yf32 + (size_t)m * ldy + n0 + c0);
#pragma unroll
                for (int j = 0; j < 4; ++j) dst[j] = make_float4(x[4 * j], x[4 * j + 1], x[4 * j + 2], x[4 * j + 3]);
            } else {
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if (n0 + c0 + j < N) yf32[(size_t)m * ldy + n0 + c0 + j] = x[j];
            }
        }
    } else if (tid == 0) {
        atomicExch(err, 1);
        // MMAs of this CTA may still run: wait once more (bounded)
        dgtc::mbar_wait_bounded(&bar[last & 1], (last >> 1) & 1, 1u << 30);
    }
    dgtc::fence_before_sync();
    __syncthreads();
    dgtc::fence_after_sync();
    if (warp == 0) dgtc::tmem_dealloc(tbase, tcols);
}

}  // namespace

int tc_linear(cudaStream_t s, int M, int N, int np, int kp, const void *X, const void *W, const float *bias, bool gelu,
              void *ybf, float *yf32, int ldy, int *err) {
    if (M < 1 || N < 1 || np < N || np % 16 || np > 256 || kp < kChunk || kp % kChunk) return -1;
    if (ybf && (ldy % 16 || ldy < np)) return -1;
    const int npc = std::min(np, kMaxCols);  // columns of the widest CTA
    uint32_t tcols = 32;
    while ((int)tcols < npc) tcols <<= 1;
    const size_t bufBytes = (size_t)kStepA * 4 + (size_t)npc * 32 * 4;
    const size_t smem = 2 * bufBytes + 32;
    // the shared-memory limit is a per-device attribute of the kernel
    static std::atomic<bool> attr_set[kMaxDevices];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return -2;
    if (!attr_set[dev].load()) {
        if (cudaFuncSetAttribute(tc_linear_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(2 * ((size_t)kStepA * 4 + (size_t)kMaxCols * 32 * 4) + 32)) != cudaSuccess)
            return -2;
        attr_set[dev].store(true);
    }
    const dim3 grid((M + kRows - 1) / kRows, (np + kMaxCols - 1) / kMaxCols);
    tc_linear_kernel<<<grid, 128, smem, s>>>(M, N, np, kp, static_cast<const __nv_bfloat16 *>(X),
                                             static_cast<const __nv_bfloat16 *>(W), bias, gelu ? 1 : 0,
                                             static_cast<__nv_bfloat16 *>(ybf), yf32, ldy, tcols, err);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

}  // namespace dgk
