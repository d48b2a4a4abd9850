// Tensor-core GEMM of MLP training (tcgen05 kind::tf32, 3xTF32 split
// products, FP32 accumulation in tensor memory).
//
// C[m][n] = sum_k op(A)[m][k] op(B)[n][k] (+ bias[n]) (+ C[m][n]), and
// optionally gelu_out = GELU(C), the three shapes training needs: the
// forward layer (A = activations, B = weights, both K-contiguous), the
// activation gradient (B = weights read transposed) and the weight gradient
// (A = output gradient transposed, B = activations transposed, K = rows).
// op(A)[m][k] = TA ? A[k*lda + m] : A[m*lda + k], op(B) likewise.
//
// One CTA of 128 threads computes 128 rows x 64 columns.  K goes in chunks
// of 32 (four K-steps of 8): the threads load a chunk of A and B from global
// memory into registers (coalesced along the contiguous dimension, zero past
// M, N, K), split every value x into hi = tf32(x) and lo = tf32(x - hi) and
// store both parts in the canonical no-swizzle K-major layout (8-row x
// 16-byte core matrices) of one of two shared-memory buffers; thread 0 then
// issues, per K-step, a_hi b_hi, a_hi b_lo and a_lo b_hi into one FP32
// accumulator and commits them to the buffer's mbarrier, and the threads
// load the next chunk while the MMAs run.  Shapes with too few tiles for
// the GPU (the weight gradients, whose K is the batch) split K over
// gridDim.z CTAs that add their partial sums atomically.  The epilogue reads
// one accumulator row per thread.
// Every wait is bounded: a wait that gives up sets *err, and the CTA still
// waits (bounded) for its own MMAs before it frees tensor memory.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>

#include "mlp_common.cuh"
#include "tc_ptx.cuh"

namespace dgk {

namespace {

constexpr int kTRows = 128;                 // rows of a CTA's tile (the MMA's M)
constexpr int kTCols = 64;                  // columns of a CTA's tile (the MMA's N)
constexpr int kTChunk = 32;                 // K per chunk (four K-steps of 8)
constexpr int kTStepA = kTRows * 32;        // bytes of one K-step of one A part
constexpr int kTStepB = kTCols * 32;        // bytes of one K-step of one B part
constexpr int kTPartA = 4 * kTStepA;        // bytes of one A part of a chunk
constexpr int kTPartB = 4 * kTStepB;
constexpr int kTBuf = 2 * kTPartA + 2 * kTPartB;  // A hi, A lo, B hi, B lo
constexpr int kTMaxDevices = 64;
// per-thread registers of one chunk: A 128 x 32 and B 64 x 32 values over
// 128 threads, as float4 (operand stored K-contiguous) or scalars (transposed)
constexpr int kVA = kTRows * kTChunk / 4 / 128, kVB = kTCols * kTChunk / 4 / 128;

// Byte offset of element (row r, k) of a chunk part of R rows (k < 32):
// K-step k/8, 8-row group, K half (LBO = 128 B), row in group, k in the
// 16-byte row.
__device__ __forceinline__ uint32_t part_off(int r, int k, int R) {
    return (uint32_t)((k >> 3) * R * 32 + (r >> 3) * 256 + ((k & 7) >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ float4 split_hi(float4 v) {
    return make_float4(dgtc::tf32_round(v.x), dgtc::tf32_round(v.y), dgtc::tf32_round(v.z), dgtc::tf32_round(v.w));
}
__device__ __forceinline__ float4 split_lo(float4 v, float4 h) {
    return make_float4(dgtc::tf32_round(v.x - h.x), dgtc::tf32_round(v.y - h.y), dgtc::tf32_round(v.z - h.z),
                       dgtc::tf32_round(v.w - h.w));
}

// Loads (into registers) an operand's chunk of R rows from row r0, column
// k0: T = false: rows K-contiguous, four consecutive k per float4, eight
// float4 per row; T = true: stored transposed, element (r, k) at k*ld + r,
// four consecutive rows per float4 slot (scalar loads, coalesced along r).
template <bool T, int R, int NV>
__device__ __forceinline__ void fetch(const float *X, int ld, int rows, int K, int r0, int k0, float4 (&v)[NV],
                                      int tid) {
#pragma unroll
    for (int j = 0; j < NV; ++j) {
        const int idx = tid + 128 * j;
        if (!T) {
            const int r = idx >> 3, k = (idx & 7) * 4;
            const int gr = r0 + r, gk = k0 + k;
            float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
            if (gr < rows) {
                const float *src = X + (size_t)gr * ld + gk;
                if (gk + 3 < K && ((reinterpret_cast<uintptr_t>(src) & 15) == 0)) {
                    x = __ldg(reinterpret_cast<const float4 *>(src));
                } else {
                    x.x = gk < K ? __ldg(src) : 0.f;
                    x.y = gk + 1 < K ? __ldg(src + 1) : 0.f;
                    x.z = gk + 2 < K ? __ldg(src + 2) : 0.f;
                    x.w = gk + 3 < K ? __ldg(src + 3) : 0.f;
                }
            }
            v[j] = x;
        } else {
            // slot idx: rows 4*(idx % (R/4)) .. +3 at column idx / (R/4)
            const int q = idx % (R / 4), k = idx / (R / 4);
            const int gk = k0 + k;
            float e[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int gr = r0 + 4 * q + i;
                e[i] = (gr < rows && gk < K) ? __ldg(X + (size_t)gk * ld + gr) : 0.f;
            }
            v[j] = make_float4(e[0], e[1], e[2], e[3]);
        }
    }
}

// Stores the registers of fetch() as hi and lo TF32 parts in the K-major
// layout of a chunk part of R rows.
template <bool T, int R, int NV>
__device__ __forceinline__ void store(const float4 (&v)[NV], unsigned char *hi, unsigned char *lo, int tid) {
#pragma unroll
    for (int j = 0; j < NV; ++j) {
        const int idx = tid + 128 * j;
        const float4 h = split_hi(v[j]), l = split_lo(v[j], h);
        if (!T) {
            const uint32_t off = part_off(idx >> 3, (idx & 7) * 4, R);
            *reinterpret_cast<float4 *>(hi + off) = h;
            *reinterpret_cast<float4 *>(lo + off) = l;
        } else {
            const int q = idx % (R / 4), k = idx / (R / 4);
            const float hh[4] = {h.x, h.y, h.z, h.w}, ll[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const uint32_t off = part_off(4 * q + i, k, R);
                *reinterpret_cast<float *>(hi + off) = hh[i];
                *reinterpret_cast<float *>(lo + off) = ll[i];
            }
        }
    }
}

// One CTA: rows [m0, m0+128) x columns [n0, n0+64) over the chunks
// [c_begin, c_end) of K.  splitk: the partial sum is added atomically into C
// (zeroed by the host unless accumulating), bias by the first split only.
template <bool TA, bool TB>
__global__ void __launch_bounds__(128) tc_gemm_kernel(int M, int N, int K, const float *__restrict__ A, int lda,
                                                      const float *__restrict__ B, int ldb, float *C, int ldc,
                                                      const float *__restrict__ bias, float *gelu_out, int accumulate,
                                                      int chunks_per_split, int *err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + 2 * kTBuf);
    uint32_t *sTmem = reinterpret_cast<uint32_t *>(smem + 2 * kTBuf + 16);
    int *sFail = reinterpret_cast<int *>(smem + 2 * kTBuf + 20);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * kTRows, n0 = blockIdx.x * kTCols;
    const bool splitk = gridDim.z > 1;
    const int nchunk_all = (K + kTChunk - 1) / kTChunk;
    const int c_begin = blockIdx.z * chunks_per_split;
    const int c_end = min(nchunk_all, c_begin + chunks_per_split);
    if (warp == 0) {
        dgtc::tmem_alloc(sTmem, kTCols);
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
    const uint32_t idesc = dgtc::idesc_tf32_f32(kTRows, kTCols);
    float4 va[kVA], vb[kVB];
    if (c_begin < c_end) {
        fetch<TA, kTRows, kVA>(A, lda, M, K, m0, c_begin * kTChunk, va, tid);
        fetch<TB, kTCols, kVB>(B, ldb, N, K, n0, c_begin * kTChunk, vb, tid);
    }
    for (int c = c_begin; c < c_end; ++c) {
        const int i = c - c_begin, b = i & 1;
        // buffer b was last read by the MMAs of local chunk i-2
        if (i >= 2 && !dgtc::mbar_wait_bounded(&bar[b], ((i - 2) >> 1) & 1, 1u << 30)) *sFail = 1;
        unsigned char *buf = smem + b * kTBuf;
        store<TA, kTRows, kVA>(va, buf, buf + kTPartA, tid);
        store<TB, kTCols, kVB>(vb, buf + 2 * kTPartA, buf + 2 * kTPartA + kTPartB, tid);
        dgtc::fence_proxy_async_smem();
        dgtc::fence_before_sync();
        __syncthreads();
        if (tid == 0 && !*sFail) {
            dgtc::fence_after_sync();
            const uint32_t ah = dgtc::smem_u32(buf), al = ah + kTPartA, bh = ah + 2 * kTPartA, bl = bh + kTPartB;
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const uint64_t dah = dgtc::desc_kmajor(ah + t * kTStepA, 128, 256);
                const uint64_t dal = dgtc::desc_kmajor(al + t * kTStepA, 128, 256);
                const uint64_t dbh = dgtc::desc_kmajor(bh + t * kTStepB, 128, 256);
                const uint64_t dbl = dgtc::desc_kmajor(bl + t * kTStepB, 128, 256);
                dgtc::mma_tf32_ss(tbase, dah, dbh, idesc, (i > 0 || t > 0) ? 1u : 0u);
                dgtc::mma_tf32_ss(tbase, dah, dbl, idesc, 1u);
                dgtc::mma_tf32_ss(tbase, dal, dbh, idesc, 1u);
            }
            dgtc::mma_commit(&bar[b]);
        }
        // the next chunk's loads run while these MMAs do
        if (c + 1 < c_end) {
            fetch<TA, kTRows, kVA>(A, lda, M, K, m0, (c + 1) * kTChunk, va, tid);
            fetch<TB, kTCols, kVB>(B, ldb, N, K, n0, (c + 1) * kTChunk, vb, tid);
        }
    }
    const int nloc = c_end - c_begin;
    bool ok = true;
    if (nloc > 0) {
        // the last chunk's MMAs complete after all earlier ones
        const int last = nloc - 1;
        ok = dgtc::mbar_wait_bounded(&bar[last & 1], (last >> 1) & 1, 1u << 30);
    }
    dgtc::fence_after_sync();
    __syncthreads();
    if (!ok) *sFail = 1;
    __syncthreads();
    if (!*sFail && nloc > 0) {
        const int m = m0 + warp * 32 + lane;
        for (int c0 = 0; c0 < kTCols && n0 + c0 < N; c0 += 16) {
            uint32_t v[16];
            dgtc::tmem_ld16(dgtc::tmem_lane_addr(tbase, warp, (uint32_t)c0), v);
            dgtc::tmem_ld_wait();
            if (m >= M) continue;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int n = n0 + c0 + j;
                if (n >= N) break;
                float x = __uint_as_float(v[j]);
                if (bias && blockIdx.z == 0) x += bias[n];
                float *dst = C + (size_t)m * ldc + n;
                if (splitk) {
                    atomicAdd(dst, x);
                } else {
                    if (accumulate) x += *dst;
                    *dst = x;
                    if (gelu_out) gelu_out[(size_t)m * ldc + n] = gelu_f(x);
                }
            }
        }
    } else if (*sFail && tid == 0) {
        atomicExch(err, 1);
        // this CTA's MMAs may still run: wait once more (bounded)
        if (nloc > 0) dgtc::mbar_wait_bounded(&bar[(nloc - 1) & 1], ((nloc - 1) >> 1) & 1, 1u << 30);
    }
    dgtc::fence_before_sync();
    __syncthreads();
    dgtc::fence_after_sync();
    if (warp == 0) dgtc::tmem_dealloc(tbase, kTCols);
}

template <bool TA, bool TB>
int launch(cudaStream_t s, int M, int N, int K, const float *A, int lda, const float *B, int ldb, float *C, int ldc,
           const float *bias, float *gelu_out, int accumulate, int *err) {
    static std::atomic<bool> attr_set[kTMaxDevices];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kTMaxDevices) return -2;
    const int smem = 2 * kTBuf + 32;
    if (!attr_set[dev].load()) {
        if (cudaFuncSetAttribute(tc_gemm_kernel<TA, TB>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
            cudaSuccess)
            return -2;
        attr_set[dev].store(true);
    }
    const int gx = (N + kTCols - 1) / kTCols, gy = (M + kTRows - 1) / kTRows;
    const int nchunks = (K + kTChunk - 1) / kTChunk;
    // too few tiles for the SMs (the weight gradients: K = rows): split K,
    // at least eight chunks per split; GELU outputs need the whole sum
    int splits = 1;
    if (!gelu_out && gx * gy < 152) splits = std::max(1, std::min((2 * 152) / (gx * gy), nchunks / 8));
    const int per = (nchunks + splits - 1) / splits;
    splits = (nchunks + per - 1) / per;
    if (splits > 1 && !accumulate) {
        // the partial sums are added into C: start it at zero
        const cudaError_t e = ldc == N ? cudaMemsetAsync(C, 0, (size_t)M * N * sizeof(float), s)
                                       : cudaMemset2DAsync(C, (size_t)ldc * sizeof(float), 0, (size_t)N * sizeof(float),
                                                           (size_t)M, s);
        if (e != cudaSuccess) return -2;
    }
    tc_gemm_kernel<TA, TB><<<dim3(gx, gy, splits), 128, smem, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, gelu_out,
                                                                    accumulate, per, err);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

}  // namespace

int tc_gemm_tf32x3(cudaStream_t s, bool ta, bool tb, int M, int N, int K, const float *A, int lda, const float *B,
                   int ldb, float *C, int ldc, const float *bias, float *gelu_out, int accumulate, int *err) {
    if (M < 1 || N < 1 || K < 1) return -1;
    if (!ta && !tb) return launch<false, false>(s, M, N, K, A, lda, B, ldb, C, ldc, bias, gelu_out, accumulate, err);
    if (!ta && tb) return launch<false, true>(s, M, N, K, A, lda, B, ldb, C, ldc, bias, gelu_out, accumulate, err);
    if (ta && tb) return launch<true, true>(s, M, N, K, A, lda, B, ldb, C, ldc, bias, gelu_out, accumulate, err);
    return launch<true, false>(s, M, N, K, A, lda, B, ldb, C, ldc, bias, gelu_out, accumulate, err);
}

}  // namespace dgk
