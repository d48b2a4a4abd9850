// Learned coarse propagator and parareal (no counterpart in the reference).
//
// A small element-local network, an MLP over one element's DOFs, its face
// neighbours' traces at its face nodes, the kinds of its boundary faces and
// its inverse Jacobian, predicts the change of the element's DOFs over
// `coarse_steps` fine RK4 steps.  It is trained on the GPU (hand-written FP32
// GEMM, GELU, MSE and Adam kernels) on pairs taken from FP64 DG trajectories,
// and serves as the coarse propagator G of parareal, whose fine propagator F
// is the plain FP64 DG RK4 run for all time slices at once as one batch
// context (member = slice):
//   U[0] = u0;  U[n+1] = G(U[n])                                   (k = 0)
//   U[n+1] <- G(U_new[n]) + F(U_old[n]) - G(U_old[n])               (k >= 1)
// After k iterations the first k slices are exact, so parareal always ends
// at the DG answer by iteration N; the DG measures its error (the update
// size) and is the fallback (iterations up to N).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "../../include/dgcuda.h"
#include "ctx.h"
#include "mlp_common.cuh"

using dgk::gelu_f;
#include "host/capi_common.h"
#include "host/layout.h"

using dg::fail;

namespace {

int cuda_fail(cudaError_t e, const char *what) {
    return fail(DG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(call)                                             \
    do {                                                     \
        cudaError_t _e = (call);                             \
        if (_e != cudaSuccess) return cuda_fail(_e, #call);  \
    } while (0)

// ---------------------------------------------------------------- kernels

// C[m][n] (+)= sum_k A(m,k) B(k,n) (+ bias[n]); A(m,k) = TA ? A[k*lda+m] :
// A[m*lda+k], B(k,n) = TB ? B[k*ldb+n] : B[n*ldb+k].  64x64 tiles, 16-deep
// K slices in shared memory, 256 threads with 4x4 outputs each.  With
// gelu_out, C receives the pre-activation and gelu_out the GELU of it.
constexpr int GB = 64, GK = 16;

__device__ __forceinline__ float gelu_grad(float x) {
    const float u = 0.7978845608028654f * (x + 0.044715f * x * x * x);
    const float t = tanhf(u);
    return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * 0.7978845608028654f * (1.0f + 3.0f * 0.044715f * x * x);
}

template <bool TA, bool TB>
__global__ void __launch_bounds__(256) gemm_kernel(int M, int N, int K, const float *__restrict__ A, int lda,
                                                   const float *__restrict__ B, int ldb, float *__restrict__ C,
                                                   int ldc, const float *__restrict__ bias, float *gelu_out,
                                                   int accumulate) {
    __shared__ float As[GK][GB + 4];
    __shared__ float Bs[GK][GB + 4];
    const int tid = threadIdx.x;
    const int m0 = blockIdx.y * GB, n0 = blockIdx.x * GB;
    const int tm = (tid / 16) * 4, tn = (tid % 16) * 4;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += GK) {
        for (int idx = tid; idx < GB * GK; idx += 256) {
            int mm, kk;
            if (TA) { kk = idx / GB; mm = idx % GB; } else { mm = idx / GK; kk = idx % GK; }
            const int m = m0 + mm, k = k0 + kk;
            float v = 0.0f;
            if (m < M && k < K) v = TA ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k];
            As[kk][mm] = v;
        }
        for (int idx = tid; idx < GB * GK; idx += 256) {
            int nn, kk;
            if (TB) { kk = idx / GB; nn = idx % GB; } else { nn = idx / GK; kk = idx % GK; }
            const int n = n0 + nn, k = k0 + kk;
            float v = 0.0f;
            if (n < N && k < K) v = TB ? B[(size_t)k * ldb + n] : B[(size_t)n * ldb + k];
            Bs[kk][nn] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][tm + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tn + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + tm + i;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int n = n0 + tn + j;
            if (n >= N) continue;
            float v = acc[i][j];
            if (bias) v += bias[n];
            if (accumulate) v += C[(size_t)m * ldc + n];
            C[(size_t)m * ldc + n] = v;
            if (gelu_out) gelu_out[(size_t)m * ldc + n] = gelu_f(v);
        }
    }
}

__global__ void gelu_backward_kernel(float *dA, const float *Z, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dA[i] *= gelu_grad(Z[i]);
}

// db[n] = sum over rows of dZ[m][n].
__global__ void column_sum_kernel(const float *dZ, int M, int N, float *db) {
    const int n = blockIdx.x;
    float s = 0.0f;
    for (int m = threadIdx.x; m < M; m += blockDim.x) s += dZ[(size_t)m * N + n];
    __shared__ float red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[n] = red[0];
}

// dY = 2 (Y - T) / count and the summed squared error (double).
__global__ void mse_kernel(const float *Y, const float *T, float *dY, long long n, float inv_count, double *loss) {
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float d = Y[i] - T[i];
        dY[i] = 2.0f * d * inv_count;
        s += (double)d * d;
    }
    __shared__ double red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0]);
}

__global__ void adam_kernel(float *p, const float *g, float *m, float *v, long long n, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    }
}

// dst[r][c] *= 1 / colscale[c / group]
__global__ void scale_columns_kernel(float *dst, long long nrows, int width, int group, float i0, float i1, float i2,
                                     float i3) {
    const float is[4] = {i0, i1, i2, i3};
    const long long n = nrows * width;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] *= is[(int)(i % width) / group];
}

// sums[f] += T[r][c]^2 over the columns of field f = c / group
__global__ void column_group_squares_kernel(const float *T, long long nrows, int width, int group, double *sums) {
    double s[4] = {0, 0, 0, 0};
    const long long n = nrows * width;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s[(int)(i % width) / group] += (double)T[i] * T[i];
    for (int f = 0; f < 4; ++f) atomicAdd(&sums[f], s[f]);
}

__global__ void gather_rows_kernel(const float *src, const int *rows, int nrows, int width, float *dst) {
    const long long n = (long long)nrows * width;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long r = i / width, c = i - r * width;
        dst[i] = src[(long long)rows[r] * width + c];
    }
}

// Element features from an FP64 state u[f*ndof + e*np + i] (member layout):
// [own DOFs by field | neighbour traces per face node by field | wall kinds
// (reflecting, absorbing) per face | inverse Jacobian], fields divided by
// their scales, the Jacobian by its scale.  The DOF and trace part is then
// divided by its own largest magnitude, escale[e] (0 for an element at
// rest), so that the network sees every element at unit amplitude and its
// prediction, multiplied back by escale[e], scales with the state as the
// linear DG propagator does.
struct FeatArgs {
    const double *u;
    long long ndof;
    int K, np, nf, nfp, nq, dim, nin;
    const int2 *conn;
    const uint8_t *tabs;  // fmask [nf][nfp], perm [nperm][nfp]
    const double *geo;    // [K][dim*dim]
    float inv_scale[4];
    float inv_geo;
};

// One warp per element (four per block): its DOFs, the neighbours' traces at
// its face nodes, wall kinds and inverse Jacobian, the DOF/trace part
// divided by its largest magnitude (written to escale).
__global__ void __launch_bounds__(128) features_kernel(FeatArgs a, float *X, float *escale) {
    const int lane = threadIdx.x & 31;
    const int e = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (e >= a.K) return;
    float *x = X + (size_t)e * a.nin;
    const uint8_t *fmask = a.tabs, *perm = a.tabs + a.nf * a.nfp;
    const int own = a.nq * a.np, tr = a.nf * a.nfp * a.nq;
    float m = 0.0f;
    for (int t = lane; t < own; t += 32) {
        const int f = t / a.np, i = t - f * a.np;
        const float v = (float)a.u[f * a.ndof + (long long)e * a.np + i] * a.inv_scale[f];
        x[t] = v;
        m = fmaxf(m, fabsf(v));
    }
    for (int t = lane; t < tr; t += 32) {
        const int lf = t / (a.nfp * a.nq), rem = t - lf * a.nfp * a.nq;
        const int k = rem / a.nq, f = rem - k * a.nq;
        const int2 cn = a.conn[(long long)e * a.nf + lf];
        float v = 0.0f;
        if (((cn.y >> 5) & 3) == 0) {
            const int nlf = cn.y & 3, pm = (cn.y >> 2) & 7;
            const int nvi = fmask[nlf * a.nfp + perm[pm * a.nfp + k]];
            v = (float)a.u[f * a.ndof + (long long)cn.x * a.np + nvi] * a.inv_scale[f];
        }
        x[own + t] = v;
        m = fmaxf(m, fabsf(v));
    }
    for (int lf = lane; lf < a.nf; lf += 32) {
        const int kind = (a.conn[(long long)e * a.nf + lf].y >> 5) & 3;
        x[own + tr + 2 * lf] = kind == 1 ? 1.0f : 0.0f;
        x[own + tr + 2 * lf + 1] = kind == 2 ? 1.0f : 0.0f;
    }
    for (int g = lane; g < a.dim * a.dim; g += 32)
        x[own + tr + 2 * a.nf + g] = (float)a.geo[(long long)e * a.dim * a.dim + g] * a.inv_geo;
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    const float inv = m > 0.0f ? 1.0f / m : 0.0f;
    __syncwarp();
    for (int t = lane; t < own + tr; t += 32) x[t] *= inv;
    if (lane == 0) escale[e] = m;
}

// u[f*ndof + e*np + i] = alpha * (u + out_scale[f] * escale[e] * Y[e][f*np + i])
__global__ void apply_increment_kernel(double *u, long long ndof, int K, int np, int nq, const float *Y,
                                       const float *escale, double s0, double s1, double s2, double s3,
                                       const double *alpha_p) {
    const double alpha = *alpha_p;
    if (alpha == 0.0) return;  // a non-finite prediction leaves the state unchanged
    const double sc[4] = {s0, s1, s2, s3};
    const long long n = (long long)K * np * nq;
    const unsigned npq = (unsigned)(np * nq);
    const bool i32 = n < (1LL << 31);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const long long e = i32 ? (long long)((unsigned)t / npq) : t / (np * nq);
        const int r = (int)(t - e * np * nq), f = r / np, i = r - f * np;
        const long long at = f * ndof + e * np + i;
        u[at] = alpha * (u[at] + sc[f] * (double)escale[e] * (double)Y[t]);
    }
}

// Energy products of the state u and the increment d (lumped: element
// Jacobian determinant times the nodal energy density p^2/(rho c^2) +
// rho |v|^2): block b writes its partial <u, d>, <d, d>, <u, u> to
// part[3b..3b+2]; sum_parts adds them in a fixed order, so that a coarse
// application is bit-reproducible (parareal's cancellation G(U) - G(U) needs
// that).
__global__ void energy_products_kernel(const double *u, long long ndof, int K, int np, int nq, const float *Y,
                                       const float *escale, double s0, double s1, double s2, double s3,
                                       const double *detj, double wp, double wv, double *part) {
    const double sc[4] = {s0, s1, s2, s3};
    const long long n = (long long)K * np * nq;
    const unsigned npq = (unsigned)(np * nq);
    const bool i32 = n < (1LL << 31);
    double ud = 0.0, dd = 0.0, uu = 0.0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        // 32-bit division while the index fits
        const long long e = i32 ? (long long)((unsigned)t / npq) : t / (np * nq);
        const int r = (int)(t - e * np * nq), f = r / np, i = r - f * np;
        const double d = sc[f] * (double)escale[e] * (double)Y[t];
        const double w = detj[e] * (f == 0 ? wp : wv);
        const double uv = u[f * ndof + e * np + i];
        ud += w * uv * d;
        dd += w * d * d;
        uu += w * uv * uv;
    }
    // fixed-order reduction: warp shuffles, then the block's warps in order
    for (int o = 16; o > 0; o >>= 1) {
        ud += __shfl_down_sync(0xffffffffu, ud, o);
        dd += __shfl_down_sync(0xffffffffu, dd, o);
        uu += __shfl_down_sync(0xffffffffu, uu, o);
    }
    __shared__ double wsum[3][8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        wsum[0][warp] = ud;
        wsum[1][warp] = dd;
        wsum[2][warp] = uu;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
            a0 += wsum[0][k];
            a1 += wsum[1][k];
            a2 += wsum[2][k];
        }
        part[3 * blockIdx.x] = a0;
        part[3 * blockIdx.x + 1] = a1;
        part[3 * blockIdx.x + 2] = a2;
    }
}

// out[k] = sum over the nparts partial triples (one block, fixed order).
__global__ void sum_parts_kernel(const double *part, int nparts, double *out) {
    __shared__ double r[3][256];
    double a[3] = {0, 0, 0};
    for (int b = threadIdx.x; b < nparts; b += blockDim.x)
        for (int k = 0; k < 3; ++k) a[k] += part[3 * b + k];
    for (int k = 0; k < 3; ++k) r[k][threadIdx.x] = a[k];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int k = 0; k < 3; ++k) r[k][threadIdx.x] += r[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 3; ++k) out[k] = r[k][0];
}

// Step factor of a coarse application from its energy products (prod =
// <u,d>, <d,d>, <u,u>): 1, or sqrt(E(u) / E(u + d)) if u + d has more energy;
// 0 when the prediction is not finite.  Running statistics in stats: sum of
// the factors, their minimum, the number of applications.
__global__ void step_factor_kernel(const double *prod, double *alpha_out, double *stats) {
    const double e_old = prod[2], e_new = prod[2] + 2.0 * prod[0] + prod[1];
    double alpha = 1.0;
    if (e_new > e_old && e_new > 0.0) alpha = sqrt(e_old / e_new);
    stats[0] += alpha;
    stats[1] = fmin(stats[1], alpha);
    stats[2] += 1.0;
    *alpha_out = (isfinite(e_new) && isfinite(alpha)) ? alpha : 0.0;
}

// Training targets: (u1 - u0) per element in output order, divided by the
// output scales and the element's input scale.
__global__ void targets_kernel(const double *u0, const double *u1, long long ndof, int K, int np, int nq,
                               const float *escale, float i0, float i1, float i2, float i3, float *T) {
    const float isc[4] = {i0, i1, i2, i3};
    const long long n = (long long)K * np * nq;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const long long e = t / (np * nq);
        const int r = (int)(t - e * np * nq), f = r / np, i = r - f * np;
        const long long at = f * ndof + e * np + i;
        const double es = escale[e];
        T[t] = es > 0.0 ? (float)((u1[at] - u0[at]) / es) * isc[f] : 0.0f;
    }
}

// dst = a + b - c (FP64, n values)
__global__ void combine_kernel(double *dst, const double *a, const double *b, const double *c, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = a[i] + b[i] - c[i];
}

// out[0] += sum (a - b)^2, out[1] += sum a^2
__global__ void diff_norm_kernel(const double *a, const double *b, long long n, double *out) {
    double s = 0.0, t = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double d = a[i] - b[i];
        s += d * d;
        t += a[i] * a[i];
    }
    __shared__ double r0[256], r1[256];
    r0[threadIdx.x] = s;
    r1[threadIdx.x] = t;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) {
            r0[threadIdx.x] += r0[threadIdx.x + k];
            r1[threadIdx.x] += r1[threadIdx.x + k];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        atomicAdd(&out[0], r0[0]);
        atomicAdd(&out[1], r1[0]);
    }
}

int grid_for(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 4096)); }
// energy products: a fixed grid (fixed reduction order, bit-reproducible)
const int kEnergyBlocks = 512;

}  // namespace

// FP32 -> BF16 (round to nearest even), zero-padded: dst[r][c] for c < kp
// (cols < width copied, the rest 0), r < rows.
// Row-major with 32-bit indices: rows * kp < 2^31 (checked by the caller).
__global__ void to_bf16_kernel(const float *src, int rows, int width, int lds, __nv_bfloat16 *dst, int kp) {
    const unsigned n = (unsigned)rows * (unsigned)kp;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned r = i / (unsigned)kp, c = i - r * (unsigned)kp;
        dst[i] = __float2bfloat16_rn((int)c < width ? src[(size_t)r * lds + c] : 0.0f);
    }
}

// ---------------------------------------------------------------- the MLP

struct dg_mlp {
    int nin = 0, width = 0, nout = 0, layers = 0;  // layers = linear layers
    std::vector<int> din, dout;                    // per layer
    std::vector<long long> woff, boff;             // parameter offsets (floats)
    long long nparam = 0;
    float *d_p = nullptr, *d_g = nullptr, *d_m = nullptr, *d_v = nullptr;
    long long adam_t = 0;
    int cap = 0;  // rows the activation buffers hold
    std::vector<float *> Z, A;  // Z[l]: pre-activation of hidden layer l, A[l]: input of layer l
    float *d_Y = nullptr, *d_dY = nullptr, *d_dA = nullptr, *d_dB = nullptr, *d_T = nullptr, *d_X = nullptr;
    int *d_rows = nullptr;
    double *d_loss = nullptr;
    cudaStream_t stream = nullptr;
    int device = 0;
    // BF16 tensor-core inference: weights rounded to BF16, padded to [np][kp]
    // (np a multiple of 16, kp of 64), refreshed when the FP32 weights change;
    // BF16 activations [cap][kp of the next layer]
    std::vector<int> npad, kpad;
    std::vector<__nv_bfloat16 *> wbf;
    bool bf_dirty = true;
    int bf_cap = 0;
    std::vector<__nv_bfloat16 *> abf;  // abf[l]: BF16 input of layer l
    int *d_err = nullptr;
    // GEMMs of training: on the tensor cores (3xTF32 split products,
    // mlp_train_tc.cu) or on the CUDA cores (gemm_kernel)
    bool gemm_tc = true;
    int *d_terr = nullptr;  // set when a tensor-core wait of those GEMMs gives up
};

namespace {

void free_bf16_buffers(dg_mlp *n) {
    for (auto *p : n->abf)
        if (p) cudaFree(p);
    n->abf.clear();
    n->bf_cap = 0;
}

void free_mlp_buffers(dg_mlp *n) {
    free_bf16_buffers(n);
    for (float *p : n->Z) cudaFree(p);
    for (size_t l = 1; l < n->A.size(); ++l) cudaFree(n->A[l]);
    n->Z.clear();
    n->A.clear();
    for (float *p : {n->d_Y, n->d_dY, n->d_dA, n->d_dB, n->d_T, n->d_X})
        if (p) cudaFree(p);
    n->d_Y = n->d_dY = n->d_dA = n->d_dB = n->d_T = n->d_X = nullptr;
    if (n->d_rows) cudaFree(n->d_rows);
    n->d_rows = nullptr;
    n->cap = 0;
}

// Activation buffers for up to `rows` rows (A[0] is set by the caller).
int ensure_rows(dg_mlp *n, int rows) {
    if (rows <= n->cap) return DG_OK;
    free_mlp_buffers(n);
    const int cap = std::max(rows, 1024);
    n->A.assign(n->layers, nullptr);
    n->Z.assign(n->layers - 1, nullptr);
    for (int l = 0; l + 1 < n->layers; ++l) {
        CK(cudaMalloc(&n->Z[l], (size_t)cap * n->dout[l] * 4));
        CK(cudaMalloc(&n->A[l + 1], (size_t)cap * n->dout[l] * 4));
    }
    CK(cudaMalloc(&n->d_Y, (size_t)cap * n->nout * 4));
    CK(cudaMalloc(&n->d_dY, (size_t)cap * std::max(n->nout, n->width) * 4));
    CK(cudaMalloc(&n->d_dA, (size_t)cap * std::max(n->nin, n->width) * 4));
    CK(cudaMalloc(&n->d_dB, (size_t)cap * std::max(n->nin, n->width) * 4));
    CK(cudaMalloc(&n->d_T, (size_t)cap * n->nout * 4));
    CK(cudaMalloc(&n->d_X, (size_t)cap * n->nin * 4));
    CK(cudaMalloc(&n->d_rows, (size_t)cap * 4));
    n->cap = cap;
    return DG_OK;
}

// BF16 weights and activation buffers of the tensor-core inference path.
int ensure_bf16(dg_mlp *n, int rows) {
    if (n->width > 256 || n->nout > 256) return fail(DG_ERR_UNSUPPORTED, "BF16 inference needs layers of at most 256");
    if ((long long)rows * ((n->nin + 63) / 64 * 64) >= (1LL << 31) || (long long)rows * 256 >= (1LL << 31))
        return fail(DG_ERR_UNSUPPORTED, "too many rows for BF16 inference");
    if (n->wbf.empty()) {
        for (int l = 0; l < n->layers; ++l) {
            n->npad.push_back((n->dout[l] + 15) / 16 * 16);
            n->kpad.push_back((n->din[l] + 63) / 64 * 64);
            __nv_bfloat16 *w = nullptr;
            CK(cudaMalloc(&w, (size_t)n->npad[l] * n->kpad[l] * 2));
            CK(cudaMemset(w, 0, (size_t)n->npad[l] * n->kpad[l] * 2));
            n->wbf.push_back(w);
        }
        CK(cudaMalloc(&n->d_err, sizeof(int)));
        CK(cudaMemset(n->d_err, 0, sizeof(int)));
        n->bf_dirty = true;
    }
    if (n->bf_dirty) {
        for (int l = 0; l < n->layers; ++l)
            to_bf16_kernel<<<grid_for((long long)n->dout[l] * n->kpad[l]), 256, 0, n->stream>>>(
                n->d_p + n->woff[l], n->dout[l], n->din[l], n->din[l], n->wbf[l], n->kpad[l]);
        CK(cudaGetLastError());
        n->bf_dirty = false;
    }
    if (rows > n->bf_cap) {
        free_bf16_buffers(n);
        const int cap = std::max(rows, 1024);
        n->abf.assign(n->layers, nullptr);
        for (int l = 0; l < n->layers; ++l) {
            // padding columns stay zero: the kernels write columns < din only
            CK(cudaMalloc(&n->abf[l], (size_t)cap * n->kpad[l] * 2));
            CK(cudaMemset(n->abf[l], 0, (size_t)cap * n->kpad[l] * 2));
        }
        n->bf_cap = cap;
    }
    return DG_OK;
}

// Inference of `rows` rows of X (device, FP32) on the tensor cores with BF16
// weights and activations and FP32 accumulation; output in n->d_Y (FP32).
int mlp_forward_bf16(dg_mlp *n, const float *X, int rows) {
    int rc = ensure_rows(n, rows);
    if (rc == DG_OK) rc = ensure_bf16(n, rows);
    if (rc != DG_OK) return rc;
    to_bf16_kernel<<<grid_for((long long)rows * n->kpad[0]), 256, 0, n->stream>>>(X, rows, n->nin, n->nin, n->abf[0],
                                                                                n->kpad[0]);
    for (int l = 0; l < n->layers; ++l) {
        const bool last = l + 1 == n->layers;
        const int r = dgk::tc_linear(n->stream, rows, n->dout[l], n->npad[l], n->kpad[l], n->abf[l], n->wbf[l],
                                     n->d_p + n->boff[l], !last, last ? nullptr : n->abf[l + 1],
                                     last ? n->d_Y : nullptr, last ? n->nout : n->kpad[l + 1], n->d_err);
        if (r != 0) return fail(DG_ERR_CUDA, "tensor-core linear layer launch failed");
    }
    CK(cudaGetLastError());
    return DG_OK;
}

// training: the GEMMs of a training step (forward, gradients), which run on
// the tensor cores when n->gemm_tc; FP32 inference stays on the CUDA cores
// (measured faster for its shapes: 0.39 against 0.52 ms for 11,028 rows).
template <bool TA, bool TB>
int gemm(dg_mlp *n, bool training, int M, int N, int K, const float *A, int lda, const float *B, int ldb, float *C,
         int ldc, const float *bias, float *gelu_out, int accumulate) {
    if (training && n->gemm_tc) {
        if (!n->d_terr) {
            CK(cudaMalloc(&n->d_terr, sizeof(int)));
            CK(cudaMemsetAsync(n->d_terr, 0, sizeof(int), n->stream));
        }
        const int r = dgk::tc_gemm_tf32x3(n->stream, TA, TB, M, N, K, A, lda, B, ldb, C, ldc, bias, gelu_out,
                                          accumulate, n->d_terr);
        if (r != 0) return fail(DG_ERR_CUDA, "tensor-core GEMM launch failed");
        return DG_OK;
    }
    dim3 grid((N + GB - 1) / GB, (M + GB - 1) / GB);
    gemm_kernel<TA, TB><<<grid, 256, 0, n->stream>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, gelu_out, accumulate);
    return DG_OK;
}

// After the stream has been synchronised: DG_ERR_CUDA if a tensor-core wait
// of the training GEMMs gave up since the last check (the flag is cleared).
int check_gemm_err(dg_mlp *n) {
    if (!n->d_terr) return DG_OK;
    int err = 0;
    CK(cudaMemcpy(&err, n->d_terr, sizeof(int), cudaMemcpyDeviceToHost));
    if (!err) return DG_OK;
    CK(cudaMemset(n->d_terr, 0, sizeof(int)));
    return fail(DG_ERR_CUDA, "tensor-core wait timed out in an MLP GEMM");
}

// Forward pass of `rows` rows of X (device); output in n->d_Y.  training:
// the forward pass of a training step.
int mlp_forward(dg_mlp *n, const float *X, int rows, bool training = false) {
    int rc = ensure_rows(n, rows);
    if (rc != DG_OK) return rc;
    n->A[0] = const_cast<float *>(X);
    for (int l = 0; l < n->layers; ++l) {
        const float *W = n->d_p + n->woff[l], *b = n->d_p + n->boff[l];
        int rc;
        if (l + 1 < n->layers)
            rc = gemm<false, false>(n, training, rows, n->dout[l], n->din[l], n->A[l], n->din[l], W, n->din[l],
                                    n->Z[l], n->dout[l], b, n->A[l + 1], 0);
        else
            rc = gemm<false, false>(n, training, rows, n->dout[l], n->din[l], n->A[l], n->din[l], W, n->din[l],
                                    n->d_Y, n->dout[l], b, nullptr, 0);
        if (rc != DG_OK) return rc;
    }
    CK(cudaGetLastError());
    return DG_OK;
}

// Loss and gradients (into d_g) of the mean squared error against T (device).
int mlp_backward(dg_mlp *n, const float *X, const float *T, int rows, double *loss) {
    int rc = mlp_forward(n, X, rows, true);
    if (rc != DG_OK) return rc;
    const long long ny = (long long)rows * n->nout;
    CK(cudaMemsetAsync(n->d_loss, 0, 8, n->stream));
    mse_kernel<<<grid_for(ny), 256, 0, n->stream>>>(n->d_Y, T, n->d_dY, ny, 1.0f / (float)ny, n->d_loss);
    float *dZ = n->d_dY;  // gradient with respect to the current layer's output (pre-activation)
    for (int l = n->layers - 1; l >= 0; --l) {
        const int din = n->din[l], dout = n->dout[l];
        // dW = dZ^T A_l  ([dout x din]), db = column sums of dZ
        rc = gemm<true, true>(n, true, dout, din, rows, dZ, dout, n->A[l], din, n->d_g + n->woff[l], din, nullptr,
                              nullptr, 0);
        if (rc != DG_OK) return rc;
        column_sum_kernel<<<dout, 256, 0, n->stream>>>(dZ, rows, dout, n->d_g + n->boff[l]);
        if (l > 0) {
            // dA_l = dZ W ([rows x din]), then through the GELU of layer l-1
            float *dA = (dZ == n->d_dA) ? n->d_dB : n->d_dA;
            rc = gemm<false, true>(n, true, rows, din, dout, dZ, dout, n->d_p + n->woff[l], din, dA, din, nullptr,
                                   nullptr, 0);
            if (rc != DG_OK) return rc;
            gelu_backward_kernel<<<grid_for((long long)rows * din), 256, 0, n->stream>>>(dA, n->Z[l - 1],
                                                                                         (long long)rows * din);
            dZ = dA;
        }
    }
    CK(cudaGetLastError());
    if (loss) {
        double h = 0;
        CK(cudaMemcpyAsync(&h, n->d_loss, 8, cudaMemcpyDeviceToHost, n->stream));
        CK(cudaStreamSynchronize(n->stream));
        *loss = h / (double)ny;
    }
    return DG_OK;
}

int mlp_adam(dg_mlp *n, float lr) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    n->adam_t += 1;
    const float c1 = 1.0f / (1.0f - std::pow(b1, (float)n->adam_t));
    const float c2 = 1.0f / (1.0f - std::pow(b2, (float)n->adam_t));
    adam_kernel<<<grid_for(n->nparam), 256, 0, n->stream>>>(n->d_p, n->d_g, n->d_m, n->d_v, n->nparam, lr, b1, b2,
                                                           eps, c1, c2);
    CK(cudaGetLastError());
    n->bf_dirty = true;
    return DG_OK;
}

}  // namespace

extern "C" {

int dg_mlp_create(int nin, int width, int nout, int hidden_layers, unsigned seed, int device, dg_mlp **out) {
    if (!out || nin < 1 || width < 1 || nout < 1 || hidden_layers < 0) return fail(DG_ERR_ARG, "bad MLP shape");
    *out = nullptr;
    dg_mlp *n = new dg_mlp();
    n->nin = nin;
    n->width = width;
    n->nout = nout;
    n->layers = hidden_layers + 1;
    n->device = device;
    for (int l = 0; l < n->layers; ++l) {
        n->din.push_back(l == 0 ? nin : width);
        n->dout.push_back(l + 1 == n->layers ? nout : width);
    }
    long long off = 0;
    for (int l = 0; l < n->layers; ++l) {
        n->woff.push_back(off);
        off += (long long)n->din[l] * n->dout[l];
        n->boff.push_back(off);
        off += n->dout[l];
    }
    n->nparam = off;
    // He-style initialisation, zero biases; the last layer starts small
    std::vector<float> p(off, 0.0f);
    std::mt19937 rng(seed);
    for (int l = 0; l < n->layers; ++l) {
        std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / n->din[l]) * (l + 1 == n->layers ? 0.1f : 1.0f));
        for (long long k = 0; k < (long long)n->din[l] * n->dout[l]; ++k) p[n->woff[l] + k] = nd(rng);
    }
    auto cleanup = [&](int rc) {
        for (float *q : {n->d_p, n->d_g, n->d_m, n->d_v})
            if (q) cudaFree(q);
        if (n->d_loss) cudaFree(n->d_loss);
        if (n->stream) cudaStreamDestroy(n->stream);
        delete n;
        return rc;
    };
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking);
    for (float **q : {&n->d_p, &n->d_g, &n->d_m, &n->d_v})
        if (e == cudaSuccess) e = cudaMalloc(q, (size_t)off * 4);
    if (e == cudaSuccess) e = cudaMalloc(&n->d_loss, 8);
    if (e == cudaSuccess) e = cudaMemcpy(n->d_p, p.data(), (size_t)off * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(n->d_m, 0, (size_t)off * 4);
    if (e == cudaSuccess) e = cudaMemset(n->d_v, 0, (size_t)off * 4);
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "MLP allocation"));
    *out = n;
    return DG_OK;
}

void dg_mlp_destroy(dg_mlp *n) {
    if (!n) return;
    cudaSetDevice(n->device);
    free_mlp_buffers(n);
    for (auto *w : n->wbf)
        if (w) cudaFree(w);
    if (n->d_err) cudaFree(n->d_err);
    if (n->d_terr) cudaFree(n->d_terr);
    for (float *q : {n->d_p, n->d_g, n->d_m, n->d_v})
        if (q) cudaFree(q);
    if (n->d_loss) cudaFree(n->d_loss);
    if (n->stream) cudaStreamDestroy(n->stream);
    delete n;
}

long long dg_mlp_num_params(const dg_mlp *n) { return n ? n->nparam : 0; }

int dg_mlp_get_params(dg_mlp *n, float *p) {
    if (!n || !p) return fail(DG_ERR_ARG, "null argument");
    CK(cudaSetDevice(n->device));
    CK(cudaMemcpy(p, n->d_p, (size_t)n->nparam * 4, cudaMemcpyDeviceToHost));
    return DG_OK;
}

int dg_mlp_set_params(dg_mlp *n, const float *p) {
    if (!n || !p) return fail(DG_ERR_ARG, "null argument");
    CK(cudaSetDevice(n->device));
    CK(cudaMemcpy(n->d_p, p, (size_t)n->nparam * 4, cudaMemcpyHostToDevice));
    n->bf_dirty = true;
    return DG_OK;
}

int dg_mlp_set_gemm(dg_mlp *n, int mode) {
    if (!n || (mode != 0 && mode != 1)) return fail(DG_ERR_ARG, "mode must be 0 (CUDA cores) or 1 (tensor cores)");
    n->gemm_tc = mode == 1;
    return DG_OK;
}

int dg_mlp_forward_bf16(dg_mlp *n, const float *X, int rows, float *Y) {
    if (!n || !X || !Y || rows < 1) return fail(DG_ERR_ARG, "bad arguments");
    CK(cudaSetDevice(n->device));
    int rc = ensure_rows(n, rows);
    if (rc != DG_OK) return rc;
    CK(cudaMemcpyAsync(n->d_X, X, (size_t)rows * n->nin * 4, cudaMemcpyHostToDevice, n->stream));
    rc = mlp_forward_bf16(n, n->d_X, rows);
    if (rc != DG_OK) return rc;
    CK(cudaMemcpyAsync(Y, n->d_Y, (size_t)rows * n->nout * 4, cudaMemcpyDeviceToHost, n->stream));
    int err = 0;
    CK(cudaMemcpyAsync(&err, n->d_err, sizeof(int), cudaMemcpyDeviceToHost, n->stream));
    CK(cudaStreamSynchronize(n->stream));
    if (err) return fail(DG_ERR_CUDA, "tensor-core wait timed out in BF16 inference");
    return DG_OK;
}

int dg_mlp_forward(dg_mlp *n, const float *X, int rows, float *Y) {
    if (!n || !X || !Y || rows < 1) return fail(DG_ERR_ARG, "bad arguments");
    CK(cudaSetDevice(n->device));
    int rc = ensure_rows(n, rows);
    if (rc != DG_OK) return rc;
    CK(cudaMemcpyAsync(n->d_X, X, (size_t)rows * n->nin * 4, cudaMemcpyHostToDevice, n->stream));
    rc = mlp_forward(n, n->d_X, rows);
    if (rc != DG_OK) return rc;
    CK(cudaMemcpyAsync(Y, n->d_Y, (size_t)rows * n->nout * 4, cudaMemcpyDeviceToHost, n->stream));
    CK(cudaStreamSynchronize(n->stream));
    return check_gemm_err(n);
}

int dg_mlp_loss_grad(dg_mlp *n, const float *X, const float *T, int rows, double *loss, float *grad) {
    if (!n || !X || !T || rows < 1) return fail(DG_ERR_ARG, "bad arguments");
    CK(cudaSetDevice(n->device));
    int rc = ensure_rows(n, rows);
    if (rc != DG_OK) return rc;
    CK(cudaMemcpyAsync(n->d_X, X, (size_t)rows * n->nin * 4, cudaMemcpyHostToDevice, n->stream));
    CK(cudaMemcpyAsync(n->d_T, T, (size_t)rows * n->nout * 4, cudaMemcpyHostToDevice, n->stream));
    rc = mlp_backward(n, n->d_X, n->d_T, rows, loss);
    if (rc != DG_OK) return rc;
    if (grad) CK(cudaMemcpy(grad, n->d_g, (size_t)n->nparam * 4, cudaMemcpyDeviceToHost));
    CK(cudaStreamSynchronize(n->stream));
    return check_gemm_err(n);
}

int dg_mlp_train_step(dg_mlp *n, const float *X, const float *T, int rows, double lr, double *loss) {
    int rc = dg_mlp_loss_grad(n, X, T, rows, loss, nullptr);
    if (rc != DG_OK) return rc;
    rc = mlp_adam(n, (float)lr);
    if (rc != DG_OK) return rc;
    CK(cudaStreamSynchronize(n->stream));
    return DG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- learned coarse propagator

struct dg_learned {
    dg_ctx *fine = nullptr;   // FP64 single-member context (trajectories)
    dg_mlp *net = nullptr;
    int coarse_steps = 1;
    double dt = 0;
    int nin = 0, nout = 0;
    float in_scale[4] = {1, 1, 1, 1};   // field scales of the inputs
    float out_scale[4] = {1, 1, 1, 1};  // field scales of the increments
    float tscale[4] = {1, 1, 1, 1};     // RMS of the training targets per field (unit-variance outputs)
    float geo_scale = 1;
    bool scaled = false;
    int2 *d_conn = nullptr;  // copies of the layout the features read
    uint8_t *d_tabs = nullptr;
    double *d_geo = nullptr;
    float *d_feat = nullptr;  // [K][nin]
    float *d_escale = nullptr;  // [K] input scale of each element
    double *d_detj = nullptr;   // [K] element Jacobian determinants
    double *d_prod = nullptr;   // energy products of a coarse application, then its step factor
    double *d_parts = nullptr;  // their per-block partial sums
    double *d_stats = nullptr;  // step factors so far: sum, minimum, count
    std::vector<float *> samples_x, samples_t;  // device blocks of training rows
    std::vector<int> sample_rows;
    long long total_rows = 0;
    double *d_u0 = nullptr, *d_u1 = nullptr;  // FP64 scratch states
    int device = 0;
    bool bf16 = false;  // coarse steps infer with BF16 tensor cores
};

namespace {

FeatArgs feat_args(dg_learned *L, const double *u) {
    dg_ctx *c = L->fine;
    FeatArgs a;
    a.u = u;
    a.ndof = c->ndof;
    a.K = c->K;
    a.np = c->np;
    a.nf = c->nf;
    a.nfp = c->nfp;
    a.nq = c->nq;
    a.dim = c->dim;
    a.nin = L->nin;
    a.conn = L->d_conn;
    a.tabs = L->d_tabs;
    a.geo = L->d_geo;
    for (int f = 0; f < 4; ++f) a.inv_scale[f] = 1.0f / L->in_scale[f];
    a.inv_geo = 1.0f / L->geo_scale;
    return a;
}

// One coarse application on an FP64 state (device, member layout), enqueued
// on the network's stream with no host synchronisation: features, network,
// energy products, step factor (on the device) and the update.
int coarse_apply(dg_learned *L, double *u) {
    dg_ctx *c = L->fine;
    dg_mlp *n = L->net;
    cudaStream_t s = n->stream;
    features_kernel<<<(c->K + 3) / 4, 128, 0, s>>>(feat_args(L, u), L->d_feat, L->d_escale);
    CK(cudaGetLastError());
    int rc = L->bf16 ? mlp_forward_bf16(n, L->d_feat, c->K) : mlp_forward(n, L->d_feat, c->K);
    if (rc != DG_OK) return rc;
    // energy-stable step: u + d, scaled back to E(u) if it has more energy
    // (the upwind DG propagator with these walls never gains energy)
    const long long nv = (long long)c->K * c->np * c->nq;
    double os[4];
    for (int f = 0; f < 4; ++f) os[f] = (double)L->out_scale[f] * L->tscale[f];
    const int nb = kEnergyBlocks;
    energy_products_kernel<<<nb, 256, 0, s>>>(u, c->ndof, c->K, c->np, c->nq, n->d_Y, L->d_escale, os[0], os[1],
                                              os[2], os[3], L->d_detj, 1.0 / (c->rho0 * c->c0 * c->c0), c->rho0,
                                              L->d_parts);
    sum_parts_kernel<<<1, 256, 0, s>>>(L->d_parts, nb, L->d_prod);
    step_factor_kernel<<<1, 1, 0, s>>>(L->d_prod, L->d_prod + 3, L->d_stats);
    apply_increment_kernel<<<grid_for(nv), 256, 0, s>>>(u, c->ndof, c->K, c->np, c->nq, n->d_Y, L->d_escale, os[0],
                                                         os[1], os[2], os[3], L->d_prod + 3);
    CK(cudaGetLastError());
    return DG_OK;
}

}  // namespace

extern "C" {

static int dg_learned_create_impl(const dg_mesh_desc *mesh, const dg_phys_desc *phys, int flux_sign, int width,
                      int hidden_layers, int coarse_steps, double dt, unsigned seed, int device, dg_learned **out) {
    if (!mesh || !phys || !out || coarse_steps < 1 || !(dt > 0)) return fail(DG_ERR_ARG, "bad arguments");
    *out = nullptr;
    dg_opts o;
    dg_default_opts(&o);
    o.flux_sign = flux_sign;
    o.device = device;
    dg_learned *L = new dg_learned();
    L->coarse_steps = coarse_steps;
    L->dt = dt;
    L->device = device;
    int rc = dg_create(mesh, phys, &o, &L->fine);
    if (rc != DG_OK) {
        delete L;
        return rc;
    }
    dg_ctx *c = L->fine;
    L->nin = c->nq * c->np + c->nf * c->nfp * c->nq + 2 * c->nf + c->dim * c->dim;
    L->nout = c->nq * c->np;
    dg::Layout lay;
    std::string err = dg::build_layout(*mesh, flux_sign, lay);
    if (err.empty() && lay.curved.C > 0) err = "the learned coarse propagator's features assume straight-sided elements";
    if (!err.empty()) {
        dg_destroy(L->fine);
        delete L;
        return fail(lay.curved.C > 0 ? DG_ERR_UNSUPPORTED : DG_ERR_MESH, err);
    }
    double gmax = 0;
    for (double g : lay.geo) gmax = std::max(gmax, std::fabs(g));
    L->geo_scale = gmax > 0 ? (float)gmax : 1.0f;
    auto bail = [&](int code) {
        dg_learned_destroy(L);
        return code;
    };
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaMalloc(&L->d_conn, lay.conn.size() * 4);
    if (e == cudaSuccess) e = cudaMemcpy(L->d_conn, lay.conn.data(), lay.conn.size() * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&L->d_tabs, lay.tabs.size());
    if (e == cudaSuccess) e = cudaMemcpy(L->d_tabs, lay.tabs.data(), lay.tabs.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&L->d_geo, lay.geo.size() * 8);
    if (e == cudaSuccess) e = cudaMemcpy(L->d_geo, lay.geo.data(), lay.geo.size() * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&L->d_feat, (size_t)c->K * L->nin * 4);
    if (e == cudaSuccess) e = cudaMalloc(&L->d_escale, (size_t)c->K * 4);
    if (e == cudaSuccess) e = cudaMalloc(&L->d_prod, 32);
    if (e == cudaSuccess) e = cudaMalloc(&L->d_stats, 24);
    if (e == cudaSuccess) {
        const double st[3] = {0.0, 1.0, 0.0};
        e = cudaMemcpy(L->d_stats, st, 24, cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMalloc(&L->d_parts, (size_t)3 * 4096 * 8);
    if (e == cudaSuccess) e = cudaMalloc(&L->d_detj, (size_t)c->K * 8);
    if (e == cudaSuccess) e = cudaMemcpy(L->d_detj, mesh->el_jacobian_dets, (size_t)c->K * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&L->d_u0, (size_t)c->ndof * c->nq * 8);
    if (e == cudaSuccess) e = cudaMalloc(&L->d_u1, (size_t)c->ndof * c->nq * 8);
    if (e != cudaSuccess) return bail(cuda_fail(e, "learned propagator allocation"));
    rc = dg_mlp_create(L->nin, width, L->nout, hidden_layers, seed, device, &L->net);
    if (rc != DG_OK) return bail(rc);
    *out = L;
    return DG_OK;
}

int dg_learned_create(const dg_mesh_desc *mesh, const dg_phys_desc *phys, int flux_sign, int width,
                      int hidden_layers, int coarse_steps, double dt, unsigned seed, int device, dg_learned **out) {
    return dg::guarded([&]() { return dg_learned_create_impl(mesh, phys, flux_sign, width, hidden_layers, coarse_steps, dt, seed, device, out); });
}

void dg_learned_destroy(dg_learned *L) {
    if (!L) return;
    cudaSetDevice(L->device);
    for (float *p : L->samples_x) cudaFree(p);
    for (float *p : L->samples_t) cudaFree(p);
    for (void *p : {(void *)L->d_conn, (void *)L->d_tabs, (void *)L->d_geo, (void *)L->d_feat, (void *)L->d_escale,
                    (void *)L->d_prod, (void *)L->d_parts, (void *)L->d_detj, (void *)L->d_u0, (void *)L->d_u1,
                    (void *)L->d_stats})
        if (p) cudaFree(p);
    if (L->net) dg_mlp_destroy(L->net);
    if (L->fine) dg_destroy(L->fine);
    delete L;
}

int dg_learned_info(dg_learned *L, int *nin, int *nout, dg_mlp **net) {
    if (!L) return fail(DG_ERR_ARG, "null argument");
    if (nin) *nin = L->nin;
    if (nout) *nout = L->nout;
    if (net) *net = L->net;
    return DG_OK;
}

int dg_learned_set_inference(dg_learned *L, int bf16) {
    if (!L) return fail(DG_ERR_ARG, "null argument");
    if (bf16 && (L->net->width > 256 || L->net->nout > 256))
        return fail(DG_ERR_UNSUPPORTED, "BF16 inference needs layers of at most 256");
    L->bf16 = bf16 != 0;
    return DG_OK;
}

int dg_learned_step_stats(dg_learned *L, long long *applications, double *alpha_mean, double *alpha_min) {
    if (!L) return fail(DG_ERR_ARG, "null argument");
    CK(cudaSetDevice(L->device));
    double st[3];
    CK(cudaMemcpyAsync(st, L->d_stats, 24, cudaMemcpyDeviceToHost, L->net->stream));
    CK(cudaStreamSynchronize(L->net->stream));
    const long long napp = (long long)st[2];
    if (applications) *applications = napp;
    if (alpha_mean) *alpha_mean = napp ? st[0] / (double)napp : 0.0;
    if (alpha_min) *alpha_min = st[1];
    return DG_OK;
}

// Runs the FP64 DG from u0 for nsnap x coarse_steps steps and keeps, after
// every coarse_steps steps, the pairs (features of the elements, their DOF
// increments) of the active elements (those whose input features are not
// all below 1e-6 of the largest), at most max_rows per snapshot.
int dg_learned_collect(dg_learned *L, const double *const u0[4], int nsnap, int max_rows) {
    if (!L || !u0 || nsnap < 1 || max_rows < 1) return fail(DG_ERR_ARG, "bad arguments");
    dg_ctx *c = L->fine;
    CK(cudaSetDevice(L->device));
    int rc = dg_set_state(c, u0);
    if (rc != DG_OK) return rc;
    const size_t sb = (size_t)c->ndof * c->nq * 8;
    if (!L->scaled) {
        // field scales from the initial state (RMS, floor 1e-30), increments
        // from the first coarse step
        std::vector<double> h(c->ndof * c->nq);
        CK(cudaMemcpy(h.data(), c->d_u, sb, cudaMemcpyDeviceToHost));
        double gmax = 0;
        for (int f = 0; f < c->nq; ++f) {
            double s = 0;
            for (long long i = 0; i < c->ndof; ++i) s = std::max(s, std::fabs(h[f * c->ndof + i]));
            gmax = std::max(gmax, s);
        }
        // pressure and velocity scales tied by the impedance rho0 c0
        const double zs = 1.0 / (c->rho0 * c->c0);
        for (int f = 0; f < c->nq; ++f) L->in_scale[f] = (float)std::max(gmax * (f == 0 ? 1.0 : zs), 1e-30);
        for (int f = 0; f < c->nq; ++f) L->out_scale[f] = L->in_scale[f];
        L->scaled = true;
    }
    double t = 0.0;
    std::vector<float> act(c->K);
    std::mt19937 rng(1234 + (unsigned)L->total_rows);
    for (int s = 0; s < nsnap; ++s) {
        CK(cudaMemcpy(L->d_u0, c->d_u, sb, cudaMemcpyDeviceToDevice));
        rc = dg_rk4_steps(c, &t, L->dt, L->coarse_steps);
        if (rc != DG_OK) return rc;
        CK(cudaMemcpy(L->d_u1, c->d_u, sb, cudaMemcpyDeviceToDevice));
        features_kernel<<<(c->K + 3) / 4, 128>>>(feat_args(L, L->d_u0), L->d_feat, L->d_escale);
        CK(cudaGetLastError());
        // activity: the elements' input scales
        CK(cudaMemcpy(act.data(), L->d_escale, (size_t)c->K * 4, cudaMemcpyDeviceToHost));
        float fmax = 0;
        for (int e = 0; e < c->K; ++e) fmax = std::max(fmax, act[e]);
        std::vector<int> rows;
        for (int e = 0; e < c->K; ++e)
            if (act[e] > 1e-6f * fmax) rows.push_back(e);
        if ((int)rows.size() > max_rows) {
            std::shuffle(rows.begin(), rows.end(), rng);
            rows.resize(max_rows);
        }
        if (rows.empty()) continue;
        const int nr = (int)rows.size();
        float *T = nullptr, *Tall = nullptr, *X = nullptr;
        int *d_rows = nullptr;
        CK(cudaMalloc(&Tall, (size_t)c->K * L->nout * 4));
        CK(cudaMalloc(&T, (size_t)nr * L->nout * 4));
        CK(cudaMalloc(&X, (size_t)nr * L->nin * 4));
        CK(cudaMalloc(&d_rows, (size_t)nr * 4));
        CK(cudaMemcpy(d_rows, rows.data(), (size_t)nr * 4, cudaMemcpyHostToDevice));
        targets_kernel<<<grid_for((long long)c->K * L->nout), 256>>>(
            L->d_u0, L->d_u1, c->ndof, c->K, c->np, c->nq, L->d_escale, 1.0f / L->out_scale[0],
            1.0f / L->out_scale[1], 1.0f / L->out_scale[2], 1.0f / L->out_scale[3], Tall);
        gather_rows_kernel<<<grid_for((long long)nr * L->nout), 256>>>(Tall, d_rows, nr, L->nout, T);
        gather_rows_kernel<<<grid_for((long long)nr * L->nin), 256>>>(L->d_feat, d_rows, nr, L->nin, X);
        CK(cudaGetLastError());
        CK(cudaDeviceSynchronize());
        cudaFree(Tall);
        cudaFree(d_rows);
        L->samples_x.push_back(X);
        L->samples_t.push_back(T);
        L->sample_rows.push_back(nr);
        L->total_rows += nr;
    }
    return DG_OK;
}

long long dg_learned_num_samples(dg_learned *L) { return L ? L->total_rows : 0; }

// Minibatch Adam over the collected pairs; *loss = mean loss of the last epoch.
int dg_learned_train(dg_learned *L, int epochs, int batch, double lr, unsigned seed, double *loss) {
    if (!L || epochs < 1 || batch < 1) return fail(DG_ERR_ARG, "bad arguments");
    if (L->total_rows == 0) return fail(DG_ERR_ARG, "no training pairs collected");
    CK(cudaSetDevice(L->device));
    dg_mlp *n = L->net;
    int rc = ensure_rows(n, batch);
    if (rc != DG_OK) return rc;
    // all pairs in one contiguous block
    float *X = nullptr, *T = nullptr;
    CK(cudaMalloc(&X, (size_t)L->total_rows * L->nin * 4));
    CK(cudaMalloc(&T, (size_t)L->total_rows * L->nout * 4));
    long long off = 0;
    for (size_t b = 0; b < L->samples_x.size(); ++b) {
        CK(cudaMemcpy(X + off * L->nin, L->samples_x[b], (size_t)L->sample_rows[b] * L->nin * 4,
                      cudaMemcpyDeviceToDevice));
        CK(cudaMemcpy(T + off * L->nout, L->samples_t[b], (size_t)L->sample_rows[b] * L->nout * 4,
                      cudaMemcpyDeviceToDevice));
        off += L->sample_rows[b];
    }
    {
        // unit-variance targets per field (the pressure increment is second
        // order in time, much smaller than the velocity one)
        dg_ctx *c = L->fine;
        double *d_sums = nullptr;
        CK(cudaMalloc(&d_sums, 32));
        CK(cudaMemset(d_sums, 0, 32));
        column_group_squares_kernel<<<grid_for(L->total_rows * L->nout), 256>>>(T, L->total_rows, L->nout, c->np,
                                                                                d_sums);
        double h[4];
        CK(cudaMemcpy(h, d_sums, 32, cudaMemcpyDeviceToHost));
        cudaFree(d_sums);
        for (int f = 0; f < 4; ++f) {
            const double rms = f < c->nq ? std::sqrt(h[f] / ((double)L->total_rows * c->np)) : 0.0;
            L->tscale[f] = rms > 0 ? (float)rms : 1.0f;
        }
        scale_columns_kernel<<<grid_for(L->total_rows * L->nout), 256>>>(
            T, L->total_rows, L->nout, c->np, 1.0f / L->tscale[0], 1.0f / L->tscale[1], 1.0f / L->tscale[2],
            1.0f / L->tscale[3]);
        CK(cudaGetLastError());
    }
    std::vector<int> order(L->total_rows);
    std::iota(order.begin(), order.end(), 0);
    std::mt19937 rng(seed);
    double last = 0;
    for (int ep = 0; ep < epochs && rc == DG_OK; ++ep) {
        std::shuffle(order.begin(), order.end(), rng);
        double sum = 0;
        long long cnt = 0;
        for (long long b0 = 0; b0 < L->total_rows; b0 += batch) {
            const int nb = (int)std::min<long long>(batch, L->total_rows - b0);
            cudaMemcpyAsync(n->d_rows, order.data() + b0, (size_t)nb * 4, cudaMemcpyHostToDevice, n->stream);
            gather_rows_kernel<<<grid_for((long long)nb * L->nin), 256, 0, n->stream>>>(X, n->d_rows, nb, L->nin,
                                                                                          n->d_X);
            gather_rows_kernel<<<grid_for((long long)nb * L->nout), 256, 0, n->stream>>>(T, n->d_rows, nb, L->nout,
                                                                                           n->d_T);
            double l = 0;
            rc = mlp_backward(n, n->d_X, n->d_T, nb, &l);
            if (rc != DG_OK) break;
            rc = mlp_adam(n, (float)lr);
            if (rc != DG_OK) break;
            sum += l * nb;
            cnt += nb;
        }
        last = cnt ? sum / cnt : 0;
    }
    cudaStreamSynchronize(n->stream);
    cudaFree(X);
    cudaFree(T);
    if (rc != DG_OK) return rc;
    rc = check_gemm_err(n);
    if (rc != DG_OK) return rc;
    if (loss) *loss = last;
    return DG_OK;
}

// napps coarse applications on a host state (in place).
int dg_learned_apply(dg_learned *L, double *const u[4], int napps) {
    if (!L || !u || napps < 0) return fail(DG_ERR_ARG, "bad arguments");
    dg_ctx *c = L->fine;
    CK(cudaSetDevice(L->device));
    for (int f = 0; f < c->nq; ++f)
        CK(cudaMemcpy(L->d_u0 + f * c->ndof, u[f], (size_t)c->ndof * 8, cudaMemcpyHostToDevice));
    for (int k = 0; k < napps; ++k) {
        int rc = coarse_apply(L, L->d_u0);
        if (rc != DG_OK) return rc;
    }
    CK(cudaStreamSynchronize(L->net->stream));
    for (int f = 0; f < c->nq; ++f)
        CK(cudaMemcpy(u[f], L->d_u0 + f * c->ndof, (size_t)c->ndof * 8, cudaMemcpyDeviceToHost));
    return check_gemm_err(L->net);
}

// Parareal over nslices slices of slice_steps fine RK4 steps from u0 (host).
// learned = NULL uses the identity as coarse propagator (the method without
// the network).  Iterates until the largest relative change of a slice end
// state falls to tol, or max_iter iterations (max_iter >= nslices reproduces
// the serial DG exactly).  uout receives the end state of the last slice;
// hist[k] the largest relative change at iteration k (max_iter entries).
int dg_parareal(dg_learned *learned, const dg_mesh_desc *mesh, const dg_phys_desc *phys, int flux_sign,
                const double *const u0[4], int nslices, int slice_steps, double dt, double tol, int max_iter,
                double *const uout[4], int *iters, double *hist) {
    if (!mesh || !phys || !u0 || nslices < 1 || slice_steps < 1 || !(dt > 0) || max_iter < 0)
        return fail(DG_ERR_ARG, "bad parareal arguments");
    if (learned && slice_steps % learned->coarse_steps != 0)
        return fail(DG_ERR_ARG, "slice steps must be a multiple of the learned propagator's coarse steps");
    dg_opts o;
    dg_default_opts(&o);
    o.flux_sign = flux_sign;
    o.device = learned ? learned->device : 0;
    dg_ctx *F = nullptr;
    int rc = dg_create_batch(mesh, phys, &o, nslices, &F);
    if (rc != DG_OK) return rc;
    const long long nv = F->bstride;  // values of one state
    const size_t sb = (size_t)nv * 8;
    std::vector<double *> U(nslices + 1, nullptr), Uold(nslices + 1, nullptr), Gold(nslices + 1, nullptr);
    double *d_norm = nullptr, *d_g = nullptr;
    cudaStream_t s = F->stream;
    auto release = [&]() {
        for (auto *v : {&U, &Uold, &Gold})
            for (double *p : *v)
                if (p) cudaFree(p);
        if (d_norm) cudaFree(d_norm);
        if (d_g) cudaFree(d_g);
        dg_destroy(F);
    };
    auto coarse = [&](double *dst, const double *src) -> int {
        CK(cudaMemcpyAsync(dst, src, sb, cudaMemcpyDeviceToDevice, s));
        if (!learned) return DG_OK;  // identity propagator
        if (learned->fine->K != F->K || learned->fine->np != F->np)
            return fail(DG_ERR_ARG, "learned propagator built for another mesh");
        CK(cudaStreamSynchronize(s));
        for (int k = 0; k < slice_steps / learned->coarse_steps; ++k) {
            int r = coarse_apply(learned, dst);
            if (r != DG_OK) return r;
        }
        CK(cudaStreamSynchronize(learned->net->stream));
        return DG_OK;
    };
    do {
        cudaError_t e = cudaSuccess;
        for (int n = 0; n <= nslices && e == cudaSuccess; ++n) {
            e = cudaMalloc(&U[n], sb);
            if (e == cudaSuccess) e = cudaMalloc(&Uold[n], sb);
            if (e == cudaSuccess) e = cudaMalloc(&Gold[n], sb);
        }
        if (e == cudaSuccess) e = cudaMalloc(&d_norm, 16);
        if (e == cudaSuccess) e = cudaMalloc(&d_g, sb);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "parareal allocation");
            break;
        }
        for (int f = 0; f < F->nq && rc == DG_OK; ++f)
            if (cudaMemcpy(U[0] + f * F->ndof, u0[f], (size_t)F->ndof * 8, cudaMemcpyHostToDevice) != cudaSuccess)
                rc = fail(DG_ERR_CUDA, "state upload");
        if (rc != DG_OK) break;
        // iteration 0: coarse sweep
        for (int n = 0; n < nslices && rc == DG_OK; ++n) {
            rc = coarse(Gold[n + 1], U[n]);
            if (rc == DG_OK && cudaMemcpyAsync(U[n + 1], Gold[n + 1], sb, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
                rc = fail(DG_ERR_CUDA, "copy");
        }
        int k = 0;
        for (; k < max_iter && rc == DG_OK; ++k) {
            // fine propagation of every slice from the previous iterate, one batch
            for (int n = 0; n < nslices; ++n)
                cudaMemcpyAsync((double *)F->d_u + (size_t)n * nv, U[n], sb, cudaMemcpyDeviceToDevice, s);
            double t = 0.0;
            rc = dg_rk4_steps(F, &t, dt, slice_steps);
            if (rc != DG_OK) break;
            for (int n = 0; n <= nslices; ++n) cudaMemcpyAsync(Uold[n], U[n], sb, cudaMemcpyDeviceToDevice, s);
            // sequential correction sweep
            double worst = 0;
            for (int n = 0; n < nslices && rc == DG_OK; ++n) {
                rc = coarse(d_g, U[n]);  // G(U_new[n])
                if (rc != DG_OK) break;
                combine_kernel<<<grid_for(nv), 256, 0, s>>>(U[n + 1], d_g, (double *)F->d_u + (size_t)n * nv,
                                                             Gold[n + 1], nv);
                cudaMemcpyAsync(Gold[n + 1], d_g, sb, cudaMemcpyDeviceToDevice, s);
                cudaMemsetAsync(d_norm, 0, 16, s);
                diff_norm_kernel<<<grid_for(nv), 256, 0, s>>>(U[n + 1], Uold[n + 1], nv, d_norm);
                double h[2];
                if (cudaMemcpyAsync(h, d_norm, 16, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                    cudaStreamSynchronize(s) != cudaSuccess) {
                    rc = fail(DG_ERR_CUDA, "parareal norm");
                    break;
                }
                worst = std::max(worst, h[1] > 0 ? std::sqrt(h[0] / h[1]) : std::sqrt(h[0]));
            }
            if (rc != DG_OK) break;
            if (hist) hist[k] = worst;
            if (worst <= tol) {
                ++k;
                break;
            }
        }
        if (rc != DG_OK) break;
        if (iters) *iters = k;
        if (uout)
            for (int f = 0; f < F->nq; ++f)
                if (uout[f] &&
                    cudaMemcpy(uout[f], U[nslices] + f * F->ndof, (size_t)F->ndof * 8, cudaMemcpyDeviceToHost) !=
                        cudaSuccess)
                    rc = fail(DG_ERR_CUDA, "state download");
    } while (0);
    release();
    return rc;
}

}  // extern "C"
