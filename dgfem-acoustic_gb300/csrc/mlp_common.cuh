// Pieces shared by the FP32 (SIMT) and BF16 (tensor-core) MLP kernels.
#pragma once
#include <cuda_runtime.h>

namespace dgk {

// GELU, tanh form (Hendrycks and Gimpel, 2016).
__device__ __forceinline__ float gelu_f(float x) {
    const float u = 0.7978845608028654f * (x + 0.044715f * x * x * x);
    return 0.5f * x * (1.0f + tanhf(u));
}

// BF16 tensor-core linear layer of MLP inference (mlp_tc.cu):
// Y[m][n] = act(sum_k X[m][k] W[n][k] + b[n]) for n < N, m < M.  X is BF16
// [M][kp] and W BF16 [np][kp], both zero-padded (kp a multiple of 64, np a
// multiple of 16, np <= 256).  gelu: apply GELU; the output is BF16 with row
// stride ldy (ybf) or FP32 with row stride ldy (yf32), whichever is not null.
// err is set to 1 if a wait on the tensor cores gives up.
int tc_linear(cudaStream_t s, int M, int N, int np, int kp, const void *X, const void *W, const float *bias, bool gelu,
              void *ybf, float *yf32, int ldy, int *err);

// FP32 GEMM of MLP training on the tensor cores (mlp_train_tc.cu), 3xTF32
// split products with FP32 accumulation: C[m][n] = sum_k op(A)[m][k]
// op(B)[n][k] (+ bias[n]) (+ C[m][n] when accumulate), gelu_out (if not
// null) = GELU of the result; op(A)[m][k] = ta ? A[k*lda + m] : A[m*lda + k],
// op(B) likewise.  Returns 0, -1 on bad sizes, -2 on a launch error; err is
// set to 1 if a wait on the tensor cores gives up.
int tc_gemm_tf32x3(cudaStream_t s, bool ta, bool tb, int M, int N, int K, const float *A, int lda, const float *B,
                   int ldb, float *C, int ldc, const float *bias, float *gelu_out, int accumulate, int *err);

}  // namespace dgk
