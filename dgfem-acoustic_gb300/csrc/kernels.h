// Kernel registry: the stage kernels compiled for each (precision, dimension,
// order), looked up by the solver at context creation.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace dgk {

struct KernelSet {
    const void *stage[4] = {nullptr, nullptr, nullptr, nullptr};
    const void *inject = nullptr;
    int epb = 0;        // elements per block
    int threads = 0;    // threads per block (epb * np)
    size_t smem = 0;    // dynamic shared memory per block
};

// prec: 0 = FP64, 1 = FP32.  Returns false if not compiled.
bool get_kernels(int prec, int dim, int order, KernelSet *out);

bool kernels_f64_2d(int order, KernelSet *out);
bool kernels_f64_3d(int order, KernelSet *out);
bool kernels_f32_2d(int order, KernelSet *out);
bool kernels_f32_3d(int order, KernelSet *out);

}  // namespace dgk
