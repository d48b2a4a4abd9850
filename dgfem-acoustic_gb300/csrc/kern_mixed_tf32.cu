// Tensor-core stage kernels of the 3xTF32 form (kind::tf32 MMAs, FP32
// accumulation).
#include "kern_mixed.cuh"

namespace dgk {

bool get_mixed_kernels_tf32(int dim, int order, bool masked, int pipes, MixedKernelSet *ks) {
    return fill_kind<kTcTf32x3>(dim, order, masked, pipes, ks);
}

}  // namespace dgk
