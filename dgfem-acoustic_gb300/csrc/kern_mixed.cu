// Tensor-core stage kernels of the exact fixed-point form (BF16 slices, exact
// accumulation) and the kind dispatch; the 3xTF32 kernels are compiled in
// kern_mixed_tf32.cu.
#include "kern_mixed.cuh"

namespace dgk {

bool get_mixed_kernels(int dim, int order, bool masked, int kind, int pipes, MixedKernelSet *ks) {
    if (kind == kTcTf32x3) return get_mixed_kernels_tf32(dim, order, masked, pipes, ks);
    return fill_kind<kTcBf16x4>(dim, order, masked, pipes, ks);
}

}  // namespace dgk
