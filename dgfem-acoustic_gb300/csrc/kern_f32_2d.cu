// Stage kernels, float, 2D, orders 1..5.
#include "kernels_inst.cuh"

namespace dgk {
bool kernels_f32_2d(int order, KernelSet *out) { return fill_for_order<2, float>(order, out); }
}  // namespace dgk
