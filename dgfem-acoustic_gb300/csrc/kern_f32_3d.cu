// Stage kernels, float, 3D, orders 1..5.
#include "kernels_inst.cuh"

namespace dgk {
bool kernels_f32_3d(int order, KernelSet *out) { return fill_for_order<3, float>(order, out); }
}  // namespace dgk
