// Stage kernels, double, 3D, orders 1..5.
#include "kernels_inst.cuh"

namespace dgk {
bool kernels_f64_3d(int order, KernelSet *out) { return fill_for_order<3, double>(order, out); }
}  // namespace dgk
