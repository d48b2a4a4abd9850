// Stage kernels of curved elements, FP64 and FP32 stage data, 2D and 3D.
#include "curved_kernel.cuh"
#include "kernels.h"

namespace dgk {

bool get_curved_kernel(int prec, int dim, const void **fn) {
    if (prec == 0 && dim == 2) *fn = (const void *)&curved_stage_kernel<2, double>;
    else if (prec == 0 && dim == 3) *fn = (const void *)&curved_stage_kernel<3, double>;
    else if (prec == 1 && dim == 2) *fn = (const void *)&curved_stage_kernel<2, float>;
    else if (prec == 1 && dim == 3) *fn = (const void *)&curved_stage_kernel<3, float>;
    else return false;
    return true;
}

}  // namespace dgk
