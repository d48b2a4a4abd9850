// Explicit instantiation helpers for the stage kernels of one precision and
// dimension; included by the kern_*.cu translation units.
#pragma once
#include "kernels.h"
#include "stage_kernel.cuh"

namespace dgk {

// Elements per block: about 128-256 threads per block.
template <int DIM, int P>
struct DefaultEpb {
    static constexpr int NP = Shape<DIM, P>::NP;
    static constexpr int value = NP <= 4 ? 32 : NP <= 6 ? 32 : NP <= 10 ? 16 : NP <= 21 ? 8 : 4;
};

template <int DIM, int P, typename Real>
bool fill_kernels(KernelSet *ks) {
    constexpr int EPB = DefaultEpb<DIM, P>::value;
    ks->stage[0] = (const void *)&stage_kernel<DIM, P, Real, 1, EPB>;
    ks->stage[1] = (const void *)&stage_kernel<DIM, P, Real, 2, EPB>;
    ks->stage[2] = (const void *)&stage_kernel<DIM, P, Real, 3, EPB>;
    ks->stage[3] = (const void *)&stage_kernel<DIM, P, Real, 4, EPB>;
    ks->euler = (const void *)&stage_kernel<DIM, P, Real, kStageEuler, EPB>;
    ks->inject = (const void *)&inject_kernel<Real>;
    ks->record = (const void *)&record_kernel<Real>;
    ks->epb = EPB;
    ks->threads = EPB * Shape<DIM, P>::NP;
    ks->smem = StageSmem<DIM, P, Real, EPB>::total;
    return true;
}

template <int DIM, typename Real>
bool fill_for_order(int order, KernelSet *ks) {
    switch (order) {
        case 1: return fill_kernels<DIM, 1, Real>(ks);
        case 2: return fill_kernels<DIM, 2, Real>(ks);
        case 3: return fill_kernels<DIM, 3, Real>(ks);
        case 4: return fill_kernels<DIM, 4, Real>(ks);
        case 5: return fill_kernels<DIM, 5, Real>(ks);
        default: return false;
    }
}

}  // namespace dgk
