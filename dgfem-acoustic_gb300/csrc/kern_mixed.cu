// Mixed-precision stage kernels (tensor-core contraction with exact
// accumulation) and the host-side slicing of the operator B.
#include <cmath>
#include <cstring>
#include <vector>

#include "kernels.h"
#include "mixed_kernel.cuh"

#ifndef MIXED_WG
#define MIXED_WG 4
#endif

namespace dgk {

namespace {

template <int DIM, int P>
void b_image(const double *ops, std::vector<uint8_t> &img, std::vector<int> &eb) {
    using MS = MixedShape<DIM, P>;
    constexpr int NP = MS::NP, KTOT = MS::KTOT, NPAD = MS::NPAD;
    const double *D = ops;                      // [u][j][i]
    const double *L = ops + DIM * NP * NP;      // [slot][i]
    img.assign(MS::BBYTES, 0);
    eb.assign(NPAD, 0);
    std::vector<double> row(KTOT);
    for (int i = 0; i < NP; ++i) {
        double amax = 0;
        for (int k = 0; k < KTOT; ++k) {
            double v;
            if (k < DIM * NP) {
                int u = k / NP, j = k % NP;
                v = D[((size_t)u * NP + j) * NP + i];
            } else {
                v = L[(size_t)(k - DIM * NP) * NP + i];
            }
            row[k] = v;
            amax = std::fmax(amax, std::fabs(v));
        }
        int e = 0;
        if (amax > 0) std::frexp(amax, &e);
        eb[i] = e;
        for (int k = 0; k < KTOT; ++k) {
            double x = std::ldexp(row[k], -e) * 256.0;
            for (int sl = 0; sl < 4; ++sl) {
                double m = std::nearbyint(x);
                x = (x - m) * 256.0;
                float val = (float)std::ldexp(m, -8 * sl);
                uint32_t bits;
                std::memcpy(&bits, &val, 4);
                uint16_t h = (uint16_t)(bits >> 16);
                // per K-step the four slices follow one another along N, so
                // that one MMA can take several slices as one wider operand
                size_t off = (size_t)((k / 16) * 4 + sl) * MS::BTILE + (i / 8) * 256 + ((k % 16) / 8) * 128 +
                             (i % 8) * 16 + (k % 8) * 2;
                std::memcpy(&img[off], &h, 2);
            }
        }
    }
}

// Warp groups per CTA: 4 (512 threads) where the per-thread state fits in
// 128 registers, else 2.
template <int DIM, int P>
struct MixedWarpGroups {
    static constexpr int value = MIXED_WG;
};

template <int DIM, int P, bool MASKED>
bool fill_variant(MixedKernelSet *ks) {
    using MS = MixedShape<DIM, P>;
    if constexpr (!MS::FITS) {
        return false;
    } else {
        constexpr int W = MixedWarpGroups<DIM, P>::value;
        ks->stage[0] = (const void *)&mixed_stage_kernel<DIM, P, 1, W, MASKED>;
        ks->stage[1] = (const void *)&mixed_stage_kernel<DIM, P, 2, W, MASKED>;
        ks->stage[2] = (const void *)&mixed_stage_kernel<DIM, P, 3, W, MASKED>;
        ks->stage[3] = (const void *)&mixed_stage_kernel<DIM, P, 4, W, MASKED>;
        ks->euler = (const void *)&mixed_stage_kernel<DIM, P, kStageEuler, W, MASKED>;
        ks->elems_per_tile = MS::ELEMS;
        ks->threads = 128 * W;
        ks->smem = MS::SMEM_LAUNCH;
        ks->b_image = &b_image<DIM, P>;
        ks->npad = MS::NPAD;
        return true;
    }
}

// Meshes with curved elements take the masked kernels (element-block list and
// per-block masks); the others the plain ones.
template <int DIM, int P>
bool fill(MixedKernelSet *ks, bool masked) {
    return masked ? fill_variant<DIM, P, true>(ks) : fill_variant<DIM, P, false>(ks);
}

}  // namespace

bool get_mixed_kernels(int dim, int order, bool masked, MixedKernelSet *ks) {
    if (dim == 2) {
        switch (order) {
            case 1: return fill<2, 1>(ks, masked);
            case 2: return fill<2, 2>(ks, masked);
            case 3: return fill<2, 3>(ks, masked);
            case 4: return fill<2, 4>(ks, masked);
            case 5: return fill<2, 5>(ks, masked);
        }
    } else if (dim == 3) {
        switch (order) {
            case 1: return fill<3, 1>(ks, masked);
            case 2: return fill<3, 2>(ks, masked);
            case 3: return fill<3, 3>(ks, masked);
            case 4: return fill<3, 4>(ks, masked);
        }
    }
    return false;
}

}  // namespace dgk
