// Tensor-core stage kernels: the exact fixed-point form (BF16 slices, exact
// accumulation) and the 3xTF32 form, and the host-side splitting of the
// operator B for each.
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
    using MS = MixedShape<DIM, P, kTcBf16x4>;
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

// 3xTF32 operator image: B[i][k] = hi + lo with hi the TF32 value nearest
// to B rounded to FP32 and lo the TF32 value nearest to the remainder; per
// K-step of 8 the hi and lo tiles follow one another along N (one MMA takes
// both), 32-bit elements in the no-swizzle K-major layout.  No exponents.
template <int DIM, int P>
void b_image_tf32(const double *ops, std::vector<uint8_t> &img, std::vector<int> &eb) {
    using MS = MixedShape<DIM, P, kTcTf32x3>;
    constexpr int NP = MS::NP, KTOT = MS::KTOT, NPAD = MS::NPAD;
    const double *D = ops;                      // [u][j][i]
    const double *L = ops + DIM * NP * NP;      // [slot][i]
    img.assign(MS::BBYTES, 0);
    eb.assign(NPAD, 0);
    for (int i = 0; i < NP; ++i)
        for (int k = 0; k < KTOT; ++k) {
            const double v = k < DIM * NP ? D[((size_t)(k / NP) * NP + k % NP) * NP + i]
                                          : L[(size_t)(k - DIM * NP) * NP + i];
            const float hi = dgtc::tf32_round((float)v);
            const float lo = dgtc::tf32_round((float)(v - (double)hi));
            const float part[2] = {hi, lo};
            for (int sl = 0; sl < 2; ++sl) {
                const size_t off = (size_t)((k / 8) * 2 + sl) * MS::BTILE + (i / 8) * 256 + ((k % 8) / 4) * 128 +
                                   (i % 8) * 16 + (k % 4) * 4;
                std::memcpy(&img[off], &part[sl], 4);
            }
        }
}

// Warp groups per CTA: 4 (512 threads) where the per-thread state fits in
// 128 registers, else 2.
template <int DIM, int P>
struct MixedWarpGroups {
    static constexpr int value = MIXED_WG;
};

template <int DIM, int P, bool MASKED, int KIND>
bool fill_variant(MixedKernelSet *ks) {
    using MS = MixedShape<DIM, P, KIND>;
    if constexpr (!MS::FITS) {
        return false;
    } else {
        constexpr int W = MixedWarpGroups<DIM, P>::value;
        ks->stage[0] = (const void *)&mixed_stage_kernel<DIM, P, 1, W, MASKED, KIND>;
        ks->stage[1] = (const void *)&mixed_stage_kernel<DIM, P, 2, W, MASKED, KIND>;
        ks->stage[2] = (const void *)&mixed_stage_kernel<DIM, P, 3, W, MASKED, KIND>;
        ks->stage[3] = (const void *)&mixed_stage_kernel<DIM, P, 4, W, MASKED, KIND>;
        ks->euler = (const void *)&mixed_stage_kernel<DIM, P, kStageEuler, W, MASKED, KIND>;
        ks->elems_per_tile = MS::ELEMS;
        ks->threads = 128 * W;
        ks->smem = MS::SMEM_LAUNCH;
        ks->b_image = KIND == kTcTf32x3 ? &b_image_tf32<DIM, P> : &b_image<DIM, P>;
        ks->npad = MS::NPAD;
        return true;
    }
}

// Meshes with curved elements take the masked kernels (element-block list and
// per-block masks); the others the plain ones.
template <int DIM, int P>
bool fill(MixedKernelSet *ks, bool masked, int kind) {
    if (kind == kTcTf32x3)
        return masked ? fill_variant<DIM, P, true, kTcTf32x3>(ks) : fill_variant<DIM, P, false, kTcTf32x3>(ks);
    return masked ? fill_variant<DIM, P, true, kTcBf16x4>(ks) : fill_variant<DIM, P, false, kTcBf16x4>(ks);
}

}  // namespace

bool get_mixed_kernels(int dim, int order, bool masked, int kind, MixedKernelSet *ks) {
    if (dim == 2) {
        switch (order) {
            case 1: return fill<2, 1>(ks, masked, kind);
            case 2: return fill<2, 2>(ks, masked, kind);
            case 3: return fill<2, 3>(ks, masked, kind);
            case 4: return fill<2, 4>(ks, masked, kind);
            case 5: return fill<2, 5>(ks, masked, kind);
        }
    } else if (dim == 3) {
        switch (order) {
            case 1: return fill<3, 1>(ks, masked, kind);
            case 2: return fill<3, 2>(ks, masked, kind);
            case 3: return fill<3, 3>(ks, masked, kind);
            case 4: return fill<3, 4>(ks, masked, kind);
        }
    }
    return false;
}

}  // namespace dgk
