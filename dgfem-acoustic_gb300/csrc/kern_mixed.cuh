// Instantiation helpers of the tensor-core stage kernels, shared by the two
// translation units that compile them (kern_mixed.cu: exact fixed-point BF16
// slices; kern_mixed_tf32.cu: 3xTF32), and the host-side splitting of the
// operator B for each kind.
#pragma once
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
            // radix 2^9 slices, |m| <= 256 (exact in BF16), as the A rows
            double x = std::ldexp(row[k], -e) * 256.0;
            for (int sl = 0; sl < MS::NSB; ++sl) {
                double m = std::nearbyint(x);
                x = (x - m) * 512.0;
                float val = (float)std::ldexp(m, -9 * sl);
                uint32_t bits;
                std::memcpy(&bits, &val, 4);
                uint16_t h = (uint16_t)(bits >> 16);
                // per K-step the four slices follow one another along N, so
                // that one MMA can take several slices as one wider operand
                size_t off = (size_t)((k / 16) * MS::NSB + sl) * MS::BTILE + (i / 8) * 256 + ((k % 16) / 8) * 128 +
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

// One tile pipeline of W warp groups per CTA, or two of W / 2 each (HALVES).
template <int DIM, int P, bool MASKED, int KIND, int HALVES>
bool fill_pipes(MixedKernelSet *ks) {
    using MS = MixedShape<DIM, P, KIND, HALVES>;
    if constexpr (!MS::RUNS) {
        return false;
    } else {
        constexpr int W = MixedWarpGroups<DIM, P>::value / HALVES;
        ks->stage[0] = (const void *)&mixed_stage_kernel<DIM, P, 1, W, MASKED, KIND, HALVES>;
        ks->stage[1] = (const void *)&mixed_stage_kernel<DIM, P, 2, W, MASKED, KIND, HALVES>;
        ks->stage[2] = (const void *)&mixed_stage_kernel<DIM, P, 3, W, MASKED, KIND, HALVES>;
        ks->stage[3] = (const void *)&mixed_stage_kernel<DIM, P, 4, W, MASKED, KIND, HALVES>;
        ks->euler = (const void *)&mixed_stage_kernel<DIM, P, kStageEuler, W, MASKED, KIND, HALVES>;
        ks->elems_per_tile = MS::ELEMS;
        ks->threads = 128 * W * HALVES;
        ks->pipes = HALVES;
        ks->smem = MS::SMEM_LAUNCH;
        ks->b_image = KIND == kTcTf32x3 ? &b_image_tf32<DIM, P> : &b_image<DIM, P>;
        ks->npad = MS::NPAD;
        return true;
    }
}

// pipes: 0 or 1 = one pipeline; 2 = two where they fit, else one
// (ks->pipes tells).  Two pipelines measured no faster on the GB300 (3D
// order 3: 66.3 against 66.9 G DOF-stage/s), so one is the default.
template <int DIM, int P, bool MASKED, int KIND>
bool fill_variant(MixedKernelSet *ks, int pipes) {
    if (pipes == 2 && fill_pipes<DIM, P, MASKED, KIND, 2>(ks)) return true;
    return fill_pipes<DIM, P, MASKED, KIND, 1>(ks);
}

// The kernels of one contraction kind for (dim, order); false if not compiled.
template <int KIND>
bool fill_kind(int dim, int order, bool masked, int pipes, MixedKernelSet *ks) {
    auto pick = [&](auto f0, auto f1) { return masked ? f1(ks, pipes) : f0(ks, pipes); };
    if (dim == 2) {
        switch (order) {
            case 1: return pick(fill_variant<2, 1, false, KIND>, fill_variant<2, 1, true, KIND>);
            case 2: return pick(fill_variant<2, 2, false, KIND>, fill_variant<2, 2, true, KIND>);
            case 3: return pick(fill_variant<2, 3, false, KIND>, fill_variant<2, 3, true, KIND>);
            case 4: return pick(fill_variant<2, 4, false, KIND>, fill_variant<2, 4, true, KIND>);
            case 5: return pick(fill_variant<2, 5, false, KIND>, fill_variant<2, 5, true, KIND>);
        }
    } else if (dim == 3) {
        switch (order) {
            case 1: return pick(fill_variant<3, 1, false, KIND>, fill_variant<3, 1, true, KIND>);
            case 2: return pick(fill_variant<3, 2, false, KIND>, fill_variant<3, 2, true, KIND>);
            case 3: return pick(fill_variant<3, 3, false, KIND>, fill_variant<3, 3, true, KIND>);
            case 4: return pick(fill_variant<3, 4, false, KIND>, fill_variant<3, 4, true, KIND>);
        }
    }
    return false;
}

}  // namespace

// defined in kern_mixed_tf32.cu
bool get_mixed_kernels_tf32(int dim, int order, bool masked, int pipes, MixedKernelSet *ks);

}  // namespace dgk
