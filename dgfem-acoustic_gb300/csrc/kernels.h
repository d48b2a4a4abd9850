// Kernel registry: the stage kernels compiled for each (precision, dimension,
// order), looked up by the solver at context creation.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <vector>

namespace dgk {

struct KernelSet {
    const void *stage[4] = {nullptr, nullptr, nullptr, nullptr};
    const void *euler = nullptr;  // forward-Euler step kernel
    const void *inject = nullptr;
    const void *record = nullptr;
    int epb = 0;        // elements per block
    int threads = 0;    // threads per block (epb * np)
    size_t smem = 0;    // dynamic shared memory per block
};

// prec: 0 = FP64, 1 = FP32.  Returns false if not compiled.
bool get_kernels(int prec, int dim, int order, KernelSet *out);

bool kernels_f64_2d(int order, KernelSet *out);
bool kernels_f64_3d(int order, KernelSet *out);
bool kernels_f32_2d(int order, KernelSet *out);
bool kernels_f32_3d(int order, KernelSet *out);

// Per-point stage kernel of curved elements (curved_kernel.cuh); prec as above.
bool get_curved_kernel(int prec, int dim, const void **fn);

}  // namespace dgk

namespace dgk {

// Mixed-precision (tensor-core) stage kernels of one (dimension, order).
struct MixedKernelSet {
    const void *stage[4] = {nullptr, nullptr, nullptr, nullptr};
    const void *euler = nullptr;  // forward-Euler step kernel
    int elems_per_tile = 0;
    int threads = 0;
    int pipes = 1;  // independent tile pipelines per CTA
    size_t smem = 0;
    int npad = 0;
    // builds the shared-memory image of the sliced operator and its row
    // exponents from the layout operators (D as [u][j][i], LIFT as [slot][i])
    void (*b_image)(const double *ops, std::vector<uint8_t> &img, std::vector<int> &eb) = nullptr;
};

// masked: the variant for meshes with curved elements (MixedArgs::blist and
// cmask in use).  kind: 0 = exact fixed-point BF16 slices, 1 = 3xTF32.
// pipes: tile pipelines per CTA, 0 or 1 = one, 2 = two where they fit.
bool get_mixed_kernels(int dim, int order, bool masked, int kind, int pipes, MixedKernelSet *out);

// Arguments of the mixed-precision stage kernels.
struct MixedArgs {
    const float *win;      // stage input
    const float *u;        // state, FP32 high part
    float *ulo;            // state, FP32 low part
    float *acc;
    float *wout;           // next stage input (stage 4: u)
    float *wlo;            // forward-Euler step: low part of the new state
    long long fstride;
    long long bstride;     // distance between batch members
    int nbatch;            // batch members (sources) on the mesh
    const float *geo;      // [K][DIM*DIM] inverse Jacobians rounded to FP32
    const float *fgeo;     // [K][NF][4]
    const int2 *conn;      // [K][NF]
    const uint8_t *bimg;   // B slices, shared-memory image
    const int *beb;        // B row exponents [NPAD]
    const uint8_t *tabs;
    int K;
    float dt;
    float rc2, inv_rho, half_c0, c0, rho;
    float v0[3];
    int *err;              // set to 1 on a wait timeout
    // meshes with curved elements: bit le of cmask[block] marks element
    // block*ELEMS + le as curved (its update comes from the per-point kernel,
    // this kernel leaves it alone); null when no element is curved
    const unsigned long long *cmask;
    const int *blist;      // element blocks to run (those with a straight element), or null: all
    int nblk;              // entries of blist
};


}  // namespace dgk
