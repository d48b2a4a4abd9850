// Mixed-precision stage kernel: FP32 state tiles and geometry factors, and
// the volume + lift contraction on the tensor cores with exact accumulation.
//
// For a tile of ELEMS elements the right-hand side of every (field, element)
// row r is one contraction over K = DIM*NP + NF*NFP columns,
//   C[r][i] = sum_k A[r][k] B[i][k],
//   A[r] = ( Fhat_u(j) for u, j | -(detJf/detJe) Fn(slot) ),
//   B[i] = ( D_u[i][j]          | LIFT[i][slot] ),
// so that dt*C is the stage increment (weak volume term minus lift, already
// multiplied by M^-1).  To keep the contraction at FP64-grade accuracy with
// FP32 accumulators, both operands are cut into fixed-point slices with one
// exponent per row and radix 2^9: a = 2^(ea-8) sum_s m_s 2^(-9s), |m_s| <= 256
// integer (at most 8 significant bits, so exact in BF16); A (FP32) in four
// slices (36 bits below the row scale; three, 27 bits, where tensor memory
// holds no more: 3D order 4), B (FP64 operators, sliced on the host per
// output node) in four (36 bits).  Slice products are integers (times
// 2^-9(i+j)); the pairs with i+j <= 3 are formed (the pairs with i+j >= 4
// lie 2^-36 below the row scales).  Level i+j = 0 sums exactly in
// its FP32 tensor-memory accumulator (|sum| <= K 2^16 < 2^24 for K <= 256),
// level 1 for K <= 128 (beyond, its rounding lies 2^-33 below the row
// scales), levels 2 and 3 in two more.  The epilogue adds them in
// double-FP32, scales by 2^(ea+eb-16) dt and applies the RK4 stage update
// with the state u kept as an FP32 pair.
//
// Roles (128*NWG threads, one CTA per SM, persistent over tiles): cp.async
// copies bring a tile's state, geometry, connectivity and neighbour traces
// into shared memory one tile ahead; warps 1.. build the next tile's A rows
// in shared memory (one task per element node for the volume fluxes, one per
// face slot for the face values) while warp 0 issues this tile's MMAs.
// Row r is sliced by lane r%32 of warps r/32 + 4g of every warp group g
// (warp w may only touch tensor-memory lanes 32(w%4)..32(w%4)+31), each
// group taking an equal share of the row's tensor-memory columns (and the
// largest magnitude of its share, for the row's exponent), two values at a
// time with paired FP32 instructions, and stored with tcgen05.st.  One
// thread issues the tcgen05.mma as one unrolled sequence and commits them to
// an mbarrier; every thread waits on it, and the warp groups read the
// accumulators of their row with tcgen05.ld, split by output node, for the
// epilogue.  Every wait is bounded; on timeout the kernel records an error,
// waits once more for the MMAs in flight, frees tensor memory and stops.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "stage_kernel.cuh"
#include "kernels.h"
#include "tc_ptx.cuh"

namespace dgk {

// Contraction kinds: the exact fixed-point form (four or three BF16 slices
// of each A value, four of each operator value, kind::f16 MMAs, exact
// accumulation)
// and 3xTF32 (each operand split into a high and a low TF32 part,
// a_hi b_hi + a_hi b_lo + a_lo b_hi by kind::tf32 MMAs, FP32 accumulation).
constexpr int kTcBf16x4 = 0, kTcTf32x3 = 1;

// HALVES = 2: the CTA runs two independent tile pipelines (one per half of
// its warps), each with half of the tensor memory and its own shared-memory
// region; the operator image is shared.  While one pipeline waits at a
// barrier or on its MMAs, the other's warps issue.
template <int DIM, int P, int KIND = kTcBf16x4, int HALVES = 1>
struct MixedShape {
    using S = Shape<DIM, P>;
    static constexpr bool TF = KIND == kTcTf32x3;
    static constexpr int NP = S::NP, NF = S::NF, NFP = S::NFP, NQ = S::NQ, NSLOT = S::NSLOT;
    static constexpr int NPERM = S::NPERM;
    static constexpr int KTOT = DIM * NP + NSLOT;
    static constexpr int KSTEP = TF ? 8 : 16;       // K of one MMA (32 bytes of a K-major row)
    static constexpr int KPAD = (KTOT + KSTEP - 1) / KSTEP * KSTEP;
    static constexpr int KSTEPS = KPAD / KSTEP;
    static constexpr int NPAD = (NP + 15) / 16 * 16;
    static constexpr int ELEMS = 128 / NQ;          // elements per tile
    static constexpr int TMEM_COLS = 512 / HALVES;  // tensor-memory columns of one pipeline
    static constexpr int NSB = TF ? 2 : 4;          // parts of each operator value
    // parts of each A value: four BF16 slices where their columns (two K
    // values per column) and the four level accumulators fit, else three
    static constexpr int NSA = TF ? 2 : (4 * (KPAD / 2) + 4 * NPAD <= TMEM_COLS ? 4 : 3);
    // Tensor-memory columns of one A part: BF16 packs two K values per
    // column, TF32 takes one.
    static constexpr int ACOLS = TF ? KPAD : KPAD / 2;
    // Level scheme: one accumulator per level L = i+j of the slice pairs
    // (0..3).  The B slices of a K-step lie side by side along N, so A slice
    // i meets B slices 0..3-i in one MMA of N = (4-i) x NPAD, accumulating
    // into levels i..3: one MMA per A slice and K-step.
    // 3xTF32: the two A parts of every K-step (one 32-bit value per column)
    // and two accumulators (a_hi b_hi + a_lo b_hi, a_hi b_lo).
    static constexpr int ACC = TF ? (2 * ACOLS + 31) / 32 * 32 : NSA * ACOLS;  // first accumulator column
    static constexpr int NACC = TF ? 2 : NSB;
    static constexpr bool FITS = ACC + NACC * NPAD <= TMEM_COLS && NSB * NPAD <= 256;
    static constexpr int NX = NACC - 2;             // accumulators past the first two
    static constexpr int BTILE = NPAD * 32;         // bytes of one (K-step, slice) B tile; image [K-step][slice]
    static constexpr int BBYTES = NSB * KSTEPS * BTILE;
    static constexpr int QS = NP;                   // element stride in the state tile
    // row stride of the staged A rows: even, so that column pairs are 8-byte
    // loads, with KSTR/2 odd, so that the 8-byte loads of 16 consecutive
    // rows fall in distinct banks
    static constexpr int KSTR = KPAD + 2;
    static constexpr int MAX_WG = 4;                // warp groups per CTA (4 warps each), at most
    // shared memory layout (bytes)
    static constexpr int r16(int x) { return (x + 15) / 16 * 16; }
    static constexpr int OFF_B = 0;                                   // sliced operator image
    // pipeline 0's region starts here; pipeline h's at + h * HSTRIDE
    static constexpr int HBASE = r16(OFF_B + BBYTES);
    static constexpr int OFF_Q = HBASE;                               // state tile [f][le][QS]
    static constexpr int OFF_NBR = r16(OFF_Q + NQ * ELEMS * QS * 4);  // neighbour traces [task][4]
    static constexpr int OFF_A = r16(OFF_NBR + ELEMS * NSLOT * 16);   // FP32 A rows [128][KSTR]
    static constexpr int OFF_GEO = OFF_A + 128 * KSTR * 4;            // [le][DIM*DIM] floats
    static constexpr int OFF_CONN = r16(OFF_GEO + ELEMS * DIM * DIM * 4);  // 2 x [le][NF] int2
    static constexpr int CONN_BYTES = r16(ELEMS * NF * 8);
    static constexpr int OFF_FGEO = OFF_CONN + 2 * CONN_BYTES;         // [le][NF] float4
    static constexpr int OFF_MAX = OFF_FGEO + ELEMS * NF * 16;
    static constexpr int OFF_TAB = OFF_MAX + MAX_WG * 128 * 4;       // [MAX_WG][128] row maxima
    static constexpr int OFF_EB = r16(OFF_TAB + S::NTAB);
    // Overlap: the next tile's A rows are built while this tile's MMAs run,
    // so the epilogue stages its outputs outside the A-row region: in a
    // region of their own where shared memory allows, else in the state-tile
    // and neighbour-trace regions (adjacent; the next tile's rows, built
    // from them, are complete before the epilogue starts, and its copies
    // into them start after it).
    static constexpr int OUT_FLOATS = 2 * NQ * ELEMS * NP;
    static constexpr int OFF_OUT_OWN = r16(OFF_EB + NPAD * 4);
    static constexpr bool OUT_OWN =
        HBASE + HALVES * (r16(OFF_OUT_OWN + OUT_FLOATS * 4 + 16) - HBASE) <= 227 * 1024;
    static constexpr bool OUT_ALIAS = !OUT_OWN && OUT_FLOATS * 4 <= OFF_A - OFF_Q;
    static constexpr bool OVERLAP = OUT_OWN || OUT_ALIAS;
    static constexpr int OFF_OUT = OUT_OWN ? OFF_OUT_OWN : OFF_Q;
    static constexpr int OFF_BAR = OUT_OWN ? r16(OFF_OUT + OUT_FLOATS * 4) : OFF_EB + NPAD * 4;
    // [OFF_BAR, +16): the mbarrier, the tensor-memory base, the error flag
    static constexpr int HSTRIDE = r16(OFF_BAR + 16) - HBASE;         // bytes of one pipeline's region
    static constexpr int SMEM = HBASE + HALVES * HSTRIDE;
    // the shape runs when both tensor memory and shared memory suffice
    static constexpr bool RUNS = FITS && SMEM <= 227 * 1024 && OVERLAP;
    // the epilogue stages the tile's two output arrays in the A-row region
    static_assert(2 * NQ * ELEMS * NP <= 128 * KSTR, "output staging fits in the A-row region");
    static_assert(HALVES == 2 || SMEM <= 227 * 1024, "tile does not fit in shared memory");
    static_assert(!OUT_ALIAS || (OFF_Q + OUT_FLOATS * 4 <= OFF_A && OFF_NBR > OFF_Q && OFF_A > OFF_NBR),
                  "aliased output staging stays inside the state-tile and neighbour-trace regions");
    // at least half of the SM's shared memory, so one CTA (the tensor-memory
    // owner) runs per SM
    static constexpr int SMEM_LAUNCH = SMEM < 118 * 1024 ? 118 * 1024 : SMEM;
    static_assert(BBYTES <= 256 * 1024 - 16, "operator image descriptors stay inside the 14-bit address field");
};

// (hi, lo) = a + b exactly (Knuth two-sum).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Exponent e with |x| < 2^e for the largest |x| of a row (frexp convention);
// 0 for a zero row.
__device__ __forceinline__ int row_exponent(float amax) {
    const unsigned bits = __float_as_uint(amax);
    if (amax == 0.0f) return 0;
    const int ef = (int)((bits >> 23) & 0xffu);
    return ef == 0 ? -126 : ef - 126;
}

// 2^k as a float for -126 <= k <= 127.
__device__ __forceinline__ float exp2i(int k) { return __uint_as_float((unsigned)(k + 127) << 23); }

// NS (3 or 4) BF16 fixed-point slices of y = x*scale (|y| < 256):
// s0 + s1 + ... with s_k a multiple of 2^-9k and |s_k| <= 256 * 2^-9k (at
// most 8 significant bits, so exact in BF16).  Rounding to a multiple of
// 2^-9k is done by adding and subtracting 1.5 * 2^(23-9k) (round to nearest
// even, as rintf of the scaled value; full-rate additions instead of
// conversions); x*scale is exact (scale is a power of two), so the first
// rounding and the first remainder are single fused multiply-adds, and each
// remainder is exact.  What is left, |y - sum s_k| <= 2^-(9 NS - 8), is
// dropped.
template <int NS>
__device__ __forceinline__ void slice_fixed(float x, float scale, float (&m)[NS]) {
    static_assert(NS == 3 || NS == 4, "three or four slices");
    m[0] = __fsub_rn(__fmaf_rn(x, scale, 12582912.0f), 12582912.0f);  // 1.5 * 2^23
    const float r1 = __fmaf_rn(x, scale, -m[0]);
    m[1] = __fsub_rn(__fadd_rn(r1, 24576.0f), 24576.0f);  // 1.5 * 2^14
    const float r2 = __fsub_rn(r1, m[1]);
    m[2] = __fsub_rn(__fadd_rn(r2, 48.0f), 48.0f);  // 1.5 * 2^5
    if constexpr (NS == 4) {
        const float r3 = __fsub_rn(r2, m[2]);
        m[3] = __fsub_rn(__fadd_rn(r3, 0.09375f), 0.09375f);  // 1.5 * 2^-4
    }
}

// slice_fixed for two values at once (paired FP32 instructions); slice s of
// both values goes to w[s] as two BF16 halves (low = first value).
template <int NS>
__device__ __forceinline__ void slice_fixed_pair(dgtc::f32x2 x, dgtc::f32x2 scale, uint32_t (&w)[NS]) {
    static_assert(NS == 3 || NS == 4, "three or four slices");
    using namespace dgtc;
    const f32x2 M0 = f2_splat(12582912.0f), M1 = f2_splat(24576.0f), M2 = f2_splat(48.0f);
    f32x2 z = f2_fma(x, scale, M0);
    f32x2 r = f2_fma(x, scale, f2_sub(M0, z));  // y - s0, exact
    f32x2 m = f2_sub(z, M0);
    w[0] = __byte_perm(f2_lo_bits(m), f2_hi_bits(m), 0x7632);
    m = f2_sub(f2_add(r, M1), M1);
    w[1] = __byte_perm(f2_lo_bits(m), f2_hi_bits(m), 0x7632);
    r = f2_sub(r, m);
    m = f2_sub(f2_add(r, M2), M2);
    w[2] = __byte_perm(f2_lo_bits(m), f2_hi_bits(m), 0x7632);
    if constexpr (NS == 4) {
        const f32x2 M3 = f2_splat(0.09375f);
        r = f2_sub(r, m);
        m = f2_sub(f2_add(r, M3), M3);
        w[3] = __byte_perm(f2_lo_bits(m), f2_hi_bits(m), 0x7632);
    }
}

// Two values exactly representable in BF16, packed low = first, high =
// second: their upper halves (a byte permute, no rounding needed).
__device__ __forceinline__ uint32_t bf16x2_bits(float lo, float hi) {
    return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632);
}

// Slices CW tensor-memory columns of row arow, from column col on, into
// the A parts and stores them at taddr (part p at taddr + p * ACOLS): BF16,
// two K values per column, NS fixed-point slices with scale sc; 3xTF32,
// one value per column, its TF32 high part and remainder.  PADDED: the staged
// rows hold zeros past KTOT and dead rows hold zeros (no guards; the BF16
// path reads column pairs as 8-byte loads and slices them with paired
// instructions); else columns past KTOT and rows that are not live get zeros.
template <int KIND, int NS, int KTOT, int ACOLS, int CW, bool PADDED>
__device__ __forceinline__ void slice_columns(const float *arow, bool live, float sc, int col, uint32_t taddr) {
    if constexpr (KIND == kTcTf32x3) {
        uint32_t wh[CW], wl[CW];
#pragma unroll
        for (int h = 0; h < CW; ++h) {
            const int k = col + h;
            const float x = PADDED ? arow[k] : (live && k < KTOT) ? arow[k] : 0.0f;
            const float xh = dgtc::tf32_round(x);
            wh[h] = __float_as_uint(xh);
            wl[h] = __float_as_uint(dgtc::tf32_round(x - xh));
        }
        __syncwarp();
        dgtc::tmem_st_n<CW>(taddr, wh);
        dgtc::tmem_st_n<CW>(taddr + ACOLS, wl);
    } else if constexpr (PADDED) {
        uint32_t w[NS][CW];
        const dgtc::f32x2 sc2 = dgtc::f2_splat(sc);
#pragma unroll
        for (int h = 0; h < CW; ++h) {
            const float2 v = *reinterpret_cast<const float2 *>(&arow[2 * (col + h)]);
            uint32_t ws[NS];
            slice_fixed_pair<NS>(dgtc::f2_make(v.x, v.y), sc2, ws);
#pragma unroll
            for (int sl = 0; sl < NS; ++sl) w[sl][h] = ws[sl];
        }
        __syncwarp();
#pragma unroll
        for (int sl = 0; sl < NS; ++sl) dgtc::tmem_st_n<CW>(taddr + sl * ACOLS, w[sl]);
    } else {
        uint32_t w[NS][CW];
#pragma unroll
        for (int h = 0; h < CW; ++h) {
            const int k = 2 * (col + h);
            const float x0 = (live && k < KTOT) ? arow[k] : 0.0f;
            const float x1 = (live && k + 1 < KTOT) ? arow[k + 1] : 0.0f;
            float m0[NS], m1[NS];
            slice_fixed<NS>(x0, sc, m0);
            slice_fixed<NS>(x1, sc, m1);
#pragma unroll
            for (int sl = 0; sl < NS; ++sl) w[sl][h] = bf16x2_bits(m0[sl], m1[sl]);
        }
        __syncwarp();
#pragma unroll
        for (int sl = 0; sl < NS; ++sl) dgtc::tmem_st_n<CW>(taddr + sl * ACOLS, w[sl]);
    }
}

// Issues the cp.async copies of a tile's connectivity words into buffer cb;
// the calling threads take words first, first + stride, ...
template <int DIM, int P, int KIND>
__device__ __forceinline__ void issue_conn_copies(const MixedArgs &a, unsigned char *smem, long long ebase, int cb,
                                                  int first, int stride) {
    using MS = MixedShape<DIM, P, KIND>;
    constexpr int NF = MS::NF, ELEMS = MS::ELEMS;
    int2 *sConn = reinterpret_cast<int2 *>(smem + MS::OFF_CONN + cb * MS::CONN_BYTES);
    static_assert(ELEMS * NF % 2 == 0, "a tile's connectivity words are whole 16-byte chunks");
    if (ebase + ELEMS <= a.K && ((uintptr_t)a.conn & 15u) == 0) {
        for (int idx = first; idx < ELEMS * NF / 2; idx += stride)
            dgtc::cp_async16(&sConn[2 * idx], &a.conn[ebase * NF + 2 * idx], 16u);
    } else {
        for (int idx = first; idx < ELEMS * NF; idx += stride) {
            const bool ok = ebase + idx / NF < a.K;
            dgtc::cp_async8(&sConn[idx], ok ? &a.conn[ebase * NF + idx] : a.conn, ok ? 8u : 0u);
        }
    }
}

// Issues the cp.async copies of a tile's element data: state, inverse
// Jacobians and face geometry (zero-filled past K).
template <int DIM, int P, int KIND>
__device__ __forceinline__ void issue_tile_copies(const MixedArgs &a, unsigned char *smem, long long ebase,
                                                  long long moff, bool vec, int first, int stride) {
    using MS = MixedShape<DIM, P, KIND>;
    constexpr int NP = MS::NP, NF = MS::NF, NQ = MS::NQ, ELEMS = MS::ELEMS, QS = MS::QS;
    static_assert(QS == NP, "the state tile is stored unpadded, as in global memory");
    float *sQ = reinterpret_cast<float *>(smem + MS::OFF_Q);
    float *sGeo = reinterpret_cast<float *>(smem + MS::OFF_GEO);
    float4 *sFgeo = reinterpret_cast<float4 *>(smem + MS::OFF_FGEO);
    if (vec && ebase + ELEMS <= a.K) {
        // a whole tile of 16-byte aligned fields: 16-byte copies
        constexpr int W = ELEMS * NP / 4;
        for (int idx = first; idx < NQ * W; idx += stride) {
            const int f = idx / W, w = idx - f * W;
            dgtc::cp_async16(&sQ[f * ELEMS * NP + 4 * w], &a.win[moff + f * a.fstride + ebase * NP + 4 * w], 16u);
        }
    } else {
        for (int idx = first; idx < NQ * ELEMS * NP; idx += stride) {
            const int f = idx / (ELEMS * NP), rem = idx - f * (ELEMS * NP);
            const bool ok = ebase + rem / NP < a.K;
            const float *src = ok ? &a.win[moff + f * a.fstride + ebase * NP + rem] : a.win;
            dgtc::cp_async4(&sQ[f * ELEMS * NP + rem], src, ok ? 4u : 0u);
        }
    }
    static_assert(ELEMS * DIM * DIM % 4 == 0, "a tile's geometry factors are whole 16-byte chunks");
    if (ebase + ELEMS <= a.K && ((uintptr_t)a.geo & 15u) == 0) {
        for (int idx = first; idx < ELEMS * DIM * DIM / 4; idx += stride)
            dgtc::cp_async16(&sGeo[4 * idx], &a.geo[ebase * DIM * DIM + 4 * idx], 16u);
    } else {
        for (int idx = first; idx < ELEMS * DIM * DIM; idx += stride) {
            const bool ok = ebase + idx / (DIM * DIM) < a.K;
            dgtc::cp_async4(&sGeo[idx], ok ? &a.geo[ebase * DIM * DIM + idx] : a.geo, ok ? 4u : 0u);
        }
    }
    for (int idx = first; idx < ELEMS * NF; idx += stride) {
        const bool ok = ebase + idx / NF < a.K;
        dgtc::cp_async16(&sFgeo[idx], ok ? &a.fgeo[(ebase * NF + idx) * 4] : a.fgeo, ok ? 16u : 0u);
    }
}

// Issues the cp.async gathers of the neighbour traces of a tile's interior
// face slots (reads the tile's connectivity words from buffer cb); the
// calling threads take tasks first, first + stride, ...
template <int DIM, int P, int KIND>
__device__ __forceinline__ void issue_neighbour_copies(const MixedArgs &a, unsigned char *smem, long long ebase,
                                                       long long moff, int cb, int first, int stride) {
    using MS = MixedShape<DIM, P, KIND>;
    constexpr int NP = MS::NP, NF = MS::NF, NFP = MS::NFP, NQ = MS::NQ, NSLOT = MS::NSLOT, ELEMS = MS::ELEMS;
    float *sNbr = reinterpret_cast<float *>(smem + MS::OFF_NBR);
    const int2 *sConn = reinterpret_cast<const int2 *>(smem + MS::OFF_CONN + cb * MS::CONN_BYTES);
    const uint8_t *sFmask = smem + MS::OFF_TAB;
    const uint8_t *sPerm = sFmask + NF * NFP;
    for (int task = first; task < ELEMS * NSLOT; task += stride) {
        const int le = task / NSLOT, s = task - le * NSLOT;
        const int lf = s / NFP, k = s - lf * NFP;
        if (ebase + le >= a.K) continue;
        const int2 cn = sConn[le * NF + lf];
        if (((cn.y >> 5) & 3) != kKindInterior) continue;
        const int nlf = cn.y & 3, pm = (cn.y >> 2) & 7;
        const long long nb = (long long)cn.x * NP + sFmask[nlf * NFP + sPerm[pm * NFP + k]];
#pragma unroll
        for (int f = 0; f < NQ; ++f) dgtc::cp_async4(&sNbr[task * 4 + f], &a.win[moff + f * a.fstride + nb], 4u);
    }
}

// Phase 2: the tile's A rows in shared memory (FP32): contravariant volume
// fluxes (one task per element node) and the face values negated and scaled
// by detJf/detJe (one task per face slot), from the tile's state, geometry,
// connectivity words (buffer cb) and neighbour traces.  The calling threads
// take the volume tasks first, first + stride, ... (stride a multiple of 32,
// first - lane the same for the lanes of a warp) and the face tasks with the
// warps in reverse order, so that the warps with one volume task more than
// others get one face task less.
template <int DIM, int P, int KIND>
__device__ __forceinline__ void build_rows(const MixedArgs &a, unsigned char *smem, long long ebase, int cb, int first,
                                           int stride) {
    using MS = MixedShape<DIM, P, KIND>;
    constexpr int NP = MS::NP, NF = MS::NF, NFP = MS::NFP, NQ = MS::NQ, NSLOT = MS::NSLOT;
    constexpr int ELEMS = MS::ELEMS, QS = MS::QS, KSTR = MS::KSTR;
    const float *sQ = reinterpret_cast<const float *>(smem + MS::OFF_Q);
    float *sA = reinterpret_cast<float *>(smem + MS::OFF_A);
    const float4 *sNbr = reinterpret_cast<const float4 *>(smem + MS::OFF_NBR);
    const float *sGeo = reinterpret_cast<const float *>(smem + MS::OFF_GEO);
    const int2 *sConn = reinterpret_cast<const int2 *>(smem + MS::OFF_CONN + cb * MS::CONN_BYTES);
    const float4 *sFgeo = reinterpret_cast<const float4 *>(smem + MS::OFF_FGEO);
    const uint8_t *sFmask = smem + MS::OFF_TAB;
    const int lane = (int)(threadIdx.x & 31);
    // 2a. contravariant fluxes, one task per element node
    for (int task = first; task < ELEMS * NP; task += stride) {
        const int le = task / NP, j = task - le * NP;
        float Bg[DIM][DIM];
#pragma unroll
        for (int x = 0; x < DIM; ++x)
#pragma unroll
            for (int u = 0; u < DIM; ++u) Bg[x][u] = sGeo[le * DIM * DIM + x * DIM + u];
        float q[NQ];
#pragma unroll
        for (int f = 0; f < NQ; ++f) q[f] = sQ[(f * ELEMS + le) * QS + j];
#pragma unroll
        for (int u = 0; u < DIM; ++u) {
            float au = 0.0f, w = 0.0f;
#pragma unroll
            for (int x = 0; x < DIM; ++x) {
                au = fmaf(Bg[x][u], a.v0[x], au);
                w = fmaf(Bg[x][u], q[1 + x], w);
            }
            sA[(0 * ELEMS + le) * KSTR + u * NP + j] = fmaf(au, q[0], a.rc2 * w);
            const float pr = a.inv_rho * q[0];
#pragma unroll
            for (int d = 0; d < DIM; ++d)
                sA[((1 + d) * ELEMS + le) * KSTR + u * NP + j] = fmaf(au, q[1 + d], pr * Bg[d][u]);
        }
    }
    // 2b. face values, negated and scaled: -(detJf/detJe) Fn
    for (int task = stride - 32 - (first - lane) + lane; task < ELEMS * NSLOT; task += stride) {
        const int le = task / NSLOT, s = task - le * NSLOT;
        const int lf = s / NFP, k = s - lf * NFP;
        float Fn[NQ];
#pragma unroll
        for (int f = 0; f < NQ; ++f) Fn[f] = 0.0f;
        float scale = 0.0f;
        if (ebase + le < a.K) {
            const int vi = sFmask[lf * NFP + k];
            float own[NQ];
#pragma unroll
            for (int f = 0; f < NQ; ++f) own[f] = sQ[(f * ELEMS + le) * QS + vi];
            const int2 cn = sConn[le * NF + lf];
            const float4 g4 = sFgeo[le * NF + lf];
            const float gg[4] = {g4.x, g4.y, g4.z, g4.w};
            float n[DIM];
#pragma unroll
            for (int x = 0; x < DIM; ++x) n[x] = gg[x];
            scale = gg[DIM];
            float vn0 = 0.0f;
#pragma unroll
            for (int x = 0; x < DIM; ++x) vn0 = fmaf(a.v0[x], n[x], vn0);
            const int kind = (cn.y >> 5) & 3;
            if (kind == kKindInterior) {
                const float4 o4 = sNbr[task];
                const float o[4] = {o4.x, o4.y, o4.z, o4.w};
                const float tau = (cn.y & 128) ? -1.0f : 1.0f;
                const float sp = own[0] + o[0];
                float svn = 0.0f;
#pragma unroll
                for (int x = 0; x < DIM; ++x) svn = fmaf(own[1 + x] + o[1 + x], n[x], svn);
                const float hj = a.half_c0 * tau;
                Fn[0] = fmaf(hj, own[0] - o[0], 0.5f * fmaf(vn0, sp, a.rc2 * svn));
#pragma unroll
                for (int d = 0; d < DIM; ++d)
                    Fn[1 + d] = fmaf(hj, own[1 + d] - o[1 + d],
                                     0.5f * fmaf(vn0, own[1 + d] + o[1 + d], a.inv_rho * sp * n[d]));
            } else if (kind == kKindReflecting) {
                float vn = 0.0f;
#pragma unroll
                for (int x = 0; x < DIM; ++x) vn = fmaf(own[1 + x], n[x], vn);
                float vw[DIM], vwn = 0.0f;
#pragma unroll
                for (int x = 0; x < DIM; ++x) {
                    vw[x] = own[1 + x] - vn * n[x];
                    vwn = fmaf(vw[x], n[x], vwn);
                }
                Fn[0] = fmaf(vn0, own[0], a.rc2 * vwn);
#pragma unroll
                for (int d = 0; d < DIM; ++d) Fn[1 + d] = fmaf(vn0, vw[d], a.inv_rho * own[0] * n[d]);
            } else {
                float vn = 0.0f;
#pragma unroll
                for (int x = 0; x < DIM; ++x) vn = fmaf(own[1 + x], n[x], vn);
                const float q0 = 0.25f * a.c0;
                Fn[0] = fmaf(q0, own[0], 0.25f * a.c0 * a.c0 * a.rho * vn);
#pragma unroll
                for (int d = 0; d < DIM; ++d) Fn[1 + d] = fmaf(0.25f * n[d] * a.inv_rho, own[0], q0 * n[d] * vn);
            }
        }
#pragma unroll
        for (int f = 0; f < NQ; ++f) sA[(f * ELEMS + le) * KSTR + DIM * NP + s] = -scale * Fn[f];
    }
}

// The MMAs of K-steps [T0, T1) into the accumulator set at dacc, every
// instruction unrolled with its operands known at compile time up to the
// tensor-memory base and the operator image's descriptor (a loop over the
// K-steps issues each tcgen05.mma at about half the rate).  3xTF32: per
// K-step a_hi against [b_hi | b_lo] into both accumulators, then a_lo
// against b_hi into the first.  Fixed-point slices: A slice i against B
// slices 0..3-i into levels i..3; A slice 0 at K-step T0 starts all four
// levels.
template <int DIM, int P, int KIND, int T0, int T1>
__device__ __forceinline__ void issue_mmas(uint32_t dacc, uint32_t tbase, uint64_t bd0) {
    using MS = MixedShape<DIM, P, KIND>;
    constexpr int NPAD = MS::NPAD, ACOLS = MS::ACOLS;
#pragma unroll
    for (int t = T0; t < T1; ++t) {
        // start address field (bits 0-13) in 16-byte units: the image stays
        // below 256 KB, so adding the offset does not carry out of the field
        const uint64_t bd = bd0 + (uint64_t)((t * MS::NSB * MS::BTILE) >> 4);
        if constexpr (MS::TF) {
            dgtc::mma_tf32_ts(dacc, tbase + t * 8, bd, dgtc::idesc_tf32_f32(128, 2 * NPAD), t > T0 ? 1u : 0u);
            dgtc::mma_tf32_ts(dacc, tbase + ACOLS + t * 8, bd, dgtc::idesc_tf32_f32(128, NPAD), 1u);
        } else {
#pragma unroll
            for (int ia = 0; ia < MS::NSA; ++ia)
                dgtc::mma_bf16_ts(dacc + ia * NPAD, tbase + ia * ACOLS + t * 8, bd,
                                  dgtc::idesc_bf16_f32(128, (MS::NSB - ia) * NPAD), (t > T0 || ia > 0) ? 1u : 0u);
        }
    }
}

// N (4 or 8) consecutive tensor-memory columns of the warp's lanes.
template <int N>
__device__ __forceinline__ void ld_cols(uint32_t taddr, uint32_t (&v)[N]) {
    static_assert(N == 4 || N == 8, "4 or 8 columns");
    if constexpr (N == 8) dgtc::tmem_ld8(taddr, v);
    else dgtc::tmem_ld4(taddr, v);
}

// Barrier of one tile pipeline: the whole CTA when it runs one pipeline, else
// named barrier `id` over that pipeline's `count` threads.
template <int HALVES>
__device__ __forceinline__ void pipe_sync(int id, int count) {
    if constexpr (HALVES == 1) {
        __syncthreads();
    } else {
        asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
    }
}

template <int DIM, int P, int STAGE, int NWG, bool MASKED, int KIND, int HALVES>
__global__ void __launch_bounds__(128 * NWG * HALVES, 1) mixed_stage_kernel(const MixedArgs a) {
    using MS = MixedShape<DIM, P, KIND, HALVES>;
    using MS1 = MixedShape<DIM, P, KIND, 1>;  // the helpers' layout: the same region offsets
    static_assert(MS1::OFF_A == MS::OFF_A && MS1::OFF_MAX == MS::OFF_MAX && MS1::OFF_TAB == MS::OFF_TAB &&
                      MS1::OFF_EB == MS::OFF_EB && MS1::OFF_CONN == MS::OFF_CONN && MS1::OFF_FGEO == MS::OFF_FGEO,
                  "per-pipeline regions keep the one-pipeline offsets");
    static_assert(MS::RUNS, "tile does not fit");
    constexpr int NP = MS::NP, NQ = MS::NQ;
    constexpr int ELEMS = MS::ELEMS, KTOT = MS::KTOT, KSTEPS = MS::KSTEPS, KSTR = MS::KSTR;
    constexpr int NPAD = MS::NPAD, ACOLS = MS::ACOLS;
    constexpr int NT = 128 * NWG;                       // threads of one pipeline
    constexpr int NTC = NT * HALVES;                    // threads of the CTA
    // tensor-memory columns of one A part that hold K values, and the
    // columns each warp group slices
    constexpr int NCOL = MS::TF ? KTOT : (KTOT + 1) / 2;
    constexpr int CPG = (NCOL + NWG - 1) / NWG;
    static_assert(NWG * CPG <= ACOLS, "the warp groups' columns stay inside each A part");
    constexpr int NPP = (NP + NWG - 1) / NWG;           // output nodes per warp group in the epilogue
    constexpr int EC = 8;                               // output nodes per tensor-memory load in the epilogue
    constexpr int NCH = (NPP + EC - 1) / EC;            // loads per accumulator
    static_assert(MS::FITS, "tile does not fit in tensor memory");
    static_assert(NWG >= 1 && NWG <= MS::MAX_WG, "warp groups");
    constexpr int NX = MS::NX;
    constexpr bool OVERLAP = MS::OVERLAP;
    constexpr int NBW = 4 * NWG - 1;                     // warps that build rows while the MMAs run
    static_assert(OVERLAP, "the next tile's rows are built while the MMAs run");
    static_assert(MS::ACC + (MS::NACC - 1) * NPAD + (NWG - 1) * NPP + EC * NCH <= MS::TMEM_COLS,
                  "epilogue loads stay inside the allocation");
    static_assert(ELEMS <= 64, "curved-element mask holds 64 elements per tile");
    extern __shared__ __align__(1024) unsigned char smem_cta[];
    // pipeline of this thread, its index and warp inside the pipeline, and
    // its pipeline's shared-memory region (the operator image is shared)
    const int pipe = HALVES == 1 ? 0 : (int)(threadIdx.x / NT);
    const int tid = (int)threadIdx.x - pipe * NT, warp = tid >> 5, lane = tid & 31;
    unsigned char *const smem = smem_cta + pipe * MS::HSTRIDE;
    // named barrier of this pipeline (all its threads)
    const int bar_all = 1 + pipe;
    // the row builders (every warp but warp 0, which issues the MMAs) and
    // their index
    const bool builder = warp != 0;
    const int bidx = tid - 32;
    float *sA = reinterpret_cast<float *>(smem + MS::OFF_A);
    float *sMax = reinterpret_cast<float *>(smem + MS::OFF_MAX);
    uint8_t *sTab = smem + MS::OFF_TAB;
    int *sEb = reinterpret_cast<int *>(smem + MS::OFF_EB);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + MS::OFF_BAR);
    uint32_t *sTmem = reinterpret_cast<uint32_t *>(smem_cta + MS::OFF_BAR + 8);  // pipeline 0's slot
    int *sFail = reinterpret_cast<int *>(smem + MS::OFF_BAR + 12);

    if (threadIdx.x < 32) {
        dgtc::tmem_alloc(sTmem, MS::TMEM_COLS * HALVES);
        dgtc::tmem_relinquish();
    }
    if (tid == 0) {
        dgtc::mbar_init(bar, 1);
        dgtc::fence_mbar_init();
        *sFail = 0;
    }
    {
        const uint4 *src = reinterpret_cast<const uint4 *>(a.bimg);
        uint4 *dst = reinterpret_cast<uint4 *>(smem_cta + MS::OFF_B);
        for (int k = threadIdx.x; k < MS::BBYTES / 16; k += NTC) dst[k] = src[k];
        for (int k = tid; k < Shape<DIM, P>::NTAB; k += NT) sTab[k] = a.tabs[k];
        for (int k = tid; k < NPAD; k += NT) sEb[k] = a.beb[k];
        // the A-row staging holds zeros past KTOT and in the rows past the
        // tile's (field, element) rows; no phase writes there afterwards (the
        // epilogue stages its outputs in a region of their own or in the
        // state-tile and neighbour-trace regions)
        for (int k = tid; k < 128 * MS::KSTR; k += NT) {
            const int rr = k / MS::KSTR, kk = k - rr * MS::KSTR;
            if (kk >= KTOT || rr >= NQ * ELEMS) sA[k] = 0.0f;
        }
    }
    dgtc::fence_proxy_async_smem();
    dgtc::fence_before_sync();
    __syncthreads();
    dgtc::fence_after_sync();
    // this pipeline's tensor-memory columns
    const uint32_t tbase = *sTmem + (uint32_t)(pipe * MS::TMEM_COLS);
    // A-part columns past the warp groups' shares hold no K values: they meet
    // zero operator rows, but must hold finite values, so they are zeroed once
    constexpr int PADC = ACOLS - NWG * CPG;
    static_assert(PADC < 16, "pad columns");
    if constexpr (PADC > 0) {
        if (warp < 4) {
            const uint32_t zero[16] = {};
#pragma unroll
            for (int pt = 0; pt < MS::NSA; ++pt)
                dgtc::tmem_st_n<PADC>(dgtc::tmem_lane_addr(tbase, warp, pt * ACOLS + NWG * CPG), zero);
            dgtc::tmem_st_wait();
        }
    }
    const uint32_t sB = dgtc::smem_u32(smem_cta + MS::OFF_B);
    // row of this thread in phases 3 and 5, and which part of the row's work
    // (K-steps when slicing, output nodes in the epilogue) its warp group takes
    const int r = (warp & 3) * 32 + lane;
    const int part = warp >> 2;
    // whole tiles move as 16-byte vectors when every field starts on 16 bytes
    float *const out_lo = STAGE <= 3 ? a.acc : STAGE == kStageEuler ? a.wlo : a.ulo;
    const bool vec = (a.fstride % 4 == 0) && (a.bstride % 4 == 0) && ((ELEMS * NP) % 4 == 0) &&
                     (((uintptr_t)a.win | (uintptr_t)a.wout | (uintptr_t)out_lo) % 16 == 0);
    const int rf = r / ELEMS, rle = r - rf * ELEMS;
    bool alive = true;
    uint32_t phase = 0;

    // Software pipeline over the CTA's tiles (cp.async groups): tile t+1's
    // connectivity words are copied while tile t's fluxes are built, its state,
    // geometry and neighbour traces while tile t is sliced, contracted and
    // written back.  Tile T covers element block T / nbatch of batch member
    // T % nbatch (members of one block are adjacent, so the block's geometry
    // is reused from L2).
    // (tile counts stay below 2^31, checked on the host: 32-bit division,
    // none at all for a single member)
    // MASKED (meshes with curved elements): only the element blocks in
    // a.blist (those with at least one straight element), curved elements
    // left alone
    const long long nblocks = MASKED ? (long long)a.nblk : (long long)((a.K + ELEMS - 1) / ELEMS);
    const long long ntiles = nblocks * a.nbatch;
    const unsigned nbu = (unsigned)a.nbatch;
    auto tile_base = [&](long long T, long long &eb, long long &mo) {
        const unsigned t32 = (unsigned)T;
        const unsigned et = nbu == 1u ? t32 : t32 / nbu;
        const unsigned blk = MASKED ? (unsigned)__ldg(&a.blist[et]) : et;
        eb = (long long)blk * ELEMS;
        mo = (long long)(t32 - et * nbu) * a.bstride;
    };
    // tiles of this pipeline: tfirst, tfirst + tstride, ...
    const long long tfirst = (long long)blockIdx.x * HALVES + pipe;
    const long long tstride = (long long)gridDim.x * HALVES;
    if (tfirst < ntiles) {
        long long eb, mo;
        tile_base(tfirst, eb, mo);
        issue_conn_copies<DIM, P, KIND>(a, smem, eb, 0, tid, NT);
        issue_tile_copies<DIM, P, KIND>(a, smem, eb, mo, vec, tid, NT);
        dgtc::cp_async_wait_all();
        pipe_sync<HALVES>(bar_all, NT);
        issue_neighbour_copies<DIM, P, KIND>(a, smem, eb, mo, 0, tid, NT);
        dgtc::cp_async_commit();
        // the first tile's rows now; every later tile's while its
        // predecessor's MMAs run
        dgtc::cp_async_wait_all();
        pipe_sync<HALVES>(bar_all, NT);
        const long long T1 = tfirst + tstride;
        if (T1 < ntiles) {
            long long e1, m1;
            tile_base(T1, e1, m1);
            issue_conn_copies<DIM, P, KIND>(a, smem, e1, 1, tid, NT);
        }
        dgtc::cp_async_commit();
        build_rows<DIM, P, KIND>(a, smem, eb, 0, tid, NT);
        pipe_sync<HALVES>(bar_all, NT);
    }
    int cb = 0;  // connectivity buffer of the current tile
    for (long long tile = tfirst; tile < ntiles && alive; tile += tstride, cb ^= 1) {
        long long ebase, moff;
        tile_base(tile, ebase, moff);
        const long long next = tile + tstride;
        long long nebase = 0, nmoff = 0;
        if (next < ntiles) tile_base(next, nebase, nmoff);
        // the tile's element data are consumed: start copying the next tile's
        // (the row builders, which wait for these copies; the MMA issuers
        // copy nothing for the next tile)
        if (next < ntiles && builder) issue_tile_copies<DIM, P, KIND>(a, smem, nebase, nmoff, vec, bidx, NBW * 32);
        dgtc::cp_async_commit();
        // this thread's connectivity copies of the next tile are complete (only
        // the group just committed may still be pending); the barrier after
        // the row maxima makes every thread's copies visible
        dgtc::cp_async_wait_group<1>();

        // 3. slices of the A rows into tensor memory (rows 0..127)
        const bool row_ok = (rf < NQ) && (ebase + rle < a.K);
        // operands of this thread's RK update, loaded now so that their latency
        // overlaps the slicing and the contraction
        const int i0 = part * NPP;
        const long long rbase = moff + rf * a.fstride + (ebase + rle) * NP;
        float pu[NPP], pl[NPP], pa[NPP];
#pragma unroll
        for (int t = 0; t < NPP; ++t) {
            pu[t] = pl[t] = pa[t] = 0.0f;
            if (row_ok && i0 + t < NP) {
                pu[t] = dgtc::ld_early(a.u + rbase + i0 + t);
                pl[t] = dgtc::ld_early(a.ulo + rbase + i0 + t);
                if (STAGE > 1 && STAGE < kStageEuler) pa[t] = dgtc::ld_early(a.acc + rbase + i0 + t);
            }
        }
        const float *arow = &sA[r * KSTR];
        if constexpr (!MS::TF) {
            // largest magnitude of this thread's slicing columns of row r (the
            // staged rows hold zeros past KTOT); the barrier below publishes it
            const float2 *ap = reinterpret_cast<const float2 *>(arow);
            float m = 0.0f;
#pragma unroll 4
            for (int c = part * CPG; c < part * CPG + CPG; ++c) {
                const float2 v = ap[c];
                m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
            }
            sMax[part * 128 + r] = m;
        }
        pipe_sync<HALVES>(bar_all, NT);
        if (next < ntiles && builder)
            issue_neighbour_copies<DIM, P, KIND>(a, smem, nebase, nmoff, cb ^ 1, bidx, NBW * 32);
        dgtc::cp_async_commit();
        int ea = 0;
        bool live = row_ok;
        float sc = 0.0f;
        if constexpr (!MS::TF) {
            float rmax = sMax[r];
#pragma unroll
            for (int g = 1; g < NWG; ++g) rmax = fmaxf(rmax, sMax[g * 128 + r]);
            ea = row_exponent(rmax);
            // rows below 2^-110 are treated as zero (their contribution is far
            // below the FP32 resolution of any non-negligible row)
            live = row_ok && ea > -110;
            sc = live ? exp2i(8 - ea) : 0.0f;
        }
        // 3 (cont.). warp group g slices columns [g*CPG, (g+1)*CPG) of the
        // row's tensor-memory columns in chunks of CH
        {
            constexpr int CH = 8;
            const int col0 = part * CPG;
            const uint32_t ta = dgtc::tmem_lane_addr(tbase, warp, col0);
#pragma unroll 1
            for (int c = 0; c < CPG / CH; ++c)
                slice_columns<KIND, MS::NSA, KTOT, ACOLS, CH, true>(arow, live, sc, col0 + CH * c, ta + CH * c);
            if constexpr (CPG % CH > 0)
                slice_columns<KIND, MS::NSA, KTOT, ACOLS, CPG % CH, true>(arow, live, sc, col0 + CPG / CH * CH,
                                                                           ta + CPG / CH * CH);
        }
        dgtc::tmem_st_wait();
        // the next tile's element data and neighbour traces (this thread's
        // copies): complete now, published by the barrier to the row builders
        dgtc::cp_async_wait_all();
        dgtc::fence_before_sync();
        pipe_sync<HALVES>(bar_all, NT);

        // 4. tensor-core contraction, issued by thread 0 (unrolled)
        if (tid == 0 && !*sFail) {
            dgtc::fence_after_sync();
            issue_mmas<DIM, P, KIND, 0, KSTEPS>(tbase + MS::ACC, tbase, dgtc::desc_kmajor(sB, 128, 256));
            dgtc::mma_commit(bar);
        }
        __syncwarp();
        // while warp 0 issues the MMAs and they run, the other warps build the
        // next tile's rows
        if (next < ntiles && builder) {
            const long long next2 = next + tstride;
            if (next2 < ntiles) {
                long long e2, m2;
                tile_base(next2, e2, m2);
                issue_conn_copies<DIM, P, KIND>(a, smem, e2, cb, bidx, NBW * 32);
            }
            build_rows<DIM, P, KIND>(a, smem, nebase, cb ^ 1, bidx, NBW * 32);
        }
        dgtc::cp_async_commit();

        // 5. epilogue: accumulators -> stage increment, RK4 stage update;
        //    warp group g takes output nodes [g*NPP, (g+1)*NPP)
        // every thread waits for the MMAs itself; a failure is published by
        // the staging barrier below, after which every thread reads the flag
        const bool mma_done = dgtc::mbar_wait_bounded(bar, phase, 1u << 30);
        if (!mma_done) *sFail = 1;
        phase ^= 1u;
        // outputs staged in the state-tile region (3D P4): every row builder
        // must have finished reading it first
        if constexpr (!MS::OUT_OWN) pipe_sync<HALVES>(bar_all, NT);
        dgtc::fence_after_sync();
        // outputs go through shared memory so that the global stores are
        // whole-tile vectors; the accumulators are read eight output nodes at
        // a time
        float *sO0 = reinterpret_cast<float *>(smem + MS::OFF_OUT);  // acc, or the new low part
        float *sO1 = sO0 + NQ * ELEMS * NP;   // next stage input / new state
        if (mma_done) {
            const float sdt = live ? a.dt * exp2i(ea - 16) : 0.0f;
            static_assert(NX <= 2, "at most two accumulators past the first two");
#pragma unroll
            for (int c = 0; c < NCH; ++c) {
                uint32_t v0[EC], v1[EC], vx[NX > 0 ? NX : 1][EC];
                const int cc = i0 + EC * c;
                ld_cols<EC>(dgtc::tmem_lane_addr(tbase, warp, MS::ACC + 0 * NPAD + cc), v0);
                ld_cols<EC>(dgtc::tmem_lane_addr(tbase, warp, MS::ACC + 1 * NPAD + cc), v1);
#pragma unroll
                for (int x = 0; x < NX; ++x) ld_cols<EC>(dgtc::tmem_lane_addr(tbase, warp, MS::ACC + (2 + x) * NPAD + cc), vx[x]);
                dgtc::tmem_ld_wait();
                if (!row_ok) continue;
#pragma unroll
                for (int h = 0; h < EC; ++h) {
                    const int t = EC * c + h;
                    const int i = i0 + t;
                    if (t >= NPP || i >= NP) break;
                    float rr;
                    if constexpr (MS::TF) {
                        rr = a.dt * (__uint_as_float(v0[h]) + __uint_as_float(v1[h]));
                    } else {
                        // levels 2 and 3 (the pairs with i+j >= 2)
                        float v2 = 0.0f;
#pragma unroll
                        for (int x = 0; x < NX; ++x) v2 += __uint_as_float(vx[x][h]);
                        float hi, lo;
                        two_sum(__uint_as_float(v0[h]), __uint_as_float(v1[h]), hi, lo);
                        lo += v2;
                        const float scl = sdt * exp2i(sEb[i]);
                        rr = fmaf(scl, hi, scl * lo);
                    }
                    const int o = r * NP + i;  // row r = (field, element) of the tile
                    if (STAGE == 1) {
                        sO0[o] = rr;
                        sO1[o] = pu[t] + (pl[t] + 0.5f * rr);
                    } else if (STAGE == 2) {
                        sO0[o] = fmaf(2.0f, rr, pa[t]);
                        sO1[o] = pu[t] + (pl[t] + 0.5f * rr);
                    } else if (STAGE == 3) {
                        sO0[o] = fmaf(2.0f, rr, pa[t]);
                        sO1[o] = pu[t] + (pl[t] + rr);
                    } else {
                        const float dlt = STAGE == kStageEuler ? rr : (pa[t] + rr) * (1.0f / 6.0f);
                        float s, e;
                        two_sum(pu[t], dlt, s, e);
                        e += pl[t];
                        const float nh = s + e;
                        sO1[o] = nh;
                        sO0[o] = e - (nh - s);
                    }
                }
            }
        }
        pipe_sync<HALVES>(bar_all, NT);
        if (*sFail) {
            alive = false;
        } else {
            const unsigned long long cm = MASKED ? a.cmask[ebase / ELEMS] : 0ull;
            if (vec && ebase + ELEMS <= a.K && cm == 0ull) {
                constexpr int W = ELEMS * NP / 4;
                for (int idx = tid; idx < NQ * W; idx += NT) {
                    const int f = idx / W, w = idx - f * W;
                    const long long g = moff + f * a.fstride + ebase * NP + 4 * w;
                    *reinterpret_cast<float4 *>(&out_lo[g]) = *reinterpret_cast<const float4 *>(&sO0[f * ELEMS * NP + 4 * w]);
                    *reinterpret_cast<float4 *>(&a.wout[g]) = *reinterpret_cast<const float4 *>(&sO1[f * ELEMS * NP + 4 * w]);
                }
            } else {
                for (int idx = tid; idx < NQ * ELEMS * NP; idx += NT) {
                    const int f = idx / (ELEMS * NP), rem = idx - f * (ELEMS * NP);
                    if (ebase + rem / NP >= a.K || ((cm >> (rem / NP)) & 1ull)) continue;
                    const long long g = moff + f * a.fstride + ebase * NP + rem;
                    out_lo[g] = sO0[idx];
                    a.wout[g] = sO1[idx];
                }
            }
        }
        dgtc::fence_before_sync();
        // with the outputs staged in a region of their own, the next tile
        // reaches that region only after several barriers; staged in the
        // state-tile region (3D P4), they must be read before the next tile's
        // copies refill it
        if constexpr (!MS::OUT_OWN) pipe_sync<HALVES>(bar_all, NT);
    }
    // no copy may still be writing shared memory when the CTA exits
    dgtc::cp_async_wait_all();
    if (!alive && tid == 0) {
        // the MMAs of the failed tile may still be in flight: wait once more
        // (bounded) before releasing tensor memory
        atomicExch(a.err, 1);
        dgtc::mbar_wait_bounded(bar, phase ^ 1u, 1u << 30);
    }
    dgtc::fence_after_sync();
    __syncthreads();
    if (threadIdx.x < 32) dgtc::tmem_dealloc(*sTmem, MS::TMEM_COLS * HALVES);
}

}  // namespace dgk
