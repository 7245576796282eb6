// leaf_raw.h — the raw inputs of a leaf's learned features, computed where the
// leaf's record and sample values are already at hand.
//
// The errors pass reads each recomputed leaf's box and sample values; in
// learned mode it also leaves these raw inputs in a dense row per recomputed
// leaf, so that the prediction that follows reads one 48-byte row instead of
// gathering the record and the values again.  The arithmetic uses only
// correctly rounded intrinsics (no contraction), so the rows are the same bits
// whichever build computes them (reference-arithmetic or strict-IEEE errors
// kernel, or the feature kernel itself).
#pragma once

#include <cuda_runtime.h>

// Floats per row: [0, 6) box extents per dimension (mx - mn, 0 past D), [6]
// samples, [7] sum of luminances, [8] sum of squared luminances, [9] smallest
// and [10] largest luminance, [11] the leaf's error.
#define MDAS_RAW_FLOATS 12

__device__ __forceinline__ float mdas_luminance(float r, float g, float b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(0.2126f, r), __fmul_rn(0.7152f, g)), __fmul_rn(0.0722f, b));
}

struct MdasLumStats {
    float n, sum, sq, mn, mx;
};

__device__ __forceinline__ MdasLumStats mdas_lum_empty() { return MdasLumStats{0.0f, 0.0f, 0.0f, 3.402823466e38f, -3.402823466e38f}; }

__device__ __forceinline__ void mdas_lum_add(MdasLumStats& s, float lum) {
    s.n = __fadd_rn(s.n, 1.0f);
    s.sum = __fadd_rn(s.sum, lum);
    s.sq = __fadd_rn(s.sq, __fmul_rn(lum, lum));
    s.mn = fminf(s.mn, lum);
    s.mx = fmaxf(s.mx, lum);
}

// One row from a leaf's box and luminance statistics (16-byte stores; the row
// is 16-byte aligned).
template <int D>
__device__ __forceinline__ void mdas_raw_store(float* __restrict__ row, const float (&mn)[D], const float (&mx)[D],
                                               const MdasLumStats& s, float error) {
    float e[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) e[j] = j < D ? __fsub_rn(mx[j < D ? j : 0], mn[j < D ? j : 0]) : 0.0f;
    float4* r4 = reinterpret_cast<float4*>(row);
    r4[0] = make_float4(e[0], e[1], e[2], e[3]);
    r4[1] = make_float4(e[4], e[5], s.n, s.sum);
    r4[2] = make_float4(s.sq, s.mn, s.mx, error);
}
