// leaf_raw.h — the raw inputs of a leaf's learned features, computed where the
// leaf's record and sample values are already at hand.
//
// In learned mode the split children of an adaptive pass get a dense row of
// these raw inputs each (row k: the k-th split's left child, row newL + k: its
// right child): the adaptive pass writes the children's box extents, the
// errors pass that recomputes them their luminance statistics and error, so
// that the prediction that follows reads one 48-byte row instead of gathering
// the record and the values again.  The arithmetic uses only
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

// A row is written in two halves (the row is 16-byte aligned): [0, 6) the box
// extents, by the adaptive pass that splits the leaf (it holds both children's
// boxes), and [6, 12) the luminance statistics and the error, by the errors
// pass that follows.
template <int D>
__device__ __forceinline__ void mdas_raw_store_extents(float* __restrict__ row, const float (&mn)[D],
                                                       const float (&mx)[D]) {
    float e[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) e[j] = j < D ? __fsub_rn(mx[j < D ? j : 0], mn[j < D ? j : 0]) : 0.0f;
    reinterpret_cast<float4*>(row)[0] = make_float4(e[0], e[1], e[2], e[3]);
    reinterpret_cast<float2*>(row)[2] = make_float2(e[4], e[5]);
}

__device__ __forceinline__ void mdas_raw_store_stats(float* __restrict__ row, const MdasLumStats& s, float error) {
    reinterpret_cast<float2*>(row)[3] = make_float2(s.n, s.sum);
    reinterpret_cast<float4*>(row)[2] = make_float4(s.sq, s.mn, s.mx, error);
}
