// kdgrid_kernels.cuh — the MDAS hot path as sm_103a CUDA kernels.
//
// This header is compiled twice, each time inside its own namespace:
//   * kdgrid_fast.cu (namespace mdas_fast) with the reference's own build flags
//     (--use_fast_math: FTZ, approximate division/sqrt, fast powf, FMA
//     contraction; SDK/CMakeLists.txt:163-180), so that every float the
//     reference computes is computed the same way here;
//   * kdgrid_ieee.cu (namespace mdas_ieee) with strict IEEE flags
//     (-fmad=false -prec-div=true -prec-sqrt=true -ftz=false) and the
//     reproducible pow of ieee_math.h, so that a CPU restatement can reproduce
//     every bit.
// The statements that produce floats follow the reference's expression order
// (SDK/lib/mdas/kdgrid.cu) so that both builds compute what the reference
// computes in the respective arithmetic.
//
// What differs from the reference is the execution design, not the results:
//   * each leaf keeps a private copy of its sample coordinates (4 x D floats)
//     in its node + box record (`nb`), so that an accepted leaf costs one
//     record (one 128-byte line at D = 4) instead of one random gather per
//     sample; the sample buffers the integrand reads and writes keep the
//     reference's AoS layout;
//   * kernels read the leaf and sample counts from device memory (no host round
//     trip is needed inside a pass);
//   * new sample and leaf slots come from a scan over the acceptance/split flags
//     in leaf order (deterministic): decide (per-tile counts + a compacted list
//     of accepted leaves), scan (one CTA over the tile counts), place (one
//     thread per accepted leaf) — instead of warp-aggregated atomics
//     (kdgrid.cu:366-378, 428-440);
//   * the errors pass after an adaptive pass visits only the split children;
//   * pixel accumulation uses one 16-byte vector atomic per pixel instead of
//     three scalar ones.
#pragma once

#include <stdint.h>
#include <float.h>
#include <cuda_runtime.h>
#include "grid_types.h"
#include "ieee_math.h"
#include "leaf_raw.h"
#include "ld_hint.h"

#ifndef MDAS_NS
#error "define MDAS_NS before including kdgrid_kernels.cuh"
#endif

namespace MDAS_NS {

#ifdef MDAS_REFERENCE_ARITH
// powf under --use_fast_math lowers exactly as in the reference build.
__device__ __forceinline__ float mdas_pow(float x, float y) { return powf(x, y); }
#else
__device__ __forceinline__ float mdas_pow(float x, float y) { return mdas_powf(x, y); }
#endif

// ---- RNG of SDK/cuda/random.h:31-67 ----------------------------------------------
__device__ __forceinline__ unsigned tea4(unsigned val0, unsigned val1) {
    unsigned v0 = val0, v1 = val1, s0 = 0;
#pragma unroll
    for (int n = 0; n < 4; n++) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}

__device__ __forceinline__ unsigned lcg(unsigned& prev) {
    prev = 1664525u * prev + 1013904223u;
    return prev & 0x00FFFFFFu;
}

__device__ __forceinline__ float rnd(unsigned& prev) { return (float)lcg(prev) / (float)0x01000000; }

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialisation may start before its predecessor ends; it waits here (in
// hardware) until the predecessor has completed and its writes are visible.
// Without that launch attribute the wait returns at once.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
// Lets the next kernel (if launched programmatically) be scheduled now.
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" :::); }

// ---- vector loads and stores of NF floats from a 16-byte aligned address ---------
template <int NF, int HINT = 0>
__device__ __forceinline__ void ld_floats(const float* __restrict__ p, float (&out)[NF]) {
#pragma unroll
    for (int k = 0; k + 4 <= NF; k += 4) {
        const float4 v = ld4_hint<HINT>(p + k);
        out[k] = v.x; out[k + 1] = v.y; out[k + 2] = v.z; out[k + 3] = v.w;
    }
    constexpr int base = NF - NF % 4;
    if constexpr (NF % 4 >= 2) {
        const float2 v = *reinterpret_cast<const float2*>(p + base);
        out[base] = v.x; out[base + 1] = v.y;
    }
    if constexpr (NF % 2) out[NF - 1] = p[NF - 1];
}

template <int NF>
__device__ __forceinline__ void st_floats(float* __restrict__ p, const float (&v)[NF]) {
#pragma unroll
    for (int k = 0; k + 4 <= NF; k += 4)
        *reinterpret_cast<float4*>(p + k) = make_float4(v[k], v[k + 1], v[k + 2], v[k + 3]);
    constexpr int base = NF - NF % 4;
    if constexpr (NF % 4 >= 2) *reinterpret_cast<float2*>(p + base) = make_float2(v[base], v[base + 1]);
    if constexpr (NF % 2) p[NF - 1] = v[NF - 1];
}

// One point of D floats at an address aligned to its natural vector (16 B for D=4,
// 8 B for even D, 4 B otherwise).
template <int D>
__device__ __forceinline__ void store_point(float* __restrict__ p, const float (&v)[D]) {
    if constexpr (D == 4) {
        *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    } else if constexpr (D % 2 == 0) {
#pragma unroll
        for (int i = 0; i < D; i += 2) *reinterpret_cast<float2*>(p + i) = make_float2(v[i], v[i + 1]);
    } else {
#pragma unroll
        for (int i = 0; i < D; ++i) p[i] = v[i];
    }
}

// ---- leaf storage ------------------------------------------------------------------
// nb:  NbLayout<D>::FLOATS floats per leaf (a multiple of 32 bytes; 128 bytes,
//      one L2 line, at D = 4):
//        [0, 4)        node: the 4 sample indices (int bits), ~D marks an empty slot
//                      (the Node union of kdgrid.h:15-40)
//        [4, 4+D)      box mn       [4+D, 4+2D)  box mx          (AABB, aabb.h:10-17)
//        [SC, SC+4D)   the coordinates of the leaf's samples in node-slot order
//                      (its private copy; SC = 4 + 2D rounded up to 4 floats)
// One record holds all that the adaptive pass reads of an accepted leaf: a
// random gather of one line pair costs less DRAM time than the same bytes
// from two arrays (measured: 73 against 93 us for 2.4 M of 6 M leaves).
template <int D>
struct NbLayout {
    static constexpr int BOX = 4;
    static constexpr int SC = (4 + 2 * D + 3) / 4 * 4;
    static constexpr int FLOATS = (SC + 4 * D + 7) / 8 * 8;
};

// the private sample copy of leaf i
template <int D>
__device__ __forceinline__ float* leaf_copy(float* nb, size_t i) {
    return nb + i * NbLayout<D>::FLOATS + NbLayout<D>::SC;
}

// node and box of a leaf
template <int D, int HINT = 0>
__device__ __forceinline__ int4 nb_load(const float* __restrict__ nb, float (&mn)[D], float (&mx)[D]) {
    float v[4 + 2 * D];
    ld_floats<4 + 2 * D, HINT>(nb, v);
#pragma unroll
    for (int i = 0; i < D; ++i) {
        mn[i] = v[4 + i];
        mx[i] = v[4 + D + i];
    }
    return make_int4(__float_as_int(v[0]), __float_as_int(v[1]), __float_as_int(v[2]), __float_as_int(v[3]));
}

template <int D>
__device__ __forceinline__ void nb_store(float* __restrict__ nb, int4 n, const float (&mn)[D], const float (&mx)[D]) {
    float v[4 + 2 * D];
    v[0] = __int_as_float(n.x);
    v[1] = __int_as_float(n.y);
    v[2] = __int_as_float(n.z);
    v[3] = __int_as_float(n.w);
#pragma unroll
    for (int i = 0; i < D; ++i) {
        v[4 + i] = mn[i];
        v[4 + D + i] = mx[i];
    }
    st_floats<4 + 2 * D>(nb, v);
}

__device__ __forceinline__ void nb_set_node(float* __restrict__ nb, int4 n) { *reinterpret_cast<int4*>(nb) = n; }

// AABB::Volume (aabb.h:20-25)
template <int D>
__device__ __forceinline__ float box_volume(const float (&mn)[D], const float (&mx)[D]) {
    float res = 1.0f;
#pragma unroll
    for (int i = 0; i < D; ++i) res *= (mx[i] - mn[i]);
    return res;
}

// PointN::Distance (point.h:172-182)
template <int D>
__device__ __forceinline__ float distance(const float (&a)[D], const float (&b)[D]) {
    float result = 0.0f;
#pragma unroll
    for (int i = 0; i < D; ++i) {
        const float d = a[i] - b[i];
        result += d * d;
    }
    return sqrtf(result);
}

__device__ __forceinline__ int node_count(const int4 n) {
    return (n.x >= 0) + (n.y >= 0) + (n.z >= 0) + (n.w >= 0);
}

__device__ __forceinline__ int node_get(const int4 n, int i) {
    return i == 0 ? n.x : i == 1 ? n.y : i == 2 ? n.z : n.w;
}

// =====================================================================================
// Initial stratified sampling — uniformSamplingKernel, kdgrid.cu:121-202.
// One thread per initial cell: Morton-decode the cell index into an n-D cell
// (bitsPerDim bits per dimension, extraImgBits more for x and y), draw 4
// samples with the cell's tea<4>/LCG stream, write record, error -1, seed.
// The AoS sample coordinates are staged in shared memory and written out as
// contiguous 16-byte vectors.
// =====================================================================================
// initial sampling of the 256 leaves [base, base + 256) of a grid with L initial leaves
// s_coords: 256 x 4 x D floats, s_box: 256 x 2 x D floats of shared memory.
template <int D>
__device__ __forceinline__ void init_chunk(const MdasDeviceGrid& g, int L, int base, float* s_coords, float* s_box) {
    constexpr int NB = NbLayout<D>::FLOATS;
    constexpr int SC = NbLayout<D>::SC;
    const int bpd = g.bitsPerDim, eib = g.extraImgBits;
    const int nodeIndex = base + threadIdx.x;
    const int n = min(256, L - base);
    if (nodeIndex < L) {
        float offset[D], extent[D];
#pragma unroll
        for (int j = 0; j < D; ++j) {
            unsigned xq = 0;
            unsigned extentInv = 1u << bpd;
            for (int k = 0; k < bpd; ++k) {
                const int i = D * k + (D - j - 1);
                xq |= (unsigned)((nodeIndex >> i) & 1) << k;
            }
            if (j < 2) {
                for (int k = bpd; k < bpd + eib; ++k) {
                    const int i = D * bpd + 2 * (k - bpd) + 1 - j;
                    xq |= (unsigned)((nodeIndex >> i) & 1) << k;
                }
                extentInv <<= eib;
            }
            extent[j] = 1.0f / float(extentInv);
            offset[j] = xq * extent[j];
        }
        offset[0] *= g.scaleX;
        offset[1] *= g.scaleY;
        extent[0] *= g.scaleX;
        extent[1] *= g.scaleY;

        unsigned seed = tea4((unsigned)nodeIndex, 0);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            float r[D];
#pragma unroll
            for (int i = 0; i < D; ++i) r[i] = rnd(seed);
#pragma unroll
            for (int i = 0; i < D; ++i) s_coords[(threadIdx.x * 4 + j) * D + i] = offset[i] + r[i] * extent[i];
        }
        g.seeds[nodeIndex] = seed;
        g.errors[nodeIndex] = -1.0f;
        g.leafCounts[nodeIndex] = 4;
#pragma unroll
        for (int i = 0; i < D; ++i) {
            s_box[threadIdx.x * 2 * D + i] = offset[i];
            s_box[threadIdx.x * 2 * D + D + i] = offset[i] + extent[i];
        }
    }
    __syncthreads();
    {
        // 4*D floats per leaf, leaf `base` starts at a 16*D-byte boundary
        float4* dst = reinterpret_cast<float4*>(g.coords + (size_t)base * 4 * D);
        const float4* src = reinterpret_cast<const float4*>(s_coords);
        for (int k = threadIdx.x; k < n * D; k += 256) dst[k] = src[k];
        // the chunk's records as consecutive 16-byte stores: node (the leaf's 4
        // samples), box, the private sample copy (an initial leaf's has the layout
        // of its 4 AoS samples), zero padding
        float4* rec = reinterpret_cast<float4*>(g.nb + (size_t)base * NB);
        for (int k = threadIdx.x; k < n * (NB / 4); k += 256) {
            const int r = k / (NB / 4), part = k - r * (NB / 4);
            float v[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int f = 4 * part + e;
                v[e] = f < 4 ? __int_as_float(4 * (base + r) + f)
                     : f < 4 + 2 * D ? s_box[r * 2 * D + (f - 4)]
                     : (f >= SC && f < SC + 4 * D) ? s_coords[r * 4 * D + (f - SC)] : 0.0f;
            }
            rec[k] = make_float4(v[0], v[1], v[2], v[3]);
        }
    }
    __syncthreads();
}

template <int D>
__global__ void __launch_bounds__(256) k_initial_sampling(MdasDeviceGrid g, int L) {
    __shared__ __align__(16) float s_coords[256 * 4 * D];
    __shared__ float s_box[256 * 2 * D];
    for (int base = blockIdx.x * 256; base < L; base += gridDim.x * 256) init_chunk<D>(g, L, base, s_coords, s_box);
}

// =====================================================================================
// Per-leaf error — computeErrorsKernel, kdgrid.cu:204-288.
// Only leaves with error < 0 (new or just split) are recomputed; stale errors
// of leaves that only gained a sample are kept, as in the reference.  The max
// over all leaves goes to counts->gerr (float bits; all errors are >= 0).
//
// Two launch shapes with the same result:
//   full  — every leaf (after InitialSampling or a loaded state);
//   dirty — only the children of the last pass's splits (the left child keeps
//           the parent's slot, listed in g.dirty; the right children are the
//           slot range [L - newL, L)); the max over all other leaves was taken
//           by the adaptive pass that left them unchanged (counts->gerrNext).
// =====================================================================================
// The error of a leaf with sample list `node` and box volume `volume`; lumOut
// (may be null) receives the luminance statistics of its samples.
template <int D>
__device__ __forceinline__ float node_error(const MdasDeviceGrid& g, const int4 node, const float volume,
                                            MdasLumStats* lumOut) {
    float3 avg = make_float3(0.0f, 0.0f, 0.0f);
    float3 loc[4];
    int sampleCount = 0;
    MdasLumStats lum = mdas_lum_empty();
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int idx = node_get(node, i);
        if (idx >= 0) {
            const float* v = g.values + 3 * (size_t)idx;
            loc[i] = make_float3(__ldg(v), __ldg(v + 1), __ldg(v + 2));
            avg.x += loc[i].x;
            avg.y += loc[i].y;
            avg.z += loc[i].z;
            sampleCount++;
            if (lumOut) mdas_lum_add(lum, mdas_luminance(loc[i].x, loc[i].y, loc[i].z));
        }
    }
    {
        // float3 /= float multiplies by the reciprocal (sutil/vec_math.h:492-496)
        const float inv = 1.0f / float(sampleCount);
        avg.x *= inv;
        avg.y *= inv;
        avg.z *= inv;
    }
    float3 diffSum = make_float3(0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (i < sampleCount) {
            diffSum.x += fabsf(loc[i].x - avg.x);
            diffSum.y += fabsf(loc[i].y - avg.y);
            diffSum.z += fabsf(loc[i].z - avg.z);
        }
    }
    float error = 0.0f;
    if (avg.x != 0.0f) error += diffSum.x / avg.x;
    if (avg.y != 0.0f) error += diffSum.y / avg.y;
    if (avg.z != 0.0f) error += diffSum.z / avg.z;
    error /= float(sampleCount);
    error += 1.0e-5f;
    error *= volume;
    if (lumOut) *lumOut = lum;
    return error;
}

template <int D>
__device__ __forceinline__ float leaf_error(const MdasDeviceGrid& g, int nodeIndex) {
    float mn[D], mx[D];
    const int4 node = nb_load<D, 64>(g.nb + (size_t)nodeIndex * NbLayout<D>::FLOATS, mn, mx);
    return node_error<D>(g, node, box_volume<D>(mn, mx), nullptr);
}

// MODE 0: full, 1: dirty, 2: dirty unless no adaptive pass ran since the
// initial sampling (the device-side budget loop, where passes alternate).
template <int D, int MODE>
__global__ void __launch_bounds__(256, 6) k_compute_errors(MdasDeviceGrid g) {
    pdl_launch_dependents();  // decide may be scheduled; it waits for this grid
    __shared__ unsigned s_max[8];
    __shared__ unsigned s_cnt[8];
    const bool DIRTY = MODE == 1 || (MODE == 2 && g.counts->passes > 0);
    int items, newL = 0, firstRight = 0;
    float maxError = 0.0f;
    if (DIRTY) {
        newL = g.counts->newL;
        firstRight = g.counts->L - newL;
        items = 2 * newL;
        maxError = __uint_as_float(g.counts->gerrCarry);
    } else {
        items = g.counts->L;
    }
    unsigned recomputed = 0;
    if (DIRTY) {
        // the split children's sample lists, slots and box volumes, as the
        // splitting pass left them (no leaf record read); learned mode also
        // completes each child's raw feature row (item k is row k)
        const int stride = gridDim.x * blockDim.x;
        // loop index m: the left (even m) and right (odd m) child of split m / 2
        // in neighbouring lanes, which often read the same value sectors (errors
        // stage -3.6 % on dof1024, -9 % on mbdof1080 against all left children
        // first)
        auto item = [&](int m) { return (m & 1) ? newL + (m >> 1) : (m >> 1); };
        int m = blockIdx.x * blockDim.x + threadIdx.x;
        int4 spNext = make_int4(0, 0, 0, 0);
        if (m < items) {
            const int kn = item(m);
            spNext = kn < newL ? g.splitL[kn] : g.splitR[kn - newL];
        }
        for (; m < items; m += stride) {
            const int k = item(m);
            const bool left = k < newL;
            const int4 sp = spNext;
            // the next item's entry, loaded while this one is computed
            if (m + stride < items) {
                const int kn = item(m + stride);
                spNext = kn < newL ? g.splitL[kn] : g.splitR[kn - newL];
            }
            const int nodeIndex = left ? sp.z : firstRight + (k - newL);
            const int4 node = make_int4(sp.x, sp.y, left ? ~D : sp.z, ~D);
            MdasLumStats lum;
            const float error = node_error<D>(g, node, __int_as_float(sp.w), g.featRaw ? &lum : nullptr);
            if (g.featRaw) mdas_raw_store_stats(g.featRaw + (size_t)k * MDAS_RAW_FLOATS, lum, error);
            g.errors[nodeIndex] = error;
            recomputed++;
            maxError = fmaxf(maxError, error);
        }
    } else {
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < items; k += gridDim.x * blockDim.x) {
            float error = g.errors[k];
            if (error < 0.0f) {
                error = leaf_error<D>(g, k);
                g.errors[k] = error;
                recomputed++;
            }
            maxError = fmaxf(maxError, error);
        }
    }
    // max of non-negative floats == max of their bit patterns
    unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(maxError));
    unsigned c = __reduce_add_sync(0xffffffffu, recomputed);
    if ((threadIdx.x & 31) == 0) {
        s_max[threadIdx.x >> 5] = m;
        s_cnt[threadIdx.x >> 5] = c;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? s_max[threadIdx.x] : 0u;
        c = threadIdx.x < (blockDim.x >> 5) ? s_cnt[threadIdx.x] : 0u;
        m = __reduce_max_sync(0xffffffffu, m);
        c = __reduce_add_sync(0xffffffffu, c);
        if (threadIdx.x == 0) {
            atomicMax(&g.counts->gerr, m);
            if (c) atomicAdd(&g.counts->recomputed, (int)c);
        }
    }
}

// =====================================================================================
// Adaptive sampling — adaptiveSamplingKernel, kdgrid.cu:290-481.
// Per leaf: accept with probability (error/g_error)^alpha against the leaf's
// LCG stream; accepted leaves place the best of candidatesNum uniform
// candidates (max of the min distance to the leaf's samples, first max wins);
// a full leaf (4 samples) splits at the median of its 5 samples along its
// largest axis: left child keeps the slot, right child takes a new slot.
//
// Slots: sample slot = N + (#accepted leaves before this one),
//        leaf slot   = L + (#split leaves before this one),
// i.e. the reference's outcome when warps retire in leaf order.  Three kernels,
// no waiting between CTAs:
//   decide — tiles of MDAS_TILE_LEAVES leaves; every thread streams
//            MDAS_LEAVES_PER_THREAD consecutive leaves (16-byte loads of errors
//            and seeds), decides acceptance, reads the node of each accepted
//            leaf, writes every final seed (the candidate draws are a fixed
//            number of LCG steps, applied by jump-ahead), and writes the tile's
//            (accepted, split) counts and its accepted leaves, compacted in leaf
//            order, to scratch;
//   scan   — one CTA: exclusive prefix of the tile counts, the new counts, and
//            for every chunk of 256 accepted leaves the tile of its first one;
//   place  — one thread per accepted leaf, in accepted-rank order (every lane
//            busy): best candidate from the leaf's box and private sample copy,
//            append or split, writes.
// decide also takes the max error of the leaves the pass does not split (their
// error is final for the next errors pass); place lists the split leaves.
// =====================================================================================

// Accepted-leaf entry: x = local leaf index in the tile (bits 0-10) | split rank
// in the tile (bits 11-21) | split flag (bit 22) | sample count (bits 23-25);
// y = the leaf's seed after the acceptance draw.
__device__ __forceinline__ unsigned acc_pack(unsigned local, unsigned splitRank, unsigned split, unsigned cnt) {
    return local | (splitRank << 11) | (split << 22) | (cnt << 23);
}

// Learned acceptance ratio (no reference counterpart): the predicted error over
// the largest predicted error, as kdgrid.cu:326 divides the error by g_error.
__device__ __forceinline__ float learned_ratio_of(float priority, float predMax, float scale) {
    return exp2f((priority - predMax) * scale);
}

// decide, one tile: acceptance of the tile's leaves, final seeds, the tile's
// counts and its compacted accepted list (shared by the single-image and the
// batched kernels).
// K: leaves per thread (4 or 8): a tile is 256 K leaves (g.tileK must be K).
// LEARNED: the grid has priorities (g.priority set; a plain grid's kernels
// carry none of their code).  keptPrio: the order bits of the largest priority
// of the leaves not split (whichever acceptance the pass takes).
template <int D, int K, bool LEARNED>
__device__ __forceinline__ void decide_tile(const MdasDeviceGrid& g, int tile, int L, float gError, unsigned jumpA,
                                            unsigned jumpC, unsigned* s_warp, float& keptMax, unsigned& gathered,
                                            unsigned& keptPrio) {
    constexpr int kMaxNodeSize = 4;  // KDGrid ctor: maxNodeSize(4), kdgrid.cu:611
    constexpr int TILE = 256 * K;
    static_assert((K == 4 || K == 8) && TILE <= 2048, "tile = 256 threads x K leaves, local index in 11 bits");
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int i0 = tile * TILE + threadIdx.x * K;
    const bool full = i0 + K <= L;
    // learned acceptance unless the judge sent this pass back to the plain one
    const bool havePrio = LEARNED && g.priority != nullptr;
    const bool learned = havePrio && !g.learned->usePlain;
    float err[K], pr[K];
    unsigned sd[K];
    int lc[K];
    if (full) {
        // the sample counts of a thread's leaves: one 8- or 4-byte load
        unsigned cw[2];
        if constexpr (K == 8) {
            const uint2 c8 = *reinterpret_cast<const uint2*>(g.leafCounts + i0);
            cw[0] = c8.x;
            cw[1] = c8.y;
        } else {
            cw[0] = *reinterpret_cast<const unsigned*>(g.leafCounts + i0);
            cw[1] = 0u;
        }
#pragma unroll
        for (int q = 0; q < K; q += 4) {
            const float4 e4 = *reinterpret_cast<const float4*>(g.errors + i0 + q);
            const uint4 s4 = *reinterpret_cast<const uint4*>(g.seeds + i0 + q);
            err[q] = e4.x; err[q + 1] = e4.y; err[q + 2] = e4.z; err[q + 3] = e4.w;
            sd[q] = s4.x; sd[q + 1] = s4.y; sd[q + 2] = s4.z; sd[q + 3] = s4.w;
            if (havePrio) {
                const float4 p4 = *reinterpret_cast<const float4*>(g.priority + i0 + q);
                pr[q] = p4.x; pr[q + 1] = p4.y; pr[q + 2] = p4.z; pr[q + 3] = p4.w;
            } else {
                pr[q] = pr[q + 1] = pr[q + 2] = pr[q + 3] = 0.0f;
            }
        }
#pragma unroll
        for (int j = 0; j < K; ++j) lc[j] = (int)((cw[j >> 2] >> (8 * (j & 3))) & 0xffu);
    } else {
#pragma unroll
        for (int j = 0; j < K; ++j) {
            const bool v = i0 + j < L;
            err[j] = v ? g.errors[i0 + j] : 0.0f;
            sd[j] = v ? g.seeds[i0 + j] : 0u;
            lc[j] = v ? (int)g.leafCounts[i0 + j] : 0;
            pr[j] = v && havePrio ? g.priority[i0 + j] : 0.0f;
        }
    }
    const float predMax = learned ? mdas_float_unorder(g.learned->predMax) : 0.0f;
    unsigned accMask = 0;
    unsigned seedAcc[K];
    // the acceptance draw of leaf j (kdgrid.cu:323-326); seed: its stream, advanced
    auto accept = [&](int j, unsigned& seed) {
        if (!learned) return mdas_pow(err[j] / gError, g.alpha) >= rnd(seed);
        return mdas_pow(learned_ratio_of(pr[j], predMax, g.priorityScale), g.alpha) >= rnd(seed);
    };
    // Almost always every leaf of the warp exists and has a drawn seed: that
    // case takes a loop without the per-leaf tests (warp-uniform choice).
    bool plain = full;
#pragma unroll
    for (int j = 0; j < K; ++j) plain = plain && sd[j] != 0u;
    if (__all_sync(0xffffffffu, plain)) {
#pragma unroll
        for (int j = 0; j < K; ++j) {
            unsigned seed = sd[j];
            const bool a = accept(j, seed);
            seedAcc[j] = seed;
            sd[j] = a ? jumpA * seed + jumpC : seed;  // the seed after the candidate draws
            accMask |= (unsigned)a << j;
        }
    } else {
#pragma unroll
        for (int j = 0; j < K; ++j) {
            const int leaf = i0 + j;
            unsigned seed = sd[j];
            if (seed == 0) seed = tea4((unsigned)leaf, 0);
            bool a = false;
            if (leaf < L) a = accept(j, seed);
            seedAcc[j] = seed;
            sd[j] = a ? jumpA * seed + jumpC : seed;
            if (a) accMask |= 1u << j;
        }
    }
    unsigned validMask = (1u << K) - 1u;
    if (!full) {
        validMask = 0u;
#pragma unroll
        for (int j = 0; j < K; ++j) validMask |= (unsigned)(i0 + j < L) << j;
    }
    int cnt[K];
#pragma unroll
    for (int j = 0; j < K; ++j) cnt[j] = ((accMask >> j) & 1u) ? lc[j] : 0;
    unsigned splitMask = 0;
#pragma unroll
    for (int j = 0; j < K; ++j) {
        gathered += (unsigned)cnt[j];
        splitMask |= (unsigned)(cnt[j] >= kMaxNodeSize) << j;
    }
    const unsigned keptMask = validMask & ~splitMask;
#pragma unroll
    for (int j = 0; j < K; ++j) {
        // (errors are >= 0: a leaf not kept contributes 0)
        keptMax = fmaxf(keptMax, ((keptMask >> j) & 1u) ? err[j] : 0.0f);
        if (havePrio && ((keptMask >> j) & 1u)) keptPrio = max(keptPrio, mdas_float_order(pr[j]));
    }
    if (full) {
#pragma unroll
        for (int q = 0; q < K; q += 4)
            *reinterpret_cast<uint4*>(g.seeds + i0 + q) = make_uint4(sd[q], sd[q + 1], sd[q + 2], sd[q + 3]);
    } else {
#pragma unroll
        for (int j = 0; j < K; ++j)
            if (i0 + j < L) g.seeds[i0 + j] = sd[j];
    }
    // The accepted leaves' new sample counts (an append adds one, a split leaves
    // 2 in the left child) and the split leaves' error (-1: recompute), written
    // here as whole vectors instead of by place at scattered slots.
    if (accMask) {
        unsigned c8[2] = {0u, 0u};
#pragma unroll
        for (int j = 0; j < K; ++j) {
            const unsigned nc = ((splitMask >> j) & 1u) ? 2u : (unsigned)(lc[j] + (int)((accMask >> j) & 1u));
            c8[j >> 2] |= nc << (8 * (j & 3));
        }
        if (full) {
            if constexpr (K == 8) *reinterpret_cast<uint2*>(g.leafCounts + i0) = make_uint2(c8[0], c8[1]);
            else *reinterpret_cast<unsigned*>(g.leafCounts + i0) = c8[0];
        } else {
#pragma unroll
            for (int j = 0; j < K; ++j)
                if (i0 + j < L) g.leafCounts[i0 + j] = (unsigned char)((c8[j >> 2] >> (8 * (j & 3))) & 0xffu);
        }
    }
    if (splitMask) {
#pragma unroll
        for (int j = 0; j < K; ++j)
            if ((splitMask >> j) & 1u) err[j] = -1.0f;
        if (full) {
#pragma unroll
            for (int q = 0; q < K; q += 4)
                *reinterpret_cast<float4*>(g.errors + i0 + q) = make_float4(err[q], err[q + 1], err[q + 2], err[q + 3]);
        } else {
#pragma unroll
            for (int j = 0; j < K; ++j)
                if (i0 + j < L && ((splitMask >> j) & 1u)) g.errors[i0 + j] = -1.0f;
        }
    }

    // block scan of (accepted, split) counts, packed lo16 | hi16
    const unsigned flag = (unsigned)__popc(accMask) | ((unsigned)__popc(splitMask) << 16);
    unsigned incl = flag;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        unsigned w = lane < 8 ? s_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < 8) s_warp[lane] = w;
    }
    __syncthreads();
    const unsigned excl = (warp ? s_warp[warp - 1] : 0u) + incl - flag;
    const unsigned tileTotal = s_warp[7];
    {
        unsigned r = excl & 0xffffu, rp = excl >> 16;
        uint2* acc = g.accepted + (size_t)tile * TILE;
#pragma unroll
        for (int j = 0; j < K; ++j) {
            const unsigned a = (accMask >> j) & 1u, sp = (splitMask >> j) & 1u;
            if (a) acc[r] = make_uint2(acc_pack((unsigned)(threadIdx.x * K + j), rp, sp, (unsigned)cnt[j]), seedAcc[j]);
            r += a;
            rp += sp;
        }
    }
    if (threadIdx.x == 0) g.tileCounts[tile] = make_uint2(tileTotal & 0xffffu, tileTotal >> 16);
    __syncthreads();  // s_warp is reused by the next tile
}

// Plain decide at 4 CTAs per SM (63 registers); measured against 3 CTAs per
// SM (70 registers): equal on dof1024, adaptive stage 2 % faster on mbdof1080.
template <int D, int K, bool LEARNED>
__global__ void __launch_bounds__(256, LEARNED ? 1 : 4) k_adaptive_decide(MdasDeviceGrid g, unsigned jumpA,
                                                                        unsigned jumpC) {
    pdl_wait();  // until the kernel before it (the errors pass or the learned judge) has completed
    pdl_launch_dependents();
    __shared__ unsigned s_warp[8];
    const int L = g.counts->L;
    const float gError = __uint_as_float(g.counts->gerr);
    const int ntiles = (L + 256 * K - 1) / (256 * K);
    float keptMax = 0.0f;   // max error of the leaves this CTA does not split
    unsigned gathered = 0;  // sample coordinates read
    unsigned keptPrio = 0;  // max priority of those leaves (learned mode)
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x)
        decide_tile<D, K, LEARNED>(g, tile, L, gError, jumpA, jumpC, s_warp, keptMax, gathered, keptPrio);
    unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(keptMax));
    unsigned c = __reduce_add_sync(0xffffffffu, gathered);
    if ((threadIdx.x & 31) == 0) {
        if (m) atomicMax(&g.counts->gerrNext, m);
        if (c) atomicAdd(&g.counts->gathered, c);
    }
    if constexpr (LEARNED) {
        const unsigned kp = __reduce_max_sync(0xffffffffu, keptPrio);
        if ((threadIdx.x & 31) == 0 && kp) atomicMax(&g.learned->keptMax, kp);
    }
}

// One CTA of 1024 threads: exclusive prefix over the tile counts, then the
// counters (N, L as the place kernel must see them go to ctl).
__device__ __forceinline__ void scan_image(const MdasDeviceGrid& g, unsigned* s_sel, unsigned* s_split) {
    const int N = g.counts->N;
    const int L = g.counts->L;
    const int tileLeaves = 256 * g.tileK;
    const int ntiles = (L + tileLeaves - 1) / tileLeaves;
    const int per = (ntiles + 1023) / 1024;
    const int t0 = threadIdx.x * per;
    const int t1 = min(t0 + per, ntiles);
    unsigned sel = 0, spl = 0;
    for (int t = t0; t < t1; ++t) {
        const uint2 c = g.tileCounts[t];
        sel += c.x;
        spl += c.y;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned is = sel, ip = spl;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned a = __shfl_up_sync(0xffffffffu, is, o);
        const unsigned b = __shfl_up_sync(0xffffffffu, ip, o);
        if (lane >= o) {
            is += a;
            ip += b;
        }
    }
    if (lane == 31) {
        s_sel[warp] = is;
        s_split[warp] = ip;
    }
    __syncthreads();
    if (warp == 0) {
        unsigned a = s_sel[lane], b = s_split[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned x = __shfl_up_sync(0xffffffffu, a, o);
            const unsigned y = __shfl_up_sync(0xffffffffu, b, o);
            if (lane >= o) {
                a += x;
                b += y;
            }
        }
        s_sel[lane] = a;
        s_split[lane] = b;
    }
    __syncthreads();
    unsigned ps = (warp ? s_sel[warp - 1] : 0u) + is - sel;
    unsigned pp = (warp ? s_split[warp - 1] : 0u) + ip - spl;
    for (int t = t0; t < t1; ++t) {
        const uint2 c = g.tileCounts[t];
        g.tilePrefix[t] = make_uint2(ps, pp);
        // chunks of 256 accepted entries whose first entry lies in this tile
        for (unsigned ch = (ps + 255u) >> 8; (ch << 8) < ps + c.x; ++ch) g.chunkTile[ch] = t;
        ps += c.x;
        pp += c.y;
    }
    if (threadIdx.x == 1023) {
        const unsigned newN = ps, newL = pp;  // the last thread ends at the totals
        g.ctl->N0 = N;
        g.ctl->L0 = L;
        g.counts->newN = (int)newN;
        g.counts->newL = (int)newL;
        g.counts->selected = (int)newN;
        g.counts->N = N + (int)newN;
        g.counts->L = L + (int)newL;
        // the pass's accumulators: kept for the host and the next errors pass,
        // cleared for the next pass (decide, their last writer, is done)
        MdasCounts* c = g.counts;
        c->gerrLast = c->gerr;
        c->recomputedLast = c->recomputed;
        c->gatheredLast = c->gathered;
        c->gerrCarry = c->gerrNext;
        c->gerr = 0u;
        c->recomputed = 0;
        c->gathered = 0u;
        c->gerrNext = 0u;
        c->passes += 1;
    }
}

__global__ void __launch_bounds__(1024) k_adaptive_scan(MdasDeviceGrid g) {
    pdl_wait();
    pdl_launch_dependents();
    __shared__ unsigned s_sel[32], s_split[32];
    scan_image(g, s_sel, s_split);
}

// Where entry k of the pass's accepted list (its new sample is N + k) lies:
// its tile (found from the first tile of its 256-entry chunk), the tile's
// prefix, its rank in the tile and its entry word.
struct PlaceLoc {
    int tile, r;
    uint2 pre, e;
};

__device__ __forceinline__ PlaceLoc place_locate(const MdasDeviceGrid& g, int k, int ntiles) {
    PlaceLoc p;
    p.tile = g.chunkTile[k >> 8];
    p.pre = g.tilePrefix[p.tile];
    while (p.tile + 1 < ntiles) {
        const uint2 next = g.tilePrefix[p.tile + 1];
        if ((int)next.x > k) break;
        ++p.tile;
        p.pre = next;
    }
    p.r = k - (int)p.pre.x;
    p.e = g.accepted[(size_t)p.tile * (256 * g.tileK) + p.r];
    return p;
}

// 16-byte chunks of a leaf record that the adaptive pass reads (node, box, padding, private copy)
template <int D>
struct RecChunks {
    static constexpr int C = (NbLayout<D>::SC + 4 * D + 3) / 4;
    static constexpr int CS = C | 1;  // shared-memory stride in chunks: odd, so lanes' chunks hit distinct banks
};

// The record read from its chunks in shared memory.
template <int D>
__device__ __forceinline__ int4 rec_from_chunks(const float4* __restrict__ ch, float (&mn)[D], float (&mx)[D],
                                                float (&scv)[4 * D]) {
    constexpr int C = RecChunks<D>::C;
    constexpr int SC = NbLayout<D>::SC;
    float v[4 * C];
#pragma unroll
    for (int c = 0; c < C; ++c) {
        const float4 t = ch[c];
        v[4 * c] = t.x; v[4 * c + 1] = t.y; v[4 * c + 2] = t.z; v[4 * c + 3] = t.w;
    }
#pragma unroll
    for (int i = 0; i < D; ++i) {
        mn[i] = v[4 + i];
        mx[i] = v[4 + D + i];
    }
#pragma unroll
    for (int k = 0; k < 4 * D; ++k) scv[k] = v[SC + k];
    return make_int4(__float_as_int(v[0]), __float_as_int(v[1]), __float_as_int(v[2]), __float_as_int(v[3]));
}

// place, one accepted leaf (entry r of `tile`, whose prefix is `pre`, entry
// word `e`): best candidate, append or split.  The leaf's record is read from
// its chunks staged in shared memory at srec, or from global memory when srec
// is null.
template <int D>
__device__ __forceinline__ void place_entry(const MdasDeviceGrid& g, int tile, int r, uint2 pre, uint2 e, int N,
                                            int L, const float4* srec = nullptr) {
    constexpr int kMaxNodeSize = 4;
    const int TILE = 256 * g.tileK;
    constexpr int NB = NbLayout<D>::FLOATS;
    (void)kMaxNodeSize;
    const int nodeIndex = tile * TILE + (int)(e.x & 0x7ffu);
    const int splitRankInTile = (int)((e.x >> 11) & 0x7ffu);
    const bool split = (e.x >> 22) & 1u;
    const int sampleCount = (int)((e.x >> 23) & 7u);
    unsigned seed = e.y;
    float* nb = g.nb + (size_t)nodeIndex * NB;
    float* sc = leaf_copy<D>(g.nb, (size_t)nodeIndex);
    float mn[D], mx[D];
    int4 node;
    float scv[4 * D];
    if (srec) {
        node = rec_from_chunks<D>(srec, mn, mx, scv);  // staged in shared memory by the warp
    } else {
        // the whole record (no hint: measured as fast as .L2::128B, faster than 64B or 256B)
        node = nb_load<D>(nb, mn, mx);
        ld_floats<4 * D>(sc, scv);
    }
    float samples[4][D];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int i = 0; i < D; ++i) samples[k][i] = scv[k * D + i];

    // best candidate (kdgrid.cu:332-361)
    float best[D];
#pragma unroll
    for (int i = 0; i < D; ++i) best[i] = 0.0f;
    float maxDistance = -1.0f;
    float diag[D];
#pragma unroll
    for (int i = 0; i < D; ++i) diag[i] = mx[i] - mn[i];
    for (int j = 0; j < g.candidatesNum; ++j) {
        float rr[D];
#pragma unroll
        for (int i = 0; i < D; ++i) rr[i] = rnd(seed);
        float candidate[D];
#pragma unroll
        for (int i = 0; i < D; ++i) candidate[i] = mn[i] + rr[i] * diag[i];
        float minDistance = FLT_MAX;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (k < sampleCount) {
                const float distance_k = distance<D>(candidate, samples[k]);
                if (minDistance > distance_k) minDistance = distance_k;
            }
        }
        if (maxDistance < minDistance) {
            maxDistance = minDistance;
#pragma unroll
            for (int i = 0; i < D; ++i) best[i] = candidate[i];
        }
    }

    const int sampleIndex = N + (int)pre.x + r;
    store_point<D>(g.coords + (size_t)sampleIndex * D, best);
    if (!split) {
        // room left: append the index (and its coordinates), the error stays as it was
        if (sampleCount == 0) node.x = sampleIndex;
        else if (sampleCount == 1) node.y = sampleIndex;
        else if (sampleCount == 2) node.z = sampleIndex;
        else node.w = sampleIndex;
        nb_set_node(nb, node);
        store_point<D>(sc + sampleCount * D, best);  // (decide wrote the new count)
    } else {
        // split dimension: AABB::LargestAxis, ties to the highest index (aabb.h:34-45)
        int axis = -1;
        float maxExtent = -FLT_MAX;
#pragma unroll
        for (int i = D - 1; i >= 0; --i) {
            const float ext = mx[i] - mn[i];
            if (maxExtent < ext) {
                maxExtent = ext;
                axis = i;
            }
        }
        // The reference bubble-sorts the 5 samples (4 old in slot order, then the
        // new one) by the split coordinate (kdgrid.cu:408-417); the sort is stable,
        // so sample k lands at rank[k] = #{m : key[m] < key[k], or key[m] == key[k]
        // and m < k}.  Each sample is written straight to its ranked slot.
        float key[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            float v = 0.0f;
#pragma unroll
            for (int i = 0; i < D; ++i) {
                const float c = k < 4 ? samples[k < 4 ? k : 0][i] : best[i];
                if (i == axis) v = c;
            }
            key[k] = v;
        }
        int rank[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            int rk = 0;
#pragma unroll
            for (int m = 0; m < 5; ++m)
                if (m != k) rk += (key[m] < key[k] || (key[m] == key[k] && m < k)) ? 1 : 0;
            rank[k] = rk;
        }
        const int idx5[5] = {node.x, node.y, node.z, node.w, sampleIndex};
        float k1 = 0.0f, k2 = 0.0f;
        int l0 = 0, l1 = 0, r0 = 0, r1 = 0, r2 = 0;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const int rk = rank[k];
            if (rk == 1) k1 = key[k];
            if (rk == 2) k2 = key[k];
            if (rk == 0) l0 = idx5[k];
            if (rk == 1) l1 = idx5[k];
            if (rk == 2) r0 = idx5[k];
            if (rk == 3) r1 = idx5[k];
            if (rk == 4) r2 = idx5[k];
        }
        const float splitPosition = 0.5f * (k1 + k2);  // md = 5 >> 1 = 2
        const int rank_ = (int)pre.y + splitRankInTile;
        const int nodeOffset = L + rank_;
        float* rnb = g.nb + (size_t)nodeOffset * NB;
        float* rsc = leaf_copy<D>(g.nb, (size_t)nodeOffset);
        // left child keeps the slot: node, mx[axis], its 2 sample coordinates;
        // right child: node, box, its 3 sample coordinates
        nb_set_node(nb, make_int4(l0, l1, ~D, ~D));
        nb[NbLayout<D>::BOX + D + axis] = splitPosition;
        float rmn[D];
#pragma unroll
        for (int i = 0; i < D; ++i) rmn[i] = (i == axis) ? splitPosition : mn[i];
        nb_store<D>(rnb, make_int4(r0, r1, r2, ~D), rmn, mx);
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            float* dst = rank[k] < 2 ? sc + rank[k] * D : rsc + (rank[k] - 2) * D;
            if (k < 4) store_point<D>(dst, samples[k < 4 ? k : 0]);
            else store_point<D>(dst, best);
        }
        // (decide wrote the left child's error -1 and count 2)
        g.errors[nodeOffset] = -1.0f;
        g.leafCounts[nodeOffset] = 3;
        // the children's sample lists and box volumes for the next errors pass
        // (the volumes of the boxes written above, by the same arithmetic)
        {
            float lmx[D];
#pragma unroll
            for (int i = 0; i < D; ++i) lmx[i] = (i == axis) ? splitPosition : mx[i];
            g.splitL[rank_] = make_int4(l0, l1, nodeIndex, __float_as_int(box_volume<D>(mn, lmx)));
            g.splitR[rank_] = make_int4(r0, r1, r2, __float_as_int(box_volume<D>(rmn, mx)));
            // learned mode: the children's box extents, the first half of their
            // raw feature rows (the errors pass writes the second)
            if (g.featRaw) {
                mdas_raw_store_extents<D>(g.featRaw + (size_t)rank_ * MDAS_RAW_FLOATS, mn, lmx);
                mdas_raw_store_extents<D>(g.featRaw + (size_t)(g.counts->newL + rank_) * MDAS_RAW_FLOATS, rmn, mx);
            }
        }
        // a new slot starts without a seed: the reference's seed buffer is zeroed
        // once at InitialSampling (kdgrid.cu:637), and a slot's first draw starts
        // from tea<4>(slot, 0) when its seed is 0 (kdgrid.cu:323-324).  The slot
        // stores that starting seed here instead of the 0, so that decide never
        // computes tea<4> (a warp paid for it whenever one of its leaves was new);
        // mdas_dump_state reports such a never-drawn seed as 0, as the reference
        // holds it (a drawn seed is tea<4>(slot, 0) advanced by >= 1 LCG steps,
        // which never returns to its start within the generator's 2^32 period)
        g.seeds[nodeOffset] = tea4((unsigned)nodeOffset, 0);
        g.dirty[rank_] = nodeIndex;  // for the next errors pass
    }
}

template <int D>
__device__ __forceinline__ void place_rank(const MdasDeviceGrid& g, int k, int N, int L) {
    const int ntiles = (L + 256 * g.tileK - 1) / (256 * g.tileK);
    const PlaceLoc p = place_locate(g, k, ntiles);
    place_entry<D>(g, p.tile, p.r, p.pre, p.e, N, L);
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_group() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// The warp's records of the leaves `leaf` (one per lane, -1: none) copied into
// shared memory at srec (record of lane l at srec + l * CS chunks).
template <int D>
__device__ __forceinline__ void stage_records(const float* __restrict__ nb, int leaf, float4* srec) {
    constexpr int C = RecChunks<D>::C, CS = RecChunks<D>::CS, NB = NbLayout<D>::FLOATS;
    const int lane = threadIdx.x & 31;
    // each record takes P lanes (P: C rounded up to a power of two), chunk = lane % P
    constexpr int P = C <= 8 ? 8 : 16;
    constexpr int RPQ = 32 / P;  // records per copy instruction
    const int c = lane & (P - 1), r0 = lane / P;
#pragma unroll
    for (int q = 0; q < P; ++q) {
        const int rr = q * RPQ + r0;
        const int src = __shfl_sync(0xffffffffu, leaf, rr);
        if (c < C && src >= 0) cp_async16(srec + rr * CS + c, nb + (size_t)src * NB + 4 * c);
    }
}

// The ranks kb + lane of a warp (kb a multiple of 32, so that all lie in one
// 256-entry chunk): each lane's tile and the tile's prefix.  The warp reads the
// prefixes of the 32 tiles from the chunk's first one in one coalesced load and
// each lane searches them (5 shuffles); ranks beyond those 32 tiles walk on.
// Every lane of the warp calls it; lanes with k >= accepted get a tile too
// (unused).
__device__ __forceinline__ void warp_locate(const MdasDeviceGrid& g, int kb, int k, int ntiles, int& tile,
                                            uint2& pre) {
    const int lane = threadIdx.x & 31;
    const int t0 = g.chunkTile[kb >> 8];
    const uint2 totals = make_uint2((unsigned)g.counts->newN, (unsigned)g.counts->newL);
    const uint2 P = t0 + lane < ntiles ? g.tilePrefix[t0 + lane] : totals;
    // largest j with P_j.x <= k (P_0.x <= kb <= k; P is non-decreasing in j)
    int j = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
        const unsigned px = __shfl_sync(0xffffffffu, P.x, j + step);
        if ((int)px <= k) j += step;
    }
    tile = t0 + j;
    pre.x = __shfl_sync(0xffffffffu, P.x, j);
    pre.y = __shfl_sync(0xffffffffu, P.y, j);
    // (only where 31 tiles in a row hold fewer than 32 accepted leaves; not for
    // the lanes past the last rank, which would walk to the last tile)
    if (j == 31 && k < (int)totals.x) {
        while (tile + 1 < ntiles) {
            const uint2 next = g.tilePrefix[tile + 1];
            if ((int)next.x > k) break;
            ++tile;
            pre = next;
        }
    }
}

// One thread per accepted leaf, in accepted-rank order; each warp places 32
// consecutive ranks per iteration, their records staged in shared memory:
//   * every 16-byte copy instruction of the warp (cp.async) covers whole
//     records (4 records of 128 bytes per instruction at D = 4) instead of one
//     16-byte piece of 32 records;
//   * double-buffered: while the warp places its current 32 leaves, the
//     records of its next 32 are on their way into the other buffer;
//   * a rank's tile comes from warp_locate (three dependent loads whatever the
//     density of accepted leaves).
// Three CTAs per SM at D <= 4 (two at D >= 5: 74-90 KB of buffers).  Measured
// against one thread per leaf loading its record when its turn comes: adaptive
// stage -4 % on dof1024, -18 % on mbdof1080.
template <int D>
__global__ void __launch_bounds__(256, D >= 5 ? 2 : 3) k_adaptive_place(MdasDeviceGrid g) {
    constexpr int CS = RecChunks<D>::CS;
    __shared__ __align__(16) float4 s_rec[2][8][32 * CS];
    pdl_wait();
    const int N = g.ctl->N0;
    const int L = g.ctl->L0;
    const int accepted = g.counts->newN;
    const int TILE = 256 * g.tileK;
    const int ntiles = (L + TILE - 1) / TILE;
    const int stride = gridDim.x * 256;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int kb = blockIdx.x * 256 + warp * 32;
    if (kb >= accepted) return;
    // the warp's ranks of one iteration, located: entry, tile, prefix
    auto fetch = [&](int kbase, uint2& e, int& tile, uint2& pre) {
        const int k = kbase + lane;
        warp_locate(g, kbase, k, ntiles, tile, pre);
        if (k < accepted) e = g.accepted[(size_t)tile * TILE + (k - (int)pre.x)];
    };
    uint2 e0 = make_uint2(0u, 0u), pre0 = make_uint2(0u, 0u);
    int tile0 = 0;
    fetch(kb, e0, tile0, pre0);
    stage_records<D>(g.nb, kb + lane < accepted ? tile0 * TILE + (int)(e0.x & 0x7ffu) : -1, s_rec[0][warp]);
    cp_async_commit();
    int buf = 0;
    for (;;) {
        const int kn = kb + stride;
        const bool more = kn < accepted;  // warp-uniform
        uint2 e1 = make_uint2(0u, 0u), pre1 = make_uint2(0u, 0u);
        int tile1 = 0;
        if (more) {
            fetch(kn, e1, tile1, pre1);
            stage_records<D>(g.nb, kn + lane < accepted ? tile1 * TILE + (int)(e1.x & 0x7ffu) : -1,
                             s_rec[buf ^ 1][warp]);
            cp_async_commit();
            cp_async_wait_group<1>();
        } else {
            cp_async_wait_group<0>();
        }
        __syncwarp();
        const int k = kb + lane;
        if (k < accepted)
            place_entry<D>(g, tile0, k - (int)pre0.x, pre0, e0, N, L, s_rec[buf][warp] + lane * CS);
        __syncwarp();  // the buffer is refilled two iterations on
        if (!more) break;
        e0 = e1;
        tile0 = tile1;
        pre0 = pre1;
        kb = kn;
        buf ^= 1;
    }
}

// =====================================================================================
// Reconstruction — integrateKernel, kdgrid.cu:483-582.
// Each leaf splats mean value * (overlap area * Volume / xyArea) / pixArea into
// the pixels its box covers; pixel edges advance incrementally as in the
// reference so that the footprint is the same to the bit.
// =====================================================================================
// reconstruction splat of one leaf
template <int D>
__device__ __forceinline__ void integrate_leaf(const MdasDeviceGrid& g, const int4 node, const float (&mn)[D],
                                               const float (&mx)[D], float4* __restrict__ pixels, int width,
                                               int height) {
    const float scaleX = g.scaleX, scaleY = g.scaleY;
    float2 pixelStep;
    pixelStep.x = scaleX / width;
    pixelStep.y = scaleY / height;
    float3 sampleValue = make_float3(0.0f, 0.0f, 0.0f);
    int sampleCount = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int idx = node_get(node, i);
        if (idx >= 0) {
            const float* v = g.values + 3 * (size_t)idx;
            sampleValue.x += __ldg(v);
            sampleValue.y += __ldg(v + 1);
            sampleValue.z += __ldg(v + 2);
            sampleCount++;
        }
    }
    {
        const float inv = 1.0f / float(sampleCount);
        sampleValue.x *= inv;
        sampleValue.y *= inv;
        sampleValue.z *= inv;
    }
    const float boxVolume = box_volume<D>(mn, mx);

    const int x0 = mn[0] * width / scaleX;
    int x1 = mx[0] * width / scaleX;
    const int y0 = mn[1] * height / scaleY;
    int y1 = mx[1] * height / scaleY;
    x1 = min(x1 + 1, width);
    y1 = min(y1 + 1, height);
    const float pixArea = (scaleX * scaleY) / float(width * height);
    const float invPixArea = 1.0f / pixArea;  // float3 / float (sutil/vec_math.h:483-487)

    float pMinX, pMaxX, pMinY, pMaxY;
    pMinY = y0 * scaleY / float(height);
    pMaxY = pMinY + pixelStep.y;
    for (int y = y0; y < y1; ++y) {
        pMinX = x0 * scaleX / float(width);
        pMaxX = pMinX + pixelStep.x;
        for (int x = x0; x < x1; ++x) {
            const float clox = fmaxf(pMinX, mn[0]);
            const float chix = fminf(pMaxX, mx[0]);
            const float cloy = fmaxf(pMinY, mn[1]);
            const float chiy = fminf(pMaxY, mx[1]);
            if (clox < chix && cloy < chiy) {
                const float volume = (chix - clox) * (chiy - cloy) * boxVolume / ((mx[0] - mn[0]) * (mx[1] - mn[1]));
                const float4 value = make_float4((sampleValue.x * volume) * invPixArea,
                                                 (sampleValue.y * volume) * invPixArea,
                                                 (sampleValue.z * volume) * invPixArea, 0.0f);
                atomicAdd(pixels + (size_t)y * width + x, value);
            }
            pMinX = pMaxX;
            pMaxX += pixelStep.x;
        }
        pMinY = pMaxY;
        pMaxY += pixelStep.y;
    }
}

// Node and box of the 32 consecutive leaves [first, first + 32), read by the
// warp into shared memory with each 16-byte load covering consecutive record
// heads (a third of the lines that 32 lanes each reading their own record
// touch, the records being a 128-byte line apart at D = 4), then this lane's
// from there.  Every lane of the warp calls it; false past the last leaf.
template <int D>
__device__ __forceinline__ bool warp_leaf_head(const float* __restrict__ nb, int first, int L, float4* wbuf,
                                               int4& node, float (&mn)[D], float (&mx)[D]) {
    constexpr int H4 = (4 + 2 * D + 3) / 4;  // 16-byte chunks of node + box
    constexpr int NB = NbLayout<D>::FLOATS;
    static_assert(4 * H4 <= NB, "the chunks stay inside the record");
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int q = 0; q < H4; ++q) {
        const int c = q * 32 + lane;
        const int rec = c / H4;
        if (first + rec < L) wbuf[c] = ld4_hint<64>(nb + (size_t)(first + rec) * NB + 4 * (c - rec * H4));
    }
    __syncwarp();
    const bool valid = first + lane < L;
    if (valid) {
        const float* h = reinterpret_cast<const float*>(wbuf + lane * H4);
        node = make_int4(__float_as_int(h[0]), __float_as_int(h[1]), __float_as_int(h[2]), __float_as_int(h[3]));
#pragma unroll
        for (int j = 0; j < D; ++j) {
            mn[j] = h[4 + j];
            mx[j] = h[4 + D + j];
        }
    }
    __syncwarp();
    return valid;
}

template <int D>
__global__ void __launch_bounds__(256) k_integrate(MdasDeviceGrid g, float4* __restrict__ pixels, int width,
                                                    int height) {
    constexpr int H4 = (4 + 2 * D + 3) / 4;
    __shared__ float4 s_head[8][32 * H4];
    const int L = g.counts->L;
    const int warp = threadIdx.x >> 5;
    for (int base = blockIdx.x * blockDim.x; base < L; base += gridDim.x * blockDim.x) {
        int4 node;
        float mn[D], mx[D];
        if (warp_leaf_head<D>(g.nb, base + 32 * warp, L, s_head[warp], node, mn, mx))
            integrate_leaf<D>(g, node, mn, mx, pixels, width, height);
    }
}

// =====================================================================================
// ConvertToBytes — convertToBytesKernel + make_color (kdgrid.cu:584-598,
// SDK/cuda/helpers.h:35-66): clamp, sRGB transfer (exponent 1/2.4), 8-bit.
// =====================================================================================
__device__ __forceinline__ unsigned char quantize_u8(float x) {
    x = fminf(fmaxf(x, 0.0f), 1.0f);
    return (unsigned char)min((unsigned int)(x * 256.0f), 255u);
}

__device__ __forceinline__ float to_srgb(float c) {
    const float invGamma = 1.0f / 2.4f;
    const float powed = mdas_pow(c, invGamma);
    return c < 0.0031308f ? 12.92f * c : 1.055f * powed - 0.055f;
}

__global__ void __launch_bounds__(256) k_convert_to_bytes(const float4* __restrict__ pixels,
                                                           uchar4* __restrict__ bytes, int P) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
        const float4 p = pixels[i];
        const float cx = fminf(fmaxf(p.x, 0.0f), 1.0f);
        const float cy = fminf(fmaxf(p.y, 0.0f), 1.0f);
        const float cz = fminf(fmaxf(p.z, 0.0f), 1.0f);
        bytes[i] = make_uchar4(quantize_u8(to_srgb(cx)), quantize_u8(to_srgb(cy)), quantize_u8(to_srgb(cz)), 255);
    }
}

// =====================================================================================
// SamplingDensity (kdgrid.cu:822-837) — host code in the reference, so its
// arithmetic is IEEE in both builds (explicitly rounded intrinsics).  Every
// sample adds 0.05 to its pixel; all addends are equal, so the float sums do not
// depend on the order of the atomics.
// =====================================================================================
template <int D>
__global__ void __launch_bounds__(256) k_sampling_density(MdasDeviceGrid g, float4* __restrict__ pixels, int width,
                                                           int height) {
    const int N = g.counts->N;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const float* c = g.coords + (size_t)i * D;
        int x = (int)__fmul_rn(__fdiv_rn(c[0], g.scaleX), (float)width);
        int y = (int)__fmul_rn(__fdiv_rn(c[1], g.scaleY), (float)height);
        x = min(x, width - 1);
        y = min(y, height - 1);
        atomicAdd(pixels + (size_t)y * width + x, make_float4(0.05f, 0.05f, 0.05f, 0.0f));
    }
}

__global__ void k_density_alpha(float4* __restrict__ pixels, int P) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) pixels[i].w = 1.0f;
}

// =====================================================================================
// Leaf records <-> the reference's node / box arrays (state dump and load).
// =====================================================================================
template <int D>
__global__ void k_unpack_records(const float* __restrict__ nb, int L, int4* __restrict__ nodes,
                                 float* __restrict__ boxes) {
    constexpr int NB = NbLayout<D>::FLOATS;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L; i += gridDim.x * blockDim.x) {
        float mn[D], mx[D];
        nodes[i] = nb_load<D>(nb + (size_t)i * NB, mn, mx);
#pragma unroll
        for (int k = 0; k < D; ++k) {
            boxes[(size_t)i * 2 * D + k] = mn[k];
            boxes[(size_t)i * 2 * D + D + k] = mx[k];
        }
    }
}

template <int D>
__global__ void k_pack_records(float* __restrict__ nb, unsigned char* __restrict__ counts, int L,
                               const int4* __restrict__ nodes, const float* __restrict__ boxes,
                               const float* __restrict__ coords) {
    constexpr int NB = NbLayout<D>::FLOATS;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L; i += gridDim.x * blockDim.x) {
        const int4 n = nodes[i];
        counts[i] = (unsigned char)node_count(n);
        float mn[D], mx[D];
#pragma unroll
        for (int k = 0; k < D; ++k) {
            mn[k] = boxes[(size_t)i * 2 * D + k];
            mx[k] = boxes[(size_t)i * 2 * D + D + k];
        }
        nb_store<D>(nb + (size_t)i * NB, n, mn, mx);
        float sc[4 * D];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int idx = node_get(n, k);
#pragma unroll
            for (int d = 0; d < D; ++d) sc[k * D + d] = idx >= 0 ? coords[(size_t)idx * D + d] : 0.0f;
        }
        st_floats<4 * D>(leaf_copy<D>(nb, (size_t)i), sc);
    }
}

// Learned mode, per pass: both schedules' acceptance of every leaf (the same
// first draw of its seed as decide's), the plain errors each leaves unrefined,
// and the verdict, set by the last block to finish (no block waits for another).
__global__ void __launch_bounds__(256) k_learned_judge(MdasDeviceGrid g, int Lhost) {
    __shared__ double s_l[8], s_p[8];
    __shared__ bool s_last;
    const int L = Lhost >= 0 ? Lhost : g.counts->L;  // < 0: the device leaf count (inside a graph)
    const float gError = __uint_as_float(g.counts->gerr);
    const float predMax = mdas_float_unorder(g.learned->predMax);
    double ul = 0.0, up = 0.0;
    // the leaf's error into the schedules' FP32 partial sums (of four leaves at
    // most: one FP64 add per schedule and four leaves, FP64 being a slow pipe)
    auto judge = [&](int i, float e, unsigned seed, float prio, float& fp, float& fl) {
        if (seed == 0) seed = tea4((unsigned)i, 0);
        const float r = rnd(seed);
        const bool plain = mdas_pow(e / gError, g.alpha) >= r;
        const bool learned = mdas_pow(learned_ratio_of(prio, predMax, g.priorityScale), g.alpha) >= r;
        if (!plain) fp = __fadd_rn(fp, e);
        if (!learned) fl = __fadd_rn(fl, e);
    };
    // four leaves per thread and iteration: 16-byte loads of errors, seeds and
    // priorities (all 256-byte aligned)
    const int L4 = L >> 2;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < L4; v += gridDim.x * blockDim.x) {
        const float4 e = reinterpret_cast<const float4*>(g.errors)[v];
        const uint4 sd = reinterpret_cast<const uint4*>(g.seeds)[v];
        const float4 p = reinterpret_cast<const float4*>(g.priority)[v];
        float fp = 0.0f, fl = 0.0f;
        judge(4 * v, e.x, sd.x, p.x, fp, fl);
        judge(4 * v + 1, e.y, sd.y, p.y, fp, fl);
        judge(4 * v + 2, e.z, sd.z, p.z, fp, fl);
        judge(4 * v + 3, e.w, sd.w, p.w, fp, fl);
        up += (double)fp;
        ul += (double)fl;
    }
    for (int i = 4 * L4 + blockIdx.x * blockDim.x + threadIdx.x; i < L; i += gridDim.x * blockDim.x) {
        float fp = 0.0f, fl = 0.0f;
        judge(i, g.errors[i], g.seeds[i], g.priority[i], fp, fl);
        up += (double)fp;
        ul += (double)fl;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ul += __shfl_xor_sync(0xffffffffu, ul, o);
        up += __shfl_xor_sync(0xffffffffu, up, o);
    }
    if ((threadIdx.x & 31) == 0) {
        s_l[threadIdx.x >> 5] = ul;
        s_p[threadIdx.x >> 5] = up;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            a += s_l[w];
            b += s_p[w];
        }
        atomicAdd(&g.learned->unrefinedLearned, a);
        atomicAdd(&g.learned->unrefinedPlain, b);
        __threadfence();
        s_last = atomicAdd(&g.learned->blocksDone, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
        __threadfence();
        MdasLearnedStats* st = g.learned;
        const double a = atomicAdd(&st->unrefinedLearned, 0.0), b = atomicAdd(&st->unrefinedPlain, 0.0);
        const int revert = a > (1.0 + (double)st->tolerance) * b ? 1 : 0;
        st->usePlain = revert;
        st->plainPasses += revert;
        st->judgedPasses += 1;
        st->blocksDone = 0;
        st->keptMax = 0u;  // taken by this pass's predMax; the adaptive pass sets it anew
    }
}

// ---- host launchers -------------------------------------------------------------
// A launch that may overlap the tail of the previous kernel on the stream (the
// kernel calls pdl_wait() before it reads what that kernel wrote).
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), int grid, int block, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

#define MDAS_SWITCH_D(D, EXPR)                 \
    switch (D) {                               \
        case 3: { constexpr int DD = 3; EXPR; } break; \
        case 4: { constexpr int DD = 4; EXPR; } break; \
        case 5: { constexpr int DD = 5; EXPR; } break; \
        case 6: { constexpr int DD = 6; EXPR; } break; \
        default: return cudaErrorInvalidValue; \
    }

cudaError_t initial_sampling(const MdasDeviceGrid& g, int L, cudaStream_t s) {
    const int grid = (L + 255) / 256;
    if (grid == 0) return cudaSuccess;
    MDAS_SWITCH_D(g.D, (k_initial_sampling<DD><<<grid, 256, 0, s>>>(g, L)));
    return cudaGetLastError();
}

cudaError_t compute_errors(const MdasDeviceGrid& g, int grid, bool dirty, cudaStream_t s) {
    // (g_error = 0, kdgrid.cu:684-685: cleared by the last pass's scan, or when
    // the counters were set)
    if (dirty) {
        MDAS_SWITCH_D(g.D, (k_compute_errors<DD, 1><<<grid, 256, 0, s>>>(g)));
    } else {
        MDAS_SWITCH_D(g.D, (k_compute_errors<DD, 0><<<grid, 256, 0, s>>>(g)));
    }
    return cudaGetLastError();
}

cudaError_t compute_errors_auto(const MdasDeviceGrid& g, int grid, cudaStream_t s) {
    MDAS_SWITCH_D(g.D, (k_compute_errors<DD, 2><<<grid, 256, 0, s>>>(g)));
    return cudaGetLastError();
}

// Condition of the device-side budget loop (optixMotionBlur.cpp:781 plus the
// capacity guard of :723-724): another pass while N < budget, the next pass
// fits, no device error, and fewer than maxPasses passes ran (a safety stop:
// every pass accepts at least the leaf with the largest error, so N grows).
__global__ void k_loop_condition(const MdasCounts* __restrict__ c, cudaGraphConditionalHandle h, int budget,
                                 int maxSamples, int maxPasses) {
    const long long N = c->N, L = c->L;
    cudaGraphSetConditional(h, (N < budget && N + L <= maxSamples && c->status == 0 && c->passes < maxPasses) ? 1u
                                                                                                             : 0u);
}

cudaError_t loop_condition(const MdasDeviceGrid& g, cudaGraphConditionalHandle h, int budget, int maxPasses,
                           cudaStream_t s) {
    k_loop_condition<<<1, 1, 0, s>>>(g.counts, h, budget, g.maxSamples, maxPasses);
    return cudaGetLastError();
}

// LCG jump-ahead: n draws take a seed s to A_n * s + C_n (mod 2^32).
static void lcg_jump(unsigned n, unsigned* A, unsigned* C) {
    unsigned a = 1u, c = 0u;
    for (unsigned k = 0; k < n; ++k) {
        a = 1664525u * a;
        c = 1664525u * c + 1013904223u;
    }
    *A = a;
    *C = c;
}

// The place kernel's shared-memory carveout: its double buffers take 56 KB per
// CTA at D = 4, three CTAs per SM need the largest carveout.
static cudaError_t place_prepare(int D) {
    static bool done[64][7] = {};  // per device ordinal (a function attribute is set per device)
    if (D < 3 || D > 6) return cudaErrorInvalidValue;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64 && done[dev][D]) return cudaSuccess;
    MDAS_SWITCH_D(D, (e = cudaFuncSetAttribute(k_adaptive_place<DD>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                               (int)cudaSharedmemCarveoutMaxShared)));
    if (e == cudaSuccess && dev >= 0 && dev < 64) done[dev][D] = true;
    return e;
}

cudaError_t adaptive_sampling(const MdasDeviceGrid& g, int gridDecide, int gridPlace, cudaStream_t s) {
    cudaError_t e = cudaSuccess;
    unsigned A, C;
    lcg_jump((unsigned)(g.candidatesNum * g.D), &A, &C);
    if (g.priority && g.tileK == 4) {
        MDAS_SWITCH_D(g.D, (e = launch_pdl(k_adaptive_decide<DD, 4, true>, gridDecide, 256, s, g, A, C)));
    } else if (g.priority) {
        MDAS_SWITCH_D(g.D, (e = launch_pdl(k_adaptive_decide<DD, 8, true>, gridDecide, 256, s, g, A, C)));
    } else if (g.tileK == 4) {
        MDAS_SWITCH_D(g.D, (e = launch_pdl(k_adaptive_decide<DD, 4, false>, gridDecide, 256, s, g, A, C)));
    } else {
        MDAS_SWITCH_D(g.D, (e = launch_pdl(k_adaptive_decide<DD, 8, false>, gridDecide, 256, s, g, A, C)));
    }
    if (e != cudaSuccess) return e;
    e = launch_pdl(k_adaptive_scan, 1, 1024, s, g);
    if (e != cudaSuccess) return e;
    e = place_prepare(g.D);
    if (e != cudaSuccess) return e;
    MDAS_SWITCH_D(g.D, (e = launch_pdl(k_adaptive_place<DD>, gridPlace, 256, s, g)));
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

cudaError_t learned_judge(const MdasDeviceGrid& g, int L, int grid, cudaStream_t s) {
    if (L == 0 || !g.learned || !g.priority) return cudaErrorInvalidValue;
    k_learned_judge<<<grid, 256, 0, s>>>(g, L);
    return cudaGetLastError();
}

cudaError_t integrate(const MdasDeviceGrid& g, int grid, float* pixels, int W, int H, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(pixels, 0, sizeof(float4) * (size_t)W * H, s);
    if (e != cudaSuccess) return e;
    MDAS_SWITCH_D(g.D, (k_integrate<DD><<<grid, 256, 0, s>>>(g, reinterpret_cast<float4*>(pixels), W, H)));
    return cudaGetLastError();
}

cudaError_t convert_to_bytes(const float* pixels, unsigned char* bytes, int P, cudaStream_t s) {
    const int grid = (P + 255) / 256;
    if (grid == 0) return cudaSuccess;
    k_convert_to_bytes<<<grid, 256, 0, s>>>(reinterpret_cast<const float4*>(pixels), reinterpret_cast<uchar4*>(bytes),
                                            P);
    return cudaGetLastError();
}

cudaError_t sampling_density(const MdasDeviceGrid& g, float* pixels, int W, int H, cudaStream_t s) {
    const int P = W * H;
    cudaError_t e = cudaMemsetAsync(pixels, 0, sizeof(float4) * (size_t)P, s);
    if (e != cudaSuccess) return e;
    MDAS_SWITCH_D(g.D, (k_sampling_density<DD><<<1024, 256, 0, s>>>(g, reinterpret_cast<float4*>(pixels), W, H)));
    k_density_alpha<<<(P + 255) / 256, 256, 0, s>>>(reinterpret_cast<float4*>(pixels), P);
    return cudaGetLastError();
}

cudaError_t unpack_records(const MdasDeviceGrid& g, int L, int* nodes, float* boxes, cudaStream_t s) {
    if (L == 0) return cudaSuccess;
    const int grid = (L + 255) / 256 < 4096 ? (L + 255) / 256 : 4096;
    MDAS_SWITCH_D(g.D, (k_unpack_records<DD><<<grid, 256, 0, s>>>(g.nb, L, reinterpret_cast<int4*>(nodes), boxes)));
    return cudaGetLastError();
}

cudaError_t pack_records(const MdasDeviceGrid& g, int L, const int* nodes, const float* boxes, cudaStream_t s) {
    if (L == 0) return cudaSuccess;
    const int grid = (L + 255) / 256 < 4096 ? (L + 255) / 256 : 4096;
    MDAS_SWITCH_D(g.D, (k_pack_records<DD><<<grid, 256, 0, s>>>(g.nb, g.leafCounts, L,
                                                               reinterpret_cast<const int4*>(nodes), boxes, g.coords)));
    return cudaGetLastError();
}

int record_floats(int D) {
    switch (D) {
        case 3: return NbLayout<3>::FLOATS;
        case 4: return NbLayout<4>::FLOATS;
        case 5: return NbLayout<5>::FLOATS;
        case 6: return NbLayout<6>::FLOATS;
    }
    return 0;
}

int max_blocks_per_sm(int D, int which) {
    int n = 0;
    cudaError_t e = cudaSuccess;
    switch (which) {
        case MDAS_K_ERRORS:
            MDAS_SWITCH_D(D, (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_compute_errors<DD, 0>, 256,
                                                                                 0)));
            break;
        case MDAS_K_ADAPTIVE:
            e = place_prepare(D);
            if (e == cudaSuccess)
                MDAS_SWITCH_D(D, (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_adaptive_place<DD>, 256, 0)));
            break;
        case MDAS_K_INTEGRATE:
            MDAS_SWITCH_D(D, (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_integrate<DD>, 256, 0)));
            break;
        case MDAS_K_DECIDE:
            MDAS_SWITCH_D(D, (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_adaptive_decide<DD, 8, false>,
                                                                                 256, 0)));
            break;
        default:
            MDAS_SWITCH_D(D, (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_initial_sampling<DD>, 256, 0)));
            break;
    }
    return e == cudaSuccess ? n : 0;
}

#undef MDAS_SWITCH_D

}  // namespace MDAS_NS
