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
//   * one pass over the leaves per stage with persistent CTAs that read the
//     leaf and sample counts from device memory (no host round trip needed);
//   * new sample and leaf slots come from a single-pass decoupled look-back scan
//     over the selection/split flags in leaf order (deterministic), not from
//     warp-aggregated atomics (kdgrid.cu:366-378, 428-440);
//   * stores of the initial samples are staged in shared memory and written
//     out as contiguous 16-byte vectors; the split writes only the one
//     coordinate of the left box that changes;
//   * pixel accumulation uses one 16-byte vector atomic per pixel instead of
//     three scalar ones.
#pragma once

#include <stdint.h>
#include <float.h>
#include <cuda_runtime.h>
#include "grid_types.h"
#include "ieee_math.h"

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

// ---- small vector helpers -----------------------------------------------------
template <int D>
__device__ __forceinline__ void load_point(const float* __restrict__ p, float (&out)[D]) {
    if constexpr (D == 4) {
        const float4 v = *reinterpret_cast<const float4*>(p);
        out[0] = v.x; out[1] = v.y; out[2] = v.z; out[3] = v.w;
    } else if constexpr (D == 6) {
        const float2 a = *reinterpret_cast<const float2*>(p);
        const float2 b = *reinterpret_cast<const float2*>(p + 2);
        const float2 c = *reinterpret_cast<const float2*>(p + 4);
        out[0] = a.x; out[1] = a.y; out[2] = b.x; out[3] = b.y; out[4] = c.x; out[5] = c.y;
    } else {
#pragma unroll
        for (int i = 0; i < D; ++i) out[i] = p[i];
    }
}

template <int D>
__device__ __forceinline__ void store_point(float* __restrict__ p, const float (&v)[D]) {
    if constexpr (D == 4) {
        *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    } else if constexpr (D == 6) {
        *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
        *reinterpret_cast<float2*>(p + 2) = make_float2(v[2], v[3]);
        *reinterpret_cast<float2*>(p + 4) = make_float2(v[4], v[5]);
    } else {
#pragma unroll
        for (int i = 0; i < D; ++i) p[i] = v[i];
    }
}

// Box = mn[D] then mx[D]; 8D bytes per leaf, 8-byte aligned for every D.
template <int D>
__device__ __forceinline__ void load_box(const float* __restrict__ b, float (&mn)[D], float (&mx)[D]) {
    if constexpr (D == 4) {
        const float4 a = *reinterpret_cast<const float4*>(b);
        const float4 c = *reinterpret_cast<const float4*>(b + 4);
        mn[0] = a.x; mn[1] = a.y; mn[2] = a.z; mn[3] = a.w;
        mx[0] = c.x; mx[1] = c.y; mx[2] = c.z; mx[3] = c.w;
    } else {
#pragma unroll
        for (int i = 0; i < D; i += 1) {
            mn[i] = b[i];
            mx[i] = b[D + i];
        }
    }
}

template <int D>
__device__ __forceinline__ void store_box(float* __restrict__ b, const float (&mn)[D], const float (&mx)[D]) {
    if constexpr (D == 4) {
        *reinterpret_cast<float4*>(b) = make_float4(mn[0], mn[1], mn[2], mn[3]);
        *reinterpret_cast<float4*>(b + 4) = make_float4(mx[0], mx[1], mx[2], mx[3]);
    } else {
#pragma unroll
        for (int i = 0; i < D; ++i) {
            b[i] = mn[i];
            b[D + i] = mx[i];
        }
    }
}

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
// samples with the cell's tea<4>/LCG stream, write leaf, box, error -1, seed.
// =====================================================================================
template <int D>
__global__ void __launch_bounds__(256) k_initial_sampling(MdasDeviceGrid g, int L) {
    __shared__ __align__(16) float s_coords[256 * 4 * D];
    __shared__ __align__(16) float s_boxes[256 * 2 * D];
    const int bpd = g.bitsPerDim, eib = g.extraImgBits;
    for (int base = blockIdx.x * 256; base < L; base += gridDim.x * 256) {
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
            const int s0 = 4 * nodeIndex;
            g.nodes[nodeIndex] = make_int4(s0, s0 + 1, s0 + 2, s0 + 3);
#pragma unroll
            for (int i = 0; i < D; ++i) {
                s_boxes[threadIdx.x * 2 * D + i] = offset[i];
                s_boxes[threadIdx.x * 2 * D + D + i] = offset[i] + extent[i];
            }
        }
        __syncthreads();
        {
            // 4*D floats per leaf, leaf `base` starts at a 16*D-byte boundary
            float4* dst = reinterpret_cast<float4*>(g.coords + (size_t)base * 4 * D);
            const float4* src = reinterpret_cast<const float4*>(s_coords);
            for (int k = threadIdx.x; k < n * D; k += 256) dst[k] = src[k];
        }
        {
            // 2*D floats per leaf, leaf `base` (a multiple of 256) starts 16-byte aligned
            const int total = n * 2 * D;
            float* dstf = g.boxes + (size_t)base * 2 * D;
            if ((total & 3) == 0) {
                float4* dst = reinterpret_cast<float4*>(dstf);
                const float4* src = reinterpret_cast<const float4*>(s_boxes);
                for (int k = threadIdx.x; k < total / 4; k += 256) dst[k] = src[k];
            } else {
                float2* dst = reinterpret_cast<float2*>(dstf);
                const float2* src = reinterpret_cast<const float2*>(s_boxes);
                for (int k = threadIdx.x; k < total / 2; k += 256) dst[k] = src[k];
            }
        }
        __syncthreads();
    }
}

// =====================================================================================
// Per-leaf error — computeErrorsKernel, kdgrid.cu:204-288.
// Only leaves with error < 0 (new or just split) are recomputed; stale errors
// of leaves that only gained a sample are kept, as in the reference.  The max
// over all leaves goes to counts->gerr (float bits; all errors are >= 0).
// =====================================================================================
template <int D>
__global__ void __launch_bounds__(256) k_compute_errors(MdasDeviceGrid g) {
    __shared__ unsigned s_max[8];
    __shared__ unsigned s_cnt[8];
    const int L = g.counts->L;
    float maxError = 0.0f;
    unsigned recomputed = 0;
    for (int nodeIndex = blockIdx.x * blockDim.x + threadIdx.x; nodeIndex < L;
         nodeIndex += gridDim.x * blockDim.x) {
        float error = g.errors[nodeIndex];
        if (error < 0.0f) {
            const int4 node = __ldg(g.nodes + nodeIndex);
            float mn[D], mx[D];
            load_box<D>(g.boxes + (size_t)nodeIndex * 2 * D, mn, mx);
            const float volume = box_volume<D>(mn, mx);
            float3 avg = make_float3(0.0f, 0.0f, 0.0f);
            float3 loc[4];
            int sampleCount = 0;
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
            error = 0.0f;
            if (avg.x != 0.0f) error += diffSum.x / avg.x;
            if (avg.y != 0.0f) error += diffSum.y / avg.y;
            if (avg.z != 0.0f) error += diffSum.z / avg.z;
            error /= float(sampleCount);
            error += 1.0e-5f;
            error *= volume;
            g.errors[nodeIndex] = error;
            recomputed++;
        }
        maxError = fmaxf(maxError, error);
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
// from a decoupled look-back scan over tiles of 256 leaves taken in ticket
// order, so a tile only ever waits on tiles that running CTAs already hold.
// =====================================================================================
__device__ __forceinline__ unsigned long long tile_pack(unsigned long long status, unsigned sel, unsigned split) {
    return (status << 62) | ((unsigned long long)split << 31) | (unsigned long long)sel;
}

__device__ __forceinline__ unsigned long long tile_load(const unsigned long long* p) {
    return *reinterpret_cast<const volatile unsigned long long*>(p);
}

__device__ __forceinline__ void tile_store(unsigned long long* p, unsigned long long v) {
    *reinterpret_cast<volatile unsigned long long*>(p) = v;
}

template <int D>
__global__ void __launch_bounds__(256) k_adaptive_sampling(MdasDeviceGrid g) {
    constexpr int kMaxNodeSize = 4;  // KDGrid ctor: maxNodeSize(4), kdgrid.cu:611
    __shared__ int s_tile;
    __shared__ unsigned s_warp[8];
    __shared__ unsigned long long s_prefix;

    const int N = g.counts->N;
    const int L = g.counts->L;
    const float gError = __uint_as_float(g.counts->gerr);
    const int ntiles = (L + MDAS_TILE_LEAVES - 1) / MDAS_TILE_LEAVES;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;

    for (;;) {
        if (threadIdx.x == 0) s_tile = (int)atomicAdd(&g.ctl->ticket, 1u);
        __syncthreads();
        const int tile = s_tile;
        if (tile >= ntiles) break;
        const int nodeIndex = tile * MDAS_TILE_LEAVES + threadIdx.x;
        const bool valid = nodeIndex < L;

        // ---- phase 1: acceptance test and split flag
        unsigned seed = 0;
        bool sel = false;
        int4 node = make_int4(0, 0, 0, 0);
        int sampleCount = 0;
        if (valid) {
            const float error = g.errors[nodeIndex];
            seed = g.seeds[nodeIndex];
            if (seed == 0) seed = tea4((unsigned)nodeIndex, 0);
            sel = mdas_pow(error / gError, g.alpha) >= rnd(seed);
            if (sel) {
                node = g.nodes[nodeIndex];
                sampleCount = node_count(node);
            }
        }
        const bool split = sel && sampleCount >= kMaxNodeSize;

        // ---- block scan of (accepted, split) packed as lo16 | hi16
        const unsigned flag = (sel ? 1u : 0u) | (split ? 0x10000u : 0u);
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
        const unsigned exclInTile = (warp ? s_warp[warp - 1] : 0u) + incl - flag;
        const unsigned tileTotal = s_warp[7];
        if (threadIdx.x == 0) {
            // publish early so that successors can look back while this tile works
            tile_store(g.tiles + tile, tile == 0 ? tile_pack(MDAS_TILE_INC, tileTotal & 0xffffu, tileTotal >> 16)
                                                 : tile_pack(MDAS_TILE_AGG, tileTotal & 0xffffu, tileTotal >> 16));
        }

        // ---- phase 2: best candidate (kdgrid.cu:332-361)
        float samples[4][D];
        float mn[D], mx[D];
        float best[D];
#pragma unroll
        for (int i = 0; i < D; ++i) best[i] = 0.0f;
        if (sel) {
            load_box<D>(g.boxes + (size_t)nodeIndex * 2 * D, mn, mx);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int idx = node_get(node, k);
                if (idx >= 0) load_point<D>(g.coords + (size_t)idx * D, samples[k]);
            }
            float maxDistance = -1.0f;
            float diag[D];
#pragma unroll
            for (int i = 0; i < D; ++i) diag[i] = mx[i] - mn[i];
            for (int j = 0; j < g.candidatesNum; ++j) {
                float r[D];
#pragma unroll
                for (int i = 0; i < D; ++i) r[i] = rnd(seed);
                float candidate[D];
#pragma unroll
                for (int i = 0; i < D; ++i) candidate[i] = mn[i] + r[i] * diag[i];
                float minDistance = FLT_MAX;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (node_get(node, k) >= 0) {
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
        }

        // ---- phase 3: look-back for the tile's exclusive prefix (warp 0)
        if (warp == 0) {
            unsigned preSel = 0, preSplit = 0;
            if (tile > 0) {
                int window = tile - 1;  // lane l inspects tile window - l
                for (;;) {
                    const int pred = window - lane;
                    unsigned long long st = tile_pack(MDAS_TILE_INC, 0, 0);
                    if (pred >= 0) {
                        unsigned spins = 0;
                        st = tile_load(g.tiles + pred);
                        while ((st >> 62) == 0ull) {
                            if (++spins > MDAS_SPIN_LIMIT) {
                                atomicCAS(&g.counts->status, 0, MDAS_ERR_TIMEOUT);
                                st = tile_pack(MDAS_TILE_INC, 0, 0);
                                break;
                            }
                            __nanosleep(64);
                            st = tile_load(g.tiles + pred);
                        }
                    }
                    const bool isInc = (st >> 62) == MDAS_TILE_INC;
                    const unsigned incMask = __ballot_sync(0xffffffffu, isInc);
                    const int firstInc = incMask ? __ffs(incMask) - 1 : 32;
                    const bool take = lane <= firstInc;
                    const unsigned s = take ? (unsigned)(st & 0x7fffffffull) : 0u;
                    const unsigned p = take ? (unsigned)((st >> 31) & 0x7fffffffull) : 0u;
                    preSel += __reduce_add_sync(0xffffffffu, s);
                    preSplit += __reduce_add_sync(0xffffffffu, p);
                    if (incMask) break;
                    window -= 32;
                }
                if (lane == 0)
                    tile_store(g.tiles + tile, tile_pack(MDAS_TILE_INC, preSel + (tileTotal & 0xffffu),
                                                         preSplit + (tileTotal >> 16)));
            }
            if (lane == 0) s_prefix = ((unsigned long long)preSplit << 32) | preSel;
        }
        __syncthreads();

        // ---- phase 4: writes (kdgrid.cu:380-477)
        if (sel) {
            const unsigned long long pre = s_prefix;
            const int sampleIndex = N + (int)(unsigned)pre + (int)(exclInTile & 0xffffu);
            store_point<D>(g.coords + (size_t)sampleIndex * D, best);
            if (!split) {
                // room left: append the index, the error stays as it was
                if (sampleCount == 0) node.x = sampleIndex;
                else if (sampleCount == 1) node.y = sampleIndex;
                else if (sampleCount == 2) node.z = sampleIndex;
                else node.w = sampleIndex;
                g.nodes[nodeIndex] = node;
            } else {
                // split dimension: AABB::LargestAxis, ties to the highest index (aabb.h:34-45)
                int axis = -1;
                float maxExtent = -FLT_MAX;
#pragma unroll
                for (int i = D - 1; i >= 0; --i) {
                    const float e = mx[i] - mn[i];
                    if (maxExtent < e) {
                        maxExtent = e;
                        axis = i;
                    }
                }
                int loc[5];
                float key[5];
                loc[0] = node.x; loc[1] = node.y; loc[2] = node.z; loc[3] = node.w; loc[4] = sampleIndex;
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
                // stable bubble sort of the 5 samples by the split coordinate (kdgrid.cu:408-417)
#pragma unroll
                for (int i = 0; i < 4; i++) {
#pragma unroll
                    for (int j = 0; j < 4 - i; j++) {
                        if (key[j] > key[j + 1]) {
                            const float tk = key[j]; key[j] = key[j + 1]; key[j + 1] = tk;
                            const int tl = loc[j]; loc[j] = loc[j + 1]; loc[j + 1] = tl;
                        }
                    }
                }
                const float splitPosition = 0.5f * (key[1] + key[2]);  // md = 5 >> 1 = 2
                const int nodeOffset = L + (int)(unsigned)(pre >> 32) + (int)(exclInTile >> 16);
                g.nodes[nodeIndex] = make_int4(loc[0], loc[1], ~D, ~D);
                g.nodes[nodeOffset] = make_int4(loc[2], loc[3], loc[4], ~D);
                // left child: only mx[axis] changes
                g.boxes[(size_t)nodeIndex * 2 * D + D + axis] = splitPosition;
                float rmn[D];
#pragma unroll
                for (int i = 0; i < D; ++i) rmn[i] = (i == axis) ? splitPosition : mn[i];
                store_box<D>(g.boxes + (size_t)nodeOffset * 2 * D, rmn, mx);
                g.errors[nodeIndex] = -1.0f;
                g.errors[nodeOffset] = -1.0f;
                // a new slot starts without a seed: the reference's seed buffer is zeroed
                // once at InitialSampling (kdgrid.cu:637) and right-child slots are never
                // written before; writing the 0 here makes that memset unnecessary
                g.seeds[nodeOffset] = 0u;
            }
        }
        if (valid) g.seeds[nodeIndex] = seed;
        // samples gathered by this tile (for the traffic accounting)
        {
            const unsigned gathered = __reduce_add_sync(0xffffffffu, sel ? (unsigned)sampleCount : 0u);
            if (lane == 0 && gathered) atomicAdd(&g.counts->gathered, gathered);
        }
        __syncthreads();
    }

    // ---- the last CTA out commits the counters and resets the tickets
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(&g.ctl->done, 1u);
        if (prev == gridDim.x - 1) {
            __threadfence();
            unsigned newN = 0, newL = 0;
            if (ntiles > 0) {
                const unsigned long long st = tile_load(g.tiles + ntiles - 1);
                newN = (unsigned)(st & 0x7fffffffull);
                newL = (unsigned)((st >> 31) & 0x7fffffffull);
            }
            g.counts->newN = (int)newN;
            g.counts->newL = (int)newL;
            g.counts->selected = (int)newN;
            g.counts->N = N + (int)newN;
            g.counts->L = L + (int)newL;
            g.counts->passes += 1;
            g.ctl->ticket = 0;
            g.ctl->done = 0;
            __threadfence();
        }
    }
}

// =====================================================================================
// Reconstruction — integrateKernel, kdgrid.cu:483-582.
// Each leaf splats mean value * (overlap area * Volume / xyArea) / pixArea into
// the pixels its box covers; pixel edges advance incrementally as in the
// reference so that the footprint is the same to the bit.
// =====================================================================================
template <int D>
__global__ void __launch_bounds__(256) k_integrate(MdasDeviceGrid g, float4* __restrict__ pixels, int width,
                                                    int height) {
    const int L = g.counts->L;
    const float scaleX = g.scaleX, scaleY = g.scaleY;
    for (int nodeIndex = blockIdx.x * blockDim.x + threadIdx.x; nodeIndex < L;
         nodeIndex += gridDim.x * blockDim.x) {
        float2 pixelStep;
        pixelStep.x = scaleX / width;
        pixelStep.y = scaleY / height;
        const int4 node = __ldg(g.nodes + nodeIndex);
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
        float mn[D], mx[D];
        load_box<D>(g.boxes + (size_t)nodeIndex * 2 * D, mn, mx);
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

// ---- host launchers -------------------------------------------------------------
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

cudaError_t compute_errors(const MdasDeviceGrid& g, int grid, cudaStream_t s) {
    // g_error = 0 (kdgrid.cu:684-685) and the recomputed-leaf counter next to it
    cudaError_t e = cudaMemsetAsync(&g.counts->gerr, 0, 2 * sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    MDAS_SWITCH_D(g.D, (k_compute_errors<DD><<<grid, 256, 0, s>>>(g)));
    return cudaGetLastError();
}

cudaError_t adaptive_sampling(const MdasDeviceGrid& g, int grid, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(g.tiles, 0, sizeof(unsigned long long) * (size_t)g.maxTiles, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(&g.counts->gathered, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    MDAS_SWITCH_D(g.D, (k_adaptive_sampling<DD><<<grid, 256, 0, s>>>(g)));
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

int max_blocks_per_sm(int D, int which) {
    int n = 0;
    cudaError_t e = cudaSuccess;
    switch (which) {
        case MDAS_K_ERRORS:
            MDAS_SWITCH_D(D, (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_compute_errors<DD>, 256, 0)));
            break;
        case MDAS_K_ADAPTIVE:
            MDAS_SWITCH_D(D, (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_adaptive_sampling<DD>, 256, 0)));
            break;
        case MDAS_K_INTEGRATE:
            MDAS_SWITCH_D(D, (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_integrate<DD>, 256, 0)));
            break;
        default:
            MDAS_SWITCH_D(D, (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_initial_sampling<DD>, 256, 0)));
            break;
    }
    return e == cudaSuccess ? n : 0;
}

#undef MDAS_SWITCH_D

}  // namespace MDAS_NS
