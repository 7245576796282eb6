// noalloc.cu — one adaptive sampling pass that allocates no memory.
//
// Some callers cannot call cudaMalloc when they run a sampling pass:
//   * a plugin host that hands out all device memory up front and forbids
//     allocations afterwards (its budget is fixed when the plugin loads);
//   * a process whose device memory belongs to another framework's caching
//     allocator, where a library's own cudaMalloc can fail for lack of memory
//     the pool is holding, or fragment it;
//   * a frame-paced renderer for which cudaMalloc/cudaFree are too costly
//     inside the frame: they can synchronise the device and stall it.
// mdas_create allocates the sampler state, so those callers cannot use a grid.
// This entry point runs one pass of KDGrid::AdaptiveSampling on buffers the
// caller already owns, in the layout of the reference's sampler (nodes as
// int4, boxes as mn[D] + mx[D], AoS sample coordinates, per-leaf errors and
// seeds), and keeps its own scratch — the per-tile counts and their prefix —
// in a fixed-size array in device memory that is part of this library (every
// GPU that loads the library holds it until the process exits).
//
// The call reads the new counts back to the host and synchronises the
// caller's stream before it returns, as mdas_adaptive_sampling does.
//
// The pass computes what mdas_adaptive_sampling computes in the reference
// arithmetic (this file is built with --use_fast_math like kdgrid_fast.cu):
// same acceptance test, candidates, splits and slot order (leaf order).
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>
#include <mutex>

#include "../../include/mdas.h"

namespace {

constexpr int kTile = 1024;                 // leaves per tile (256 threads x 4)
constexpr int kMaxLeaves = MDAS_STATIC_MAX_LEAVES;
constexpr int kMaxTiles = kMaxLeaves / kTile;

struct StaticScratch {
    uint2 tileCounts[kMaxTiles];  // (accepted, split) per tile
    uint2 tilePrefix[kMaxTiles];  // exclusive prefix of tileCounts
    int totals[4];                // new samples, new leaves
};

// The scratch.  In host code this name is only a stand-in for the device
// array; the kernels get its device address from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_mdasStaticScratch[sizeof(StaticScratch)];

// ---- RNG of SDK/cuda/random.h:31-67 and the point helpers (reference arithmetic)
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

__device__ __forceinline__ float rnd(unsigned& prev) {
    prev = 1664525u * prev + 1013904223u;
    return (float)(prev & 0x00FFFFFFu) / (float)0x01000000;
}

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

__device__ __forceinline__ int node_get(const int4 n, int i) {
    return i == 0 ? n.x : i == 1 ? n.y : i == 2 ? n.z : n.w;
}

__device__ __forceinline__ int node_count(const int4 n) {
    return (n.x >= 0) + (n.y >= 0) + (n.z >= 0) + (n.w >= 0);
}

struct PassArgs {
    int N, L, candidatesNum;
    float alpha, gError;
    float* coords;
    int4* nodes;
    float* boxes;
    float* errors;
    unsigned* seeds;
    StaticScratch* scratch;
};

// The acceptance test of kdgrid.cu:323-326 for the 4 leaves of one thread;
// returns the accepted mask, the seeds after the draw and the sample counts.
__device__ __forceinline__ unsigned decide4(const PassArgs& a, int i0, unsigned (&seed)[4], int (&cnt)[4]) {
    unsigned acc = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int leaf = i0 + j;
        cnt[j] = 0;
        seed[j] = 0;
        if (leaf < a.L) {
            unsigned s = a.seeds[leaf];
            if (s == 0) s = tea4((unsigned)leaf, 0);
            if (powf(a.errors[leaf] / a.gError, a.alpha) >= rnd(s)) {
                acc |= 1u << j;
                cnt[j] = node_count(a.nodes[leaf]);
            }
            seed[j] = s;
        }
    }
    return acc;
}

// Block-wide exclusive scan of v (lo16 accepted | hi16 split), 256 threads.
__device__ __forceinline__ unsigned block_scan(unsigned v, unsigned* s_warp, unsigned* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned incl = v;
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
    const unsigned excl = (warp ? s_warp[warp - 1] : 0u) + incl - v;
    *total = s_warp[7];
    __syncthreads();
    return excl;
}

__global__ void __launch_bounds__(256) k_static_decide(PassArgs a) {
    __shared__ unsigned s_warp[8];
    const int ntiles = (a.L + kTile - 1) / kTile;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        unsigned seed[4];
        int cnt[4];
        const unsigned acc = decide4(a, tile * kTile + threadIdx.x * 4, seed, cnt);
        unsigned split = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) split += (cnt[j] >= 4) ? 1u : 0u;
        unsigned total;
        block_scan((unsigned)__popc(acc) | (split << 16), s_warp, &total);
        if (threadIdx.x == 0) a.scratch->tileCounts[tile] = make_uint2(total & 0xffffu, total >> 16);
    }
}

__global__ void __launch_bounds__(1024) k_static_scan(PassArgs a) {
    __shared__ unsigned s_a[32], s_b[32];
    const int ntiles = (a.L + kTile - 1) / kTile;
    const int per = (ntiles + 1023) / 1024;
    const int t0 = threadIdx.x * per, t1 = min(t0 + per, ntiles);
    unsigned sa = 0, sb = 0;
    for (int t = t0; t < t1; ++t) {
        sa += a.scratch->tileCounts[t].x;
        sb += a.scratch->tileCounts[t].y;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned ia = sa, ib = sb;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned x = __shfl_up_sync(0xffffffffu, ia, o);
        const unsigned y = __shfl_up_sync(0xffffffffu, ib, o);
        if (lane >= o) {
            ia += x;
            ib += y;
        }
    }
    if (lane == 31) {
        s_a[warp] = ia;
        s_b[warp] = ib;
    }
    __syncthreads();
    if (warp == 0) {
        unsigned x = s_a[lane], y = s_b[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned p = __shfl_up_sync(0xffffffffu, x, o);
            const unsigned q = __shfl_up_sync(0xffffffffu, y, o);
            if (lane >= o) {
                x += p;
                y += q;
            }
        }
        s_a[lane] = x;
        s_b[lane] = y;
    }
    __syncthreads();
    unsigned pa = (warp ? s_a[warp - 1] : 0u) + ia - sa;
    unsigned pb = (warp ? s_b[warp - 1] : 0u) + ib - sb;
    for (int t = t0; t < t1; ++t) {
        const uint2 c = a.scratch->tileCounts[t];
        a.scratch->tilePrefix[t] = make_uint2(pa, pb);
        pa += c.x;
        pb += c.y;
    }
    if (threadIdx.x == 1023) {
        a.scratch->totals[0] = (int)pa;
        a.scratch->totals[1] = (int)pb;
    }
}

// Re-runs the (deterministic) acceptance test of its tile, then does the work of
// kdgrid.cu:332-477 for each accepted leaf, with the slots of the scan.
template <int D>
__global__ void __launch_bounds__(256) k_static_place(PassArgs a) {
    __shared__ unsigned s_warp[8];
    const int ntiles = (a.L + kTile - 1) / kTile;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int i0 = tile * kTile + threadIdx.x * 4;
        unsigned seed[4];
        int cnt[4];
        const unsigned acc = decide4(a, i0, seed, cnt);
        unsigned split = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) split += (cnt[j] >= 4) ? 1u : 0u;
        unsigned total;
        const unsigned excl = block_scan((unsigned)__popc(acc) | (split << 16), s_warp, &total);
        const uint2 pre = a.scratch->tilePrefix[tile];
        unsigned rs = excl & 0xffffu, rp = excl >> 16;
#pragma unroll 1
        for (int j = 0; j < 4; ++j) {
            const int leaf = i0 + j;
            if (leaf >= a.L) break;
            unsigned s = seed[j];
            if ((acc >> j) & 1u) {
                int4 node = a.nodes[leaf];
                float mn[D], mx[D], samples[4][D];
#pragma unroll
                for (int i = 0; i < D; ++i) {
                    mn[i] = a.boxes[(size_t)leaf * 2 * D + i];
                    mx[i] = a.boxes[(size_t)leaf * 2 * D + D + i];
                }
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int idx = node_get(node, k);
#pragma unroll
                    for (int i = 0; i < D; ++i) samples[k][i] = idx >= 0 ? a.coords[(size_t)idx * D + i] : 0.0f;
                }
                float best[D], diag[D];
#pragma unroll
                for (int i = 0; i < D; ++i) {
                    best[i] = 0.0f;
                    diag[i] = mx[i] - mn[i];
                }
                float maxDistance = -1.0f;
                for (int c = 0; c < a.candidatesNum; ++c) {
                    float rr[D], candidate[D];
#pragma unroll
                    for (int i = 0; i < D; ++i) rr[i] = rnd(s);
#pragma unroll
                    for (int i = 0; i < D; ++i) candidate[i] = mn[i] + rr[i] * diag[i];
                    float minDistance = FLT_MAX;
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        if (node_get(node, k) >= 0) {
                            const float dk = distance<D>(candidate, samples[k]);
                            if (minDistance > dk) minDistance = dk;
                        }
                    }
                    if (maxDistance < minDistance) {
                        maxDistance = minDistance;
#pragma unroll
                        for (int i = 0; i < D; ++i) best[i] = candidate[i];
                    }
                }
                const int sampleIndex = a.N + (int)pre.x + (int)rs;
                rs++;
#pragma unroll
                for (int i = 0; i < D; ++i) a.coords[(size_t)sampleIndex * D + i] = best[i];
                const int sampleCount = cnt[j];
                if (sampleCount < 4) {
                    if (sampleCount == 0) node.x = sampleIndex;
                    else if (sampleCount == 1) node.y = sampleIndex;
                    else if (sampleCount == 2) node.z = sampleIndex;
                    else node.w = sampleIndex;
                    a.nodes[leaf] = node;
                } else {
                    int axis = -1;
                    float maxExtent = -FLT_MAX;
#pragma unroll
                    for (int i = D - 1; i >= 0; --i) {
                        if (maxExtent < diag[i]) {
                            maxExtent = diag[i];
                            axis = i;
                        }
                    }
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
                    // positions after the reference's stable bubble sort (kdgrid.cu:408-417)
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
                        if (rank[k] == 1) k1 = key[k];
                        if (rank[k] == 2) k2 = key[k];
                        if (rank[k] == 0) l0 = idx5[k];
                        if (rank[k] == 1) l1 = idx5[k];
                        if (rank[k] == 2) r0 = idx5[k];
                        if (rank[k] == 3) r1 = idx5[k];
                        if (rank[k] == 4) r2 = idx5[k];
                    }
                    const float splitPosition = 0.5f * (k1 + k2);
                    const int nodeOffset = a.L + (int)pre.y + (int)rp;
                    rp++;
                    a.nodes[leaf] = make_int4(l0, l1, ~D, ~D);
                    a.nodes[nodeOffset] = make_int4(r0, r1, r2, ~D);
                    float* lb = a.boxes + (size_t)leaf * 2 * D;
                    float* rb = a.boxes + (size_t)nodeOffset * 2 * D;
#pragma unroll
                    for (int i = 0; i < D; ++i) {
                        rb[i] = (i == axis) ? splitPosition : mn[i];
                        rb[D + i] = mx[i];
                    }
                    lb[D + axis] = splitPosition;
                    a.errors[leaf] = -1.0f;
                    a.errors[nodeOffset] = -1.0f;
                    a.seeds[nodeOffset] = 0u;
                }
            }
            a.seeds[leaf] = s;
        }
        __syncthreads();  // s_warp is reused by the next tile
    }
}

// Device address of the scratch array, looked up once per device (at the first
// call with that device current) and kept for the life of the process.  After
// cudaDeviceReset the library's module is loaded again and the kept address
// is stale, so the call must not be used across a device reset.
std::mutex g_scratchMutex;
void* g_scratchPtr[64] = {nullptr};

int scratch_for_current_device(StaticScratch** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return MDAS_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_scratchMutex);
    if (!g_scratchPtr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_mdasStaticScratch) != cudaSuccess || !p) return MDAS_ERR_CUDA;
        g_scratchPtr[dev] = p;
    }
    *out = static_cast<StaticScratch*>(g_scratchPtr[dev]);
    return MDAS_OK;
}

}  // namespace

extern "C" int mdas_adaptive_sampling_static(int dim, int numberOfSamples, int numberOfNodes, int candidatesNum,
                                             float alpha, float gError, int maxSamples, int nodeCapacity,
                                             float* coords, int* nodes, float* boxes, float* errors, uint32_t* seeds,
                                             int* newSamples, int* newNodes, void* stream) {
    if (dim < 3 || dim > 6 || numberOfSamples < 0 || numberOfNodes < 0 || candidatesNum < 1 || !coords || !nodes ||
        !boxes || !errors || !seeds || !newSamples || !newNodes)
        return MDAS_ERR_INVALID;
    if (numberOfNodes > kMaxLeaves) return MDAS_ERR_INVALID;  // beyond the fixed scratch
    // the pass adds at most one sample and one leaf per leaf
    if ((int64_t)numberOfSamples + numberOfNodes > maxSamples || 2 * (int64_t)numberOfNodes > nodeCapacity)
        return MDAS_ERR_CAPACITY;
    StaticScratch* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    *newSamples = 0;
    *newNodes = 0;
    if (numberOfNodes == 0) return MDAS_OK;
    cudaStream_t s = (cudaStream_t)stream;
    PassArgs a{numberOfSamples, numberOfNodes, candidatesNum, alpha, gError, coords,
               reinterpret_cast<int4*>(nodes), boxes, errors, seeds, scratch};
    int nsm = 1, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int ntiles = (numberOfNodes + kTile - 1) / kTile;
    const int grid = ntiles < nsm * 4 ? ntiles : nsm * 4;
    k_static_decide<<<grid, 256, 0, s>>>(a);
    k_static_scan<<<1, 1024, 0, s>>>(a);
    switch (dim) {
        case 3: k_static_place<3><<<grid, 256, 0, s>>>(a); break;
        case 4: k_static_place<4><<<grid, 256, 0, s>>>(a); break;
        case 5: k_static_place<5><<<grid, 256, 0, s>>>(a); break;
        default: k_static_place<6><<<grid, 256, 0, s>>>(a); break;
    }
    int totals[2] = {0, 0};
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(totals, scratch->totals, sizeof(totals), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    *newSamples = totals[0];
    *newNodes = totals[1];
    return MDAS_OK;
}
