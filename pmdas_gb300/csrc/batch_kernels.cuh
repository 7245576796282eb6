// batch_kernels.cuh — many images of uneven size, dimension and budget in one
// launch per stage (compiled inside MDAS_NS after kdgrid_kernels.cuh).
//
// Each stage enumerates its work items (initial cells, error leaves, tiles of
// 1024 leaves, accepted leaves, reconstruction leaves) across all images of the
// launch: every CTA computes the per-image item counts from the images' device
// counters and their prefix in shared memory, then walks the global item range
// with a grid stride, mapping each chunk of items to its image by binary search.
// A chunk never spans two images, so every block-wide step (scan, reduction)
// stays within one image.  Per image the work and its results are exactly those
// of the single-image kernels: the item bodies are the same device functions.
//
// Images that reached their budget keep `counts->active == 0` and are skipped;
// the loop condition kernel clears the flag after a pass.
#pragma once

#include "kdgrid_kernels.cuh"

namespace MDAS_NS {

#define MDAS_MAX_BATCH 256

// Exclusive prefix of per-image chunk counts (n <= 256) in s_pre[0..n]; returns the total.
template <class F>
__device__ __forceinline__ int batch_prefix(int n, int* s_pre, unsigned* s_warp, F chunks_of) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned v = threadIdx.x < (unsigned)n ? (unsigned)chunks_of((int)threadIdx.x) : 0u;
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
    if (threadIdx.x < (unsigned)n) s_pre[threadIdx.x] = (int)excl;
    if (threadIdx.x == 0) s_pre[n] = (int)s_warp[7];
    __syncthreads();
    return s_pre[n];
}

// The image whose chunk range holds chunk c: the last i with s_pre[i] <= c.
__device__ __forceinline__ int batch_image_of(const int* s_pre, int n, int c) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_pre[mid] <= c) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ int ceil_div(int a, int b) { return (a + b - 1) / b; }

// ---- initial sampling of every image
template <int D>
__global__ void __launch_bounds__(256) k_batch_init(const MdasBatchImage* __restrict__ imgs, int n) {
    __shared__ __align__(16) float s_coords[256 * 4 * D];
    __shared__ float s_box[256 * 2 * D];
    __shared__ int s_pre[MDAS_MAX_BATCH + 1];
    __shared__ unsigned s_warp[8];
    const int total = batch_prefix(n, s_pre, s_warp, [&](int i) { return ceil_div(imgs[i].initialLeaves, 256); });
    for (int c = blockIdx.x; c < total; c += gridDim.x) {
        const int i = batch_image_of(s_pre, n, c);
        init_chunk<D>(imgs[i].g, imgs[i].initialLeaves, (c - s_pre[i]) * 256, s_coords, s_box);
    }
}

// Counters after the initial sampling; an image takes passes while N < budget
// and the next pass fits (optixMotionBlur.cpp:781, 723-724).
__global__ void k_batch_set_counts(const MdasBatchImage* __restrict__ imgs, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    MdasCounts* c = imgs[i].g.counts;
    const int L = imgs[i].initialLeaves, N = 4 * L;
    c->N = N;
    c->L = L;
    c->newN = 0;
    c->newL = 0;
    c->gerr = c->gerrLast = 0u;
    c->recomputed = c->recomputedLast = 0;
    c->status = 0;
    c->selected = 0;
    c->passes = 0;
    c->gathered = c->gatheredLast = 0u;
    c->gerrNext = c->gerrCarry = 0u;
    c->active = (N < imgs[i].budget && (long long)N + L <= imgs[i].g.maxSamples) ? 1 : 0;
}

// Clears the per-pass statistics of the active learned images before their
// predictions (which = 2; the pass accumulators of MdasCounts need no clearing:
// each pass's scan clears them for the next pass).
__global__ void k_batch_reset(const MdasBatchImage* __restrict__ imgs, int n, int which) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    MdasCounts* c = imgs[i].g.counts;
    if (!c->active) return;
    if (which == 2 && imgs[i].mlp) {
        MdasLearnedStats* st = imgs[i].g.learned;
        // after the first pass the predictions cover only the split children:
        // the largest priority starts from that of the leaves the last pass kept
        st->predMax = c->passes > 0 ? st->keptMax : 0u;
        st->blocksDone = 0u;
        st->usePlain = 0;
        st->unrefinedLearned = 0.0;
        st->unrefinedPlain = 0.0;
    }
}

// ---- learned images: the plain errors each schedule leaves unrefined, over
// chunks of 256 leaves across the active learned images (the largest priority
// came with the predictions).  A block keeps its partial results while its
// chunks stay in one image and adds them to that image's statistics when it
// moves on (a few atomics per block and image); the verdicts follow in
// k_batch_verdict.
// Compensated FP32 sum (Kahan): a thread's unrefined errors over any number of
// leaves within about an ulp, without a per-leaf FP64 add (a slow pipe).
struct KahanF {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        const float y = __fsub_rn(x, c);
        const float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

__device__ __forceinline__ void flush_learned(MdasLearnedStats* st, double ul, double up) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ul += __shfl_xor_sync(0xffffffffu, ul, o);
        up += __shfl_xor_sync(0xffffffffu, up, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (ul != 0.0) atomicAdd(&st->unrefinedLearned, ul);
        if (up != 0.0) atomicAdd(&st->unrefinedPlain, up);
    }
}

__global__ void __launch_bounds__(256) k_batch_learned_reduce(const MdasBatchImage* __restrict__ imgs, int n) {
    __shared__ int s_pre[MDAS_MAX_BATCH + 1];
    __shared__ unsigned s_warp[8];
    // chunks of 1024 leaves: four per thread, 16-byte loads of errors, seeds and
    // priorities (all 256-byte aligned)
    const int total = batch_prefix(n, s_pre, s_warp, [&](int i) {
        return imgs[i].mlp && imgs[i].g.counts->active ? ceil_div(imgs[i].g.counts->L, 1024) : 0;
    });
    int cur = -1;  // the image the block's partial results belong to (uniform across the block)
    KahanF ul, up;
    for (int ch = blockIdx.x; ch < total; ch += gridDim.x) {
        const int img = batch_image_of(s_pre, n, ch);
        if (img != cur) {
            if (cur >= 0) flush_learned(imgs[cur].g.learned, ul.value(), up.value());
            cur = img;
            ul = KahanF();
            up = KahanF();
        }
        const MdasDeviceGrid& g = imgs[img].g;
        const int L = g.counts->L;
        const int i0 = (ch - s_pre[img]) * 1024 + 4 * (int)threadIdx.x;
        if (i0 >= L) continue;
        const float gError = __uint_as_float(g.counts->gerr);
        const float predMax = mdas_float_unorder(g.learned->predMax);
        float e[4], p[4];
        unsigned sd[4];
        const int m = L - i0 < 4 ? L - i0 : 4;
        if (m == 4) {
            const float4 e4 = *reinterpret_cast<const float4*>(g.errors + i0);
            const uint4 s4 = *reinterpret_cast<const uint4*>(g.seeds + i0);
            const float4 p4 = *reinterpret_cast<const float4*>(g.priority + i0);
            e[0] = e4.x; e[1] = e4.y; e[2] = e4.z; e[3] = e4.w;
            sd[0] = s4.x; sd[1] = s4.y; sd[2] = s4.z; sd[3] = s4.w;
            p[0] = p4.x; p[1] = p4.y; p[2] = p4.z; p[3] = p4.w;
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                e[j] = j < m ? g.errors[i0 + j] : 0.0f;
                sd[j] = j < m ? g.seeds[i0 + j] : 0u;
                p[j] = j < m ? g.priority[i0 + j] : 0.0f;
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (j >= m) break;
            unsigned seed = sd[j];
            if (seed == 0) seed = tea4((unsigned)(i0 + j), 0);
            const float r = rnd(seed);
            if (!(mdas_pow(e[j] / gError, g.alpha) >= r)) up.add(e[j]);
            if (!(mdas_pow(learned_ratio_of(p[j], predMax, g.priorityScale), g.alpha) >= r)) ul.add(e[j]);
        }
    }
    if (cur >= 0) flush_learned(imgs[cur].g.learned, ul.value(), up.value());
}

// One thread per image: the verdict of a learned image's pass.
__global__ void k_batch_verdict(const MdasBatchImage* __restrict__ imgs, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !imgs[i].mlp || !imgs[i].g.counts->active) return;
    MdasLearnedStats* st = imgs[i].g.learned;
    const int revert = st->unrefinedLearned > (1.0 + (double)st->tolerance) * st->unrefinedPlain ? 1 : 0;
    st->usePlain = revert;
    st->plainPasses += revert;
    st->judgedPasses += 1;
    st->keptMax = 0u;  // taken by this pass's predMax; the adaptive pass sets it anew
}

// ---- errors: full on an image's first pass, its split children after
template <int D>
__global__ void __launch_bounds__(256) k_batch_errors(const MdasBatchImage* __restrict__ imgs, int n) {
    __shared__ int s_pre[MDAS_MAX_BATCH + 1];
    __shared__ unsigned s_warp[8];
    __shared__ unsigned s_max[8], s_cnt[8];
    const int total = batch_prefix(n, s_pre, s_warp, [&](int i) {
        const MdasCounts* c = imgs[i].g.counts;
        if (!c->active) return 0;
        const int items = c->passes == 0 ? c->L : 2 * c->newL;
        return ceil_div(items, 256) > 0 ? ceil_div(items, 256) : 1;  // one chunk carries gerrNext
    });
    for (int ch = blockIdx.x; ch < total; ch += gridDim.x) {
        const int i = batch_image_of(s_pre, n, ch);
        const MdasDeviceGrid& g = imgs[i].g;
        const MdasCounts* cnt = g.counts;
        const bool dirty = cnt->passes > 0;
        const int newL = cnt->newL;
        const int items = dirty ? 2 * newL : cnt->L;
        const int firstRight = cnt->L - newL;
        const int k = (ch - s_pre[i]) * 256 + threadIdx.x;
        float maxError = dirty ? __uint_as_float(cnt->gerrCarry) : 0.0f;
        unsigned recomputed = 0;
        if (k < items && dirty) {
            // split children from the splitting pass's lists (no leaf record read);
            // learned images also complete the child's raw feature row.  The two
            // children of a split in neighbouring lanes (item kk: left children
            // first, then right ones, as the lists and rows are laid out)
            const int kk = (k & 1) ? newL + (k >> 1) : (k >> 1);
            const bool left = kk < newL;
            const int4 sp = left ? g.splitL[kk] : g.splitR[kk - newL];
            const int nodeIndex = left ? sp.z : firstRight + (kk - newL);
            MdasLumStats lum;
            const float error = node_error<D>(g, make_int4(sp.x, sp.y, left ? ~D : sp.z, ~D), __int_as_float(sp.w),
                                              g.featRaw ? &lum : nullptr);
            if (g.featRaw) mdas_raw_store_stats(g.featRaw + (size_t)kk * MDAS_RAW_FLOATS, lum, error);
            g.errors[nodeIndex] = error;
            recomputed = 1;
            maxError = fmaxf(maxError, error);
        } else if (k < items) {
            float error = g.errors[k];
            if (error < 0.0f) {
                error = leaf_error<D>(g, k);
                g.errors[k] = error;
                recomputed = 1;
            }
            maxError = fmaxf(maxError, error);
        }
        unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(maxError));
        unsigned r = __reduce_add_sync(0xffffffffu, recomputed);
        if ((threadIdx.x & 31) == 0) {
            s_max[threadIdx.x >> 5] = m;
            s_cnt[threadIdx.x >> 5] = r;
        }
        __syncthreads();
        if (threadIdx.x < 32) {
            m = threadIdx.x < 8 ? s_max[threadIdx.x] : 0u;
            r = threadIdx.x < 8 ? s_cnt[threadIdx.x] : 0u;
            m = __reduce_max_sync(0xffffffffu, m);
            r = __reduce_add_sync(0xffffffffu, r);
            if (threadIdx.x == 0) {
                atomicMax(&g.counts->gerr, m);
                if (r) atomicAdd(&g.counts->recomputed, (int)r);
            }
        }
        __syncthreads();
    }
}

// ---- adaptive pass: decide
// LEARNED: some image of the batch is learned (else the lean plain kernel).
template <int D, int K, bool LEARNED>
__global__ void __launch_bounds__(256, LEARNED ? 3 : 4) k_batch_decide(const MdasBatchImage* __restrict__ imgs, int n) {
    pdl_launch_dependents();
    __shared__ int s_pre[MDAS_MAX_BATCH + 1];
    __shared__ unsigned s_warp[8];
    const int total = batch_prefix(n, s_pre, s_warp, [&](int i) {
        const MdasCounts* c = imgs[i].g.counts;
        return c->active ? ceil_div(c->L, 256 * K) : 0;
    });
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int i = batch_image_of(s_pre, n, t);
        const MdasDeviceGrid& g = imgs[i].g;
        const int L = g.counts->L;
        const float gError = __uint_as_float(g.counts->gerr);
        float keptMax = 0.0f;
        unsigned gathered = 0, keptPrio = 0;
        decide_tile<D, K, LEARNED>(g, t - s_pre[i], L, gError, imgs[i].jumpA, imgs[i].jumpC, s_warp, keptMax,
                                   gathered, keptPrio);
        const unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(keptMax));
        const unsigned c = __reduce_add_sync(0xffffffffu, gathered);
        if ((threadIdx.x & 31) == 0) {
            if (m) atomicMax(&g.counts->gerrNext, m);
            if (c) atomicAdd(&g.counts->gathered, c);
        }
        if constexpr (LEARNED) {
            const unsigned kp = __reduce_max_sync(0xffffffffu, keptPrio);
            if ((threadIdx.x & 31) == 0 && kp) atomicMax(&g.learned->keptMax, kp);
        }
    }
}

// ---- adaptive pass: scan (one CTA of 1024 threads per image)
__global__ void __launch_bounds__(1024) k_batch_scan(const MdasBatchImage* __restrict__ imgs, int n) {
    pdl_wait();
    pdl_launch_dependents();
    __shared__ unsigned s_sel[32], s_split[32];
    if ((int)blockIdx.x >= n) return;
    const MdasDeviceGrid& g = imgs[blockIdx.x].g;
    if (!g.counts->active) return;
    scan_image(g, s_sel, s_split);
}

// ---- adaptive pass: place (one thread per accepted leaf)
template <int D>
__global__ void __launch_bounds__(256, 4) k_batch_place(const MdasBatchImage* __restrict__ imgs, int n) {
    pdl_wait();
    __shared__ int s_pre[MDAS_MAX_BATCH + 1];
    __shared__ unsigned s_warp[8];
    const int total = batch_prefix(n, s_pre, s_warp, [&](int i) {
        const MdasDeviceGrid& g = imgs[i].g;
        return g.counts->active ? ceil_div(g.counts->newN, 256) : 0;
    });
    for (int c = blockIdx.x; c < total; c += gridDim.x) {
        const int i = batch_image_of(s_pre, n, c);
        const MdasDeviceGrid& g = imgs[i].g;
        const int k = (c - s_pre[i]) * 256 + threadIdx.x;
        if (k < g.counts->newN) place_rank<D>(g, k, g.ctl->N0, g.ctl->L0);
    }
}

// ---- loop condition over all images of the batch (one CTA of 256 threads)
// anyOut: where the host-driven loop reads the verdict (nullptr: the graph's
// conditional handle h takes it).
__global__ void __launch_bounds__(256) k_batch_condition(const MdasBatchImage* __restrict__ imgs, int n,
                                                          cudaGraphConditionalHandle h, int maxPasses, int* anyOut) {
    __shared__ int s_any[8];
    int act = 0;
    if (threadIdx.x < (unsigned)n) {
        MdasCounts* c = imgs[threadIdx.x].g.counts;
        if (c->active) {
            const long long N = c->N, L = c->L;
            act = (N < imgs[threadIdx.x].budget && N + L <= imgs[threadIdx.x].g.maxSamples && c->status == 0 &&
                   c->passes < maxPasses) ? 1 : 0;
            c->active = act;
        }
    }
    const int any = __reduce_or_sync(0xffffffffu, (unsigned)act);
    if ((threadIdx.x & 31) == 0) s_any[threadIdx.x >> 5] = any;
    __syncthreads();
    if (threadIdx.x == 0) {
        int a = 0;
        for (int w = 0; w < 8; ++w) a |= s_any[w];
        if (anyOut) *anyOut = a;
        else cudaGraphSetConditional(h, a ? 1u : 0u);
    }
}

// ---- reconstruction of every image
__global__ void k_batch_clear_pixels(const MdasBatchImage* __restrict__ imgs, int n) {
    const int i = blockIdx.y;
    if (i >= n) return;
    const int P = imgs[i].width * imgs[i].height;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x)
        imgs[i].pixels[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

template <int D>
__global__ void __launch_bounds__(256) k_batch_integrate(const MdasBatchImage* __restrict__ imgs, int n) {
    constexpr int H4 = (4 + 2 * D + 3) / 4;
    __shared__ int s_pre[MDAS_MAX_BATCH + 1];
    __shared__ unsigned s_warp[8];
    __shared__ float4 s_head[8][32 * H4];
    const int total = batch_prefix(n, s_pre, s_warp, [&](int i) { return ceil_div(imgs[i].g.counts->L, 256); });
    const int warp = threadIdx.x >> 5;
    for (int c = blockIdx.x; c < total; c += gridDim.x) {
        const int i = batch_image_of(s_pre, n, c);
        const int first = (c - s_pre[i]) * 256 + 32 * warp;
        int4 node;
        float mn[D], mx[D];
        if (warp_leaf_head<D>(imgs[i].g.nb, first, imgs[i].g.counts->L, s_head[warp], node, mn, mx))
            integrate_leaf<D>(imgs[i].g, node, mn, mx, imgs[i].pixels, imgs[i].width, imgs[i].height);
    }
}

// ---- host launchers (one group of images of one point dimension)
#define MDAS_BATCH_SWITCH_D(D, EXPR)           \
    switch (D) {                               \
        case 3: { constexpr int DD = 3; EXPR; } break; \
        case 4: { constexpr int DD = 4; EXPR; } break; \
        case 5: { constexpr int DD = 5; EXPR; } break; \
        case 6: { constexpr int DD = 6; EXPR; } break; \
        default: return cudaErrorInvalidValue; \
    }

cudaError_t batch_init(const MdasBatchImage* imgs, int n, int D, int grid, cudaStream_t s) {
    MDAS_BATCH_SWITCH_D(D, (k_batch_init<DD><<<grid, 256, 0, s>>>(imgs, n)));
    return cudaGetLastError();
}

cudaError_t batch_set_counts(const MdasBatchImage* imgs, int n, cudaStream_t s) {
    k_batch_set_counts<<<(n + 255) / 256, 256, 0, s>>>(imgs, n);
    return cudaGetLastError();
}

cudaError_t batch_errors(const MdasBatchImage* imgs, int n, int D, int grid, cudaStream_t s) {
    MDAS_BATCH_SWITCH_D(D, (k_batch_errors<DD><<<grid, 256, 0, s>>>(imgs, n)));
    return cudaGetLastError();
}

cudaError_t batch_reset(const MdasBatchImage* imgs, int n, int which, cudaStream_t s) {
    k_batch_reset<<<(n + 255) / 256, 256, 0, s>>>(imgs, n, which);
    return cudaGetLastError();
}

cudaError_t batch_learned_judge(const MdasBatchImage* imgs, int n, int grid, cudaStream_t s) {
    k_batch_learned_reduce<<<grid, 256, 0, s>>>(imgs, n);
    k_batch_verdict<<<(n + 255) / 256, 256, 0, s>>>(imgs, n);
    return cudaGetLastError();
}

// K: leaves per thread of decide (4 or 8); every image of the group has tileK == K.
// learned: some image of the batch takes the learned acceptance.
cudaError_t batch_decide(const MdasBatchImage* imgs, int n, int D, int K, bool learned, int grid, cudaStream_t s) {
    if (learned && K == 4) {
        MDAS_BATCH_SWITCH_D(D, (k_batch_decide<DD, 4, true><<<grid, 256, 0, s>>>(imgs, n)));
    } else if (learned) {
        MDAS_BATCH_SWITCH_D(D, (k_batch_decide<DD, 8, true><<<grid, 256, 0, s>>>(imgs, n)));
    } else if (K == 4) {
        MDAS_BATCH_SWITCH_D(D, (k_batch_decide<DD, 4, false><<<grid, 256, 0, s>>>(imgs, n)));
    } else {
        MDAS_BATCH_SWITCH_D(D, (k_batch_decide<DD, 8, false><<<grid, 256, 0, s>>>(imgs, n)));
    }
    return cudaGetLastError();
}

cudaError_t batch_scan(const MdasBatchImage* imgs, int n, cudaStream_t s) {
    cudaError_t e = launch_pdl(k_batch_scan, n, 1024, s, imgs, n);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

cudaError_t batch_place(const MdasBatchImage* imgs, int n, int D, int grid, cudaStream_t s) {
    cudaError_t e = cudaSuccess;
    MDAS_BATCH_SWITCH_D(D, (e = launch_pdl(k_batch_place<DD>, grid, 256, s, imgs, n)));
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

cudaError_t batch_condition(const MdasBatchImage* imgs, int n, cudaGraphConditionalHandle h, int maxPasses,
                            int* anyOut, cudaStream_t s) {
    k_batch_condition<<<1, 256, 0, s>>>(imgs, n, h, maxPasses, anyOut);
    return cudaGetLastError();
}

cudaError_t batch_integrate(const MdasBatchImage* imgs, int n, int D, int grid, cudaStream_t s) {
    MDAS_BATCH_SWITCH_D(D, (k_batch_integrate<DD><<<grid, 256, 0, s>>>(imgs, n)));
    return cudaGetLastError();
}

cudaError_t batch_clear_pixels(const MdasBatchImage* imgs, int n, cudaStream_t s) {
    k_batch_clear_pixels<<<dim3(64, n), 256, 0, s>>>(imgs, n);
    return cudaGetLastError();
}

unsigned batch_jump(int candidatesNum, int D, unsigned* C) {
    unsigned A;
    lcg_jump((unsigned)(candidatesNum * D), &A, C);
    return A;
}

#undef MDAS_BATCH_SWITCH_D

}  // namespace MDAS_NS
