// integrand.cu — the analytic integrand kernel and the seeded scene generators.
//
// Stands in for the reference's OptiX launch over the sample buffer
// (launchSubframe, SDK/optixMotionBlur/optixMotionBlur.cpp:420-470): evaluates
// samples [offset, offset + count) of a grid's coordinate buffer into its value
// buffer.  Compiled with strict IEEE flags so the CPU oracle, which shares
// integrand.h, gets identical values.
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>
#include <algorithm>
#include <vector>
#include "integrand.h"
#include "grid_types.h"
#include "scene.h"

namespace {

// ---- disc culling ---------------------------------------------------------------------
__host__ __device__ inline bool mdas_culled_kind(int kind) {
    return kind == MDAS_SCENE_DISCS_MB || kind == MDAS_SCENE_DISCS_DOF || kind == MDAS_SCENE_DISCS_MBDOF;
}

// Can disc p cover a sample whose image point lies in [x0, x1] x [y0, y1] (in
// [0, 1] image units)?  Motion blur: the disc's centre sweeps the box between
// its positions at t = 0 and t = 1.  Depth of field: the ray meets the disc's
// plane at s * focal * (nx * filmHalfW, ny * filmHalfH) + (1 - s) * lens point,
// s = depth / focal, |lens point| <= lensRadius.  So the disc can be hit only
// if the distance between those two boxes is within r (+ |1 - s| * lensRadius).
// NaNs keep the disc (only a certain miss drops it).
__device__ bool cull_may_cover(const MdasScene& sc, const float* p, float x0, float x1, float y0, float y1) {
    const bool moving = sc.kind != MDAS_SCENE_DISCS_DOF;
    const float vx = moving ? p[4] : 0.0f, vy = moving ? p[5] : 0.0f;
    const float cx0 = p[0] + fminf(0.0f, vx), cx1 = p[0] + fmaxf(0.0f, vx);
    const float cy0 = p[1] + fminf(0.0f, vy), cy1 = p[1] + fmaxf(0.0f, vy);
    float bx0 = x0, bx1 = x1, by0 = y0, by1 = y1, reach = sqrtf(fmaxf(p[7], 0.0f));
    float scale = 1.0f;
    if (sc.kind != MDAS_SCENE_DISCS_MB) {
        const float s = p[6];
        const float ax = s * sc.focalDistance * sc.filmHalfW, ay = s * sc.focalDistance * sc.filmHalfH;
        const float ux0 = ax * (2.0f * x0 - 1.0f), ux1 = ax * (2.0f * x1 - 1.0f);
        const float uy0 = ay * (2.0f * y0 - 1.0f), uy1 = ay * (2.0f * y1 - 1.0f);
        bx0 = fminf(ux0, ux1);
        bx1 = fmaxf(ux0, ux1);
        by0 = fminf(uy0, uy1);
        by1 = fmaxf(uy0, uy1);
        reach += fabsf(1.0f - s) * fabsf(sc.lensRadius);
        scale += fabsf(ax) + fabsf(ay) + fabsf(sc.lensRadius);
    }
    scale += fabsf(cx0) + fabsf(cx1) + fabsf(cy0) + fabsf(cy1) + reach;
    const float dx = fmaxf(fmaxf(cx0 - bx1, bx0 - cx1), 0.0f);
    const float dy = fmaxf(fmaxf(cy0 - by1, by0 - cy1), 0.0f);
    const float dist = sqrtf(dx * dx + dy * dy);
    return !(dist > reach + 1.0e-3f * scale);
}

// One warp per (tile, mask word): lane b tests disc 32 * word + b, the
// ballot is the word.
__global__ void __launch_bounds__(256) k_build_cull(MdasScene sc, const float* __restrict__ prims,
                                                     unsigned* __restrict__ masks) {
    constexpr int T = MDAS_CULL_TILES;
    const int words = (sc.count + 31) / 32;
    const int total = T * T * words;
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < total; i += warps) {
        const int tile = i / words, w = i - tile * words;
        const int tx = tile % T, ty = tile / T;
        const float pad = 1.0e-4f;
        const float x0 = (float)tx / T - pad, x1 = (float)(tx + 1) / T + pad;
        const float y0 = (float)ty / T - pad, y1 = (float)(ty + 1) / T + pad;
        const int k = 32 * w + lane;
        const bool may = k < sc.count && cull_may_cover(sc, prims + MDAS_PRIM_STRIDE * k, x0, x1, y0, y1);
        const unsigned m = __ballot_sync(0xffffffffu, may);
        if (lane == 0) masks[i] = m;
    }
}

__device__ __forceinline__ int cull_tile(float px, float py) {
    constexpr int T = MDAS_CULL_TILES;
    const int tx = min(max((int)(px * (float)T), 0), T - 1);
    const int ty = min(max((int)(py * (float)T), 0), T - 1);
    return ty * T + tx;
}

// mdas_shade over the tile's candidate discs: the same tests in the same order
// as the full scans of integrand.h (the direct-light kind is not culled).
__device__ void shade_culled(const MdasScene& sc, const float* prims, const unsigned* __restrict__ cull,
                             const float* c, float* out) {
    const int words = (sc.count + 31) / 32;
    float R = sc.background, G = sc.background, B = sc.background;
    if (sc.kind == MDAS_SCENE_DISCS_MB) {
        const float px = c[0] / sc.scaleX;
        const float py = c[1] / sc.scaleY;
        const float t = c[2];
        const unsigned* m = cull + (size_t)cull_tile(px, py) * words;
        // the last listed covering disc wins: from the back
        for (int w = words - 1; w >= 0; --w) {
            unsigned bits = m[w];
            while (bits) {
                const int b = 31 - __clz(bits);
                bits &= ~(1u << b);
                const float* p = prims + MDAS_PRIM_STRIDE * (32 * w + b);
                if (mdas_disc_mb_covers(p, px, py, t)) {
                    R = p[8];
                    G = p[9];
                    B = p[10];
                    goto done;
                }
            }
        }
    } else if (sc.kind == MDAS_SCENE_DISCS_DOF || sc.kind == MDAS_SCENE_DISCS_MBDOF) {
        const int moving = sc.kind == MDAS_SCENE_DISCS_MBDOF;
        float t, lx, ly, wx, wy;
        mdas_dof_ray(&sc, c, moving, &t, &lx, &ly, &wx, &wy);
        const unsigned* m = cull + (size_t)cull_tile(c[0] / sc.scaleX, c[1] / sc.scaleY) * words;
        for (int w = 0; w < words; ++w) {
            unsigned bits = m[w];
            while (bits) {
                const int b = __ffs(bits) - 1;
                bits &= bits - 1u;
                const float* p = prims + MDAS_PRIM_STRIDE * (32 * w + b);
                if (mdas_disc_dof_covers(p, lx, ly, wx, wy, t, moving)) {
                    R = p[8];
                    G = p[9];
                    B = p[10];
                    goto done;
                }
            }
        }
    } else {
        mdas_shade(&sc, prims, c, out);
        return;
    }
done:
    out[0] = R;
    out[1] = G;
    out[2] = B;
}

template <int D>
__global__ void __launch_bounds__(256) k_evaluate(MdasScene sc, const float* __restrict__ prims,
                                                   const unsigned* __restrict__ cull, const float* __restrict__ coords,
                                                   float* __restrict__ values, const MdasCounts* __restrict__ counts,
                                                   int offset, int count) {
    // a full scan reads every primitive for every sample: staged in shared
    // memory; a culled scan reads a few, straight from the (L1-resident) table
    extern __shared__ float s_prims[];
    if (!cull) {
        const int nfl = sc.count * MDAS_PRIM_STRIDE;
        for (int k = threadIdx.x; k < nfl; k += blockDim.x) s_prims[k] = prims[k];
        __syncthreads();
    }
    if (counts) {  // the samples the last adaptive pass added
        offset = counts->N - counts->newN;
        count = counts->newN;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const size_t s = (size_t)offset + i;
        float c[D];
#pragma unroll
        for (int d = 0; d < D; ++d) c[d] = coords[s * D + d];
        float out[3];
        if (cull) shade_culled(sc, prims, cull, c, out);
        else mdas_shade(&sc, s_prims, c, out);
        values[3 * s + 0] = out[0];
        values[3 * s + 1] = out[1];
        values[3 * s + 2] = out[2];
    }
}

// Batched integrand: chunks of 256 samples across the images of one launch
// (same enumeration scheme as the batched MDAS kernels); primitives are read
// from global memory (L1/L2-resident), as several scenes share a launch.
template <int D>
__global__ void __launch_bounds__(256) k_evaluate_batch(const MdasBatchScene* __restrict__ scenes, int n, int all) {
    __shared__ int s_pre[257];
    __shared__ unsigned s_warp[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned v = 0;
    if (threadIdx.x < (unsigned)n) {
        const MdasCounts* c = scenes[threadIdx.x].counts;
        const int items = all ? scenes[threadIdx.x].initialSamples : (c->active ? c->newN : 0);
        v = (unsigned)((items + 255) / 256);
    }
    unsigned incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        unsigned w = lane < 8 ? s_warp[lane] : 0u;
        for (int o = 1; o < 8; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < 8) s_warp[lane] = w;
    }
    __syncthreads();
    if (threadIdx.x < (unsigned)n) s_pre[threadIdx.x] = (int)((warp ? s_warp[warp - 1] : 0u) + incl - v);
    if (threadIdx.x == 0) s_pre[n] = (int)s_warp[7];
    __syncthreads();
    const int total = s_pre[n];
    for (int ch = blockIdx.x; ch < total; ch += gridDim.x) {
        int lo = 0, hi = n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_pre[mid] <= ch) lo = mid;
            else hi = mid - 1;
        }
        const MdasBatchScene& b = scenes[lo];
        const int offset = all ? 0 : b.counts->N - b.counts->newN;
        const int count = all ? b.initialSamples : b.counts->newN;
        const int k = (ch - s_pre[lo]) * 256 + threadIdx.x;
        if (k < count) {
            const size_t s = (size_t)offset + k;
            float c[D];
#pragma unroll
            for (int d = 0; d < D; ++d) c[d] = b.coords[s * D + d];
            float out[3];
            if (b.cull) shade_culled(b.sc, b.prims, b.cull, c, out);
            else mdas_shade(&b.sc, b.prims, c, out);
            b.values[3 * s + 0] = out[0];
            b.values[3 * s + 1] = out[1];
            b.values[3 * s + 2] = out[2];
        }
    }
}

// Reference image of an integrand: `spp` samples per pixel, the image plane
// stratified on a sqrt(spp) x sqrt(spp) grid with jitter, the other dimensions
// uniform, radiance accumulated in FP64 (the only FP64 work on the GPU).  One
// thread per pixel; the sample stream is a per-pixel 64-bit LCG (Knuth's
// MMIX constants), 24 random bits per float.
struct Lcg64 {
    unsigned long long s;
    __device__ float next() {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        return (float)(unsigned)(s >> 40) * (1.0f / 16777216.0f);
    }
};

template <int D>
__global__ void __launch_bounds__(256) k_reference_image(MdasScene sc, const float* __restrict__ prims, int width,
                                                          int height, int strata, unsigned long long seed,
                                                          double* __restrict__ out) {
    extern __shared__ float s_prims[];
    const int nfl = sc.count * MDAS_PRIM_STRIDE;
    for (int k = threadIdx.x; k < nfl; k += blockDim.x) s_prims[k] = prims[k];
    __syncthreads();
    const int P = width * height;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
        const int x = p % width, y = p / width;
        Lcg64 rng{seed ^ (0x9E3779B97F4A7C15ull * (unsigned long long)(p + 1))};
        double acc[3] = {0.0, 0.0, 0.0};
        const float px = sc.scaleX / (float)width, py = sc.scaleY / (float)height;
        for (int i = 0; i < strata; ++i) {
            for (int j = 0; j < strata; ++j) {
                float c[D];
                c[0] = ((float)x + ((float)i + rng.next()) / (float)strata) * px;
                c[1] = ((float)y + ((float)j + rng.next()) / (float)strata) * py;
#pragma unroll
                for (int d = 2; d < D; ++d) c[d] = rng.next();
                float v[3];
                mdas_shade(&sc, s_prims, c, v);
                acc[0] += (double)v[0];
                acc[1] += (double)v[1];
                acc[2] += (double)v[2];
            }
        }
        const double inv = 1.0 / ((double)strata * (double)strata);
        out[3 * (size_t)p + 0] = acc[0] * inv;
        out[3 * (size_t)p + 1] = acc[1] * inv;
        out[3 * (size_t)p + 2] = acc[2] * inv;
    }
}

// True reconstruction error of each leaf (the training target of the learned
// leaf priority): the leaf's mean sample value against the integrand's mean
// over the leaf's box, estimated from `samples` uniform points with FP64
// accumulation; err = volume * sum_c |mean_c - ref_c| / sqrt(ref_c^2 + 1e-2),
// in the units of the plain error (a relative deviation times the volume,
// image axes in pixels).
template <int D>
__global__ void __launch_bounds__(256) k_leaf_true_errors(MdasScene sc, const float* __restrict__ prims,
                                                           MdasDeviceGrid g, const int* __restrict__ leaves, int L,
                                                           int samples, unsigned long long seed,
                                                           float* __restrict__ out) {
    extern __shared__ float s_prims[];
    const int nfl = sc.count * MDAS_PRIM_STRIDE;
    for (int k = threadIdx.x; k < nfl; k += blockDim.x) s_prims[k] = prims[k];
    __syncthreads();
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < L; row += gridDim.x * blockDim.x) {
        const int i = leaves ? leaves[row] : row;
        const float* nb = g.nb + (size_t)i * g.nbFloats;
        const int idx[4] = {reinterpret_cast<const int*>(nb)[0], reinterpret_cast<const int*>(nb)[1],
                            reinterpret_cast<const int*>(nb)[2], reinterpret_cast<const int*>(nb)[3]};
        float mn[D], mx[D];
        float volume = 1.0f;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            mn[d] = nb[4 + d];
            mx[d] = nb[4 + D + d];
            volume *= mx[d] - mn[d];
        }
        float mean[3] = {0.0f, 0.0f, 0.0f};
        int n = 0;
        for (int k = 0; k < 4; ++k) {
            if (idx[k] < 0) continue;
            for (int c = 0; c < 3; ++c) mean[c] += g.values[3 * (size_t)idx[k] + c];
            ++n;
        }
        for (int c = 0; c < 3; ++c) mean[c] = n ? mean[c] / (float)n : 0.0f;
        Lcg64 rng{seed ^ (0x9E3779B97F4A7C15ull * (unsigned long long)(i + 1))};
        double acc[3] = {0.0, 0.0, 0.0};
        for (int s = 0; s < samples; ++s) {
            float c[D];
#pragma unroll
            for (int d = 0; d < D; ++d) c[d] = mn[d] + rng.next() * (mx[d] - mn[d]);
            float v[3];
            mdas_shade(&sc, s_prims, c, v);
            acc[0] += (double)v[0];
            acc[1] += (double)v[1];
            acc[2] += (double)v[2];
        }
        double e = 0.0;
        for (int c = 0; c < 3; ++c) {
            const double ref = acc[c] / (double)samples;
            e += fabs((double)mean[c] - ref) / sqrt(ref * ref + 1e-2);
        }
        out[row] = (float)(e * (double)volume);
    }
}

// splitmix64 (Steele, Lea & Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014): the documented stream every scene is drawn from.
struct SplitMix64 {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    // 24 random bits -> [0, 1)
    float uniform() { return (float)(next() >> 40) * (1.0f / 16777216.0f); }
    float range(float a, float b) { return a + (b - a) * uniform(); }
};

}  // namespace

cudaError_t mdas_launch_leaf_true_errors(const MdasScene& sc, const float* d_prims, const MdasDeviceGrid& g,
                                         const int* leaves, int L, int samples, unsigned long long seed, float* out,
                                         cudaStream_t s) {
    if (L <= 0) return cudaSuccess;
    const size_t smem = sizeof(float) * MDAS_PRIM_STRIDE * (size_t)sc.count;
    const int grid = (L + 255) / 256 < 65535 ? (L + 255) / 256 : 65535;
    switch (g.D) {
        case 3: k_leaf_true_errors<3><<<grid, 256, smem, s>>>(sc, d_prims, g, leaves, L, samples, seed, out); break;
        case 4: k_leaf_true_errors<4><<<grid, 256, smem, s>>>(sc, d_prims, g, leaves, L, samples, seed, out); break;
        case 5: k_leaf_true_errors<5><<<grid, 256, smem, s>>>(sc, d_prims, g, leaves, L, samples, seed, out); break;
        case 6: k_leaf_true_errors<6><<<grid, 256, smem, s>>>(sc, d_prims, g, leaves, L, samples, seed, out); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

size_t mdas_cull_words(const MdasScene& sc) {
    if (!mdas_culled_kind(sc.kind) || sc.count <= 0) return 0;
    return (size_t)MDAS_CULL_TILES * MDAS_CULL_TILES * (size_t)((sc.count + 31) / 32);
}

cudaError_t mdas_launch_build_cull(const MdasScene& sc, const float* d_prims, unsigned* masks, cudaStream_t s) {
    const size_t words = mdas_cull_words(sc);
    if (words == 0) return cudaSuccess;
    if (!masks) return cudaErrorInvalidValue;
    const size_t blocks = (words + 7) / 8;  // 8 warps per block, one mask word per warp
    k_build_cull<<<(unsigned)(blocks < 8192 ? blocks : 8192), 256, 0, s>>>(sc, d_prims, masks);
    return cudaGetLastError();
}

cudaError_t mdas_launch_evaluate(const MdasScene& sc, const float* d_prims, const unsigned* cull, const float* coords,
                                 float* values, int dim, const MdasCounts* counts, int offset, int count, int grid,
                                 cudaStream_t s) {
    if (grid <= 0) grid = 1;
    if (dim < sc.dim) return cudaErrorInvalidValue;
    if (!mdas_culled_kind(sc.kind)) cull = nullptr;
    const size_t smem = cull ? 0 : sizeof(float) * MDAS_PRIM_STRIDE * (size_t)sc.count;
    switch (dim) {
        case 3: k_evaluate<3><<<grid, 256, smem, s>>>(sc, d_prims, cull, coords, values, counts, offset, count); break;
        case 4: k_evaluate<4><<<grid, 256, smem, s>>>(sc, d_prims, cull, coords, values, counts, offset, count); break;
        case 5: k_evaluate<5><<<grid, 256, smem, s>>>(sc, d_prims, cull, coords, values, counts, offset, count); break;
        case 6: k_evaluate<6><<<grid, 256, smem, s>>>(sc, d_prims, cull, coords, values, counts, offset, count); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t mdas_launch_evaluate_batch(const MdasBatchScene* scenes, int n, int D, int all, int grid, cudaStream_t s) {
    switch (D) {
        case 3: k_evaluate_batch<3><<<grid, 256, 0, s>>>(scenes, n, all); break;
        case 4: k_evaluate_batch<4><<<grid, 256, 0, s>>>(scenes, n, all); break;
        case 5: k_evaluate_batch<5><<<grid, 256, 0, s>>>(scenes, n, all); break;
        case 6: k_evaluate_batch<6><<<grid, 256, 0, s>>>(scenes, n, all); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t mdas_launch_reference_image(const MdasScene& sc, const float* d_prims, int width, int height, int strata,
                                        unsigned long long seed, double* out, int grid, cudaStream_t s) {
    const size_t smem = sizeof(float) * MDAS_PRIM_STRIDE * (size_t)sc.count;
    switch (sc.dim) {
        case 3: k_reference_image<3><<<grid, 256, smem, s>>>(sc, d_prims, width, height, strata, seed, out); break;
        case 4: k_reference_image<4><<<grid, 256, smem, s>>>(sc, d_prims, width, height, strata, seed, out); break;
        case 5: k_reference_image<5><<<grid, 256, smem, s>>>(sc, d_prims, width, height, strata, seed, out); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// Scene generators.  Draw order is part of the format: the same seed gives the
// same primitives on every machine (host code is built with -ffp-contract=off).
int mdas_generate_scene(int kind, uint64_t seed, int count, float scaleX, float scaleY, int width, int height,
                        MdasScene* sc, std::vector<float>* prims) {
    if (count < 0 || count > MDAS_MAX_PRIMS || width <= 0 || height <= 0) return MDAS_ERR_INVALID;
    *sc = MdasScene();
    sc->kind = kind;
    sc->count = count;
    sc->scaleX = scaleX;
    sc->scaleY = scaleY;
    sc->background = 0.1f;
    // fovy = 45 degrees: tan(pi/8) = sqrt(2) - 1 exactly in real arithmetic
    const float tanHalf = (float)(sqrt(2.0) - 1.0);
    sc->filmHalfH = tanHalf;
    sc->filmHalfW = tanHalf * ((float)width / (float)height);
    sc->focalDistance = 4.0f;
    sc->lensRadius = 0.1f;
    prims->assign((size_t)count * MDAS_PRIM_STRIDE, 0.0f);
    SplitMix64 rng{seed};
    float* p = prims->data();
    switch (kind) {
        case MDAS_SCENE_DISCS_MB: {
            sc->dim = 3;
            for (int k = 0; k < count; ++k) {
                float* q = p + MDAS_PRIM_STRIDE * k;
                q[0] = rng.uniform();             // center x in [0,1)
                q[1] = rng.uniform();             // center y
                q[3] = rng.range(0.02f, 0.08f);   // radius
                q[8] = rng.uniform();             // R
                q[9] = rng.uniform();             // G
                q[10] = rng.uniform();            // B
                q[4] = rng.range(-0.1f, 0.1f);    // velocity x per unit shutter time
                q[5] = rng.range(-0.1f, 0.1f);    // velocity y
                q[7] = q[3] * q[3];
            }
            break;
        }
        case MDAS_SCENE_DISCS_DOF:
        case MDAS_SCENE_DISCS_MBDOF: {
            sc->dim = kind == MDAS_SCENE_DISCS_DOF ? 4 : 5;
            for (int k = 0; k < count; ++k) {
                float* q = p + MDAS_PRIM_STRIDE * k;
                q[2] = rng.range(1.0f, 10.0f);    // depth
                q[3] = rng.range(0.05f, 0.3f);    // radius (world units)
                q[8] = rng.uniform();
                q[9] = rng.uniform();
                q[10] = rng.uniform();
                // center uniform over the view frustum's cross-section at that depth
                q[0] = (2.0f * rng.uniform() - 1.0f) * (q[2] * sc->filmHalfW);
                q[1] = (2.0f * rng.uniform() - 1.0f) * (q[2] * sc->filmHalfH);
                q[6] = q[2] / sc->focalDistance;
                q[7] = q[3] * q[3];
            }
            // list by increasing depth (stable), so that shading can stop at the first cover
            std::vector<float> sorted(prims->size());
            std::vector<int> order(count);
            for (int k = 0; k < count; ++k) order[k] = k;
            std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
                return p[MDAS_PRIM_STRIDE * a + 2] < p[MDAS_PRIM_STRIDE * b + 2];
            });
            for (int k = 0; k < count; ++k)
                for (int f = 0; f < MDAS_PRIM_STRIDE; ++f)
                    sorted[MDAS_PRIM_STRIDE * k + f] = p[MDAS_PRIM_STRIDE * order[k] + f];
            *prims = sorted;
            p = prims->data();
            if (kind == MDAS_SCENE_DISCS_MBDOF) {
                for (int k = 0; k < count; ++k) {
                    float* q = p + MDAS_PRIM_STRIDE * k;
                    q[4] = rng.range(-0.1f, 0.1f);
                    q[5] = rng.range(-0.1f, 0.1f);
                }
            }
            break;
        }
        case MDAS_SCENE_DIRECT_LIGHT: {
            sc->dim = 4;
            sc->background = 0.0f;
            for (int k = 0; k < count; ++k) {
                float* q = p + MDAS_PRIM_STRIDE * k;
                q[3] = rng.range(0.3f, 1.0f);
                q[0] = rng.range(-2.0f, 2.0f);
                q[1] = rng.range(-2.0f, 2.0f);
                q[2] = rng.range(0.5f, 2.0f);
                q[6] = 1.0f / q[3];
                q[7] = q[3] * q[3];
            }
            // pinhole at (0,-6,3) looking at the origin, up = +z
            const double eye[3] = {0.0, -6.0, 3.0};
            const double wl = sqrt(eye[0] * eye[0] + eye[1] * eye[1] + eye[2] * eye[2]);
            const double w[3] = {-eye[0] / wl, -eye[1] / wl, -eye[2] / wl};
            // u = w x up, normalised
            double u[3] = {w[1] * 1.0 - w[2] * 0.0, w[2] * 0.0 - w[0] * 1.0, w[0] * 0.0 - w[1] * 0.0};
            const double ul = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
            for (double& x : u) x /= ul;
            // v = u x w
            const double v[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
            const double th = sqrt(2.0) - 1.0;
            const double aspect = (double)width / (double)height;
            for (int i = 0; i < 3; ++i) {
                sc->eye[i] = (float)eye[i];
                sc->W[i] = (float)w[i];
                sc->U[i] = (float)(u[i] * th * aspect);
                sc->V[i] = (float)(v[i] * th);
            }
            sc->lightCorner[0] = -0.5f;
            sc->lightCorner[1] = -0.5f;
            sc->lightCorner[2] = 4.0f;
            sc->lightSize = 1.0f;
            sc->emission = 10.0f;
            sc->albedo = 0.7f;
            break;
        }
        default:
            return MDAS_ERR_INVALID;
    }
    return MDAS_OK;
}
