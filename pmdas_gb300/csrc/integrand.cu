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

template <int D>
__global__ void __launch_bounds__(256) k_evaluate(MdasScene sc, const float* __restrict__ prims,
                                                   const float* __restrict__ coords, float* __restrict__ values,
                                                   const MdasCounts* __restrict__ counts, int offset, int count) {
    extern __shared__ float s_prims[];
    const int nfl = sc.count * MDAS_PRIM_STRIDE;
    for (int k = threadIdx.x; k < nfl; k += blockDim.x) s_prims[k] = prims[k];
    __syncthreads();
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
        mdas_shade(&sc, s_prims, c, out);
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
            mdas_shade(&b.sc, b.prims, c, out);
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

cudaError_t mdas_launch_evaluate(const MdasScene& sc, const float* d_prims, const float* coords, float* values,
                                 int dim, const MdasCounts* counts, int offset, int count, int grid, cudaStream_t s) {
    const size_t smem = sizeof(float) * MDAS_PRIM_STRIDE * (size_t)sc.count;
    if (grid <= 0) grid = 1;
    if (dim < sc.dim) return cudaErrorInvalidValue;
    switch (dim) {
        case 3: k_evaluate<3><<<grid, 256, smem, s>>>(sc, d_prims, coords, values, counts, offset, count); break;
        case 4: k_evaluate<4><<<grid, 256, smem, s>>>(sc, d_prims, coords, values, counts, offset, count); break;
        case 5: k_evaluate<5><<<grid, 256, smem, s>>>(sc, d_prims, coords, values, counts, offset, count); break;
        case 6: k_evaluate<6><<<grid, 256, smem, s>>>(sc, d_prims, coords, values, counts, offset, count); break;
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
