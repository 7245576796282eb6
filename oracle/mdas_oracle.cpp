// mdas_oracle.cpp — CPU restatement of the MDAS sampler (Meister & Hachisuka,
// "Lightweight Multidimensional Adaptive Sampling"), following the reference's
// SDK/lib/mdas/kdgrid.cu kernel bodies line by line.
//
// THIS IS TEST INFRASTRUCTURE: the checker for the CUDA kernels in pmdas_gb300
// and the timed CPU baseline.  Nothing in the product links, loads or calls it.
//
// Arithmetic: IEEE-754 binary32, round to nearest, no contraction
// (build with -ffp-contract=off), subnormals kept, and the reproducible pow of
// pmdas_gb300/csrc/ieee_math.h in place of powf.  This is the strict-IEEE
// arithmetic of the GPU build `MDAS_ARITH_IEEE`, which must match this file bit
// for bit.  The reference itself is compiled with --use_fast_math (approximate
// division, square root and powf); results of that arithmetic are compared
// against this oracle with the tolerances stated in the tests.
//
// Allocation order: the reference hands out new sample and node slots with
// warp-aggregated atomicAdd (kdgrid.cu:366-378, 428-440), so the slot order
// depends on warp scheduling.  Here slots are handed out in leaf-index order
// (an exclusive scan of the selection and split flags), which is the outcome of
// the reference when warps retire in index order.

#include <stdint.h>
#include <string.h>
#include <math.h>
#include <float.h>
#include <stdlib.h>
#include <vector>
#include <chrono>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../pmdas_gb300/csrc/ieee_math.h"
#include "../pmdas_gb300/csrc/integrand.h"

namespace {

// ---- SDK/cuda/random.h:31-67 -------------------------------------------------
inline uint32_t tea4(uint32_t val0, uint32_t val1) {
    uint32_t v0 = val0, v1 = val1, s0 = 0;
    for (int n = 0; n < 4; n++) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}

inline uint32_t lcg(uint32_t& prev) {
    prev = 1664525u * prev + 1013904223u;
    return prev & 0x00FFFFFFu;
}

inline float rnd(uint32_t& prev) { return (float)lcg(prev) / (float)0x01000000; }

// Empty index marker `~Point::DIM` written by the Node constructor (kdgrid.h:26-29).
inline int empty_marker(int D) { return ~D; }

// AABB::Volume (aabb.h:20-25): product of the diagonal, left to right from 1.
template <int D>
inline float box_volume(const float* box) {
    float res = 1.0f;
    for (int i = 0; i < D; ++i) res *= (box[D + i] - box[i]);
    return res;
}

// AABB::LargestAxis (aabb.h:34-45): scan from the last axis down, strict <,
// so ties go to the highest index.
template <int D>
inline int largest_axis(const float* box) {
    int maxAxis = -1;
    float maxExtent = -FLT_MAX;
    for (int i = D - 1; i >= 0; --i) {
        const float e = box[D + i] - box[i];
        if (maxExtent < e) {
            maxExtent = e;
            maxAxis = i;
        }
    }
    return maxAxis;
}

// PointN::Distance (point.h:172-182): sqrt of the running sum of squares.
template <int D>
inline float distance(const float* a, const float* b) {
    float result = 0.0f;
    for (int i = 0; i < D; ++i) {
        const float d = a[i] - b[i];
        result += d * d;
    }
    return sqrtf(result);
}

// ---- uniformSamplingKernel, kdgrid.cu:121-202 -----------------------------------
template <int D>
void initial_sampling(int L, int bpd, int eib, float sx, float sy, float* coords, int* nodes, float* boxes,
                      float* errors, uint32_t* seeds) {
#pragma omp parallel for schedule(static)
    for (int nodeIndex = 0; nodeIndex < L; ++nodeIndex) {
        float offset[D], extent[D];
        for (int j = 0; j < D; ++j) {
            uint32_t xq = 0;
            uint32_t extentInv = 1u << bpd;
            for (int k = 0; k < bpd; ++k) {
                const int i = D * k + (D - j - 1);
                xq |= (uint32_t)((nodeIndex >> i) & 1) << k;
            }
            if (j < 2) {
                for (int k = bpd; k < bpd + eib; ++k) {
                    const int i = D * bpd + 2 * (k - bpd) + 1 - j;
                    xq |= (uint32_t)((nodeIndex >> i) & 1) << k;
                }
                extentInv <<= eib;
            }
            extent[j] = 1.0f / (float)extentInv;
            offset[j] = (float)xq * extent[j];
        }
        offset[0] *= sx;
        offset[1] *= sy;
        extent[0] *= sx;
        extent[1] *= sy;

        uint32_t seed = tea4((uint32_t)nodeIndex, 0);
        for (int j = 0; j < 4; ++j) {
            float r[D];
            for (int i = 0; i < D; ++i) r[i] = rnd(seed);
            const int64_t sampleIndex = 4 * (int64_t)nodeIndex + j;
            for (int i = 0; i < D; ++i) coords[sampleIndex * D + i] = offset[i] + r[i] * extent[i];
            nodes[4 * (int64_t)nodeIndex + j] = (int)sampleIndex;
        }
        seeds[nodeIndex] = seed;
        errors[nodeIndex] = -1.0f;
        float* box = boxes + (int64_t)nodeIndex * 2 * D;
        for (int i = 0; i < D; ++i) {
            box[i] = offset[i];
            box[D + i] = offset[i] + extent[i];
        }
    }
}

// ---- computeErrorsKernel, kdgrid.cu:204-288 --------------------------------------
template <int D>
float compute_errors(int L, float* errors, const int* nodes, const float* boxes, const float* values) {
    float gmax = 0.0f;
#pragma omp parallel for schedule(static) reduction(max : gmax)
    for (int nodeIndex = 0; nodeIndex < L; ++nodeIndex) {
        float error = errors[nodeIndex];
        if (error < 0.0f) {
            const int* node = nodes + 4 * (int64_t)nodeIndex;
            const float volume = box_volume<D>(boxes + (int64_t)nodeIndex * 2 * D);
            float avg[3] = {0.0f, 0.0f, 0.0f};
            float loc[4][3];
            int sampleCount = 0;
            for (int i = 0; i < 4; ++i) {
                if (node[i] >= 0) {
                    for (int c = 0; c < 3; ++c) {
                        loc[i][c] = values[3 * (int64_t)node[i] + c];
                        avg[c] += loc[i][c];
                    }
                    sampleCount++;
                }
            }
            // float3 /= float is a multiply by the reciprocal (sutil/vec_math.h:492-496)
            const float inv = 1.0f / (float)sampleCount;
            for (int c = 0; c < 3; ++c) avg[c] *= inv;
            float diff[3] = {0.0f, 0.0f, 0.0f};
            for (int i = 0; i < sampleCount; ++i)
                for (int c = 0; c < 3; ++c) diff[c] += fabsf(loc[i][c] - avg[c]);
            error = 0.0f;
            for (int c = 0; c < 3; ++c)
                if (avg[c] != 0.0f) error += diff[c] / avg[c];
            error /= (float)sampleCount;
            error += 1.0e-5f;
            error *= volume;
            errors[nodeIndex] = error;
        }
        gmax = std::max(gmax, error);  // warp max + atomicMax on the float bits
    }
    return gmax;
}

// ---- adaptiveSamplingKernel, kdgrid.cu:290-481 -----------------------------------
// Phase 1 (per leaf, independent): selection, best candidate, split flag.
// Phase 2: exclusive scan of the flags in leaf order -> slot indices.
// Phase 3 (per leaf, independent): writes.
template <int D>
int adaptive_sampling(int N, int L, int maxNodeSize, int candidatesNum, float alpha, float gerr, float* errors,
                      int* nodes, float* boxes, float* coords, uint32_t* seeds, int* newN, int* newL,
                      uint8_t* selMask) {
    std::vector<uint8_t> flags((size_t)L);
    std::vector<float> cand((size_t)L * D);
#pragma omp parallel for schedule(static)
    for (int nodeIndex = 0; nodeIndex < L; ++nodeIndex) {
        const float error = errors[nodeIndex];
        const float* box = boxes + (int64_t)nodeIndex * 2 * D;
        uint32_t seed = seeds[nodeIndex];
        if (seed == 0) seed = tea4((uint32_t)nodeIndex, 0);
        uint8_t f = 0;
        if (mdas_powf(error / gerr, alpha) >= rnd(seed)) {
            f = 1;
            const int* node = nodes + 4 * (int64_t)nodeIndex;
            float maxDistance = -1.0f;
            float best[D];
            for (int i = 0; i < D; ++i) best[i] = 0.0f;  // PointN() zero-initialises
            float diag[D];
            for (int i = 0; i < D; ++i) diag[i] = box[D + i] - box[i];
            for (int j = 0; j < candidatesNum; ++j) {
                float r[D], c[D];
                for (int i = 0; i < D; ++i) r[i] = rnd(seed);
                for (int i = 0; i < D; ++i) c[i] = box[i] + r[i] * diag[i];
                float minDistance = FLT_MAX;
                for (int i = 0; i < 4; ++i) {
                    if (node[i] >= 0) {
                        const float d = distance<D>(c, coords + (int64_t)node[i] * D);
                        if (minDistance > d) minDistance = d;
                    }
                }
                if (maxDistance < minDistance) {
                    maxDistance = minDistance;
                    for (int i = 0; i < D; ++i) best[i] = c[i];
                }
            }
            int sampleCount = 0;
            for (int i = 0; i < 4; ++i)
                if (node[i] >= 0) sampleCount++;
            if (sampleCount >= maxNodeSize) f |= 2;
            for (int i = 0; i < D; ++i) cand[(size_t)nodeIndex * D + i] = best[i];
        }
        flags[nodeIndex] = f;
        seeds[nodeIndex] = seed;
    }

    // Phase 2: slots in leaf order
    std::vector<int> sampleSlot((size_t)L), nodeSlot((size_t)L);
    int ns = 0, nn = 0;
    for (int i = 0; i < L; ++i) {
        sampleSlot[i] = ns;
        nodeSlot[i] = nn;
        ns += flags[i] & 1;
        nn += (flags[i] >> 1) & 1;
    }

#pragma omp parallel for schedule(static)
    for (int nodeIndex = 0; nodeIndex < L; ++nodeIndex) {
        const uint8_t f = flags[nodeIndex];
        if (selMask) selMask[nodeIndex] = f;
        if (!(f & 1)) continue;
        int* node = nodes + 4 * (int64_t)nodeIndex;
        float* box = boxes + (int64_t)nodeIndex * 2 * D;
        const int sampleIndex = N + sampleSlot[nodeIndex];
        for (int i = 0; i < D; ++i) coords[(int64_t)sampleIndex * D + i] = cand[(size_t)nodeIndex * D + i];
        int loc[5];
        int sampleCount = 0;
        for (int i = 0; i < 4; ++i) {
            if (node[i] >= 0) {
                loc[i] = node[i];
                sampleCount++;
            }
        }
        if (!(f & 2)) {  // room left: append the index, keep the (stale) error
            node[sampleCount] = sampleIndex;
            continue;
        }
        loc[sampleCount++] = sampleIndex;
        const int axis = largest_axis<D>(box);
        // stable bubble sort by the split-axis coordinate (kdgrid.cu:408-417)
        for (int i = 0; i < sampleCount - 1; i++) {
            for (int j = 0; j < sampleCount - i - 1; j++) {
                const int a = loc[j], b = loc[j + 1];
                if (coords[(int64_t)a * D + axis] > coords[(int64_t)b * D + axis]) std::swap(loc[j], loc[j + 1]);
            }
        }
        const int md = sampleCount >> 1;
        const float pos = 0.5f * (coords[(int64_t)loc[md - 1] * D + axis] + coords[(int64_t)loc[md] * D + axis]);
        const int nodeOffset = L + nodeSlot[nodeIndex];
        int* right = nodes + 4 * (int64_t)nodeOffset;
        float* rbox = boxes + (int64_t)nodeOffset * 2 * D;
        for (int i = 0; i < 4; ++i) {
            right[i] = i < sampleCount - md ? loc[md + i] : empty_marker(D);
        }
        for (int i = 0; i < 4; ++i) node[i] = i < md ? loc[i] : empty_marker(D);
        for (int i = 0; i < 2 * D; ++i) rbox[i] = box[i];
        box[D + axis] = pos;
        rbox[axis] = pos;
        errors[nodeIndex] = -1.0f;
        errors[nodeOffset] = -1.0f;
    }
    *newN = ns;
    *newL = nn;
    return 0;
}

// ---- integrateKernel, kdgrid.cu:483-582 (serial, leaf order) ----------------------
template <int D>
void integrate_leaf(int nodeIndex, int W, int H, float sx, float sy, const int* nodes, const float* boxes,
                    const float* values, float* pixels) {
    const float stepX = sx / (float)W;
    const float stepY = sy / (float)H;
    const int* node = nodes + 4 * (int64_t)nodeIndex;
    float val[3] = {0.0f, 0.0f, 0.0f};
    int sampleCount = 0;
    for (int i = 0; i < 4; ++i) {
        if (node[i] >= 0) {
            for (int c = 0; c < 3; ++c) val[c] += values[3 * (int64_t)node[i] + c];
            sampleCount++;
        }
    }
    const float inv = 1.0f / (float)sampleCount;
    for (int c = 0; c < 3; ++c) val[c] *= inv;
    const float* box = boxes + (int64_t)nodeIndex * 2 * D;
    const float mn0 = box[0], mn1 = box[1], mx0 = box[D], mx1 = box[D + 1];
    const int x0 = (int)(mn0 * (float)W / sx);
    int x1 = (int)(mx0 * (float)W / sx);
    const int y0 = (int)(mn1 * (float)H / sy);
    int y1 = (int)(mx1 * (float)H / sy);
    x1 = std::min(x1 + 1, W);
    y1 = std::min(y1 + 1, H);
    const float pixArea = (sx * sy) / (float)(W * H);
    const float invPixArea = 1.0f / pixArea;
    const float volume = box_volume<D>(box);
    float pMinY = (float)y0 * sy / (float)H;
    float pMaxY = pMinY + stepY;
    for (int y = y0; y < y1; ++y) {
        float pMinX = (float)x0 * sx / (float)W;
        float pMaxX = pMinX + stepX;
        for (int x = x0; x < x1; ++x) {
            const float clox = fmaxf(pMinX, mn0);
            const float chix = fminf(pMaxX, mx0);
            const float cloy = fmaxf(pMinY, mn1);
            const float chiy = fminf(pMaxY, mx1);
            if (clox < chix && cloy < chiy) {
                const float v = (chix - clox) * (chiy - cloy) * volume / ((mx0 - mn0) * (mx1 - mn1));
                float* px = pixels + 4 * ((int64_t)y * W + x);
                // float3 * float, then float3 / float = * (1/pixArea) (vec_math.h:483-487)
                for (int c = 0; c < 3; ++c) px[c] += (val[c] * v) * invPixArea;
            }
            pMinX = pMaxX;
            pMaxX += stepX;
        }
        pMinY = pMaxY;
        pMaxY += stepY;
    }
}

template <int D>
void integrate(int L, int W, int H, float sx, float sy, const int* nodes, const float* boxes, const float* values,
               float* pixels, int threads) {
    memset(pixels, 0, sizeof(float) * 4 * (size_t)W * H);
    if (threads <= 1) {
        for (int i = 0; i < L; ++i) integrate_leaf<D>(i, W, H, sx, sy, nodes, boxes, values, pixels);
        return;
    }
#ifdef _OPENMP
    // private images per thread, then a reduction (the timed CPU baseline)
    std::vector<float> priv((size_t)threads * 4 * W * H, 0.0f);
#pragma omp parallel num_threads(threads)
    {
        const int t = omp_get_thread_num();
        float* mine = priv.data() + (size_t)t * 4 * W * H;
#pragma omp for schedule(static)
        for (int i = 0; i < L; ++i) integrate_leaf<D>(i, W, H, sx, sy, nodes, boxes, values, mine);
#pragma omp for schedule(static)
        for (int64_t p = 0; p < (int64_t)4 * W * H; ++p) {
            float s = 0.0f;
            for (int k = 0; k < threads; ++k) s += priv[(size_t)k * 4 * W * H + p];
            pixels[p] = s;
        }
    }
#else
    for (int i = 0; i < L; ++i) integrate_leaf<D>(i, W, H, sx, sy, nodes, boxes, values, pixels);
#endif
}

// ---- KDGrid::Validate, kdgrid.cu:848-961 -------------------------------------------
// The leaf volumes are summed in double: the reference's float sum (:858, :903) drifts
// past its own 1 % tolerance (:910) at a few million leaves (about 1.2 % at 6 M
// leaves of similar size), which would fail a valid partition.
template <int D>
int validate(int N, int L, float sx, float sy, const float* coords, const int* nodes, const float* boxes) {
    int bad = 0;
    std::vector<int> hist((size_t)N, 0);
    double totalVolume = 0.0;
    int64_t total = 0;
    for (int k = 0; k < L; ++k) {
        const float* box = boxes + (int64_t)k * 2 * D;
        for (int i = 0; i < 4; ++i) {
            const int s = nodes[4 * (int64_t)k + i];
            if (s >= 0) {
                if (s >= N) {
                    bad |= 8;
                    continue;
                }
                for (int d = 0; d < D; ++d) {
                    const float c = coords[(int64_t)s * D + d];
                    if (c < box[d] || c > box[D + d]) bad |= 1;
                }
                hist[s]++;
                total++;
            }
        }
        totalVolume += box_volume<D>(box);
    }
    const double rootVolume = (double)(sx * sy);
    if (fabs(totalVolume - rootVolume) > 1.0e-2 * rootVolume) bad |= 2;
    if (total != N) bad |= 4;
    for (int i = 0; i < N; ++i)
        if (hist[i] != 1) bad |= 4;
    return bad;
}

template <int D>
void sampling_density(int N, float sx, float sy, const float* coords, float* pixels, int W, int H) {
    memset(pixels, 0, sizeof(float) * 4 * (size_t)W * H);
    for (int i = 0; i < N; ++i) {
        int x = (int)(coords[(int64_t)i * D + 0] / sx * (float)W);
        int y = (int)(coords[(int64_t)i * D + 1] / sy * (float)H);
        x = std::min(x, W - 1);
        y = std::min(y, H - 1);
        float* p = pixels + 4 * ((int64_t)y * W + x);
        for (int c = 0; c < 4; ++c) p[c] += 0.05f;
    }
    for (int64_t i = 0; i < (int64_t)W * H; ++i) pixels[4 * i + 3] = 1.0f;
}

// make_color (SDK/cuda/helpers.h:35-66) with the reproducible pow.
inline unsigned char quantize(float x) {
    x = std::min(std::max(x, 0.0f), 1.0f);
    const unsigned int q = (unsigned int)(x * 256.0f);
    return (unsigned char)std::min(q, 255u);
}

inline float to_srgb(float c) {
    const float invGamma = 1.0f / 2.4f;
    const float powed = mdas_powf(c, invGamma);
    return c < 0.0031308f ? 12.92f * c : 1.055f * powed - 0.055f;
}

}  // namespace

#define ORC_DISPATCH(D, CALL)          \
    switch (D) {                       \
        case 3: { constexpr int DD = 3; CALL; } break; \
        case 4: { constexpr int DD = 4; CALL; } break; \
        case 5: { constexpr int DD = 5; CALL; } break; \
        case 6: { constexpr int DD = 6; CALL; } break; \
        default: return -1;            \
    }

extern "C" {

int orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

// KDGrid::InitialSampling (kdgrid.cu:633-674): L = (1 << bpd*D) << 2*eib leaves
// of 4 samples each.  seeds must hold capNodes entries; all are zeroed first
// (kdgrid.cu:637), so slots that are not leaves yet keep a zero seed.
int orc_initial_sampling(int D, int bpd, int eib, float sx, float sy, int capNodes, float* coords, int* nodes,
                         float* boxes, float* errors, uint32_t* seeds, int* outN, int* outL) {
    const int64_t L = ((int64_t)1 << (bpd * D)) << (2 * eib);
    if (L > capNodes) return -2;
    memset(seeds, 0, sizeof(uint32_t) * (size_t)capNodes);
    ORC_DISPATCH(D, initial_sampling<DD>((int)L, bpd, eib, sx, sy, coords, nodes, boxes, errors, seeds));
    *outL = (int)L;
    *outN = (int)(4 * L);
    return 0;
}

float orc_compute_errors(int D, int L, float* errors, const int* nodes, const float* boxes, const float* values) {
    switch (D) {
        case 3: return compute_errors<3>(L, errors, nodes, boxes, values);
        case 4: return compute_errors<4>(L, errors, nodes, boxes, values);
        case 5: return compute_errors<5>(L, errors, nodes, boxes, values);
        case 6: return compute_errors<6>(L, errors, nodes, boxes, values);
    }
    return -1.0f;
}

int orc_adaptive_sampling(int D, int N, int L, int maxNodeSize, int candidatesNum, float alpha, float gerr,
                          float* errors, int* nodes, float* boxes, float* coords, uint32_t* seeds, int* newN,
                          int* newL, uint8_t* selMask) {
    ORC_DISPATCH(D, adaptive_sampling<DD>(N, L, maxNodeSize, candidatesNum, alpha, gerr, errors, nodes, boxes,
                                          coords, seeds, newN, newL, selMask));
    return 0;
}

int orc_integrate(int D, int L, int W, int H, float sx, float sy, const int* nodes, const float* boxes,
                  const float* values, float* pixels, int threads) {
    ORC_DISPATCH(D, integrate<DD>(L, W, H, sx, sy, nodes, boxes, values, pixels, threads));
    return 0;
}

int orc_convert_to_bytes(int P, const float* pixels, unsigned char* bytes) {
    for (int64_t i = 0; i < P; ++i) {
        for (int c = 0; c < 3; ++c) {
            const float v = std::min(std::max(pixels[4 * i + c], 0.0f), 1.0f);
            bytes[4 * i + c] = quantize(to_srgb(v));
        }
        bytes[4 * i + 3] = 255;
    }
    return 0;
}

int orc_sampling_density(int D, int N, float sx, float sy, const float* coords, float* pixels, int W, int H) {
    ORC_DISPATCH(D, sampling_density<DD>(N, sx, sy, coords, pixels, W, H));
    return 0;
}

int orc_validate(int D, int N, int L, float sx, float sy, const float* coords, const int* nodes, const float* boxes) {
    int r = 0;
    ORC_DISPATCH(D, r = validate<DD>(N, L, sx, sy, coords, nodes, boxes));
    return r;
}

int orc_evaluate(const MdasScene* scene, const float* prims, int D, const float* coords, float* values, int offset,
                 int count) {
#pragma omp parallel for schedule(dynamic, 4096)
    for (int i = 0; i < count; ++i) {
        const int64_t s = (int64_t)offset + i;
        mdas_shade(scene, prims, coords + s * D, values + 3 * s);
    }
    return 0;
}

float orc_powf(float x, float y) { return mdas_powf(x, y); }
float orc_log2f(float x) { return mdas_log2f(x); }
float orc_exp2f(float x) { return mdas_exp2f(x); }
void orc_sincos(float phi, float* s, float* c) { mdas_sincos_quarter(phi, s, c); }

// The whole headless MDAS loop (optixMotionBlur.cpp:768-793) on the CPU:
// initial sampling, integrand, then `while N < budget` passes of errors +
// adaptive sampling + integrand for the new samples, then integrate.
// Stops early, like the interactive loop (optixMotionBlur.cpp:723-724), when a
// pass could overrun the buffers (N + L > capSamples or 2L > capNodes).
// times_ms[0..4] = initial sampling, errors, adaptive, integrate, integrand.
int orc_render(int D, int bpd, int eib, int candidatesNum, float alpha, float sx, float sy, int budget,
               int capSamples, int capNodes, const MdasScene* scene, const float* prims, int W, int H,
               float* coords, float* values, int* nodes, float* boxes, float* errors, uint32_t* seeds,
               float* pixels, int threads, int* outN, int* outL, int* outPasses, double* times_ms) {
    using clk = std::chrono::steady_clock;
    auto ms = [](clk::time_point a, clk::time_point b) {
        return std::chrono::duration<double, std::milli>(b - a).count();
    };
    for (int i = 0; i < 5; ++i) times_ms[i] = 0.0;
    int N = 0, L = 0;
    auto t0 = clk::now();
    int rc = orc_initial_sampling(D, bpd, eib, sx, sy, capNodes, coords, nodes, boxes, errors, seeds, &N, &L);
    if (rc) return rc;
    auto t1 = clk::now();
    times_ms[0] += ms(t0, t1);
    orc_evaluate(scene, prims, D, coords, values, 0, N);
    times_ms[4] += ms(t1, clk::now());
    int passes = 0;
    while (N < budget) {
        if ((int64_t)N + L > capSamples || 2 * (int64_t)L > capNodes) break;
        t0 = clk::now();
        const float g = orc_compute_errors(D, L, errors, nodes, boxes, values);
        t1 = clk::now();
        int nN = 0, nL = 0;
        orc_adaptive_sampling(D, N, L, 4, candidatesNum, alpha, g, errors, nodes, boxes, coords, seeds, &nN, &nL,
                              nullptr);
        auto t2 = clk::now();
        orc_evaluate(scene, prims, D, coords, values, N, nN);
        auto t3 = clk::now();
        times_ms[1] += ms(t0, t1);
        times_ms[2] += ms(t1, t2);
        times_ms[4] += ms(t2, t3);
        N += nN;
        L += nL;
        passes++;
    }
    t0 = clk::now();
    orc_integrate(D, L, W, H, sx, sy, nodes, boxes, values, pixels, threads);
    times_ms[3] += ms(t0, clk::now());
    *outN = N;
    *outL = L;
    *outPasses = passes;
    return 0;
}


// ---- Leaf ordering (no reference counterpart) ----------------------------------
// Keys number the cells of a finer grid the way uniformSamplingKernel numbers
// its initial cells (kdgrid.cu:144-157), with K = bitsPerDim + fineBits bits
// per dimension: key bit pos < D*K holds bit pos/D of dimension D-1 - pos%D;
// key bit D*K + r holds bit K + r/2 of image dimension 1 - r%2.  Restated here
// position by position (the CUDA kernels place coordinate bits instead).

static uint32_t orc_cell_coord(float x, float scale, bool image, int B) {
    const float u = image ? x / scale : x;
    const float top = (float)(1u << B);
    const float s = u * top;
    if (!(s > 0.0f)) return 0u;
    if (s >= top) return (1u << B) - 1u;
    return (uint32_t)s;
}

static uint64_t orc_key(const float* p, int D, int bpd, int eib, int F, float sx, float sy) {
    const int K = bpd + F;
    uint32_t q[8];
    for (int j = 0; j < D; ++j)
        q[j] = orc_cell_coord(p[j], j == 0 ? sx : sy, j < 2, K + (j < 2 ? eib : 0));
    uint64_t key = 0;
    const int total = D * K + 2 * eib;
    for (int pos = 0; pos < total; ++pos) {
        int j, k;
        if (pos < D * K) {
            k = pos / D;
            j = D - 1 - pos % D;
        } else {
            const int r = pos - D * K;
            k = K + r / 2;
            j = 1 - r % 2;
        }
        key |= (uint64_t)((q[j] >> k) & 1u) << pos;
    }
    return key;
}

// Prefix length of sorted keys i and j, positions breaking ties.
static int orc_prefix(const uint64_t* k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    if (k[i] == k[j]) {
        const uint32_t x = (uint32_t)(i ^ j);
        return 64 + (x ? __builtin_clz(x) : 32);
    }
    return __builtin_clzll(k[i] ^ k[j]);
}

int orc_morton_encode(int D, int bpd, int eib, int F, float sx, float sy, const float* points, int n,
                      uint64_t* keys) {
    if (D > 8 || D * (bpd + F) + 2 * eib > 64 || bpd + F + eib > 31) return -1;
    for (int i = 0; i < n; ++i) keys[i] = orc_key(points + (size_t)i * D, D, bpd, eib, F, sx, sy);
    return 0;
}

// Cell boxes as uniformSamplingKernel computes them (kdgrid.cu:142-164, 191-196).
int orc_morton_decode(int D, int bpd, int eib, float sx, float sy, const uint64_t* cells, int n, float* boxes) {
    if (D > 8 || D * bpd + 2 * eib > 64 || bpd + eib > 31) return -1;
    for (int i = 0; i < n; ++i) {
        uint32_t xq[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        const int total = D * bpd + 2 * eib;
        for (int pos = 0; pos < total; ++pos) {
            int j, k;
            if (pos < D * bpd) {
                k = pos / D;
                j = D - 1 - pos % D;
            } else {
                const int r = pos - D * bpd;
                k = bpd + r / 2;
                j = 1 - r % 2;
            }
            xq[j] |= (uint32_t)((cells[i] >> pos) & 1u) << k;
        }
        float* b = boxes + (size_t)i * 2 * D;
        for (int j = 0; j < D; ++j) {
            const unsigned extentInv = (1u << bpd) << (j < 2 ? eib : 0);
            float extent = 1.0f / float(extentInv);
            float offset = xq[j] * extent;
            if (j < 2) {
                const float sc = j == 0 ? sx : sy;
                offset *= sc;
                extent *= sc;
            }
            b[j] = offset;
            b[D + j] = offset + extent;
        }
    }
    return 0;
}

// Key of each leaf's box centre (boxes: L x (mn[D], mx[D])).
int orc_leaf_keys(int D, int bpd, int eib, int F, float sx, float sy, const float* boxes, int L, uint64_t* keys) {
    if (D > 8 || D * (bpd + F) + 2 * eib > 64 || bpd + F + eib > 31) return -1;
    float c[8];
    for (int i = 0; i < L; ++i) {
        const float* b = boxes + (size_t)i * 2 * D;
        for (int j = 0; j < D; ++j) c[j] = 0.5f * (b[j] + b[D + j]);
        keys[i] = orc_key(c, D, bpd, eib, F, sx, sy);
    }
    return 0;
}

// Stable sort by key bits [beginBit, endBit): sorted keys and the permutation.
int orc_sort_pairs(const uint64_t* keys, int n, int beginBit, int endBit, uint64_t* sortedKeys, uint32_t* order) {
    if (beginBit < 0 || endBit > 64 || beginBit > endBit) return -1;
    const int w = endBit - beginBit;
    const uint64_t mask = w == 64 ? ~0ull : ((1ull << w) - 1ull);
    std::vector<uint32_t> idx((size_t)n);
    for (int i = 0; i < n; ++i) idx[i] = (uint32_t)i;
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) {
        const uint64_t ka = w ? (keys[a] >> beginBit) & mask : 0, kb = w ? (keys[b] >> beginBit) & mask : 0;
        return ka < kb;
    });
    for (int i = 0; i < n; ++i) {
        order[i] = idx[i];
        sortedKeys[i] = keys[idx[i]];
    }
    return 0;
}

// Radix tree over n sorted keys, built top-down: a node spanning [first, last]
// splits after the last position whose prefix with `first` is longer than the
// node's own prefix; its children are the leaf or the internal node numbered
// by the split (gamma, gamma + 1), the numbering of Karras (HPG 2012).
int orc_karras(const uint64_t* k, int n, int* children, int* parents) {
    if (n <= 0) return 0;
    parents[0] = -1;
    if (n == 1) return 0;
    struct Span { int node, first, last; };
    std::vector<Span> stack;
    stack.push_back({0, 0, n - 1});
    while (!stack.empty()) {
        const Span s = stack.back();
        stack.pop_back();
        const int dnode = orc_prefix(k, n, s.first, s.last);
        int lo = s.first, hi = s.last - 1;  // largest g in [first, last-1] with prefix(first, g) > dnode
        while (lo < hi) {
            const int mid = lo + (hi - lo + 1) / 2;
            if (orc_prefix(k, n, s.first, mid) > dnode) lo = mid;
            else hi = mid - 1;
        }
        const int g = lo;
        const int left = g == s.first ? ~g : g;
        const int right = g + 1 == s.last ? ~(g + 1) : g + 1;
        children[2 * s.node] = left;
        children[2 * s.node + 1] = right;
        parents[left >= 0 ? left : (n - 1) + ~left] = s.node;
        parents[right >= 0 ? right : (n - 1) + ~right] = s.node;
        if (left >= 0) stack.push_back({left, s.first, g});
        if (right >= 0) stack.push_back({right, g + 1, s.last});
    }
    return 0;
}

// Internal node boxes: componentwise min / max over each node's leaves
// (leafBoxes by leaf slot, order = slots by sorted position).
int orc_refit(int D, const float* leafBoxes, const uint32_t* order, int n, const int* children, float* boxes) {
    if (n <= 1) return 0;
    // children have larger spans' sub-ranges; a post-order walk from the root
    std::vector<int> post;
    std::vector<int> st{0};
    while (!st.empty()) {
        const int v = st.back();
        st.pop_back();
        post.push_back(v);
        for (int c = 0; c < 2; ++c)
            if (children[2 * v + c] >= 0) st.push_back(children[2 * v + c]);
    }
    for (size_t t = post.size(); t-- > 0;) {
        const int v = post[t];
        float* out = boxes + (size_t)v * 2 * D;
        for (int c = 0; c < 2; ++c) {
            const int ch = children[2 * v + c];
            const float* b = ch >= 0 ? boxes + (size_t)ch * 2 * D : leafBoxes + (size_t)order[~ch] * 2 * D;
            for (int j = 0; j < D; ++j) {
                out[j] = c == 0 ? b[j] : std::min(out[j], b[j]);
                out[D + j] = c == 0 ? b[D + j] : std::max(out[D + j], b[D + j]);
            }
        }
    }
    return 0;
}

// For each point the first leaf in key order whose box holds it (mn <= p < mx,
// p <= mx on the domain's upper faces), -1 if none; brute force.
int orc_locate(int D, const float* leafBoxes, const uint32_t* order, int n, const float* points, int m, int* out) {
    std::vector<float> dom((size_t)D, -INFINITY);
    for (int p = 0; p < n; ++p)
        for (int j = 0; j < D; ++j) dom[j] = std::max(dom[j], leafBoxes[(size_t)p * 2 * D + D + j]);
#pragma omp parallel for schedule(dynamic, 64)
    for (int q = 0; q < m; ++q) {
        const float* x = points + (size_t)q * D;
        int found = -1;
        for (int p = 0; p < n && found < 0; ++p) {
            const float* b = leafBoxes + (size_t)order[p] * 2 * D;
            bool in = true;
            for (int j = 0; j < D && in; ++j)
                in = b[j] <= x[j] && (x[j] < b[D + j] || (x[j] == b[D + j] && b[D + j] >= dom[j]));
            if (in) found = (int)order[p];
        }
        out[q] = found;
    }
    return 0;
}

}  // extern "C"
