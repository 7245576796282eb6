// scene.h — host-side scene object and the integrand launcher (internal).
#pragma once

#include <stdint.h>
#include <vector>
#include <cuda_runtime.h>
#include "integrand.h"
#include "grid_types.h"

#define MDAS_MAX_PRIMS 1024  // 48 KB of shared memory in the integrand kernel

// Disc culling: the image is cut into MDAS_CULL_TILES x MDAS_CULL_TILES tiles
// and every tile keeps a bit mask (one bit per disc, ceil(count/32) words) of
// the discs that may cover a sample in it, with a margin that absorbs rounding.
// Shading then tests only those discs, in list order, so the first covering
// disc (and every value) is the one the full scan finds.
#define MDAS_CULL_TILES 64
size_t mdas_cull_words(const MdasScene& sc);  // 0: the scene kind is not culled
cudaError_t mdas_launch_build_cull(const MdasScene& sc, const float* d_prims, unsigned* masks, cudaStream_t s);

// Evaluates samples [offset, offset+count) of an AoS coordinate buffer with `dim`
// floats per sample (dim >= the scene's own dimension; extra coordinates are
// ignored).  With `counts`, the range is the last adaptive pass's new samples.
// `cull` (may be null) is the scene's tile masks.
cudaError_t mdas_launch_evaluate(const MdasScene& sc, const float* d_prims, const unsigned* cull, const float* coords,
                                 float* values, int dim, const MdasCounts* counts, int offset, int count, int grid,
                                 cudaStream_t s);

cudaError_t mdas_launch_leaf_true_errors(const MdasScene& sc, const float* d_prims, const MdasDeviceGrid& g,
                                         const int* leaves, int L, int samples, unsigned long long seed, float* out,
                                         cudaStream_t s);

cudaError_t mdas_launch_reference_image(const MdasScene& sc, const float* d_prims, int width, int height, int strata,
                                        unsigned long long seed, double* out, int grid, cudaStream_t s);

int mdas_generate_scene(int kind, uint64_t seed, int count, float scaleX, float scaleY, int width, int height,
                        MdasScene* sc, std::vector<float>* prims);

// The integrand side of one image of a batched render (device-side descriptor).
struct MdasBatchScene {
    MdasScene sc;
    const float* prims;
    const unsigned* cull;  // tile masks of the discs, or null
    const MdasCounts* counts;
    const float* coords;
    float* values;
    int dim;
    int initialSamples;
};

// Batched integrand: every image's initial samples (all = 1) or the samples the
// last pass added to each still-active image (all = 0).  Images of one launch
// share the coordinate stride D.
cudaError_t mdas_launch_evaluate_batch(const MdasBatchScene* scenes, int n, int D, int all, int grid, cudaStream_t s);

struct mdas_scene {
    MdasScene desc;
    std::vector<float> prims;  // host copy
    float* d_prims = nullptr;  // device copy
    unsigned* d_cull = nullptr;  // tile masks of the discs (culled kinds only), rebuilt with every upload
};
