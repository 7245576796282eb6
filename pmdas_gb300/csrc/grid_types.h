// grid_types.h — device-side state shared by the MDAS kernels and the C-ABI layer.
#pragma once

#include <stdint.h>
#include <cuda_runtime.h>

// Counters kept in device memory so that a pass never needs the host to know
// how many leaves there are (the reference reads them back with
// cudaMemcpyFromSymbol after every pass, kdgrid.cu:753-759).
struct MdasCounts {
    int N;          // samples
    int L;          // leaves
    int newN;       // samples added by the last adaptive pass
    int newL;       // leaves added by the last adaptive pass
    unsigned gerr;   // bits of g_error, the max leaf error of the last errors pass
    int recomputed;  // leaf errors recomputed by the last errors pass (reset with gerr)
    int status;      // first device-side error (MDAS_ERR_*), 0 if none
    int selected;    // leaves selected by the last adaptive pass (== newN)
    int passes;      // adaptive passes since the initial sampling
    unsigned gathered;  // sample coordinates read by the last adaptive pass
    int pad[2];
};

// Per-launch scratch of the persistent kernels: tile tickets and exit counter.
struct MdasCtl {
    unsigned ticket;
    unsigned done;
    unsigned pad[2];
};

struct MdasDeviceGrid {
    int D;
    int maxSamples;
    int maxNodes;
    int candidatesNum;
    int maxNodeSize;
    int bitsPerDim;
    int extraImgBits;
    float alpha;
    float scaleX;
    float scaleY;
    float* coords;        // [capSamples * D], AoS like the reference's Point buffer
    float* values;        // [capSamples * 3], float3
    int4* nodes;          // [maxNodes], 4 sample indices, ~D = empty
    float* boxes;         // [maxNodes * 2D], mn[D] then mx[D]
    float* errors;        // [maxNodes], < 0 = needs recomputation
    unsigned* seeds;      // [maxNodes], 0 = not drawn yet
    MdasCounts* counts;   // device counters
    MdasCtl* ctl;         // persistent-kernel scratch
    unsigned long long* tiles;  // decoupled look-back tile states, one per 256 leaves
    int maxTiles;
};

// Decoupled look-back tile state: [63:62] status, [61:31] split count, [30:0] selected count.
#define MDAS_TILE_AGG 1ull
#define MDAS_TILE_INC 2ull
#define MDAS_TILE_LEAVES 256
// Spin limit of the look-back wait; on expiry the kernel records MDAS_ERR_TIMEOUT and moves on.
#define MDAS_SPIN_LIMIT (1u << 22)

#define MDAS_OK 0
#define MDAS_ERR_INVALID 1
#define MDAS_ERR_CUDA 2
#define MDAS_ERR_CAPACITY 3
#define MDAS_ERR_TIMEOUT 4
#define MDAS_ERR_ALLOC 5
#define MDAS_ERR_STATE 6

// Host launchers, one set per arithmetic build (namespace mdas_fast / mdas_ieee).
#define MDAS_DECLARE_LAUNCHERS(NS)                                                                          \
    namespace NS {                                                                                          \
    cudaError_t initial_sampling(const MdasDeviceGrid& g, int L, cudaStream_t s);                           \
    cudaError_t compute_errors(const MdasDeviceGrid& g, int grid, cudaStream_t s);                          \
    cudaError_t adaptive_sampling(const MdasDeviceGrid& g, int grid, cudaStream_t s);                       \
    cudaError_t integrate(const MdasDeviceGrid& g, int grid, float* pixels, int W, int H, cudaStream_t s);  \
    cudaError_t convert_to_bytes(const float* pixels, unsigned char* bytes, int P, cudaStream_t s);         \
    cudaError_t sampling_density(const MdasDeviceGrid& g, float* pixels, int W, int H, cudaStream_t s);     \
    int max_blocks_per_sm(int D, int which);                                                                \
    }

MDAS_DECLARE_LAUNCHERS(mdas_fast)
MDAS_DECLARE_LAUNCHERS(mdas_ieee)

enum { MDAS_K_INIT = 0, MDAS_K_ERRORS = 1, MDAS_K_ADAPTIVE = 2, MDAS_K_INTEGRATE = 3 };
