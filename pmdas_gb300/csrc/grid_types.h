// grid_types.h — device-side state shared by the MDAS kernels and the C-ABI layer.
#pragma once

#include <stdint.h>
#include <cuda_runtime.h>

// Counters kept in device memory so that a pass never needs the host to know
// how many leaves there are (the reference reads them back with
// cudaMemcpyFromSymbol after every pass, kdgrid.cu:753-759).
//
// The accumulators of a pass need no memset before it: the adaptive pass's
// scan, which runs once the pass's decide kernel is done, moves each to its
// `...Last` copy (or, for gerrNext, to gerrCarry for the next errors pass) and
// clears it for the next pass.
struct MdasCounts {
    int N;          // samples
    int L;          // leaves
    int newN;       // samples added by the last adaptive pass
    int newL;       // leaves added by the last adaptive pass
    unsigned gerr;   // bits of g_error, the max leaf error of the errors pass since the last adaptive pass
    int recomputed;  // leaf errors recomputed by that errors pass
    int status;      // first device-side error (MDAS_ERR_*), 0 if none
    int selected;    // leaves selected by the last adaptive pass (== newN)
    int passes;      // adaptive passes since the initial sampling
    unsigned gathered;  // sample coordinates read by the running adaptive pass
    unsigned gerrNext;  // max error of the leaves the running adaptive pass does not split
    int active;         // batched rendering: 1 while this image still takes passes
    unsigned gerrLast;      // gerr of the last adaptive pass
    int recomputedLast;     // recomputed of the last adaptive pass
    unsigned gatheredLast;  // gathered of the last adaptive pass
    unsigned gerrCarry;     // gerrNext of the last adaptive pass (where the next errors pass starts)
};

// Learned acceptance, one pass: the largest prediction, and the judge's sums of
// the plain errors that each schedule leaves unrefined (leaves it does not
// accept) and its verdict.
struct MdasLearnedStats {
    unsigned predMax;            // order-preserving bits of the largest prediction
    unsigned blocksDone;         // judge blocks finished (the last one decides)
    int usePlain;                // 1: this pass takes the plain acceptance
    int plainPasses;             // passes the judge sent back to the plain acceptance
    double unrefinedLearned;     // sum of plain errors of the leaves the learned schedule does not accept
    double unrefinedPlain;       // the same for the plain schedule
    float tolerance;             // revert when unrefinedLearned > (1 + tolerance) * unrefinedPlain
    int judgedPasses;
    // order-preserving bits of the largest priority of the leaves the last
    // adaptive pass did not split (their priorities carry over to the next
    // pass, whose predictions of the split children complete predMax); set by
    // decide, cleared by the judge once the predictions have taken it
    unsigned keptMax;
};

// Order-preserving unsigned image of a float (for atomicMax over floats of any sign).
__host__ __device__ inline unsigned mdas_float_order(float f) {
    union { float f; unsigned u; } c;
    c.f = f;
    return (c.u & 0x80000000u) ? ~c.u : (c.u | 0x80000000u);
}
__host__ __device__ inline float mdas_float_unorder(unsigned u) {
    union { float f; unsigned u; } c;
    c.u = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    return c.f;
}

// Scratch of one adaptive pass: the counts before it, for the place kernel.
struct MdasCtl {
    int N0;
    int L0;
    int pad[2];
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
    float* nb;            // [maxNodes * nbFloats], per leaf: node (4 sample indices), box, and the
                          // coordinates of its samples in node-slot order
    int nbFloats;         // floats per leaf record
    float* errors;        // [maxNodes], < 0 = needs recomputation
    unsigned char* leafCounts;  // [maxNodes + 16], samples per leaf (the node's non-empty slots)
    unsigned* seeds;      // [maxNodes], 0 = not drawn yet
    MdasCounts* counts;   // device counters
    MdasCtl* ctl;         // per-pass scratch
    uint2* tileCounts;    // [maxTiles] (accepted, split) per tile of MDAS_TILE_LEAVES leaves
    uint2* tilePrefix;    // [maxTiles] exclusive prefix of tileCounts
    uint2* accepted;      // [maxTiles * MDAS_TILE_LEAVES] accepted leaves, compacted per tile
    int* chunkTile;       // [maxNodes/256 + 2] tile of the first entry of each 256-entry chunk of accepted leaves
    int maxTiles;
    int* dirty;           // [maxNodes/2 + 1], slots of the left children of the last pass's splits
    // [maxNodes/2 + 1] per split of the last pass, for the next errors pass:
    // left child {sample 0, sample 1, slot, volume bits}, right child
    // {sample 0, sample 1, sample 2, volume bits} (its slot is L - newL + split rank)
    int4* splitL;
    int4* splitR;
    // learned acceptance (nullptr: the reference's plain error ratio): predicted
    // log2(error) / priorityScale per leaf, and the pass's statistics and verdict
    const float* priority;
    float priorityScale;
    MdasLearnedStats* learned;
    // learned mode: [maxNodes * MDAS_RAW_FLOATS] the raw feature inputs of each
    // leaf the last split-children errors pass recomputed, in its item order
    // (nullptr: not written)
    float* featRaw;
    // leaves per thread of decide (4 or 8): its tiles are 256 * tileK leaves
    int tileK;
};

// One image of a batched render (device-side descriptor).
struct MdasBatchImage {
    MdasDeviceGrid g;
    float4* pixels;
    int width, height;
    int budget;
    int initialLeaves;
    unsigned jumpA, jumpC;  // LCG jump-ahead over the candidate draws of one accepted leaf
    const void* mlp;        // packed weights of a learned image (g.priority set), nullptr: plain acceptance
};

// Leaves per thread and per tile of the adaptive pass (the default; the
// batched renders may take 4 per thread: MdasDeviceGrid::tileK), and the
// smallest tile, which sizes the per-tile scratch.
#define MDAS_LEAVES_PER_THREAD 8
#define MDAS_TILE_LEAVES (256 * MDAS_LEAVES_PER_THREAD)
#define MDAS_TILE_LEAVES_MIN 1024

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
    cudaError_t compute_errors(const MdasDeviceGrid& g, int grid, bool dirty, cudaStream_t s);              \
    cudaError_t adaptive_sampling(const MdasDeviceGrid& g, int gridDecide, int gridPlace, cudaStream_t s);  \
    cudaError_t integrate(const MdasDeviceGrid& g, int grid, float* pixels, int W, int H, cudaStream_t s);  \
    cudaError_t convert_to_bytes(const float* pixels, unsigned char* bytes, int P, cudaStream_t s);         \
    cudaError_t sampling_density(const MdasDeviceGrid& g, float* pixels, int W, int H, cudaStream_t s);     \
    cudaError_t unpack_records(const MdasDeviceGrid& g, int L, int* nodes, float* boxes, cudaStream_t s);   \
    cudaError_t pack_records(const MdasDeviceGrid& g, int L, const int* nodes, const float* boxes,          \
                             cudaStream_t s);                                                               \
    int record_floats(int D);                                                                               \
    cudaError_t compute_errors_auto(const MdasDeviceGrid& g, int grid, cudaStream_t s);                     \
    cudaError_t batch_init(const MdasBatchImage* imgs, int n, int D, int grid, cudaStream_t s);              \
    cudaError_t batch_set_counts(const MdasBatchImage* imgs, int n, cudaStream_t s);                         \
    cudaError_t batch_errors(const MdasBatchImage* imgs, int n, int D, int grid, cudaStream_t s);            \
    cudaError_t batch_reset(const MdasBatchImage* imgs, int n, int which, cudaStream_t s);                   \
    cudaError_t batch_decide(const MdasBatchImage* imgs, int n, int D, int K, bool learned, int grid,        \
                             cudaStream_t s);                                                                 \
    cudaError_t batch_scan(const MdasBatchImage* imgs, int n, cudaStream_t s);                               \
    cudaError_t batch_place(const MdasBatchImage* imgs, int n, int D, int grid, cudaStream_t s);             \
    cudaError_t batch_condition(const MdasBatchImage* imgs, int n, cudaGraphConditionalHandle h,             \
                                int maxPasses, int* anyOut, cudaStream_t s);                                 \
    cudaError_t batch_integrate(const MdasBatchImage* imgs, int n, int D, int grid, cudaStream_t s);         \
    cudaError_t batch_clear_pixels(const MdasBatchImage* imgs, int n, cudaStream_t s);                       \
    unsigned batch_jump(int candidatesNum, int D, unsigned* C);                                              \
    cudaError_t loop_condition(const MdasDeviceGrid& g, cudaGraphConditionalHandle h, int budget,           \
                               int maxPasses, cudaStream_t s);                                              \
    int max_blocks_per_sm(int D, int which);                                                                \
    cudaError_t learned_judge(const MdasDeviceGrid& g, int L, int grid, cudaStream_t s);                     \
    cudaError_t batch_learned_judge(const MdasBatchImage* imgs, int n, int grid, cudaStream_t s);            \
    }

MDAS_DECLARE_LAUNCHERS(mdas_fast)
MDAS_DECLARE_LAUNCHERS(mdas_ieee)

enum {
    MDAS_K_INIT = 0,
    MDAS_K_ERRORS = 1,
    MDAS_K_ADAPTIVE = 2,
    MDAS_K_INTEGRATE = 3,
    MDAS_K_DECIDE = 4,
    MDAS_K_COUNT = 5
};
