/* mdas.h — C ABI of the GB300-native MDAS sampler (libpmdas_gb300.so).
 *
 * Drop-in for the reference's sampler class template
 *   mdas::KDGrid<PointN<D>>           SDK/lib/mdas/kdgrid.h:10-107
 * whose methods are implemented in     SDK/lib/mdas/kdgrid.cu:600-961.
 * The point dimension D (3..6, SDK/lib/mdas/point.h:196-199) is a runtime
 * argument instead of a template parameter.
 *
 * Conventions
 *   - Every function returns an int status (MDAS_OK == 0) unless stated;
 *     nothing throws across the ABI.  The reference prints CUDA errors and
 *     continues (SDK/lib/mdas/buffer.h:6-16); this library returns them.
 *   - The grid owns its device buffers (device memory, not managed memory).
 *     Callers own the pixel buffers they pass in.
 *   - All work is queued on the grid's stream (default: the legacy default
 *     stream, like the reference).  Calls that must report counts to the host
 *     (mdas_adaptive_sampling, mdas_sampling_pass) synchronise that stream,
 *     as the reference does with cudaMemcpyFromSymbol (kdgrid.cu:753-759).
 *   - Device pointers are plain `float*`; a float3 buffer is 3 floats per
 *     sample, a float4 pixel buffer 4 floats per pixel.
 */
#ifndef PMDAS_GB300_MDAS_H
#define PMDAS_GB300_MDAS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mdas_grid mdas_grid;
typedef struct mdas_scene mdas_scene;

#define MDAS_OK 0
#define MDAS_ERR_INVALID 1   /* bad argument or configuration */
#define MDAS_ERR_CUDA 2      /* a CUDA call failed */
#define MDAS_ERR_CAPACITY 3  /* a pass could write past maxSamples samples */
#define MDAS_ERR_TIMEOUT 4   /* a bounded device-side wait gave up */
#define MDAS_ERR_ALLOC 5     /* device or host allocation failed */
#define MDAS_ERR_STATE 6     /* call out of order (e.g. a pass before InitialSampling) */

/* Arithmetic of the float work.
 * REFERENCE: the reference's own build flags (--use_fast_math); results match
 *            the reference's CUDA kernels bit for bit.
 * IEEE:      correctly rounded binary32 without contraction and a reproducible
 *            pow; results match a CPU restatement bit for bit. */
#define MDAS_ARITH_REFERENCE 0
#define MDAS_ARITH_IEEE 1

/* Replaces KDGrid::KDGrid(maxSamples, candidatesNum, bitsPerDim, extraImgBits,
 * alpha, scaleX, scaleY, std::ofstream* log)   (kdgrid.h:42-51, kdgrid.cu:600-631).
 * logPath may be NULL; otherwise the per-stage keys of the reference's log
 * (INITIAL SAMPLES, INITIAL SAMPLING TIME, COMPUTE ERRORS TIME, SAMPLES,
 * ADAPTIVE SAMPLING TIME, TOTAL SAMPLES, INTEGRATE TIME) are appended to it. */
int mdas_create(mdas_grid** out, int dim, int maxSamples, int candidatesNum, int bitsPerDim, int extraImgBits,
                float alpha, float scaleX, float scaleY, const char* logPath);

/* mdas_create with the arithmetic mode and a CUDA stream (cudaStream_t, may be NULL). */
int mdas_create_ex(mdas_grid** out, int dim, int maxSamples, int candidatesNum, int bitsPerDim, int extraImgBits,
                   float alpha, float scaleX, float scaleY, const char* logPath, int arith, void* stream);

/* Replaces KDGrid::~KDGrid (buffers freed, buffer.h:37-38). */
int mdas_destroy(mdas_grid* g);

/* Changes the stream later calls queue their work on. */
int mdas_set_stream(mdas_grid* g, void* stream);

/* Replaces KDGrid::InitialSampling (kdgrid.cu:633-674). */
int mdas_initial_sampling(mdas_grid* g);

/* Replaces KDGrid::ComputeErrors (kdgrid.cu:676-716). */
int mdas_compute_errors(mdas_grid* g);

/* Replaces KDGrid::AdaptiveSampling (kdgrid.cu:718-773).  Returns
 * MDAS_ERR_CAPACITY instead of writing out of bounds when N + L > maxSamples
 * (the pass could add one sample per leaf). */
int mdas_adaptive_sampling(mdas_grid* g);

/* Replaces KDGrid::SamplingPass (kdgrid.cu:775-779). */
int mdas_sampling_pass(mdas_grid* g);

/* Replaces KDGrid::Integrate(float4* pixels, int width, int height)
 * (kdgrid.cu:781-820); pixels is a device float4 buffer of width*height. */
int mdas_integrate(mdas_grid* g, float* pixels, int width, int height);

/* Replaces KDGrid::ConvertToBytes(float4*, uchar4*, w, h) (kdgrid.cu:839-846);
 * both are device buffers. */
int mdas_convert_to_bytes(mdas_grid* g, const float* pixels, unsigned char* bytes, int width, int height);

/* Replaces KDGrid::SamplingDensity(float4* pixels, w, h) (kdgrid.cu:822-837);
 * pixels is a HOST float4 buffer, as in the reference. */
int mdas_sampling_density(mdas_grid* g, float* hostPixels, int width, int height);

/* Same result into a device float4 buffer. */
int mdas_sampling_density_device(mdas_grid* g, float* pixels, int width, int height);

/* Replaces KDGrid::Validate (kdgrid.cu:848-961): *valid = 1 if every sample
 * lies in its leaf, the leaf volumes add up to scaleX*scaleY within 1%, and
 * every sample is referenced exactly once; *valid = 0 otherwise. */
int mdas_validate(mdas_grid* g, int* valid);

/* Replace GetSampleCoordinates().Data() / GetSampleValues().Data()
 * (kdgrid.h:65-66): device buffers the caller's integrand reads (AoS, dim
 * floats per sample) and writes (3 floats per sample) in place. */
float* mdas_sample_coordinates(mdas_grid* g);
float* mdas_sample_values(mdas_grid* g);

/* Replace GetNumberOfSamples / GetNewSamples / GetNumberOfNodes / GetNewNodes
 * (kdgrid.h:69-72). */
int mdas_get_counts(mdas_grid* g, int* numberOfSamples, int* newSamples, int* numberOfNodes, int* newNodes);

/* Replace GetCandidatesNum / GetMaxNodeSize / GetMaxSamples / GetScaleX / GetScaleY
 * (kdgrid.h:67-76), plus the dimension and arithmetic mode. */
int mdas_get_info(mdas_grid* g, int* dim, int* maxSamples, int* candidatesNum, int* maxNodeSize, float* scaleX,
                  float* scaleY, int* arith);

/* g_error of the last ComputeErrors (the __device__ float of kdgrid.cu:21). */
int mdas_get_gerror(mdas_grid* g, float* gError);

/* Copy the complete sampler state to host buffers: coords [N*dim], values [N*3],
 * nodes [L*4], boxes [L*2*dim], errors [L], seeds [L] (any may be NULL). */
int mdas_dump_state(mdas_grid* g, float* coords, float* values, int* nodes, float* boxes, float* errors,
                    uint32_t* seeds);

/* Load a complete state from host buffers (a checkpoint, or a parity case). */
int mdas_load_state(mdas_grid* g, int numberOfSamples, int numberOfNodes, const float* coords, const float* values,
                    const int* nodes, const float* boxes, const float* errors, const uint32_t* seeds);

/* One adaptive sampling pass that allocates no memory (no counterpart in the
 * reference; it exists for callers of this library that cannot allocate).
 *
 * mdas_create allocates the sampler's state with cudaMalloc.  Some callers
 * cannot allocate when they sample: a plugin host that hands out all device
 * memory up front and forbids allocations afterwards, a process whose device
 * memory belongs to another framework's caching allocator (a library's own
 * cudaMalloc can fail for memory the pool holds, or fragment it), or a
 * frame-paced renderer for which cudaMalloc/cudaFree inside a frame cost too
 * much (they can synchronise the device).  This call runs one pass of
 * KDGrid::AdaptiveSampling on buffers the caller owns, laid out like the
 * reference's sampler: coords (dim floats per sample, room for maxSamples
 * samples), nodes (4 ints per leaf, ~dim = empty), boxes (mn[dim] then
 * mx[dim] per leaf), errors and seeds (one per leaf; nodes, boxes, errors and
 * seeds with room for nodeCapacity leaves).  gError is the max leaf error of
 * the caller's errors pass.  The results equal mdas_adaptive_sampling's in
 * the reference arithmetic; the new counts are returned in *newSamples and
 * *newNodes: the call copies them to the host and synchronises `stream`
 * before it returns, like mdas_adaptive_sampling.
 *
 * Its only scratch (per-tile counts of 1024 leaves, 64 KB) lives in a fixed
 * array of device memory inside this library, so a pass takes at most
 * MDAS_STATIC_MAX_LEAVES leaves; larger passes return MDAS_ERR_INVALID.  The
 * capacity check is the worst case, stricter than the reference's own sizes:
 * every leaf may take one sample and split into one more leaf, so it needs
 * maxSamples >= numberOfSamples + numberOfNodes and nodeCapacity >=
 * 2 * numberOfNodes, and returns MDAS_ERR_CAPACITY otherwise, before any
 * work.  Nothing in the array needs clearing between calls: every call
 * overwrites the entries it reads.  All calls share that one array, so calls
 * that overlap on the GPU (two streams, two threads) race and must be
 * serialised by the caller.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress) and keeps it; the call must not be
 * used across a cudaDeviceReset. */
#define MDAS_STATIC_MAX_LEAVES (1 << 22)
int mdas_adaptive_sampling_static(int dim, int numberOfSamples, int numberOfNodes, int candidatesNum, float alpha,
                                  float gError, int maxSamples, int nodeCapacity, float* coords, int* nodes,
                                  float* boxes, float* errors, uint32_t* seeds, int* newSamples, int* newNodes,
                                  void* stream);

/* Test hook (no counterpart in the reference): the number of polls after which
 * the library's bounded device-side waits report MDAS_ERR_TIMEOUT (polls <= 0
 * restores their own limits).  The radix sort's look-back then gives up and
 * its output is incomplete (its scatter stays in bounds); the waits for the
 * tensor-core MMAs of the priority MLP record the timeout and wait on with
 * their own limit, so their results stay complete and no MMA is in flight
 * when a kernel ends.  Process-wide; needs a current CUDA device. */
int mdas_test_set_wait_limit(int polls);

/* Per-stage CUDA-event times accumulated since the last reset, in ms:
 * [0] initial sampling, [1] compute errors, [2] adaptive sampling,
 * [3] integrate, [4] integrand.  Timing is off until mdas_set_timing(g, 1). */
int mdas_set_timing(mdas_grid* g, int on);
int mdas_get_stage_times(mdas_grid* g, double* ms5, int reset);
/* The same n <= 6 times; [5] is the adaptive pass as the caller sees it, from
 * its launch until the host holds the new counts (the window of the
 * reference's own ADAPTIVE SAMPLING TIME, which ends after its two blocking
 * counter reads, kdgrid.cu:753-768); [2] is its kernels' device time only. */
int mdas_get_stage_times_ex(mdas_grid* g, double* ms, int n, int reset);

/* Tallies of the last sampling pass (for traffic accounting): leaves whose error
 * was recomputed, leaves accepted, leaves split, and sample coordinates the
 * adaptive pass read.  Valid after mdas_adaptive_sampling returns. */
int mdas_get_pass_stats(mdas_grid* g, int* recomputed, int* selected, int* splits, int64_t* gathered);

/* Number of kernels this grid has launched (all of them this library's own). */
int mdas_get_launch_count(mdas_grid* g, uint64_t* launches);

const char* mdas_status_string(int status);

/* ---- analytic integrand (stands in for the OptiX ray-generation programs,
 *      SDK/cuda/whitted.cu:164-293, SDK/cuda/direct.cu:116-152) ---- */
#define MDAS_SCENE_DISCS_MB 0     /* (x, y, t)       */
#define MDAS_SCENE_DISCS_DOF 1    /* (x, y, u, v)    */
#define MDAS_SCENE_DISCS_MBDOF 2  /* (x, y, t, u, v) */
#define MDAS_SCENE_DIRECT_LIGHT 3 /* (x, y, u, v)    */

/* Seeded scene: kind, seed, primitive count, the grid's scaleX/scaleY and the image size. */
int mdas_scene_create(mdas_scene** out, int kind, uint64_t seed, int count, float scaleX, float scaleY, int width,
                      int height);
int mdas_scene_destroy(mdas_scene* s);
/* Copy the scene descriptor (descBytes >= mdas_scene_desc_size()) and its
 * primitives (12 floats each) to host memory. */
int mdas_scene_desc_size(void);
int mdas_scene_export(mdas_scene* s, void* desc, int descBytes, float* prims, int maxPrims, int* dim, int* count);

/* Evaluate samples [offset, offset+count) of the grid in place — the
 * reference's launchSubframe with sample_offset/sample_count
 * (optixMotionBlur.cpp:420-470).  count < 0 evaluates the samples the last
 * adaptive pass added. */
int mdas_evaluate(mdas_grid* g, mdas_scene* s, int offset, int count);

/* The same integrand over any device buffers: coords AoS with `dim` floats per
 * sample (dim >= the scene's dimension), values 3 floats per sample. */
int mdas_scene_evaluate(mdas_scene* s, const float* coords, float* values, int dim, int offset, int count,
                        void* stream);

/* Reference image of the scene for quality measurement: `spp` (a square
 * number) samples per pixel, image plane stratified with jitter, radiance
 * accumulated in FP64; `out` is a device buffer of width*height*3 doubles.
 * The rel-MSE of an MDAS image is measured against it, as the reference's
 * scripts measure against a high-spp render (SDK/data/Scripts/parse_logs.py:48-50). */
int mdas_scene_reference_image(mdas_scene* s, int width, int height, int spp, uint64_t seed, double* out,
                               void* stream);

/* ---- the headless budget loop of the sample apps (optixMotionBlur.cpp:768-793) ----
 * initial sampling, integrand, then while N < budget: sampling pass + integrand
 * for the new samples, then integrate into a device float4 image.  Stops early
 * (like the interactive loop's guard, optixMotionBlur.cpp:723-724) when the
 * next pass could overrun the buffers. */
typedef struct mdas_render_stats {
    int numberOfSamples;
    int numberOfNodes;
    int passes;
    int reserved;
    double stageMs[5];  /* as mdas_get_stage_times, when timing is on */
} mdas_render_stats;

int mdas_render(mdas_grid* g, mdas_scene* s, int budget, float* pixels, int width, int height,
                mdas_render_stats* stats);

/* The same budget loop as one CUDA graph: the loop runs on the device (a
 * conditional while node around errors + adaptive pass + integrand for the new
 * samples + the loop condition), so a whole render costs one launch and one
 * synchronisation instead of one per pass.  Results are identical to
 * mdas_render.  The graph is built on the first call and reused while the
 * scene, budget and pixel buffer stay the same; stats->stageMs stays zero
 * (no per-stage events inside the graph). */
int mdas_render_graph(mdas_grid* g, mdas_scene* s, int budget, float* pixels, int width, int height,
                      mdas_render_stats* stats);

/* mdas_render_graph with HOST input and output: the scene primitives are uploaded
 * from `hostPrims` (12 floats each, may be NULL to keep the scene's) and the
 * float4 image is copied back into `hostPixels`. */
int mdas_render_host(mdas_grid* g, mdas_scene* s, const float* hostPrims, int budget, float* hostPixels, int width,
                     int height, mdas_render_stats* stats);

/* ---- batched rendering: many images of uneven size, dimension and budget ----
 * One render of all images of the batch in one CUDA graph: every stage is one
 * launch per point dimension present (the work items of all images share
 * each launch), and a device-side loop runs passes until every image reached
 * its budget (or its capacity).  Each image's result equals what mdas_render
 * gives for it alone.  The grids and scenes stay owned by the caller; a grid
 * may appear once; all grids use the same arithmetic and device; up to 256
 * images.  pixels[i] is a device float4 buffer of widths[i] * heights[i]. */
typedef struct mdas_batch mdas_batch;
int mdas_batch_create(mdas_batch** out, int n, mdas_grid* const* grids, mdas_scene* const* scenes,
                      const int* budgets, float* const* pixels, const int* widths, const int* heights);
int mdas_batch_destroy(mdas_batch* b);
/* Renders every image; stats (n entries, caller order) may be NULL. */
int mdas_batch_render(mdas_batch* b, mdas_render_stats* stats);
/* The same render with the loop over passes on the host: the same kernels
 * launched on the stream one pass at a time (one 4-byte read of the loop's
 * verdict per pass) instead of the graph's device-side loop.  Same results;
 * for tools that cannot look inside a graph's conditional node (profilers). */
int mdas_batch_render_stepped(mdas_batch* b, mdas_render_stats* stats);
/* Persistent CTAs per SM of the errors, decide, place and integrate/integrand
 * launches (rebuilds the graph). */
int mdas_batch_set_tuning(mdas_batch* b, const int* ctasPerSm4);
/* mdas_batch_set_tuning plus the tile size of the adaptive pass's decide
 * kernel (leavesPerTile: 1024 or 2048 leaves per 256-thread tile).  The
 * results do not depend on it. */
int mdas_batch_set_tiling(mdas_batch* b, const int* ctasPerSm4, int leavesPerTile);
/* The batch's autotuner: times candidate tunings on this batch (`repeats`
 * renders each after a warm one) by coordinate descent from the default — the
 * decide tile size, then each stage's CTAs per SM in turn — keeps the fastest
 * and returns it (each pointer optional) with its time per render and the
 * number of candidates timed. */
int mdas_batch_autotune_ex(mdas_batch* b, int repeats, int* best4, int* bestLeavesPerTile, double* bestMs,
                           int* evaluated);
/* mdas_batch_autotune_ex without the tile size and the count. */
int mdas_batch_autotune(mdas_batch* b, int repeats, int* best4, double* bestMs);

/* ---- Leaf ordering: Morton keys, radix sort, Karras hierarchy, point location.
 *
 * No reference counterpart (the reference keeps its leaves in allocation order
 * and stores no tree); none of these calls changes the grid.  A key numbers the
 * cells of a finer grid the way the reference numbers its initial cells
 * (uniformSamplingKernel, kdgrid.cu:144-160), at bitsPerDim + fineBits bits per
 * dimension (+ extraImgBits for the two image dimensions):
 *   bit k < bitsPerDim + fineBits of the cell coordinate of dimension j is key
 *   bit dim*k + (dim-1-j); image bit k >= bitsPerDim + fineBits is key bit
 *   dim*(bitsPerDim + fineBits) + 2*(k - bitsPerDim - fineBits) + 1-j.
 * So key >> (dim * fineBits) is the reference's index of the initial cell
 * holding the point, and keys sort points along a Z-order curve whose top
 * levels are the image plane.  The cell coordinate of coordinate x of
 * dimension j is floor(x / scale_j * 2^bits_j) clamped to the grid (scale =
 * scaleX, scaleY, then 1). */

/* Bits of a key (<= 64), or -1 if the parameters need more. */
int mdas_morton_key_bits(int dim, int bitsPerDim, int extraImgBits, int fineBits);

/* Keys of n points (device pointers: points [n * dim] floats, keys [n]). */
int mdas_morton_encode(int dim, int bitsPerDim, int extraImgBits, int fineBits, float scaleX, float scaleY,
                       const float* points, int n, uint64_t* keys, void* stream);

/* The boxes (mn[dim], mx[dim]) of n cells at bitsPerDim bits per dimension,
 * computed as uniformSamplingKernel computes the initial cells' boxes
 * (kdgrid.cu:142-164, 191-196).  Device pointers. */
int mdas_morton_decode(int dim, int bitsPerDim, int extraImgBits, float scaleX, float scaleY, const uint64_t* cells,
                       int n, float* boxes, void* stream);

/* Stable LSD radix sort of (key, value) pairs on key bits [beginBit, endBit),
 * 8 bits per pass.  Device pointers; valuesIn == NULL sorts the values 0..n-1;
 * keysIn must not be keysOut.  Call with temp == NULL to get *tempBytes.
 * Synchronises `stream`; MDAS_ERR_TIMEOUT if a bounded inter-CTA wait gave up
 * (the output is then incomplete). */
int mdas_radix_sort_pairs(void* temp, size_t* tempBytes, const uint64_t* keysIn, uint64_t* keysOut,
                          const uint32_t* valuesIn, uint32_t* valuesOut, int n, int beginBit, int endBit,
                          void* stream);

/* The grid's leaves in key order: key of each leaf's box centre (fineBits < 0:
 * the most that fit in 64 bits), sorted; `order` receives the leaf slots, ties
 * in slot order.  Device pointers of numberOfNodes entries, each optional. */
int mdas_leaf_order(mdas_grid* g, int fineBits, uint64_t* keys, uint32_t* order);

/* Orders the leaves (as mdas_leaf_order) and builds a Karras radix tree over
 * them: numberOfNodes - 1 internal nodes, root 0, with boxes that bound their
 * leaves.  Valid until the grid changes. */
int mdas_build_hierarchy(mdas_grid* g, int fineBits);

/* Host copies of the hierarchy, each pointer optional: n = numberOfNodes sorted
 * keys and leaf slots; children [2 (n-1)] (c >= 0: internal node c, c < 0: the
 * leaf at sorted position ~c); parents [2n - 1] (internal nodes, then leaves by
 * sorted position; -1 for the root); boxes [(n-1) * 2 dim] of the internal
 * nodes.  MDAS_ERR_STATE if the grid changed since mdas_build_hierarchy. */
int mdas_get_hierarchy(mdas_grid* g, int* numLeaves, uint64_t* keys, uint32_t* order, int* children, int* parents,
                       float* boxes);

/* For each of n points (device [n * dim]) the leaf slot whose box holds it
 * (mn <= x < mx per dimension, x <= mx on the domain's upper faces), the first
 * in key order if several do, -1 if none (device [n]).  Needs a current
 * hierarchy (MDAS_ERR_STATE otherwise).  Synchronises the grid's stream. */
int mdas_locate(mdas_grid* g, const float* points, int n, int* leaves);

/* ---- Learned acceptance: a leaf-priority MLP on the tensor cores.
 *
 * No reference counterpart.  The reference accepts a leaf with probability
 * powf(error / g_error, alpha) (kdgrid.cu:326).  In learned mode the error is
 * replaced by an estimate of the leaf's true reconstruction error: the plain
 * error times 2^(32 c), c the output of a 16 -> 64 -> 64 -> 1 ReLU MLP (BF16
 * tcgen05 GEMMs, FP32 accumulation) of per-leaf features: log2 box extents of
 * the first five dimensions (image axes relative to the image), the sample
 * count, log2(1 + x) of the samples' luminance mean, deviation, minimum and
 * maximum, the plain error, the depth below the initial cell, and the plain
 * errors of the four neighbouring leaf slots; the ratio is the estimate over
 * the largest one.  The model is trained offline (mdas_leaf_features,
 * mdas_leaf_true_errors, mdas_mlp_gradients, mdas_mlp_adam) on
 * log2(true error / plain error) / 32.  The plain error still judges every
 * pass: both schedules' acceptance is drawn from the same random number, and a
 * pass in which the learned schedule leaves more than (1 + tolerance) x the
 * plain schedule's plain error unrefined takes the plain acceptance.
 * Predictions are refreshed for the leaves whose error a pass recomputes.
 * Learned mode runs in mdas_sampling_pass, mdas_render and mdas_render_graph. */
#define MDAS_MLP_PARAMS 5313 /* W1[64][16], b1[64], W2[64][64], b2[64], w3[64], b3 */

typedef struct mdas_learned_config {
    float tolerance;      /* default 0.05 */
    uint64_t seed;        /* initial weights when params is NULL (default 1) */
    const float* params;  /* host, MDAS_MLP_PARAMS trained weights (NULL: seeded initial weights) */
} mdas_learned_config;

int mdas_learned_defaults(mdas_learned_config* cfg);
/* Turns learned mode on (cfg == NULL: off). */
int mdas_learned_enable(mdas_grid* g, const mdas_learned_config* cfg);
/* Predicts every leaf and judges the pass (needs the leaves' errors: after
 * mdas_compute_errors); mdas_sampling_pass calls it between its halves. */
int mdas_learned_update(mdas_grid* g);
/* Predicts every leaf, without judging (tests, inspection). */
int mdas_learned_predict(mdas_grid* g);
/* Passes judged, passes sent back to the plain acceptance, the last pass's
 * verdict (1 = plain) and its unrefined plain error of each schedule (each
 * pointer optional). */
int mdas_learned_stats(mdas_grid* g, int* judgedPasses, int* plainPasses, int* lastPlain, double* unrefinedLearned,
                       double* unrefinedPlain);
/* The largest priority the last update scaled the acceptance by (the maximum
 * over every leaf's current prediction). */
int mdas_learned_pred_max(mdas_grid* g, float* predMax);
/* Host copies of the FP32 parameters (MDAS_MLP_PARAMS floats). */
int mdas_learned_get_params(mdas_grid* g, float* params);
int mdas_learned_set_params(mdas_grid* g, const float* params);
/* Device copy of the current predictions (numberOfNodes floats). */
int mdas_learned_predictions(mdas_grid* g, float* pred);
/* Device copy of the leaves' features (numberOfNodes x 16 floats). */
int mdas_leaf_features(mdas_grid* g, float* features);
/* Training targets: the true reconstruction error of leaves against the
 * integrand's mean over each box from samplesPerLeaf uniform points (FP64
 * accumulation): volume * sum_c |mean_c - ref_c| / sqrt(ref_c^2 + 1e-2).  For
 * the `count` leaf slots in `leaves` (device), or every leaf if leaves is
 * NULL; device output, one float per row. */
int mdas_leaf_true_errors(mdas_grid* g, mdas_scene* s, int samplesPerLeaf, uint64_t seed, const int* leaves,
                          int count, float* errors);

/* The MLP on its own (device pointers): pred[m] of features[m x 16];
 * gradients of mean((pred - target)^2) into grads[MDAS_MLP_PARAMS] and the
 * loss into *loss (host); one bias-corrected Adam step (step >= 1) that also
 * zeroes grads. */
int mdas_mlp_forward(const float* params, const float* features, int m, float* pred, void* stream);
int mdas_mlp_gradients(const float* params, const float* features, const float* targets, int m, float* grads,
                       float* loss, void* stream);
int mdas_mlp_adam(float* params, float* m1, float* m2, float* grads, int step, float learningRate, void* stream);

/* ---- env configuration (SDK/sutil/Environment.{h,cpp}; the options the MDAS
 *      apps register, optixMotionBlur.cpp:104-137) ---- */
typedef struct mdas_config {
    int mdas;            /* Sampler.mdas        (bool, default 0)    */
    float samples;       /* Sampler.samples     (float, default 1)   */
    float scaleFactor;   /* Mdas.scaleFactor    (float, default 1.0) */
    float alpha;         /* Mdas.alpha          (float, default 0.25)*/
    int bitsPerDim;      /* Mdas.bitsPerDim     (int, default 0)     */
    int extraImgBits;    /* Mdas.extraImgBits   (int, default 8)     */
    int candidatesNum;   /* Mdas.candidatesNum  (int, default 4)     */
    int width;           /* Film.width          (int, default 1024)  */
    int height;          /* Film.height         (int, default 768)   */
    float focalDistance; /* Camera.focalDistance (float, default 0)  */
    float lensRadius;    /* Camera.lensRadius   (float, default 0)   */
    float fovy;          /* Camera.fovy         (float, default 45)  */
    int sceneKind;       /* Scene.kind (this library's synthetic scenes, default -1 = unset) */
    int sceneCount;      /* Scene.count   (int, default 0)  */
    int64_t sceneSeed;   /* Scene.seed    (int, default 0)  */
    char filmFilename[256]; /* Film.filename */
} mdas_config;

/* Defaults of the registered options. */
int mdas_config_defaults(mdas_config* cfg);

/* Parse an .env file with the reference's rules (blocks `Name { key value }`,
 * '#' comments, unknown keys are an error, numbers round-tripped through
 * std::to_string, the first occurrence of a key wins).  `err` receives a
 * message on failure. */
int mdas_config_read(const char* path, mdas_config* cfg, char* err, int errBytes);

/* ---- image files (replace sutil::saveImage in the sample apps,
 *      SDK/optixMotionBlur/optixMotionBlur.cpp:795-840) ---- */
#define MDAS_IMAGE_FLOAT4 0 /* float4 pixels (the film, the sampling density) -> PFM */
#define MDAS_IMAGE_UCHAR4 1 /* uchar4 pixels (after mdas_convert_to_bytes)     -> PPM */

/* Write width x height pixels from HOST memory, row-major from the top, to
 * `path`: float4 as a Portable Float Map (RGB float32, little-endian; in place
 * of the reference's OpenEXR output), uchar4 as a binary PPM (RGB).  Alpha is
 * dropped.  MDAS_ERR_INVALID if the file cannot be written. */
int mdas_save_image(const char* path, const void* pixels, int width, int height, int format);

#ifdef __cplusplus
}
#endif

#endif /* PMDAS_GB300_MDAS_H */
