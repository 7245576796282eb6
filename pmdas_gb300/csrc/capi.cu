// capi.cu — host side of libpmdas_gb300: the C ABI declared in include/mdas.h.
//
// Mirrors the host drivers of mdas::KDGrid (SDK/lib/mdas/kdgrid.cu:600-961)
// and the headless budget loop of the sample apps
// (SDK/optixMotionBlur/optixMotionBlur.cpp:768-793), over device memory and a
// caller-chosen stream.  The kernels live in kdgrid_fast.cu (the reference's
// arithmetic) and kdgrid_ieee.cu (strict IEEE); a grid picks one at creation.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include <stddef.h>
#include <math.h>
#include <fstream>
#include <string>
#include <vector>
#include <new>

#include "../../include/mdas.h"
#include "grid_types.h"
#include "scene.h"
#include "order.h"
#include "mlp.h"
#include "leaf_raw.h"

namespace {

__global__ void k_set_counts(MdasCounts* c, int N, int L) {
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
    c->active = 1;
}

struct PendingTiming {
    int stage;
    cudaEvent_t a, b;
};

// An instantiated device-side render (mdas_render_graph) and what it was built for.
struct RenderGraph {
    cudaGraphExec_t exec = nullptr;
    const void* scene = nullptr;
    int budget = 0;
    float* pixels = nullptr;
    int width = 0, height = 0;
    cudaStream_t stream = nullptr;
};

}  // namespace

struct mdas_grid {
    MdasDeviceGrid dg{};
    int arith = MDAS_ARITH_REFERENCE;
    cudaStream_t stream = nullptr;
    int device = 0;
    int numSMs = 1;
    int occ[MDAS_K_COUNT] = {1, 1, 1, 1, 1};
    int N = 0, L = 0, newN = 0, newL = 0;
    bool initialized = false;
    // errorsClean: every leaf error is >= 0 (an errors pass ran since the last change).
    // dirtyValid: the last adaptive pass ran on a clean state, so the leaves needing an
    // error are exactly its split children and the next errors pass can visit only those.
    bool errorsClean = false;
    bool dirtyValid = false;
    MdasCounts* hcounts = nullptr;  // pinned mirror of the device counters
    std::ofstream* log = nullptr;
    bool timing = false;
    // [0..4] device time of the stages' kernels; [5] the adaptive pass as the
    // caller sees it: from its launch until the host holds the new counts
    double stageMs[6] = {0, 0, 0, 0, 0, 0};
    uint64_t launches = 0;
    float* scratch = nullptr;  // density / host-render image
    size_t scratchBytes = 0;
    std::vector<cudaEvent_t> eventPool;
    std::vector<PendingTiming> pending;
    RenderGraph graph;
    cudaStream_t captureStream = nullptr, bodyStream = nullptr;
    // leaf order and hierarchy (mdas_leaf_order, mdas_build_hierarchy)
    uint64_t version = 0;             // bumped by every call that changes the leaves
    uint64_t hierVersion = ~0ull;     // version the hierarchy was built for
    int hierN = 0, hierCap = 0, hierFineBits = 0;
    uint64_t* hKeys = nullptr;        // [cap] key of each leaf slot
    uint64_t* hSorted = nullptr;      // [cap] keys in ascending order
    uint32_t* hOrder = nullptr;       // [cap] leaf slots in key order
    int2* hChildren = nullptr;        // [cap] children of the internal nodes
    int* hParents = nullptr;          // [2 cap] parents of the internal nodes, then of the leaves
    float* hBoxes = nullptr;          // [cap * 2D] boxes of the internal nodes
    unsigned* hVisits = nullptr;      // [cap + 1] refit arrival counters, then the locate status word
    void* sortTemp = nullptr;
    size_t sortTempBytes = 0;
    // point location: coarse keys of the queries (2 cap), their order, sort scratch
    int qCap = 0;
    uint64_t* qKeys = nullptr;
    uint32_t* qPerm = nullptr;
    void* qTemp = nullptr;
    size_t qTempBytes = 0;
    // learned acceptance (mdas_learned_enable)
    bool learned = false;
    float* lState = nullptr;            // FP32 params (MDAS_MLP_PARAMS), then a status word
    mdas_mlp::Packed* lPacked = nullptr;
    float* lPred = nullptr;             // [maxNodes] predicted log2(error) / MDAS_MLP_TARGET_SCALE
    float* lRaw = nullptr;              // [maxNodes * MDAS_RAW_FLOATS] raw feature rows of the split-children errors pass
    bool rawValid = false;              // the last errors pass wrote lRaw for the leaves it recomputed
    bool extentsValid = false;          // the last adaptive pass wrote the box extents of its split children's rows
    MdasLearnedStats* lStats = nullptr;
    uint64_t lPredVersion = ~0ull;      // grid version the predictions (and the verdict) belong to
    bool lastErrorsDirty = false;       // the last errors pass visited only the split children
};

namespace {

int status_of(cudaError_t e) { return e == cudaSuccess ? MDAS_OK : MDAS_ERR_CUDA; }

// tea<4>(v, 0) of SDK/cuda/random.h:31-46: the seed a leaf slot's first draw
// starts from.  The grid stores it in slots that were never drawn from; the
// reference stores 0 there (kdgrid.cu:323-324, 637), and the state dump and
// load translate between the two.
uint32_t host_tea4(uint32_t val0) {
    uint32_t v0 = val0, v1 = 0, s0 = 0;
    for (int n = 0; n < 4; n++) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}

cudaEvent_t pool_get(mdas_grid* g) {
    if (!g->eventPool.empty()) {
        cudaEvent_t e = g->eventPool.back();
        g->eventPool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void flush_timing(mdas_grid* g) {
    for (const PendingTiming& p : g->pending) {
        float ms = 0.0f;
        if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess)
            g->stageMs[p.stage] += ms;
        g->eventPool.push_back(p.a);
        g->eventPool.push_back(p.b);
    }
    g->pending.clear();
}

// Runs `launch` between two events of the given stage when timing is on.
template <class F>
int timed(mdas_grid* g, int stage, F&& launch) {
    cudaEvent_t a = nullptr, b = nullptr;
    if (g->timing) {
        a = pool_get(g);
        b = pool_get(g);
        cudaEventRecord(a, g->stream);
    }
    const cudaError_t e = launch();
    if (g->timing) {
        cudaEventRecord(b, g->stream);
        g->pending.push_back({stage, a, b});
    }
    return status_of(e);
}

// Time of the most recent pending event pair of `stage` (syncs), for the log.
double last_stage_ms(mdas_grid* g, int stage) {
    double before = g->stageMs[stage];
    flush_timing(g);
    return g->stageMs[stage] - before;
}

int grid_for(mdas_grid* g, int which, int64_t items) {
    const int64_t want = (items + 255) / 256;
    const int64_t cap = (int64_t)g->numSMs * (g->occ[which] > 0 ? g->occ[which] : 1);
    int64_t n = want < cap ? want : cap;
    return (int)(n < 1 ? 1 : n);
}

cudaError_t launch_initial(mdas_grid* g, int L) {
    return g->arith == MDAS_ARITH_IEEE ? mdas_ieee::initial_sampling(g->dg, L, g->stream)
                                       : mdas_fast::initial_sampling(g->dg, L, g->stream);
}
cudaError_t launch_errors(mdas_grid* g, int grid, bool dirty) {
    return g->arith == MDAS_ARITH_IEEE ? mdas_ieee::compute_errors(g->dg, grid, dirty, g->stream)
                                       : mdas_fast::compute_errors(g->dg, grid, dirty, g->stream);
}
cudaError_t launch_adaptive(mdas_grid* g, int gridDecide, int gridPlace) {
    return g->arith == MDAS_ARITH_IEEE ? mdas_ieee::adaptive_sampling(g->dg, gridDecide, gridPlace, g->stream)
                                       : mdas_fast::adaptive_sampling(g->dg, gridDecide, gridPlace, g->stream);
}
cudaError_t launch_integrate(mdas_grid* g, int grid, float* pixels, int W, int H) {
    return g->arith == MDAS_ARITH_IEEE ? mdas_ieee::integrate(g->dg, grid, pixels, W, H, g->stream)
                                       : mdas_fast::integrate(g->dg, grid, pixels, W, H, g->stream);
}

int ensure_scratch(mdas_grid* g, size_t bytes) {
    if (g->scratchBytes >= bytes) return MDAS_OK;
    if (g->scratch) cudaFree(g->scratch);
    g->scratch = nullptr;
    g->scratchBytes = 0;
    if (cudaMalloc(&g->scratch, bytes) != cudaSuccess) return MDAS_ERR_ALLOC;
    g->scratchBytes = bytes;
    return MDAS_OK;
}

// The device counters to the page-locked host copy, queued on the grid's stream.
cudaError_t counts_copy_async(mdas_grid* g) {
    return cudaMemcpyAsync(g->hcounts, g->dg.counts, sizeof(MdasCounts), cudaMemcpyDeviceToHost, g->stream);
}

// The host copy of the counters (the stream has completed the copy) into the grid's state.
int counts_apply(mdas_grid* g) {
    g->N = g->hcounts->N;
    g->L = g->hcounts->L;
    g->version += 1;
    g->newN = g->hcounts->newN;
    g->newL = g->hcounts->newL;
    return g->hcounts->status ? g->hcounts->status : MDAS_OK;
}

int read_counts(mdas_grid* g) {
    cudaError_t e = counts_copy_async(g);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    return counts_apply(g);
}

void free_grid(mdas_grid* g) {
    if (!g) return;
    flush_timing(g);
    if (g->graph.exec) cudaGraphExecDestroy(g->graph.exec);
    if (g->captureStream) cudaStreamDestroy(g->captureStream);
    if (g->bodyStream) cudaStreamDestroy(g->bodyStream);
    for (cudaEvent_t e : g->eventPool) cudaEventDestroy(e);
    cudaFree(g->dg.coords);
    cudaFree(g->dg.values);
    cudaFree(g->dg.nb);
    cudaFree(g->dg.errors);
    cudaFree(g->dg.leafCounts);
    cudaFree(g->dg.seeds);
    cudaFree(g->dg.counts);
    cudaFree(g->dg.ctl);
    cudaFree(g->dg.tileCounts);
    cudaFree(g->dg.tilePrefix);
    cudaFree(g->dg.accepted);
    cudaFree(g->dg.chunkTile);
    cudaFree(g->dg.dirty);
    cudaFree(g->dg.splitL);
    cudaFree(g->dg.splitR);
    cudaFree(g->hKeys);
    cudaFree(g->hSorted);
    cudaFree(g->hOrder);
    cudaFree(g->hChildren);
    cudaFree(g->hParents);
    cudaFree(g->hBoxes);
    cudaFree(g->hVisits);
    cudaFree(g->sortTemp);
    cudaFree(g->qKeys);
    cudaFree(g->qPerm);
    cudaFree(g->qTemp);
    cudaFree(g->lState);
    cudaFree(g->lPacked);
    cudaFree(g->lPred);
    cudaFree(g->lRaw);
    cudaFree(g->lStats);
    if (g->scratch) cudaFree(g->scratch);
    if (g->hcounts) cudaFreeHost(g->hcounts);
    delete g->log;
    delete g;
}

int scene_upload(mdas_scene* s, cudaStream_t stream) {
    if (s->d_prims) return MDAS_OK;
    const size_t bytes = sizeof(float) * (s->prims.size() ? s->prims.size() : 1);
    if (cudaMalloc(&s->d_prims, bytes) != cudaSuccess) {
        s->d_prims = nullptr;
        return MDAS_ERR_ALLOC;
    }
    if (!s->prims.empty() && cudaMemcpyAsync(s->d_prims, s->prims.data(), sizeof(float) * s->prims.size(),
                                             cudaMemcpyHostToDevice, stream) != cudaSuccess)
        return MDAS_ERR_CUDA;
    const size_t cullWords = mdas_cull_words(s->desc);
    if (cullWords) {
        if (cudaMalloc(&s->d_cull, sizeof(unsigned) * cullWords) != cudaSuccess) {
            s->d_cull = nullptr;
            return MDAS_ERR_ALLOC;
        }
        if (mdas_launch_build_cull(s->desc, s->d_prims, s->d_cull, stream) != cudaSuccess) return MDAS_ERR_CUDA;
    }
    return cudaStreamSynchronize(stream) == cudaSuccess ? MDAS_OK : MDAS_ERR_CUDA;
}

}  // namespace

extern "C" {

const char* mdas_status_string(int s) {
    switch (s) {
        case MDAS_OK: return "ok";
        case MDAS_ERR_INVALID: return "invalid argument or configuration";
        case MDAS_ERR_CUDA: return "CUDA error";
        case MDAS_ERR_CAPACITY: return "sample or leaf capacity exceeded";
        case MDAS_ERR_TIMEOUT: return "device-side wait timed out";
        case MDAS_ERR_ALLOC: return "allocation failed";
        case MDAS_ERR_STATE: return "call out of order";
    }
    return "unknown status";
}

int mdas_create_ex(mdas_grid** out, int dim, int maxSamples, int candidatesNum, int bitsPerDim, int extraImgBits,
                   float alpha, float scaleX, float scaleY, const char* logPath, int arith, void* stream) {
    if (!out) return MDAS_ERR_INVALID;
    *out = nullptr;
    if (dim < 3 || dim > 6 || maxSamples < 1 || maxSamples >= (1 << 30) || candidatesNum < 1 || bitsPerDim < 0 ||
        extraImgBits < 0 || bitsPerDim * dim + 2 * extraImgBits > 28 || !(scaleX > 0.0f) || !(scaleY > 0.0f) ||
        !isfinite(alpha) || !isfinite(scaleX) || !isfinite(scaleY) ||
        (arith != MDAS_ARITH_REFERENCE && arith != MDAS_ARITH_IEEE))
        return MDAS_ERR_INVALID;
    mdas_grid* g = new (std::nothrow) mdas_grid();
    if (!g) return MDAS_ERR_ALLOC;
    g->arith = arith;
    g->stream = (cudaStream_t)stream;
    if (cudaGetDevice(&g->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&g->numSMs, cudaDevAttrMultiProcessorCount, g->device) != cudaSuccess) {
        delete g;
        return MDAS_ERR_CUDA;
    }
    for (int k = 0; k < MDAS_K_COUNT; ++k)
        g->occ[k] = arith == MDAS_ARITH_IEEE ? mdas_ieee::max_blocks_per_sm(dim, k) : mdas_fast::max_blocks_per_sm(dim, k);

    MdasDeviceGrid& d = g->dg;
    d.D = dim;
    d.maxSamples = maxSamples;
    // every leaf holds at least 2 samples (initial leaves 4, split children 2 and 3),
    // so L <= N/2 and maxSamples/2 + 1 leaf slots always suffice (the reference
    // allocates 2 * maxSamples - 1, kdgrid.cu:627-629)
    d.maxNodes = maxSamples / 2 + 1;
    d.nbFloats = mdas_fast::record_floats(dim);
    d.candidatesNum = candidatesNum;
    d.maxNodeSize = 4;                // kdgrid.cu:611
    d.bitsPerDim = bitsPerDim;
    d.extraImgBits = extraImgBits;
    d.alpha = alpha;
    d.scaleX = scaleX;
    d.scaleY = scaleY;
    d.tileK = MDAS_LEAVES_PER_THREAD;
    d.maxTiles = (d.maxNodes + MDAS_TILE_LEAVES_MIN - 1) / MDAS_TILE_LEAVES_MIN;  // (room for the smallest tiles)
    const size_t capSamples = ((size_t)maxSamples + 127) / 128 * 128;  // roundUp(maxSamples, 128), kdgrid.cu:625-626
    bool ok = cudaMalloc(&d.coords, sizeof(float) * capSamples * dim) == cudaSuccess &&
              cudaMalloc(&d.values, sizeof(float) * 3 * capSamples) == cudaSuccess &&
              cudaMalloc(&d.nb, sizeof(float) * (size_t)d.nbFloats * (size_t)d.maxNodes) == cudaSuccess &&
              cudaMalloc(&d.errors, sizeof(float) * (size_t)d.maxNodes) == cudaSuccess &&
              cudaMalloc(&d.leafCounts, (size_t)d.maxNodes + 16) == cudaSuccess &&
              cudaMalloc(&d.seeds, sizeof(unsigned) * (size_t)d.maxNodes) == cudaSuccess &&
              cudaMalloc(&d.counts, sizeof(MdasCounts)) == cudaSuccess &&
              cudaMalloc(&d.ctl, sizeof(MdasCtl)) == cudaSuccess &&
              cudaMalloc(&d.tileCounts, sizeof(uint2) * (size_t)d.maxTiles) == cudaSuccess &&
              cudaMalloc(&d.tilePrefix, sizeof(uint2) * (size_t)d.maxTiles) == cudaSuccess &&
              cudaMalloc(&d.accepted, sizeof(uint2) * (size_t)d.maxTiles * MDAS_TILE_LEAVES_MIN) == cudaSuccess &&
              cudaMalloc(&d.chunkTile, sizeof(int) * ((size_t)d.maxNodes / 256 + 2)) == cudaSuccess &&
              cudaMalloc(&d.dirty, sizeof(int) * ((size_t)d.maxNodes / 2 + 1)) == cudaSuccess &&
              cudaMalloc(&d.splitL, sizeof(int4) * ((size_t)d.maxNodes / 2 + 1)) == cudaSuccess &&
              cudaMalloc(&d.splitR, sizeof(int4) * ((size_t)d.maxNodes / 2 + 1)) == cudaSuccess &&
              cudaMallocHost(&g->hcounts, sizeof(MdasCounts)) == cudaSuccess;
    if (ok) {
        ok = cudaMemset(d.counts, 0, sizeof(MdasCounts)) == cudaSuccess &&
             cudaMemset(d.ctl, 0, sizeof(MdasCtl)) == cudaSuccess &&
             cudaDeviceSynchronize() == cudaSuccess;
    }
    if (!ok) {
        cudaGetLastError();
        free_grid(g);
        return MDAS_ERR_ALLOC;
    }
    memset(g->hcounts, 0, sizeof(MdasCounts));
    if (logPath && logPath[0]) {
        g->log = new (std::nothrow) std::ofstream(logPath, std::ios::app);
        if (!g->log || !g->log->good()) {
            free_grid(g);
            return MDAS_ERR_INVALID;
        }
        g->timing = true;
    }
    *out = g;
    return MDAS_OK;
}

int mdas_create(mdas_grid** out, int dim, int maxSamples, int candidatesNum, int bitsPerDim, int extraImgBits,
                float alpha, float scaleX, float scaleY, const char* logPath) {
    return mdas_create_ex(out, dim, maxSamples, candidatesNum, bitsPerDim, extraImgBits, alpha, scaleX, scaleY,
                          logPath, MDAS_ARITH_REFERENCE, nullptr);
}

int mdas_destroy(mdas_grid* g) {
    if (!g) return MDAS_ERR_INVALID;
    cudaStreamSynchronize(g->stream);
    free_grid(g);
    return MDAS_OK;
}

int mdas_set_stream(mdas_grid* g, void* stream) {
    if (!g) return MDAS_ERR_INVALID;
    g->stream = (cudaStream_t)stream;
    return MDAS_OK;
}

int mdas_initial_sampling(mdas_grid* g) {
    if (!g) return MDAS_ERR_INVALID;
    const MdasDeviceGrid& d = g->dg;
    const int64_t L = ((int64_t)1 << (d.bitsPerDim * d.D)) << (2 * d.extraImgBits);  // kdgrid.cu:641
    const int64_t N = 4 * L;                                                        // kdgrid.cu:642
    if (N > d.maxSamples) return MDAS_ERR_CAPACITY;
    int rc = timed(g, 0, [&]() {
        // the reference zeroes the seed buffer here (kdgrid.cu:637); the kernels write every
        // leaf slot's seed when the slot is created instead, so no memset is needed
        cudaError_t e = launch_initial(g, (int)L);
        if (e != cudaSuccess) return e;
        k_set_counts<<<1, 1, 0, g->stream>>>(d.counts, (int)N, (int)L);
        return cudaGetLastError();
    });
    g->launches += 2;
    if (rc) return rc;
    g->N = (int)N;
    g->L = (int)L;
    g->version += 1;
    g->newN = 0;
    g->newL = 0;
    g->initialized = true;
    g->errorsClean = false;
    g->dirtyValid = false;
    g->extentsValid = false;
    if (g->log) {
        const double t = last_stage_ms(g, 0);
        *g->log << "INITIAL SAMPLES\n" << g->N << std::endl;
        *g->log << "INITIAL SAMPLING TIME\n" << t << std::endl;
    }
    return MDAS_OK;
}

int mdas_compute_errors(mdas_grid* g) {
    if (!g) return MDAS_ERR_INVALID;
    if (!g->initialized) return MDAS_ERR_STATE;
    const bool dirty = g->dirtyValid;
    const int grid = grid_for(g, MDAS_K_ERRORS, dirty ? 2 * (int64_t)g->newL : (int64_t)g->L);
    int rc = timed(g, 1, [&]() { return launch_errors(g, grid, dirty); });
    g->launches += 1;
    if (rc) return rc;
    g->errorsClean = true;
    g->lastErrorsDirty = dirty;
    g->rawValid = dirty && g->dg.featRaw != nullptr && g->extentsValid;
    if (g->log) *g->log << "COMPUTE ERRORS TIME\n" << last_stage_ms(g, 1) << std::endl;
    return MDAS_OK;
}

int mdas_adaptive_sampling(mdas_grid* g) {
    if (!g) return MDAS_ERR_INVALID;
    if (!g->initialized) return MDAS_ERR_STATE;
    // A pass adds at most one sample per leaf.  Leaves then still hold >= 2 samples
    // each, so the leaf count stays <= (N + L) / 2 <= maxSamples / 2 < maxNodes.
    if ((int64_t)g->N + g->L > g->dg.maxSamples) return MDAS_ERR_CAPACITY;
    // one CTA iteration per tile of MDAS_TILE_LEAVES leaves
    const int64_t tiles = ((int64_t)g->L + 256 * g->dg.tileK - 1) / (256 * g->dg.tileK);
    const int gridDecide = grid_for(g, MDAS_K_DECIDE, tiles * 256);
    const int gridPlace = grid_for(g, MDAS_K_ADAPTIVE, g->L);  // one thread per accepted leaf (<= L)
    g->dg.priority = g->learned && g->lPredVersion == g->version ? g->lPred : nullptr;
    cudaEvent_t apiA = nullptr;
    if (g->timing) {
        apiA = pool_get(g);
        cudaEventRecord(apiA, g->stream);
    }
    int rc = timed(g, 2, [&]() { return launch_adaptive(g, gridDecide, gridPlace); });
    g->dg.priority = nullptr;
    g->dirtyValid = g->errorsClean;
    g->extentsValid = g->dg.featRaw != nullptr;
    g->errorsClean = false;
    g->launches += 3;
    if (rc) {
        if (apiA) g->eventPool.push_back(apiA);
        return rc;
    }
    rc = read_counts(g);
    if (apiA) {
        // recorded once the host holds the counts, as the reference's log records its
        // stop event after its two blocking counter reads (kdgrid.cu:753-768)
        cudaEvent_t apiB = pool_get(g);
        cudaEventRecord(apiB, g->stream);
        g->pending.push_back({5, apiA, apiB});
    }
    if (g->log) {
        const double t = last_stage_ms(g, 2);
        *g->log << "SAMPLES\n" << g->newN << std::endl;
        *g->log << "ADAPTIVE SAMPLING TIME\n" << t << std::endl;
    }
    return rc;
}

int mdas_sampling_pass(mdas_grid* g) {
    int rc = mdas_compute_errors(g);
    if (rc) return rc;
    if (g->learned) {
        rc = mdas_learned_update(g);
        if (rc) return rc;
    }
    return mdas_adaptive_sampling(g);
}

int mdas_integrate(mdas_grid* g, float* pixels, int width, int height) {
    if (!g || !pixels || width <= 0 || height <= 0) return MDAS_ERR_INVALID;
    if (!g->initialized) return MDAS_ERR_STATE;
    const int grid = grid_for(g, MDAS_K_INTEGRATE, g->L);
    int rc = timed(g, 3, [&]() { return launch_integrate(g, grid, pixels, width, height); });
    g->launches += 1;
    if (rc) return rc;
    if (g->log) {
        const double t = last_stage_ms(g, 3);
        *g->log << "TOTAL SAMPLES\n" << g->N << std::endl;
        *g->log << "INTEGRATE TIME\n" << t << std::endl;
    }
    return MDAS_OK;
}

int mdas_convert_to_bytes(mdas_grid* g, const float* pixels, unsigned char* bytes, int width, int height) {
    if (!g || !pixels || !bytes || width <= 0 || height <= 0) return MDAS_ERR_INVALID;
    const cudaError_t e = g->arith == MDAS_ARITH_IEEE
                              ? mdas_ieee::convert_to_bytes(pixels, bytes, width * height, g->stream)
                              : mdas_fast::convert_to_bytes(pixels, bytes, width * height, g->stream);
    g->launches += 1;
    return status_of(e);
}

int mdas_sampling_density_device(mdas_grid* g, float* pixels, int width, int height) {
    if (!g || !pixels || width <= 0 || height <= 0) return MDAS_ERR_INVALID;
    if (!g->initialized) return MDAS_ERR_STATE;
    const cudaError_t e = g->arith == MDAS_ARITH_IEEE
                              ? mdas_ieee::sampling_density(g->dg, pixels, width, height, g->stream)
                              : mdas_fast::sampling_density(g->dg, pixels, width, height, g->stream);
    g->launches += 2;
    return status_of(e);
}

int mdas_sampling_density(mdas_grid* g, float* hostPixels, int width, int height) {
    if (!g || !hostPixels || width <= 0 || height <= 0) return MDAS_ERR_INVALID;
    const size_t bytes = sizeof(float) * 4 * (size_t)width * height;
    int rc = ensure_scratch(g, bytes);
    if (rc) return rc;
    rc = mdas_sampling_density_device(g, g->scratch, width, height);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(hostPixels, g->scratch, bytes, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    return status_of(e);
}

float* mdas_sample_coordinates(mdas_grid* g) { return g ? g->dg.coords : nullptr; }
float* mdas_sample_values(mdas_grid* g) { return g ? g->dg.values : nullptr; }

int mdas_get_counts(mdas_grid* g, int* numberOfSamples, int* newSamples, int* numberOfNodes, int* newNodes) {
    if (!g) return MDAS_ERR_INVALID;
    if (numberOfSamples) *numberOfSamples = g->N;
    if (newSamples) *newSamples = g->newN;
    if (numberOfNodes) *numberOfNodes = g->L;
    if (newNodes) *newNodes = g->newL;
    return MDAS_OK;
}

int mdas_get_info(mdas_grid* g, int* dim, int* maxSamples, int* candidatesNum, int* maxNodeSize, float* scaleX,
                  float* scaleY, int* arith) {
    if (!g) return MDAS_ERR_INVALID;
    if (dim) *dim = g->dg.D;
    if (maxSamples) *maxSamples = g->dg.maxSamples;
    if (candidatesNum) *candidatesNum = g->dg.candidatesNum;
    if (maxNodeSize) *maxNodeSize = g->dg.maxNodeSize;
    if (scaleX) *scaleX = g->dg.scaleX;
    if (scaleY) *scaleY = g->dg.scaleY;
    if (arith) *arith = g->arith;
    return MDAS_OK;
}

int mdas_get_gerror(mdas_grid* g, float* gError) {
    if (!g || !gError) return MDAS_ERR_INVALID;
    cudaError_t e = cudaMemcpyAsync(g->hcounts, g->dg.counts, sizeof(MdasCounts), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    // the last errors pass's: this pass's, or (after an adaptive pass) the last pass's
    unsigned bits = g->errorsClean || g->hcounts->passes == 0 ? g->hcounts->gerr : g->hcounts->gerrLast;
    memcpy(gError, &bits, 4);
    return MDAS_OK;
}

int mdas_dump_state(mdas_grid* g, float* coords, float* values, int* nodes, float* boxes, float* errors,
                    uint32_t* seeds) {
    if (!g) return MDAS_ERR_INVALID;
    const MdasDeviceGrid& d = g->dg;
    cudaError_t e = cudaSuccess;
    const size_t N = (size_t)g->N, L = (size_t)g->L;
    auto cp = [&](void* dst, const void* src, size_t bytes) {
        if (dst && bytes && e == cudaSuccess) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, g->stream);
    };
    cp(coords, d.coords, sizeof(float) * N * d.D);
    cp(values, d.values, sizeof(float) * 3 * N);
    cp(errors, d.errors, sizeof(float) * L);
    cp(seeds, d.seeds, sizeof(unsigned) * L);
    // nodes and boxes live inside the leaf records: unpack into a staging buffer
    void* stage = nullptr;
    if ((nodes || boxes) && L && e == cudaSuccess) {
        const size_t nb = sizeof(int4) * L, bb = sizeof(float) * 2 * d.D * L;
        e = cudaMalloc(&stage, nb + bb);
        if (e == cudaSuccess) {
            int* dn = reinterpret_cast<int*>(stage);
            float* db = reinterpret_cast<float*>(reinterpret_cast<char*>(stage) + nb);
            e = g->arith == MDAS_ARITH_IEEE ? mdas_ieee::unpack_records(d, (int)L, dn, db, g->stream)
                                            : mdas_fast::unpack_records(d, (int)L, dn, db, g->stream);
            g->launches += 1;
            cp(nodes, dn, nb);
            cp(boxes, db, bb);
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (stage) cudaFree(stage);
    if (e == cudaSuccess && seeds)
        for (size_t i = 0; i < L; ++i)
            if (seeds[i] == host_tea4((uint32_t)i)) seeds[i] = 0u;  // never drawn: the reference's 0
    return status_of(e);
}

int mdas_load_state(mdas_grid* g, int numberOfSamples, int numberOfNodes, const float* coords, const float* values,
                    const int* nodes, const float* boxes, const float* errors, const uint32_t* seeds) {
    if (!g || numberOfSamples < 0 || numberOfNodes < 0 || numberOfSamples > g->dg.maxSamples ||
        numberOfNodes > g->dg.maxNodes || !coords || !values || !nodes || !boxes || !errors || !seeds)
        return MDAS_ERR_INVALID;
    const MdasDeviceGrid& d = g->dg;
    const size_t N = (size_t)numberOfSamples, L = (size_t)numberOfNodes;
    for (size_t k = 0; k < 4 * L; ++k)
        if (nodes[k] >= (int)N) return MDAS_ERR_INVALID;  // a node names a sample that does not exist
    cudaError_t e = cudaSuccess;
    auto cp = [&](void* dst, const void* src, size_t bytes) {
        if (bytes && e == cudaSuccess) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, g->stream);
    };
    cp(d.coords, coords, sizeof(float) * N * d.D);
    cp(d.values, values, sizeof(float) * 3 * N);
    cp(d.errors, errors, sizeof(float) * L);
    // a never-drawn seed (0) is stored as the seed its first draw starts from
    std::vector<uint32_t> stored(seeds, seeds + L);
    for (size_t i = 0; i < L; ++i)
        if (stored[i] == 0u) stored[i] = host_tea4((uint32_t)i);
    cp(d.seeds, stored.data(), sizeof(unsigned) * L);
    // build the leaf records from the nodes, boxes and (already loaded) coordinates
    void* stage = nullptr;
    if (L && e == cudaSuccess) {
        const size_t nb = sizeof(int4) * L, bb = sizeof(float) * 2 * d.D * L;
        e = cudaMalloc(&stage, nb + bb);
        if (e == cudaSuccess) {
            int* dn = reinterpret_cast<int*>(stage);
            float* db = reinterpret_cast<float*>(reinterpret_cast<char*>(stage) + nb);
            cp(dn, nodes, nb);
            cp(db, boxes, bb);
            if (e == cudaSuccess)
                e = g->arith == MDAS_ARITH_IEEE ? mdas_ieee::pack_records(d, (int)L, dn, db, g->stream)
                                                : mdas_fast::pack_records(d, (int)L, dn, db, g->stream);
            g->launches += 1;
        }
    }
    if (e == cudaSuccess && (size_t)d.maxNodes > L)
        e = cudaMemsetAsync(d.seeds + L, 0, sizeof(unsigned) * ((size_t)d.maxNodes - L), g->stream);
    if (e == cudaSuccess) {
        k_set_counts<<<1, 1, 0, g->stream>>>(d.counts, (int)N, (int)L);
        g->launches += 1;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);  // host buffers may go away after return
    if (stage) cudaFree(stage);
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    g->N = (int)N;
    g->L = (int)L;
    g->version += 1;
    g->newN = 0;
    g->newL = 0;
    g->initialized = true;
    g->errorsClean = false;
    g->dirtyValid = false;
    g->extentsValid = false;
    return MDAS_OK;
}

int mdas_validate(mdas_grid* g, int* valid) {
    if (!g || !valid) return MDAS_ERR_INVALID;
    const int D = g->dg.D;
    const size_t N = (size_t)g->N, L = (size_t)g->L;
    std::vector<float> coords(N * D), boxes(L * 2 * D);
    std::vector<int> nodes(L * 4);
    int rc = mdas_dump_state(g, coords.data(), nullptr, nodes.data(), boxes.data(), nullptr, nullptr);
    if (rc) return rc;
    bool ok = true;
    std::vector<int> hist(N, 0);
    // summed in double: the reference's float sum (kdgrid.cu:858, :903) drifts past its
    // own 1 % tolerance (:910) at a few million leaves
    double totalVolume = 0.0;
    size_t total = 0;
    for (size_t k = 0; k < L; ++k) {
        const float* box = boxes.data() + k * 2 * D;
        float vol = 1.0f;
        for (int i = 0; i < D; ++i) vol *= box[D + i] - box[i];
        totalVolume += vol;
        for (int i = 0; i < 4; ++i) {
            const int s = nodes[k * 4 + i];
            if (s < 0) continue;
            if ((size_t)s >= N) {
                ok = false;
                continue;
            }
            for (int j = 0; j < D; ++j) {
                const float c = coords[(size_t)s * D + j];
                if (c < box[j] || c > box[D + j]) ok = false;
            }
            hist[s]++;
            total++;
        }
    }
    const double rootVolume = (double)(g->dg.scaleX * g->dg.scaleY);
    if (fabs(totalVolume - rootVolume) > 1.0e-2 * rootVolume) ok = false;
    if (total != N) ok = false;
    for (size_t i = 0; i < N; ++i)
        if (hist[i] != 1) ok = false;
    *valid = ok ? 1 : 0;
    return MDAS_OK;
}

int mdas_test_set_wait_limit(int polls) {
    mdas_order::set_test_wait_limit(polls);
    return status_of(mdas_mlp::set_test_wait_limit(polls));
}

int mdas_set_timing(mdas_grid* g, int on) {
    if (!g) return MDAS_ERR_INVALID;
    g->timing = on != 0 || g->log != nullptr;
    return MDAS_OK;
}

int mdas_get_stage_times(mdas_grid* g, double* ms5, int reset) {
    if (!g || !ms5) return MDAS_ERR_INVALID;
    flush_timing(g);
    for (int i = 0; i < 5; ++i) ms5[i] = g->stageMs[i];
    if (reset)
        for (double& x : g->stageMs) x = 0.0;
    return MDAS_OK;
}

int mdas_get_stage_times_ex(mdas_grid* g, double* ms, int n, int reset) {
    if (!g || !ms || n < 0) return MDAS_ERR_INVALID;
    flush_timing(g);
    for (int i = 0; i < n && i < 6; ++i) ms[i] = g->stageMs[i];
    if (reset)
        for (double& x : g->stageMs) x = 0.0;
    return MDAS_OK;
}

int mdas_get_pass_stats(mdas_grid* g, int* recomputed, int* selected, int* splits, int64_t* gathered) {
    if (!g) return MDAS_ERR_INVALID;
    if (recomputed) *recomputed = g->hcounts->recomputedLast;
    if (selected) *selected = g->hcounts->selected;
    if (splits) *splits = g->hcounts->newL;
    if (gathered) *gathered = (int64_t)g->hcounts->gatheredLast;
    return MDAS_OK;
}

int mdas_get_launch_count(mdas_grid* g, uint64_t* launches) {
    if (!g || !launches) return MDAS_ERR_INVALID;
    *launches = g->launches;
    return MDAS_OK;
}

// ---- scenes and the integrand ------------------------------------------------------

int mdas_scene_create(mdas_scene** out, int kind, uint64_t seed, int count, float scaleX, float scaleY, int width,
                      int height) {
    if (!out) return MDAS_ERR_INVALID;
    *out = nullptr;
    mdas_scene* s = new (std::nothrow) mdas_scene();
    if (!s) return MDAS_ERR_ALLOC;
    int rc = mdas_generate_scene(kind, seed, count, scaleX, scaleY, width, height, &s->desc, &s->prims);
    if (rc) {
        delete s;
        return rc;
    }
    *out = s;  // the device copy is made on first use, so scenes can be generated without a GPU
    return MDAS_OK;
}

int mdas_scene_destroy(mdas_scene* s) {
    if (!s) return MDAS_ERR_INVALID;
    if (s->d_prims) cudaFree(s->d_prims);
    if (s->d_cull) cudaFree(s->d_cull);
    delete s;
    return MDAS_OK;
}

int mdas_scene_desc_size(void) { return (int)sizeof(MdasScene); }

int mdas_scene_export(mdas_scene* s, void* desc, int descBytes, float* prims, int maxPrims, int* dim, int* count) {
    if (!s) return MDAS_ERR_INVALID;
    if (desc) {
        if (descBytes < (int)sizeof(MdasScene)) return MDAS_ERR_INVALID;
        memcpy(desc, &s->desc, sizeof(MdasScene));
    }
    if (prims) {
        if (maxPrims < s->desc.count) return MDAS_ERR_INVALID;
        memcpy(prims, s->prims.data(), sizeof(float) * s->prims.size());
    }
    if (dim) *dim = s->desc.dim;
    if (count) *count = s->desc.count;
    return MDAS_OK;
}

int mdas_evaluate(mdas_grid* g, mdas_scene* s, int offset, int count) {
    if (!g || !s || s->desc.dim > g->dg.D) return MDAS_ERR_INVALID;
    if (!g->initialized) return MDAS_ERR_STATE;
    if (count >= 0 && (offset < 0 || (int64_t)offset + count > g->dg.maxSamples)) return MDAS_ERR_INVALID;
    const int grid = count >= 0 ? grid_for(g, MDAS_K_INIT, count) : g->numSMs * 8;
    if (count == 0) return MDAS_OK;
    int rc = scene_upload(s, g->stream);
    if (rc) return rc;
    rc = timed(g, 4, [&]() {
        return mdas_launch_evaluate(s->desc, s->d_prims, s->d_cull, g->dg.coords, g->dg.values, g->dg.D,
                                    count < 0 ? g->dg.counts : nullptr, offset, count, grid, g->stream);
    });
    g->launches += 1;
    return rc;
}

int mdas_scene_evaluate(mdas_scene* s, const float* coords, float* values, int dim, int offset, int count,
                        void* stream) {
    if (!s || !coords || !values || dim < s->desc.dim || dim > 6 || offset < 0 || count < 0)
        return MDAS_ERR_INVALID;
    if (count == 0) return MDAS_OK;
    int rc = scene_upload(s, (cudaStream_t)stream);
    if (rc) return rc;
    int nsm = 1, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = ((int64_t)count + 255) / 256;
    const int grid = (int)(want < (int64_t)nsm * 8 ? want : (int64_t)nsm * 8);
    return status_of(mdas_launch_evaluate(s->desc, s->d_prims, s->d_cull, coords, values, dim, nullptr, offset, count,
                                          grid, (cudaStream_t)stream));
}

int mdas_scene_reference_image(mdas_scene* s, int width, int height, int spp, uint64_t seed, double* out,
                               void* stream) {
    if (!s || !out || width <= 0 || height <= 0 || spp < 1) return MDAS_ERR_INVALID;
    int strata = 1;
    while ((strata + 1) * (strata + 1) <= spp) ++strata;
    if (strata * strata != spp) return MDAS_ERR_INVALID;  // a square number of samples per pixel
    int rc = scene_upload(s, (cudaStream_t)stream);
    if (rc) return rc;
    int nsm = 1, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = ((int64_t)width * height + 255) / 256;
    const int grid = (int)(want < (int64_t)nsm * 16 ? want : (int64_t)nsm * 16);
    return status_of(mdas_launch_reference_image(s->desc, s->d_prims, width, height, strata, seed, out, grid,
                                                 (cudaStream_t)stream));
}

int mdas_render(mdas_grid* g, mdas_scene* s, int budget, float* pixels, int width, int height,
                mdas_render_stats* stats) {
    if (!g || !s || !pixels) return MDAS_ERR_INVALID;
    int rc = mdas_initial_sampling(g);
    if (rc) return rc;
    rc = mdas_evaluate(g, s, 0, g->N);
    if (rc) return rc;
    int passes = 0;
    while (g->N < budget) {
        if ((int64_t)g->N + g->L > g->dg.maxSamples) break;
        rc = mdas_sampling_pass(g);
        if (rc) return rc;
        rc = mdas_evaluate(g, s, g->N - g->newN, g->newN);
        if (rc) return rc;
        passes++;
    }
    rc = mdas_integrate(g, pixels, width, height);
    if (rc) return rc;
    if (stats) {
        stats->numberOfSamples = g->N;
        stats->numberOfNodes = g->L;
        stats->passes = passes;
        stats->reserved = 0;
        mdas_get_stage_times(g, stats->stageMs, 0);
    }
    return MDAS_OK;
}

// ---- the device-side budget loop ----------------------------------------------------
namespace {

constexpr int kMaxGraphPasses = 1 << 20;  // safety stop of the device-side loop

cudaError_t launch_errors_auto(mdas_grid* g, int grid, cudaStream_t s) {
    return g->arith == MDAS_ARITH_IEEE ? mdas_ieee::compute_errors_auto(g->dg, grid, s)
                                       : mdas_fast::compute_errors_auto(g->dg, grid, s);
}

cudaError_t launch_adaptive_on(mdas_grid* g, int gridDecide, int gridPlace, cudaStream_t s) {
    return g->arith == MDAS_ARITH_IEEE ? mdas_ieee::adaptive_sampling(g->dg, gridDecide, gridPlace, s)
                                       : mdas_fast::adaptive_sampling(g->dg, gridDecide, gridPlace, s);
}

// Builds the whole render as one graph: initial sampling, integrand, a
// conditional while node around {errors, adaptive pass, integrand for the new
// samples, loop condition}, integrate.  Every kernel has a fixed persistent
// grid and reads the leaf and sample counts from device memory.
cudaError_t learned_queue(mdas_grid* g, int L, cudaStream_t s);

int build_render_graph(mdas_grid* g, mdas_scene* s, int budget, float* pixels, int width, int height) {
    if (g->graph.exec) {
        cudaGraphExecDestroy(g->graph.exec);
        g->graph.exec = nullptr;
    }
    if (!g->captureStream && cudaStreamCreateWithFlags(&g->captureStream, cudaStreamNonBlocking) != cudaSuccess)
        return MDAS_ERR_CUDA;
    if (!g->bodyStream && cudaStreamCreateWithFlags(&g->bodyStream, cudaStreamNonBlocking) != cudaSuccess)
        return MDAS_ERR_CUDA;
    const MdasDeviceGrid& d = g->dg;
    const int64_t L0 = ((int64_t)1 << (d.bitsPerDim * d.D)) << (2 * d.extraImgBits);
    const int64_t N0 = 4 * L0;
    if (N0 > d.maxSamples) return MDAS_ERR_CAPACITY;
    const unsigned firstPass = (N0 < budget && N0 + L0 <= d.maxSamples) ? 1u : 0u;
    const int gErr = g->numSMs * (g->occ[MDAS_K_ERRORS] > 0 ? g->occ[MDAS_K_ERRORS] : 1);
    const int gDecide = g->numSMs * (g->occ[MDAS_K_DECIDE] > 0 ? g->occ[MDAS_K_DECIDE] : 1);
    const int gPlace = g->numSMs * (g->occ[MDAS_K_ADAPTIVE] > 0 ? g->occ[MDAS_K_ADAPTIVE] : 1);
    const int gInt = g->numSMs * (g->occ[MDAS_K_INTEGRATE] > 0 ? g->occ[MDAS_K_INTEGRATE] : 1);
    const int gEval = g->numSMs * 16;  // integrand CTAs (16 per SM measured 1 % faster per render than 8)
    cudaStream_t cs = g->captureStream, bs = g->bodyStream;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    auto fail = [&](cudaError_t err) {
        cudaGraph_t junk = nullptr;
        cudaStreamEndCapture(cs, &junk);
        if (junk) cudaGraphDestroy(junk);
        cudaGetLastError();
        return err == cudaSuccess ? MDAS_ERR_CUDA : MDAS_ERR_CUDA;
    };
    // prologue: initial sampling + integrand for all initial samples
    e = g->arith == MDAS_ARITH_IEEE ? mdas_ieee::initial_sampling(d, (int)L0, cs)
                                    : mdas_fast::initial_sampling(d, (int)L0, cs);
    if (e != cudaSuccess) return fail(e);
    k_set_counts<<<1, 1, 0, cs>>>(d.counts, (int)N0, (int)L0);
    e = mdas_launch_evaluate(s->desc, s->d_prims, s->d_cull, d.coords, d.values, d.D, nullptr, 0, (int)N0, gEval, cs);
    if (e != cudaSuccess) return fail(e);
    // the conditional while node
    cudaStreamCaptureStatus status;
    cudaGraph_t capGraph = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    e = cudaStreamGetCaptureInfo(cs, &status, nullptr, &capGraph, &deps, nullptr, &ndeps);
    if (e != cudaSuccess) return fail(e);
    cudaGraphConditionalHandle handle;
    e = cudaGraphConditionalHandleCreate(&handle, capGraph, firstPass, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return fail(e);
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t condNode;
    e = cudaGraphAddNode(&condNode, capGraph, deps, nullptr, ndeps, &cp);
    if (e != cudaSuccess) return fail(e);
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    e = cudaStreamUpdateCaptureDependencies(cs, &condNode, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e != cudaSuccess) return fail(e);
    // loop body, captured into the conditional node's child graph
    e = cudaStreamBeginCaptureToGraph(bs, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return fail(e);
    cudaError_t eb = launch_errors_auto(g, gErr, bs);
    if (eb == cudaSuccess && g->learned) {
        eb = learned_queue(g, -1, bs);  // predictions and the judge's verdict for this pass
        g->dg.priority = g->lPred;
    }
    if (eb == cudaSuccess) eb = launch_adaptive_on(g, gDecide, gPlace, bs);
    g->dg.priority = nullptr;
    if (eb == cudaSuccess)
        eb = mdas_launch_evaluate(s->desc, s->d_prims, s->d_cull, d.coords, d.values, d.D, d.counts, 0, 0, gEval, bs);
    if (eb == cudaSuccess)
        eb = g->arith == MDAS_ARITH_IEEE ? mdas_ieee::loop_condition(d, handle, budget, kMaxGraphPasses, bs)
                                         : mdas_fast::loop_condition(d, handle, budget, kMaxGraphPasses, bs);
    cudaGraph_t bodyOut = nullptr;
    e = cudaStreamEndCapture(bs, &bodyOut);
    if (eb != cudaSuccess || e != cudaSuccess) return fail(eb != cudaSuccess ? eb : e);
    // epilogue: reconstruction
    e = g->arith == MDAS_ARITH_IEEE ? mdas_ieee::integrate(d, gInt, pixels, width, height, cs)
                                    : mdas_fast::integrate(d, gInt, pixels, width, height, cs);
    if (e != cudaSuccess) return fail(e);
    e = cudaStreamEndCapture(cs, &graph);
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    e = cudaGraphInstantiate(&g->graph.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        g->graph.exec = nullptr;
        return MDAS_ERR_CUDA;
    }
    g->graph.scene = s;
    g->graph.budget = budget;
    g->graph.pixels = pixels;
    g->graph.width = width;
    g->graph.height = height;
    return MDAS_OK;
}

}  // namespace

namespace {

// The render graph launched and the counter read queued behind it (no wait).
int render_graph_launch(mdas_grid* g, mdas_scene* s, int budget, float* pixels, int width, int height) {
    if (!g || !s || !pixels || width <= 0 || height <= 0 || s->desc.dim > g->dg.D) return MDAS_ERR_INVALID;
    int rc = scene_upload(s, g->stream);
    if (rc) return rc;
    flush_timing(g);
    const RenderGraph& rg = g->graph;
    if (!rg.exec || rg.scene != s || rg.budget != budget || rg.pixels != pixels || rg.width != width ||
        rg.height != height) {
        rc = build_render_graph(g, s, budget, pixels, width, height);
        if (rc) return rc;
    }
    cudaError_t e = cudaGraphLaunch(g->graph.exec, g->stream);
    g->launches += 1;
    if (e == cudaSuccess) e = counts_copy_async(g);
    return e == cudaSuccess ? MDAS_OK : MDAS_ERR_CUDA;
}

// After the stream completed a launched render: the grid's state and the stats.
int render_graph_finish(mdas_grid* g, mdas_render_stats* stats) {
    const int rc = counts_apply(g);
    if (rc) return rc;
    g->initialized = true;
    g->errorsClean = false;
    g->dirtyValid = g->hcounts->passes > 0;
    g->extentsValid = g->dirtyValid && g->dg.featRaw != nullptr;
    if (stats) {
        stats->numberOfSamples = g->N;
        stats->numberOfNodes = g->L;
        stats->passes = g->hcounts->passes;
        stats->reserved = 0;
        for (double& x : stats->stageMs) x = 0.0;
    }
    return MDAS_OK;
}

}  // namespace

int mdas_render_graph(mdas_grid* g, mdas_scene* s, int budget, float* pixels, int width, int height,
                      mdas_render_stats* stats) {
    int rc = render_graph_launch(g, s, budget, pixels, width, height);
    if (rc) return rc;
    if (cudaStreamSynchronize(g->stream) != cudaSuccess) return MDAS_ERR_CUDA;
    return render_graph_finish(g, stats);
}

// ---- batched rendering ------------------------------------------------------------------
struct mdas_batch {
    int n = 0;
    int arith = 0;
    int numSMs = 1;
    std::vector<mdas_grid*> grids;  // caller order
    std::vector<int> order;          // batch slot -> caller index (images grouped by dimension)
    struct Group {
        int D, offset, count;
    };
    std::vector<Group> groups;
    std::vector<MdasBatchImage> himgs;
    std::vector<MdasBatchScene> hscenes;
    MdasBatchImage* d_imgs = nullptr;
    MdasBatchScene* d_scenes = nullptr;
    bool anyActive = false;
    cudaStream_t stream = nullptr, captureStream = nullptr, bodyStream = nullptr;
    cudaGraphExec_t exec = nullptr;
    int tune[4] = {4, 4, 4, 8};  // persistent CTAs per SM: errors, decide, place, integrate/integrand
    int tileK = MDAS_LEAVES_PER_THREAD;  // leaves per thread of decide (tiles of 256 * tileK leaves)
    uint64_t launches = 0;
    bool anyLearned = false;     // some image takes the learned acceptance
    unsigned* status = nullptr;  // bounded waits of the batched learned kernels
};

namespace {

#define MDAS_ARITH_CALL(b, FN, ...) \
    ((b)->arith == MDAS_ARITH_IEEE ? mdas_ieee::FN(__VA_ARGS__) : mdas_fast::FN(__VA_ARGS__))

// The stages of one batched render.  Every stage is one launch per point
// dimension present.  prologue: initial sampling and integrand of every image;
// body: one pass over the still-active images, ending in the loop's verdict
// (into the graph's conditional handle, or into anyOut when the host drives
// the loop); epilogue: reconstruction.
cudaError_t enqueue_batch_prologue(mdas_batch* b, cudaStream_t s) {
    const int gInt = b->numSMs * b->tune[3];
    cudaError_t e = cudaSuccess;
    for (const auto& gr : b->groups)
        if (e == cudaSuccess) e = MDAS_ARITH_CALL(b, batch_init, b->d_imgs + gr.offset, gr.count, gr.D, gInt, s);
    if (e == cudaSuccess) e = MDAS_ARITH_CALL(b, batch_set_counts, b->d_imgs, b->n, s);
    for (const auto& gr : b->groups)
        if (e == cudaSuccess) e = mdas_launch_evaluate_batch(b->d_scenes + gr.offset, gr.count, gr.D, 1, gInt, s);
    return e;
}

cudaError_t enqueue_batch_body(mdas_batch* b, cudaGraphConditionalHandle handle, int* anyOut, cudaStream_t s) {
    const int gErr = b->numSMs * b->tune[0], gDec = b->numSMs * b->tune[1], gPl = b->numSMs * b->tune[2];
    const int gInt = b->numSMs * b->tune[3];
    // (the accumulators of this pass were cleared by the last pass's scan, or
    // when the counters were set)
    cudaError_t e = cudaSuccess;
    for (const auto& gr : b->groups)
        if (e == cudaSuccess) e = MDAS_ARITH_CALL(b, batch_errors, b->d_imgs + gr.offset, gr.count, gr.D, gErr, s);
    if (e == cudaSuccess && b->anyLearned) {
        // learned images: priorities of the leaves whose error was recomputed, then the judge
        e = MDAS_ARITH_CALL(b, batch_reset, b->d_imgs, b->n, 2, s);
        for (const auto& gr : b->groups)
            if (e == cudaSuccess) e = mdas_mlp::batch_predict(b->d_imgs + gr.offset, gr.count, gr.D, b->status, s);
        if (e == cudaSuccess) e = MDAS_ARITH_CALL(b, batch_learned_judge, b->d_imgs, b->n, b->numSMs * 4, s);
    }
    for (const auto& gr : b->groups)
        if (e == cudaSuccess)
            e = MDAS_ARITH_CALL(b, batch_decide, b->d_imgs + gr.offset, gr.count, gr.D, b->tileK, b->anyLearned, gDec,
                                s);
    if (e == cudaSuccess) e = MDAS_ARITH_CALL(b, batch_scan, b->d_imgs, b->n, s);
    for (const auto& gr : b->groups)
        if (e == cudaSuccess) e = MDAS_ARITH_CALL(b, batch_place, b->d_imgs + gr.offset, gr.count, gr.D, gPl, s);
    for (const auto& gr : b->groups)
        if (e == cudaSuccess) e = mdas_launch_evaluate_batch(b->d_scenes + gr.offset, gr.count, gr.D, 0, gInt, s);
    if (e == cudaSuccess) e = MDAS_ARITH_CALL(b, batch_condition, b->d_imgs, b->n, handle, kMaxGraphPasses, anyOut, s);
    return e;
}

cudaError_t enqueue_batch_epilogue(mdas_batch* b, cudaStream_t s) {
    const int gInt = b->numSMs * b->tune[3];
    cudaError_t e = MDAS_ARITH_CALL(b, batch_clear_pixels, b->d_imgs, b->n, s);
    for (const auto& gr : b->groups)
        if (e == cudaSuccess) e = MDAS_ARITH_CALL(b, batch_integrate, b->d_imgs + gr.offset, gr.count, gr.D, gInt, s);
    return e;
}

// Graph of one batched render: the prologue, a device-side loop (a conditional
// WHILE node) over the body, the epilogue.
int build_batch_graph(mdas_batch* b) {
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    cudaStream_t cs = b->captureStream, bs = b->bodyStream;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    auto fail = [&]() {
        cudaGraph_t junk = nullptr;
        cudaStreamEndCapture(cs, &junk);
        if (junk) cudaGraphDestroy(junk);
        cudaGetLastError();
        return MDAS_ERR_CUDA;
    };
    if (enqueue_batch_prologue(b, cs) != cudaSuccess) return fail();
    cudaStreamCaptureStatus status;
    cudaGraph_t capGraph = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    if (cudaStreamGetCaptureInfo(cs, &status, nullptr, &capGraph, &deps, nullptr, &ndeps) != cudaSuccess) return fail();
    cudaGraphConditionalHandle handle;
    if (cudaGraphConditionalHandleCreate(&handle, capGraph, b->anyActive ? 1u : 0u, cudaGraphCondAssignDefault) !=
        cudaSuccess)
        return fail();
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t condNode;
    if (cudaGraphAddNode(&condNode, capGraph, deps, nullptr, ndeps, &cp) != cudaSuccess) return fail();
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    if (cudaStreamUpdateCaptureDependencies(cs, &condNode, nullptr, 1, cudaStreamSetCaptureDependencies) != cudaSuccess)
        return fail();
    if (cudaStreamBeginCaptureToGraph(bs, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) != cudaSuccess)
        return fail();
    const cudaError_t eb = enqueue_batch_body(b, handle, nullptr, bs);
    cudaGraph_t bodyOut = nullptr;
    e = cudaStreamEndCapture(bs, &bodyOut);
    if (eb != cudaSuccess || e != cudaSuccess) return fail();
    if (enqueue_batch_epilogue(b, cs) != cudaSuccess) return fail();
    cudaGraph_t graph = nullptr;
    if (cudaStreamEndCapture(cs, &graph) != cudaSuccess) return MDAS_ERR_CUDA;
    e = cudaGraphInstantiate(&b->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        b->exec = nullptr;
        return MDAS_ERR_CUDA;
    }
    return MDAS_OK;
}

void free_batch(mdas_batch* b) {
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->captureStream) cudaStreamDestroy(b->captureStream);
    if (b->bodyStream) cudaStreamDestroy(b->bodyStream);
    cudaFree(b->d_imgs);
    cudaFree(b->d_scenes);
    cudaFree(b->status);
    delete b;
}

}  // namespace

int mdas_batch_create(mdas_batch** out, int n, mdas_grid* const* grids, mdas_scene* const* scenes,
                      const int* budgets, float* const* pixels, const int* widths, const int* heights) {
    if (!out || n < 1 || n > 256 || !grids || !scenes || !budgets || !pixels || !widths || !heights)
        return MDAS_ERR_INVALID;
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        if (!grids[i] || !scenes[i] || !pixels[i] || widths[i] <= 0 || heights[i] <= 0 ||
            scenes[i]->desc.dim > grids[i]->dg.D || grids[i]->arith != grids[0]->arith ||
            grids[i]->device != grids[0]->device)
            return MDAS_ERR_INVALID;
        for (int j = 0; j < i; ++j)
            if (grids[j] == grids[i]) return MDAS_ERR_INVALID;  // one image per grid
    }
    mdas_batch* b = new (std::nothrow) mdas_batch();
    if (!b) return MDAS_ERR_ALLOC;
    b->n = n;
    b->arith = grids[0]->arith;
    b->numSMs = grids[0]->numSMs;
    b->stream = grids[0]->stream;
    b->grids.assign(grids, grids + n);
    for (int D = 3; D <= 6; ++D) {
        const int off = (int)b->order.size();
        for (int i = 0; i < n; ++i)
            if (grids[i]->dg.D == D) b->order.push_back(i);
        if ((int)b->order.size() > off) b->groups.push_back({D, off, (int)b->order.size() - off});
    }
    for (int slot = 0; slot < n; ++slot) {
        const int i = b->order[slot];
        mdas_grid* g = grids[i];
        int rc = scene_upload(scenes[i], g->stream);
        if (rc) {
            free_batch(b);
            return rc;
        }
        MdasBatchImage im{};
        im.g = g->dg;
        im.g.priority = g->learned ? g->lPred : nullptr;  // learned images keep their weights and statistics
        im.g.featRaw = g->learned ? g->lRaw : nullptr;    // raw feature rows of the batched errors pass
        im.g.learned = g->learned ? g->lStats : nullptr;
        im.mlp = g->learned ? g->lPacked : nullptr;
        if (g->learned) b->anyLearned = true;
        im.pixels = reinterpret_cast<float4*>(pixels[i]);
        im.width = widths[i];
        im.height = heights[i];
        im.budget = budgets[i];
        const int64_t L0 = ((int64_t)1 << (g->dg.bitsPerDim * g->dg.D)) << (2 * g->dg.extraImgBits);
        if (4 * L0 > g->dg.maxSamples) {
            free_batch(b);
            return MDAS_ERR_CAPACITY;
        }
        im.initialLeaves = (int)L0;
        im.jumpA = (b->arith == MDAS_ARITH_IEEE) ? mdas_ieee::batch_jump(g->dg.candidatesNum, g->dg.D, &im.jumpC)
                                                 : mdas_fast::batch_jump(g->dg.candidatesNum, g->dg.D, &im.jumpC);
        if (4 * L0 < budgets[i] && 5 * L0 <= g->dg.maxSamples) b->anyActive = true;
        b->himgs.push_back(im);
        MdasBatchScene bs{};
        bs.sc = scenes[i]->desc;
        bs.prims = scenes[i]->d_prims;
        bs.cull = scenes[i]->d_cull;
        bs.counts = g->dg.counts;
        bs.coords = g->dg.coords;
        bs.values = g->dg.values;
        bs.dim = g->dg.D;
        bs.initialSamples = (int)(4 * L0);
        b->hscenes.push_back(bs);
    }
    bool ok = cudaMalloc(&b->d_imgs, sizeof(MdasBatchImage) * n) == cudaSuccess &&
              cudaMalloc(&b->d_scenes, sizeof(MdasBatchScene) * n) == cudaSuccess &&
              cudaMemcpy(b->d_imgs, b->himgs.data(), sizeof(MdasBatchImage) * n, cudaMemcpyHostToDevice) ==
                  cudaSuccess &&
              cudaMemcpy(b->d_scenes, b->hscenes.data(), sizeof(MdasBatchScene) * n, cudaMemcpyHostToDevice) ==
                  cudaSuccess &&
              cudaMalloc(&b->status, sizeof(unsigned)) == cudaSuccess &&
              cudaMemset(b->status, 0, sizeof(unsigned)) == cudaSuccess &&
              cudaStreamCreateWithFlags(&b->captureStream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&b->bodyStream, cudaStreamNonBlocking) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        free_batch(b);
        return MDAS_ERR_ALLOC;
    }
    int rc = build_batch_graph(b);
    if (rc) {
        free_batch(b);
        return rc;
    }
    *out = b;
    return MDAS_OK;
}

int mdas_batch_destroy(mdas_batch* b) {
    if (!b) return MDAS_ERR_INVALID;
    cudaStreamSynchronize(b->stream);
    free_batch(b);
    return MDAS_OK;
}

namespace {
// After a batched render: the status, every grid's counts and the stats.
int batch_finish(mdas_batch* b, mdas_render_stats* stats) {
    int status = MDAS_OK;
    if (b->anyLearned) {
        unsigned st = 0;
        if (cudaMemcpy(&st, b->status, sizeof(st), cudaMemcpyDeviceToHost) != cudaSuccess) return MDAS_ERR_CUDA;
        if (st) status = MDAS_ERR_TIMEOUT;
    }
    for (int i = 0; i < b->n; ++i) {
        mdas_grid* g = b->grids[i];
        const int rc = read_counts(g);
        if (rc && !status) status = rc;
        g->initialized = true;
        g->errorsClean = false;
        g->dirtyValid = g->hcounts->passes > 0;
        g->extentsValid = g->dirtyValid && g->dg.featRaw != nullptr;
        if (stats) {
            stats[i].numberOfSamples = g->N;
            stats[i].numberOfNodes = g->L;
            stats[i].passes = g->hcounts->passes;
            stats[i].reserved = 0;
            for (double& x : stats[i].stageMs) x = 0.0;
        }
    }
    return status;
}
}  // namespace

int mdas_batch_render(mdas_batch* b, mdas_render_stats* stats) {
    if (!b || !b->exec) return MDAS_ERR_INVALID;
    cudaError_t e = cudaGraphLaunch(b->exec, b->stream);
    b->launches += 1;
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return MDAS_ERR_CUDA;
    return batch_finish(b, stats);
}

int mdas_batch_render_stepped(mdas_batch* b, mdas_render_stats* stats) {
    if (!b || !b->exec) return MDAS_ERR_INVALID;
    int* any = nullptr;  // the loop's verdict, read by the host after every pass
    if (cudaMallocHost(&any, sizeof(int)) != cudaSuccess) return MDAS_ERR_ALLOC;
    int* dAny = nullptr;
    cudaError_t e = cudaMalloc(&dAny, sizeof(int));
    if (e == cudaSuccess) e = enqueue_batch_prologue(b, b->stream);
    bool more = b->anyActive;
    for (int pass = 0; e == cudaSuccess && more && pass < kMaxGraphPasses; ++pass) {
        e = enqueue_batch_body(b, cudaGraphConditionalHandle{}, dAny, b->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(any, dAny, sizeof(int), cudaMemcpyDeviceToHost, b->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
        more = *any != 0;
    }
    if (e == cudaSuccess) e = enqueue_batch_epilogue(b, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    cudaFree(dAny);
    cudaFreeHost(any);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return MDAS_ERR_CUDA;
    }
    return batch_finish(b, stats);
}

int mdas_batch_set_tiling(mdas_batch* b, const int* ctasPerSm4, int leavesPerTile) {
    if (!b || !ctasPerSm4 || (leavesPerTile != 1024 && leavesPerTile != 2048)) return MDAS_ERR_INVALID;
    for (int k = 0; k < 4; ++k)
        if (ctasPerSm4[k] < 1 || ctasPerSm4[k] > 32) return MDAS_ERR_INVALID;
    for (int k = 0; k < 4; ++k) b->tune[k] = ctasPerSm4[k];
    const int K = leavesPerTile / 256;
    if (K != b->tileK) {
        // every image's decide tiles (the grid's own passes keep theirs)
        b->tileK = K;
        for (auto& im : b->himgs) im.g.tileK = K;
        if (cudaMemcpy(b->d_imgs, b->himgs.data(), sizeof(MdasBatchImage) * b->himgs.size(), cudaMemcpyHostToDevice) !=
            cudaSuccess)
            return MDAS_ERR_CUDA;
    }
    return build_batch_graph(b);
}

int mdas_batch_set_tuning(mdas_batch* b, const int* ctasPerSm4) {
    if (!b) return MDAS_ERR_INVALID;
    return mdas_batch_set_tiling(b, ctasPerSm4, 256 * b->tileK);
}

namespace {
// one render of the batch's graph after a warm one, `repeats` times: ms per render
int batch_time(mdas_batch* b, int repeats, cudaEvent_t e0, cudaEvent_t e1, double* ms) {
    if (cudaGraphLaunch(b->exec, b->stream) != cudaSuccess) return MDAS_ERR_CUDA;  // warm
    cudaEventRecord(e0, b->stream);
    for (int r = 0; r < repeats; ++r) cudaGraphLaunch(b->exec, b->stream);
    cudaEventRecord(e1, b->stream);
    if (cudaEventSynchronize(e1) != cudaSuccess) return MDAS_ERR_CUDA;
    float t = 0.0f;
    cudaEventElapsedTime(&t, e0, e1);
    b->launches += repeats + 1;
    *ms = t / repeats;
    return MDAS_OK;
}
}  // namespace

int mdas_batch_autotune_ex(mdas_batch* b, int repeats, int* best4, int* bestLeavesPerTile, double* bestMs,
                           int* evaluated) {
    if (!b || repeats < 1) return MDAS_ERR_INVALID;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return MDAS_ERR_CUDA;
    // coordinate descent from the default: the decide tile size, then each stage's
    // persistent grid (CTAs per SM) in turn, keeping every improvement
    int cur[4] = {4, 4, 4, 8}, curTile = MDAS_TILE_LEAVES;
    double best = 1e30;
    int evals = 0, rc = MDAS_OK;
    auto eval = [&](const int* t4, int tile, double* ms) {
        int r = mdas_batch_set_tiling(b, t4, tile);
        if (!r) r = batch_time(b, repeats, e0, e1, ms);
        ++evals;
        return r;
    };
    for (int tile : {MDAS_TILE_LEAVES, MDAS_TILE_LEAVES_MIN}) {
        double ms = 0.0;
        if ((rc = eval(cur, tile, &ms))) break;
        if (ms < best) {
            best = ms;
            curTile = tile;
        }
    }
    static const int choices[4][3] = {{2, 4, 8}, {2, 4, 8}, {2, 4, 6}, {4, 8, 16}};
    for (int k = 0; k < 4 && !rc; ++k) {
        for (int v : choices[k]) {
            if (v == cur[k]) continue;
            int t4[4] = {cur[0], cur[1], cur[2], cur[3]};
            t4[k] = v;
            double ms = 0.0;
            if ((rc = eval(t4, curTile, &ms))) break;
            if (ms < best) {
                best = ms;
                cur[k] = v;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    rc = mdas_batch_set_tiling(b, cur, curTile);
    if (best4)
        for (int k = 0; k < 4; ++k) best4[k] = cur[k];
    if (bestLeavesPerTile) *bestLeavesPerTile = curTile;
    if (bestMs) *bestMs = best;
    if (evaluated) *evaluated = evals;
    return rc;
}

int mdas_batch_autotune(mdas_batch* b, int repeats, int* best4, double* bestMs) {
    return mdas_batch_autotune_ex(b, repeats, best4, nullptr, bestMs, nullptr);
}

int mdas_render_host(mdas_grid* g, mdas_scene* s, const float* hostPrims, int budget, float* hostPixels, int width,
                     int height, mdas_render_stats* stats) {
    if (!g || !s || !hostPixels || width <= 0 || height <= 0) return MDAS_ERR_INVALID;
    const size_t bytes = sizeof(float) * 4 * (size_t)width * height;
    int rc = ensure_scratch(g, bytes);
    if (rc) return rc;
    rc = scene_upload(s, g->stream);
    if (rc) return rc;
    if (hostPrims && s->desc.count > 0) {
        cudaError_t e = cudaMemcpyAsync(s->d_prims, hostPrims, sizeof(float) * MDAS_PRIM_STRIDE * s->desc.count,
                                        cudaMemcpyHostToDevice, g->stream);
        if (e == cudaSuccess) e = mdas_launch_build_cull(s->desc, s->d_prims, s->d_cull, g->stream);  // new primitives
        if (e != cudaSuccess) return MDAS_ERR_CUDA;
    }
    // the image copy queued behind the render and its counter read: one wait
    rc = render_graph_launch(g, s, budget, g->scratch, width, height);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(hostPixels, g->scratch, bytes, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    return render_graph_finish(g, stats);
}

// ---- Morton keys, radix sort, leaf order, hierarchy, point location

int mdas_morton_key_bits(int dim, int bitsPerDim, int extraImgBits, int fineBits) {
    return mdas_order::key_bits(dim, bitsPerDim, extraImgBits, fineBits);
}

int mdas_morton_encode(int dim, int bitsPerDim, int extraImgBits, int fineBits, float scaleX, float scaleY,
                       const float* points, int n, uint64_t* keys, void* stream) {
    if (dim < 1 || n < 0 || (n > 0 && (!points || !keys)) || !(scaleX > 0.0f) || !(scaleY > 0.0f) ||
        mdas_order::key_bits(dim, bitsPerDim, extraImgBits, fineBits) < 0)
        return MDAS_ERR_INVALID;
    return status_of(mdas_order::morton_encode(points, n, dim, bitsPerDim, extraImgBits, fineBits, scaleX, scaleY,
                                               keys, static_cast<cudaStream_t>(stream)));
}

int mdas_morton_decode(int dim, int bitsPerDim, int extraImgBits, float scaleX, float scaleY, const uint64_t* cells,
                       int n, float* boxes, void* stream) {
    if (dim < 1 || n < 0 || (n > 0 && (!cells || !boxes)) || mdas_order::key_bits(dim, bitsPerDim, extraImgBits, 0) < 0 ||
        bitsPerDim + extraImgBits > 31)
        return MDAS_ERR_INVALID;
    return status_of(mdas_order::morton_decode(cells, n, dim, bitsPerDim, extraImgBits, scaleX, scaleY, boxes,
                                               static_cast<cudaStream_t>(stream)));
}

int mdas_radix_sort_pairs(void* temp, size_t* tempBytes, const uint64_t* keysIn, uint64_t* keysOut,
                          const uint32_t* valuesIn, uint32_t* valuesOut, int n, int beginBit, int endBit,
                          void* stream) {
    if (!tempBytes || n < 0 || beginBit < 0 || endBit > 64 || beginBit > endBit) return MDAS_ERR_INVALID;
    const size_t need = mdas_order::sort_temp_bytes(n, beginBit, endBit);
    if (!temp) {
        *tempBytes = need;
        return MDAS_OK;
    }
    if (*tempBytes < need || (n > 0 && (!keysIn || !keysOut || !valuesOut)) || (n > 0 && keysIn == keysOut))
        return MDAS_ERR_INVALID;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned* status = nullptr;
    cudaError_t e = mdas_order::radix_sort(temp, *tempBytes, keysIn, keysOut, valuesIn, valuesOut, n, beginBit, endBit,
                                           s, &status);
    unsigned h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, status, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    return h ? MDAS_ERR_TIMEOUT : MDAS_OK;
}

}  // extern "C"

namespace {

int ensure_hierarchy(mdas_grid* g, int n) {
    if (g->hierCap >= n && g->hKeys) return MDAS_OK;
    const int cap = n > 1 ? n : 1;
    cudaFree(g->hKeys);
    cudaFree(g->hSorted);
    cudaFree(g->hOrder);
    cudaFree(g->hChildren);
    cudaFree(g->hParents);
    cudaFree(g->hBoxes);
    cudaFree(g->hVisits);
    cudaFree(g->sortTemp);
    g->hKeys = g->hSorted = nullptr;
    g->hOrder = nullptr;
    g->hChildren = nullptr;
    g->hParents = nullptr;
    g->hBoxes = nullptr;
    g->hVisits = nullptr;
    g->sortTemp = nullptr;
    g->hierCap = 0;
    g->hierVersion = ~0ull;
    const size_t c = (size_t)cap;
    g->sortTempBytes = mdas_order::sort_temp_bytes(cap, 0, 64);
    const bool ok = cudaMalloc(&g->hKeys, sizeof(uint64_t) * c) == cudaSuccess &&
                    cudaMalloc(&g->hSorted, sizeof(uint64_t) * c) == cudaSuccess &&
                    cudaMalloc(&g->hOrder, sizeof(uint32_t) * c) == cudaSuccess &&
                    cudaMalloc(&g->hChildren, sizeof(int2) * c) == cudaSuccess &&
                    cudaMalloc(&g->hParents, sizeof(int) * 2 * c) == cudaSuccess &&
                    cudaMalloc(&g->hBoxes, sizeof(float) * 2 * g->dg.D * c) == cudaSuccess &&
                    cudaMalloc(&g->hVisits, sizeof(unsigned) * (c + 1)) == cudaSuccess &&
                    cudaMalloc(&g->sortTemp, g->sortTempBytes) == cudaSuccess;
    if (!ok) return MDAS_ERR_ALLOC;
    g->hierCap = cap;
    return MDAS_OK;
}

// Point locations of at least this many queries order them by a coarse key first.
constexpr int kLocateSortMin = 1 << 16;

// Scratch of a point location over n >= kLocateSortMin queries.
int ensure_query_scratch(mdas_grid* g, int n) {
    if (g->qCap >= n && g->qKeys) return MDAS_OK;
    cudaFree(g->qKeys);
    cudaFree(g->qPerm);
    cudaFree(g->qTemp);
    g->qKeys = nullptr;
    g->qPerm = nullptr;
    g->qTemp = nullptr;
    g->qCap = 0;
    const size_t c = (size_t)n;
    g->qTempBytes = mdas_order::sort_temp_bytes(n, 0, 64);
    const bool ok = cudaMalloc(&g->qKeys, sizeof(uint64_t) * 2 * c) == cudaSuccess &&
                    cudaMalloc(&g->qPerm, sizeof(uint32_t) * c) == cudaSuccess &&
                    cudaMalloc(&g->qTemp, g->qTempBytes) == cudaSuccess;
    if (!ok) return MDAS_ERR_ALLOC;
    g->qCap = n;
    return MDAS_OK;
}

// Leaf keys and their order (sorted keys in hSorted, slots in hOrder).
int order_leaves(mdas_grid* g, int fineBits) {
    if (!g->initialized) return MDAS_ERR_STATE;
    const MdasDeviceGrid& d = g->dg;
    if (fineBits < 0) fineBits = mdas_order::max_fine_bits(d.D, d.bitsPerDim, d.extraImgBits);
    const int bits = mdas_order::key_bits(d.D, d.bitsPerDim, d.extraImgBits, fineBits);
    if (bits < 0) return MDAS_ERR_INVALID;
    int rc = ensure_hierarchy(g, g->L);
    if (rc) return rc;
    cudaError_t e = mdas_order::leaf_keys(d, g->L, fineBits, g->hKeys, g->stream);
    unsigned* status = nullptr;
    if (e == cudaSuccess)
        e = mdas_order::radix_sort(g->sortTemp, g->sortTempBytes, g->hKeys, g->hSorted, nullptr, g->hOrder, g->L, 0,
                                   bits, g->stream, &status);
    g->launches += 1 + mdas_order::sort_launches(g->L, 0, bits);
    unsigned h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, status, sizeof(unsigned), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    if (h) return MDAS_ERR_TIMEOUT;
    g->hierFineBits = fineBits;
    g->hierN = g->L;
    return MDAS_OK;
}

}  // namespace

extern "C" {

int mdas_leaf_order(mdas_grid* g, int fineBits, uint64_t* keys, uint32_t* order) {
    if (!g) return MDAS_ERR_INVALID;
    g->hierVersion = ~0ull;  // the hierarchy buffers are reused
    int rc = order_leaves(g, fineBits);
    if (rc) return rc;
    cudaError_t e = cudaSuccess;
    if (keys && g->L) e = cudaMemcpyAsync(keys, g->hSorted, sizeof(uint64_t) * g->L, cudaMemcpyDeviceToDevice, g->stream);
    if (order && g->L && e == cudaSuccess)
        e = cudaMemcpyAsync(order, g->hOrder, sizeof(uint32_t) * g->L, cudaMemcpyDeviceToDevice, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    return status_of(e);
}

int mdas_build_hierarchy(mdas_grid* g, int fineBits) {
    if (!g) return MDAS_ERR_INVALID;
    g->hierVersion = ~0ull;
    int rc = order_leaves(g, fineBits);
    if (rc) return rc;
    const int n = g->L;
    cudaError_t e = mdas_order::karras_build(g->hSorted, n, g->hChildren, g->hParents, g->stream);
    if (e == cudaSuccess)
        e = mdas_order::karras_refit(g->dg, g->hOrder, n, g->hChildren, g->hParents, g->hVisits, g->hBoxes, g->stream);
    g->launches += 2;
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    g->hierVersion = g->version;
    return MDAS_OK;
}

int mdas_get_hierarchy(mdas_grid* g, int* numLeaves, uint64_t* keys, uint32_t* order, int* children, int* parents,
                       float* boxes) {
    if (!g) return MDAS_ERR_INVALID;
    if (g->hierVersion != g->version) return MDAS_ERR_STATE;
    const size_t n = (size_t)g->hierN;
    if (numLeaves) *numLeaves = (int)n;
    cudaError_t e = cudaSuccess;
    auto cp = [&](void* dst, const void* src, size_t bytes) {
        if (dst && bytes && e == cudaSuccess) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, g->stream);
    };
    cp(keys, g->hSorted, sizeof(uint64_t) * n);
    cp(order, g->hOrder, sizeof(uint32_t) * n);
    if (n > 1) {
        cp(children, g->hChildren, sizeof(int2) * (n - 1));
        cp(boxes, g->hBoxes, sizeof(float) * 2 * g->dg.D * (n - 1));
    }
    cp(parents, g->hParents, sizeof(int) * (2 * n - 1));
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    return status_of(e);
}

int mdas_locate(mdas_grid* g, const float* points, int n, int* leaves) {
    if (!g || n < 0 || (n > 0 && (!points || !leaves))) return MDAS_ERR_INVALID;
    if (g->hierVersion != g->version) return MDAS_ERR_STATE;
    unsigned* status = g->hVisits + g->hierCap;
    cudaError_t e = cudaMemsetAsync(status, 0, sizeof(unsigned), g->stream);
    // Many queries: threads take them in the order of a coarse Morton key, so
    // that the points of a warp lie close together and walk the same nodes.
    const uint32_t* perm = nullptr;
    unsigned* sortStatus = nullptr;
    if (e == cudaSuccess && n >= kLocateSortMin) {
        const int rc = ensure_query_scratch(g, n);
        if (rc) return rc;
        const MdasDeviceGrid& d = g->dg;
        const int fine = mdas_order::query_fine_bits(d.D, d.bitsPerDim, d.extraImgBits);
        const int bits = mdas_order::key_bits(d.D, d.bitsPerDim, d.extraImgBits, fine);
        e = mdas_order::morton_encode(points, n, d.D, d.bitsPerDim, d.extraImgBits, fine, d.scaleX, d.scaleY,
                                      g->qKeys, g->stream);
        if (e == cudaSuccess)
            e = mdas_order::radix_sort(g->qTemp, g->qTempBytes, g->qKeys, g->qKeys + g->qCap, nullptr, g->qPerm, n, 0,
                                       bits, g->stream, &sortStatus);
        g->launches += 1 + mdas_order::sort_launches(n, 0, bits);
        perm = g->qPerm;
    }
    if (e == cudaSuccess)
        e = mdas_order::locate(g->dg, g->hOrder, g->hierN, g->hChildren, g->hBoxes, points, n, perm, leaves, status,
                               g->stream);
    g->launches += 1;
    unsigned h[2] = {0u, 0u};
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h[0], status, sizeof(unsigned), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess && sortStatus)
        e = cudaMemcpyAsync(&h[1], sortStatus, sizeof(unsigned), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    if (h[1]) return MDAS_ERR_TIMEOUT;
    return h[0] ? MDAS_ERR_CAPACITY : MDAS_OK;
}


// ---- learned acceptance: the tcgen05 MLP

int mdas_learned_defaults(mdas_learned_config* cfg) {
    if (!cfg) return MDAS_ERR_INVALID;
    cfg->tolerance = 0.05f;
    cfg->seed = 1;
    cfg->params = nullptr;
    return MDAS_OK;
}

}  // extern "C"

namespace {

uint64_t splitmix(uint64_t& x) {
    uint64_t z = (x += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) for every weight and bias of a layer.
void mlp_init(std::vector<float>& p, uint64_t seed) {
    p.assign(MDAS_MLP_PARAMS, 0.0f);
    uint64_t st = seed;
    auto fill = [&](int off, int n, int fanIn) {
        const float b = 1.0f / sqrtf((float)fanIn);
        for (int i = 0; i < n; ++i) {
            const double u = (double)(splitmix(st) >> 11) * (1.0 / 9007199254740992.0);
            p[off + i] = (float)((2.0 * u - 1.0) * b);
        }
    };
    fill(MDAS_MLP_OFF_W1, MDAS_MLP_HIDDEN * MDAS_MLP_IN, MDAS_MLP_IN);
    fill(MDAS_MLP_OFF_B1, MDAS_MLP_HIDDEN, MDAS_MLP_IN);
    fill(MDAS_MLP_OFF_W2, MDAS_MLP_HIDDEN * MDAS_MLP_HIDDEN, MDAS_MLP_HIDDEN);
    fill(MDAS_MLP_OFF_B2, MDAS_MLP_HIDDEN, MDAS_MLP_HIDDEN);
    fill(MDAS_MLP_OFF_W3, MDAS_MLP_HIDDEN, MDAS_MLP_HIDDEN);
    fill(MDAS_MLP_OFF_B3, 1, MDAS_MLP_HIDDEN);
}

unsigned* learned_status(mdas_grid* g) { return reinterpret_cast<unsigned*>(g->lState + MDAS_MLP_PARAMS); }

int learned_upload(mdas_grid* g, const float* hostParams) {
    cudaError_t e = cudaMemcpyAsync(g->lState, hostParams, sizeof(float) * MDAS_MLP_PARAMS, cudaMemcpyHostToDevice,
                                    g->stream);
    if (e == cudaSuccess) e = mdas_mlp::pack(g->lState, g->lPacked, g->stream);
    g->launches += 1;
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    g->lPredVersion = ~0ull;
    return status_of(e);
}

// Queues the per-pass learned work on stream s: clear the pass's statistics,
// predict every leaf (L < 0: the device leaf count), judge both schedules.
cudaError_t learned_queue(mdas_grid* g, int L, cudaStream_t s) {
    MdasLearnedStats* st = g->lStats;
    cudaError_t e = cudaMemsetAsync(st, 0, offsetof(MdasLearnedStats, plainPasses), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(&st->unrefinedLearned, 0, 2 * sizeof(double), s);
    // refresh the leaves whose error was recomputed (every leaf when the last
    // errors pass was a full one or the predictions are not from the previous
    // pass), then the exact maximum
    const int mode = L < 0 ? 2
                           : (g->lastErrorsDirty && g->lPredVersion + 1 == g->version ? (g->rawValid ? 3 : 1) : 0);
    if (e == cudaSuccess)
        e = mdas_mlp::predict_leaves(g->dg, L, mode, g->lPacked, g->lPred, &st->predMax, learned_status(g), s);
    MdasDeviceGrid dg = g->dg;
    dg.priority = g->lPred;
    const int grid = g->numSMs * 4;
    if (e == cudaSuccess)
        e = g->arith == MDAS_ARITH_IEEE ? mdas_ieee::learned_judge(dg, L, grid, s)
                                        : mdas_fast::learned_judge(dg, L, grid, s);
    g->launches += 2;
    return e;
}

}  // namespace

extern "C" {

int mdas_learned_enable(mdas_grid* g, const mdas_learned_config* cfg) {
    if (!g) return MDAS_ERR_INVALID;
    if (g->graph.exec) cudaGraphExecDestroy(g->graph.exec);  // a cached device-side render was built for the other mode
    g->graph = RenderGraph{};
    if (!cfg) {
        g->learned = false;
        g->lPredVersion = ~0ull;
        g->dg.priority = nullptr;
        g->dg.learned = nullptr;
        g->dg.featRaw = nullptr;
        g->rawValid = false;
        g->extentsValid = false;
        return MDAS_OK;
    }
    if (!(cfg->tolerance >= 0.0f)) return MDAS_ERR_INVALID;
    if (!g->lState) {
        const bool ok = cudaMalloc(&g->lState, sizeof(float) * (MDAS_MLP_PARAMS + 1)) == cudaSuccess &&
                        cudaMalloc(&g->lPacked, sizeof(mdas_mlp::Packed)) == cudaSuccess &&
                        cudaMalloc(&g->lPred, sizeof(float) * (size_t)g->dg.maxNodes) == cudaSuccess &&
                        cudaMalloc(&g->lRaw, sizeof(float) * MDAS_RAW_FLOATS * (size_t)g->dg.maxNodes) == cudaSuccess &&
                        cudaMalloc(&g->lStats, sizeof(MdasLearnedStats)) == cudaSuccess;
        if (!ok) return MDAS_ERR_ALLOC;
    }
    MdasLearnedStats h{};
    h.tolerance = cfg->tolerance;
    cudaError_t e = cudaMemcpyAsync(g->lStats, &h, sizeof(h), cudaMemcpyHostToDevice, g->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(learned_status(g), 0, sizeof(unsigned), g->stream);
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    std::vector<float> p;
    if (cfg->params) p.assign(cfg->params, cfg->params + MDAS_MLP_PARAMS);
    else mlp_init(p, cfg->seed);
    const int rc = learned_upload(g, p.data());
    if (rc) return rc;
    g->dg.priorityScale = MDAS_MLP_TARGET_SCALE;
    g->dg.learned = g->lStats;
    g->dg.featRaw = g->lRaw;
    g->rawValid = false;
    g->extentsValid = false;
    g->learned = true;
    return MDAS_OK;
}

int mdas_learned_update(mdas_grid* g) {
    if (!g || !g->learned) return MDAS_ERR_INVALID;
    if (!g->initialized || !g->errorsClean) return MDAS_ERR_STATE;  // needs current leaf errors
    cudaError_t e = learned_queue(g, g->L, g->stream);
    unsigned st = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&st, learned_status(g), sizeof(st), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    if (st) return MDAS_ERR_TIMEOUT;
    g->lPredVersion = g->version;
    return MDAS_OK;
}

int mdas_learned_predict(mdas_grid* g) {
    if (!g || !g->learned) return MDAS_ERR_INVALID;
    if (!g->initialized) return MDAS_ERR_STATE;
    cudaError_t e = mdas_mlp::predict_leaves(g->dg, g->L, 0, g->lPacked, g->lPred, &g->lStats->predMax,
                                             learned_status(g), g->stream);
    g->launches += 1;
    unsigned st = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&st, learned_status(g), sizeof(st), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    return st ? MDAS_ERR_TIMEOUT : MDAS_OK;
}

int mdas_learned_stats(mdas_grid* g, int* judgedPasses, int* plainPasses, int* lastPlain, double* unrefinedLearned,
                       double* unrefinedPlain) {
    if (!g || !g->lStats) return MDAS_ERR_INVALID;
    MdasLearnedStats h;
    cudaError_t e = cudaMemcpyAsync(&h, g->lStats, sizeof(h), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    if (judgedPasses) *judgedPasses = h.judgedPasses;
    if (plainPasses) *plainPasses = h.plainPasses;
    if (lastPlain) *lastPlain = h.usePlain;
    if (unrefinedLearned) *unrefinedLearned = h.unrefinedLearned;
    if (unrefinedPlain) *unrefinedPlain = h.unrefinedPlain;
    return MDAS_OK;
}

int mdas_learned_pred_max(mdas_grid* g, float* predMax) {
    if (!g || !g->lStats || !predMax) return MDAS_ERR_INVALID;
    unsigned bits = 0;
    cudaError_t e = cudaMemcpyAsync(&bits, &g->lStats->predMax, sizeof(bits), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    *predMax = mdas_float_unorder(bits);
    return MDAS_OK;
}

int mdas_learned_get_params(mdas_grid* g, float* params) {
    if (!g || !g->lState || !params) return MDAS_ERR_INVALID;
    cudaError_t e = cudaMemcpyAsync(params, g->lState, sizeof(float) * MDAS_MLP_PARAMS, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    return status_of(e);
}

int mdas_learned_set_params(mdas_grid* g, const float* params) {
    if (!g || !g->lState || !params) return MDAS_ERR_INVALID;
    return learned_upload(g, params);
}

int mdas_learned_predictions(mdas_grid* g, float* pred) {
    if (!g || !pred) return MDAS_ERR_INVALID;
    if (!g->learned) return MDAS_ERR_STATE;
    cudaError_t e = cudaMemcpyAsync(pred, g->lPred, sizeof(float) * (size_t)g->L, cudaMemcpyDeviceToDevice, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    return status_of(e);
}

int mdas_leaf_true_errors(mdas_grid* g, mdas_scene* s, int samplesPerLeaf, uint64_t seed, const int* leaves,
                          int count, float* errors) {
    if (!g || !s || !errors || samplesPerLeaf < 1 || s->desc.dim > g->dg.D || (leaves && count < 0)) return MDAS_ERR_INVALID;
    if (!g->initialized) return MDAS_ERR_STATE;
    int rc = scene_upload(s, g->stream);
    if (rc) return rc;
    cudaError_t e = mdas_launch_leaf_true_errors(s->desc, s->d_prims, g->dg, leaves, leaves ? count : g->L,
                                                 samplesPerLeaf, seed, errors, g->stream);
    g->launches += 1;
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    return status_of(e);
}

int mdas_leaf_features(mdas_grid* g, float* features) {
    if (!g || !features) return MDAS_ERR_INVALID;
    if (!g->initialized) return MDAS_ERR_STATE;
    cudaError_t e = mdas_mlp::leaf_features(g->dg, g->L, features, g->stream);
    g->launches += 1;
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    return status_of(e);
}

}  // extern "C"

namespace {

// scratch of the standalone MLP calls: packed weights + status word
struct MlpScratch {
    mdas_mlp::Packed* packed = nullptr;
    unsigned* status = nullptr;
    float* loss = nullptr;
    ~MlpScratch() {
        cudaFree(packed);
        cudaFree(status);
    }
    bool open() {
        if (cudaMalloc(&packed, sizeof(mdas_mlp::Packed)) != cudaSuccess) return false;
        if (cudaMalloc(&status, 2 * sizeof(unsigned)) != cudaSuccess) return false;
        loss = reinterpret_cast<float*>(status + 1);
        return true;
    }
};

}  // namespace

extern "C" {

int mdas_mlp_forward(const float* params, const float* features, int m, float* pred, void* stream) {
    if (!params || m < 0 || (m > 0 && (!features || !pred))) return MDAS_ERR_INVALID;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    MlpScratch sc;
    if (!sc.open()) return MDAS_ERR_ALLOC;
    cudaError_t e = cudaMemsetAsync(sc.status, 0, 2 * sizeof(unsigned), s);
    if (e == cudaSuccess) e = mdas_mlp::pack(params, sc.packed, s);
    if (e == cudaSuccess) e = mdas_mlp::forward(sc.packed, features, m, pred, sc.status, s);
    unsigned st = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&st, sc.status, sizeof(st), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    return st ? MDAS_ERR_TIMEOUT : MDAS_OK;
}

int mdas_mlp_adam(float* params, float* m1, float* m2, float* grads, int step, float learningRate, void* stream) {
    if (!params || !m1 || !m2 || !grads || step < 1 || !(learningRate >= 0.0f)) return MDAS_ERR_INVALID;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    MlpScratch sc;
    if (!sc.open()) return MDAS_ERR_ALLOC;
    cudaError_t e = mdas_mlp::adam(params, m1, m2, grads, step, learningRate, sc.packed, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return status_of(e);
}

int mdas_mlp_gradients(const float* params, const float* features, const float* targets, int m, float* grads,
                       float* loss, void* stream) {
    if (!params || !grads || m < 1 || !features || !targets) return MDAS_ERR_INVALID;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    MlpScratch sc;
    if (!sc.open()) return MDAS_ERR_ALLOC;
    cudaError_t e = cudaMemsetAsync(sc.status, 0, 2 * sizeof(unsigned), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(grads, 0, sizeof(float) * MDAS_MLP_PARAMS, s);
    if (e == cudaSuccess) e = mdas_mlp::pack(params, sc.packed, s);
    if (e == cudaSuccess)
        e = mdas_mlp::gradients(sc.packed, features, targets, nullptr, 0, 0, 1, m, grads, sc.loss, sc.status, s);
    unsigned h[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, sc.status, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return MDAS_ERR_CUDA;
    if (h[0]) return MDAS_ERR_TIMEOUT;
    float l;
    memcpy(&l, &h[1], sizeof(l));
    if (loss) *loss = l / (float)m;
    return MDAS_OK;
}

}  // extern "C"
