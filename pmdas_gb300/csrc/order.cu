// order.cu — Morton keys, one-sweep LSD radix sort, Karras hierarchy and point
// location over the MDAS leaves (compiled with strict IEEE flags: the keys
// depend on one division and one multiplication per coordinate, which a CPU
// restatement must be able to repeat bit for bit).
#include "order.h"
#include "ld_hint.h"

namespace mdas_order {

// ---------------------------------------------------------------------------------
// Keys.  The reference numbers its initial cells (uniformSamplingKernel,
// kdgrid.cu:144-157): bit k < bitsPerDim of the cell coordinate of dimension j is
// bit D*k + (D-1-j) of the index, and for the two image dimensions bit
// k in [bitsPerDim, bitsPerDim + extraImgBits) is bit
// D*bitsPerDim + 2*(k - bitsPerDim) + 1-j.  A key is that index at
// K = bitsPerDim + fineBits bits per dimension, so key >> (D * fineBits) is
// the reference's index of the initial cell.
// ---------------------------------------------------------------------------------

// (a cell coordinate has at most 31 bits: bitsPerDim + fineBits + extraImgBits <= 31)
int key_bits(int D, int bitsPerDim, int extraImgBits, int fineBits) {
    if (D < 1 || D > 16 || bitsPerDim < 0 || extraImgBits < 0 || fineBits < 0) return -1;
    if ((long long)bitsPerDim + fineBits + extraImgBits > 31) return -1;
    const long long b = (long long)D * (bitsPerDim + fineBits) + 2LL * extraImgBits;
    return b <= 64 ? (int)b : -1;
}

int max_fine_bits(int D, int bitsPerDim, int extraImgBits) {
    if (D < 1 || D > 16 || bitsPerDim < 0 || extraImgBits < 0) return -1;
    const int rest = 64 - D * bitsPerDim - 2 * extraImgBits;
    const int f = rest < 0 ? -1 : rest / D;
    const int cap = 31 - bitsPerDim - extraImgBits;
    return f < cap ? f : cap;
}

struct KeyParams {
    int D, K, eib;
    float scaleX, scaleY;
};

// Cell coordinate of u in [0, 1) at B bits: floor(u * 2^B), clamped to [0, 2^B - 1].
__device__ __forceinline__ uint32_t quantize(float u, int B) {
    const float top = (float)(1u << B);
    const float s = __fmul_rn(u, top);  // exact: a power-of-two scaling
    if (!(s > 0.0f)) return 0u;         // negative, zero or NaN
    if (s >= top) return (1u << B) - 1u;
    return (uint32_t)s;  // truncation = floor for s > 0
}

// The 8 bits of v spread D apart (bit i to bit D * i): one entry of the table a
// key kernel keeps in shared memory, so that a key takes one lookup per byte of
// each coordinate instead of one step per bit.
__device__ __forceinline__ uint64_t spread_byte(unsigned v, int D) {
    uint64_t r = 0;
    for (int i = 0; i < 8 && D * i < 64; ++i) r |= (uint64_t)((v >> i) & 1u) << (D * i);
    return r;
}

// The bits of x at the even positions (bit i to bit 2i).
__device__ __forceinline__ uint64_t spread_two(uint32_t x) {
    uint64_t v = x;
    v = (v | (v << 16)) & 0x0000FFFF0000FFFFull;
    v = (v | (v << 8)) & 0x00FF00FF00FF00FFull;
    v = (v | (v << 4)) & 0x0F0F0F0F0F0F0F0Full;
    v = (v | (v << 2)) & 0x3333333333333333ull;
    v = (v | (v << 1)) & 0x5555555555555555ull;
    return v;
}

// Key of point p: bit b < K of dimension j's cell coordinate goes to bit
// D * b + (D - 1 - j); the extra image bits b in [K, K + eib) of the two image
// axes go to bit D * K + 2 (b - K) + 1 - j (the initial-cell numbering of
// uniformSamplingKernel, kdgrid.cu:144-160, extended to K bits).  `spread`:
// spread_byte(v, D) for v < 256.
__device__ __forceinline__ uint64_t point_key(const float* p, const KeyParams& k, const uint64_t* spread) {
    uint64_t key = 0;
    const uint32_t lowMask = k.K >= 32 ? 0xffffffffu : ((1u << k.K) - 1u);
    for (int j = 0; j < k.D; ++j) {
        float u = p[j];
        if (j == 0) u = __fdiv_rn(u, k.scaleX);
        if (j == 1) u = __fdiv_rn(u, k.scaleY);
        const int B = k.K + (j < 2 ? k.eib : 0);
        const uint32_t q = quantize(u, B);
        const uint32_t low = q & lowMask;
        for (int m = 0; 8 * m < k.K; ++m)
            key |= spread[(low >> (8 * m)) & 0xffu] << (k.D * 8 * m + (k.D - 1 - j));
        if (j < 2 && k.eib > 0) key |= spread_two(q >> k.K) << (k.D * k.K + 1 - j);
    }
    return key;
}

__device__ __forceinline__ void load_spread(uint64_t* s_spread, int D) {
    for (int v = threadIdx.x; v < 256; v += blockDim.x) s_spread[v] = spread_byte((unsigned)v, D);
    __syncthreads();
}

__global__ void k_morton_encode(const float* __restrict__ points, int n, KeyParams kp, uint64_t* __restrict__ keys) {
    __shared__ uint64_t s_spread[256];
    load_spread(s_spread, kp.D);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        keys[i] = point_key(points + (size_t)i * kp.D, kp, s_spread);
}

// The box of cell c at K bits per dimension, as uniformSamplingKernel
// computes it (kdgrid.cu:142-164, 191-196): mn = offset, mx = offset + extent.
__global__ void k_morton_decode(const uint64_t* __restrict__ cells, int n, KeyParams kp, float* __restrict__ boxes) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint64_t c = cells[i];
        float* box = boxes + (size_t)i * 2 * kp.D;
        for (int j = 0; j < kp.D; ++j) {
            uint32_t xq = 0, extentInv = 1u << kp.K;
            for (int b = 0; b < kp.K; ++b) xq |= (uint32_t)((c >> (kp.D * b + (kp.D - j - 1))) & 1u) << b;
            if (j < 2) {
                for (int b = kp.K; b < kp.K + kp.eib; ++b)
                    xq |= (uint32_t)((c >> (kp.D * kp.K + 2 * (b - kp.K) + 1 - j)) & 1u) << b;
                extentInv <<= kp.eib;
            }
            float extent = __fdiv_rn(1.0f, (float)extentInv);
            float offset = __fmul_rn((float)xq, extent);
            if (j == 0) {
                offset = __fmul_rn(offset, kp.scaleX);
                extent = __fmul_rn(extent, kp.scaleX);
            } else if (j == 1) {
                offset = __fmul_rn(offset, kp.scaleY);
                extent = __fmul_rn(extent, kp.scaleY);
            }
            box[j] = offset;
            box[kp.D + j] = __fadd_rn(offset, extent);
        }
    }
}

template <int D>
__global__ void k_leaf_keys(const float* __restrict__ nb, int nbFloats, int L, KeyParams kp,
                            uint64_t* __restrict__ keys) {
    __shared__ uint64_t s_spread[256];
    load_spread(s_spread, kp.D);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L; i += gridDim.x * blockDim.x) {
        float h[(4 + 2 * D + 3) / 4 * 4];  // node and box of the record (it extends past them)
        ld_head64<4 + 2 * D>(nb + (size_t)i * nbFloats, h);
        float c[D];
#pragma unroll
        for (int j = 0; j < D; ++j) c[j] = __fmul_rn(0.5f, __fadd_rn(h[4 + j], h[4 + D + j]));
        keys[i] = point_key(c, kp, s_spread);
    }
}

static int blocks_for(int n, int threads) {
    const int b = (n + threads - 1) / threads;
    return b < 1 ? 1 : (b > 65535 * 4 ? 65535 * 4 : b);
}

cudaError_t morton_encode(const float* points, int n, int D, int bpd, int eib, int F, float sx, float sy,
                          uint64_t* keys, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const KeyParams kp{D, bpd + F, eib, sx, sy};
    k_morton_encode<<<blocks_for(n, 256), 256, 0, s>>>(points, n, kp, keys);
    return cudaGetLastError();
}

cudaError_t morton_decode(const uint64_t* cells, int n, int D, int bpd, int eib, float sx, float sy, float* boxes,
                          cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const KeyParams kp{D, bpd, eib, sx, sy};
    k_morton_decode<<<blocks_for(n, 256), 256, 0, s>>>(cells, n, kp, boxes);
    return cudaGetLastError();
}

#define ORDER_SWITCH_D(D, CALL)                         \
    switch (D) {                                        \
        case 3: { constexpr int DD = 3; CALL; } break;  \
        case 4: { constexpr int DD = 4; CALL; } break;  \
        case 5: { constexpr int DD = 5; CALL; } break;  \
        case 6: { constexpr int DD = 6; CALL; } break;  \
        default: return cudaErrorInvalidValue;          \
    }

cudaError_t leaf_keys(const MdasDeviceGrid& g, int L, int F, uint64_t* keys, cudaStream_t s) {
    if (L <= 0) return cudaSuccess;
    const KeyParams kp{g.D, g.bitsPerDim + F, g.extraImgBits, g.scaleX, g.scaleY};
    ORDER_SWITCH_D(g.D, (k_leaf_keys<DD><<<blocks_for(L, 256), 256, 0, s>>>(g.nb, g.nbFloats, L, kp, keys)));
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// Radix sort: 8-bit digits, least significant first.  One histogram kernel counts
// every digit position in one read of the keys; a tiny kernel turns the counts
// into each digit's global start; then one kernel per digit position ranks a
// tile of keys in shared memory and scatters it, taking the tile's offsets from
// its predecessors' published digit counts (chained scan with look-back).
// Tiles are numbered in launch order by an atomic counter, so every tile a CTA
// waits for already runs and never waits for a later one; each wait is bounded
// and records a timeout in `status` instead of waiting on.
// ---------------------------------------------------------------------------------

constexpr int kBins = 256;
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
#ifndef MDAS_SORT_ITEMS
#define MDAS_SORT_ITEMS 12
#endif
constexpr int kItems = MDAS_SORT_ITEMS;    // keys per thread
constexpr int kTile = kThreads * kItems;  // keys per tile
// the tile staged in digit order: static shared memory up to 12 keys per
// thread, dynamic (keys, then values) above
#ifndef MDAS_SORT_DYNAMIC_SMEM
#define MDAS_SORT_DYNAMIC_SMEM (MDAS_SORT_ITEMS > 12)
#endif
constexpr size_t kSweepSmem = MDAS_SORT_DYNAMIC_SMEM ? (size_t)kTile * (sizeof(uint64_t) + sizeof(uint32_t)) : 0;
constexpr unsigned kFlagAggregate = 1u << 30;
constexpr unsigned kFlagInclusive = 2u << 30;
constexpr unsigned kCountMask = (1u << 30) - 1u;
constexpr int kSpinLimit = 1 << 18;  // polls of one look-back word before giving up
constexpr int kMaxPasses = 8;
#ifndef MDAS_SORT_WINDOW
#define MDAS_SORT_WINDOW 4
#endif
constexpr int kWindow = MDAS_SORT_WINDOW;  // predecessor words read per look-back round trip

__device__ __forceinline__ unsigned ld_relaxed(const unsigned* p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(unsigned* p, unsigned v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__global__ void __launch_bounds__(kThreads) k_histogram(const uint64_t* __restrict__ keys, int n, int beginBit,
                                                        int endBit, int passes, unsigned* __restrict__ hist) {
    __shared__ unsigned s_hist[kMaxPasses][kBins];
    for (int i = threadIdx.x; i < passes * kBins; i += kThreads) s_hist[i / kBins][i % kBins] = 0u;
    __syncthreads();
    for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
        const uint64_t k = keys[i];
        for (int p = 0; p < passes; ++p) {
            const int shift = beginBit + 8 * p;
            const int bits = min(8, endBit - shift);
            const unsigned d = (unsigned)(k >> shift) & ((1u << bits) - 1u);
            atomicAdd(&s_hist[p][d], 1u);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * kBins; i += kThreads) {
        const unsigned c = s_hist[i / kBins][i % kBins];
        if (c) atomicAdd(&hist[i], c);
    }
}

// exclusive prefix of each pass's 256 digit counts, in place (one CTA per pass)
__global__ void __launch_bounds__(kBins) k_digit_starts(unsigned* __restrict__ hist) {
    __shared__ unsigned s_warp[kBins / 32];
    unsigned* h = hist + blockIdx.x * kBins;
    const unsigned v = h[threadIdx.x];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    unsigned base = 0;
    for (int w = 0; w < warp; ++w) base += s_warp[w];
    h[threadIdx.x] = base + incl - v;
}

struct SweepArgs {
    const uint64_t* keysIn;
    const uint32_t* valuesIn;  // nullptr: value = index
    uint64_t* keysOut;
    uint32_t* valuesOut;
    int n;
    int shift;
    int bits;
    const unsigned* digitStart;  // [256]
    unsigned* lookback;          // [tiles * 256], zeroed
    unsigned* tileCounter;       // zeroed
    unsigned* status;
    int spinLimit;               // polls of one look-back word before giving up
};

// The look-back's poll limit (0: kSpinLimit); a test sets it small to drive the
// timeout path (set_test_wait_limit).
int g_sortSpinLimit = 0;

#ifndef MDAS_SORT_MIN_CTAS
#define MDAS_SORT_MIN_CTAS 4  // 64 registers: 4 CTAs per SM (3 at 80 registers: 12 % slower)
#endif
__global__ void __launch_bounds__(kThreads, MDAS_SORT_MIN_CTAS) k_onesweep(SweepArgs a) {
    __shared__ unsigned s_warpHist[kWarps][kBins];  // per-warp digit counts, then per-warp offsets
    __shared__ unsigned s_localStart[kBins];         // digit start within the tile
    __shared__ unsigned s_globalBase[kBins];         // output position of the tile's first key of each digit
#if MDAS_SORT_DYNAMIC_SMEM
    extern __shared__ __align__(16) unsigned char s_tileBuf[];
    uint64_t* s_keys = reinterpret_cast<uint64_t*>(s_tileBuf);
    uint32_t* s_values = reinterpret_cast<uint32_t*>(s_tileBuf + sizeof(uint64_t) * kTile);
#else
    __shared__ __align__(16) uint64_t s_keys[kTile];
    __shared__ uint32_t s_values[kTile];
#endif
    __shared__ int s_tile;

    if (threadIdx.x == 0) s_tile = (int)atomicAdd(a.tileCounter, 1u);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int b = lane; b < kBins; b += 32) s_warpHist[warp][b] = 0u;
    __syncthreads();
    const int tile = s_tile;
    const int tileBase = tile * kTile;
    const int warpBase = tileBase + warp * 32 * kItems;
    const unsigned mask = (1u << a.bits) - 1u;

    // load (striped per warp: item i of lane l is key warpBase + 32 i + l) and rank within the warp
    uint64_t key[kItems];
    uint32_t val[kItems];
    unsigned digit[kItems], rank[kItems];
    const unsigned lowerLanes = (1u << lane) - 1u;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        const int idx = warpBase + 32 * i + lane;
        const bool valid = idx < a.n;
        key[i] = valid ? a.keysIn[idx] : 0ull;
        val[i] = valid ? (a.valuesIn ? a.valuesIn[idx] : (uint32_t)idx) : 0u;
        const unsigned d = valid ? ((unsigned)(key[i] >> a.shift) & mask) : (unsigned)kBins;  // kBins: no digit
        digit[i] = d;
        // lanes holding the same digit: the AND over the digit's bits of the
        // matching ballots (cheaper than match.any, which runs on a slow pipe)
        unsigned peers = __ballot_sync(0xffffffffu, valid);
#pragma unroll
        for (int bit = 0; bit < 8; ++bit) {
            const bool set = (d >> bit) & 1u;
            const unsigned bal = __ballot_sync(0xffffffffu, set);
            peers &= set ? bal : ~bal;
        }
        const int leader = __ffs(peers) - 1;
        const unsigned base = valid ? s_warpHist[warp][d] : 0u;
        __syncwarp();
        if (valid && lane == leader) s_warpHist[warp][d] = base + __popc(peers);
        __syncwarp();
        rank[i] = base + __popc(peers & lowerLanes);
    }
    __syncthreads();

    // per digit: offsets of the warps, the tile's count, publish it, look back
    const int b = threadIdx.x;  // kThreads == kBins
    unsigned count = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
        const unsigned c = s_warpHist[w][b];
        s_warpHist[w][b] = count;
        count += c;
    }
    unsigned* mine = a.lookback + (size_t)tile * kBins + b;
    st_relaxed(mine, (tile == 0 ? kFlagInclusive : kFlagAggregate) | count);
    unsigned exclusive = 0;
    if (tile > 0) {
        // walk back over the predecessors' words, four per round trip: add
        // aggregates until an inclusive prefix; re-poll from a word not yet published
        int t = tile - 1;
        int spins = 0;
        bool done = false;
        while (!done && t >= 0) {
            unsigned w[kWindow];
#pragma unroll
            for (int q = 0; q < kWindow; ++q)
                w[q] = t - q >= 0 ? ld_relaxed(a.lookback + (size_t)(t - q) * kBins + b) : kFlagInclusive;
            int q = 0;
            for (; q < kWindow; ++q) {
                if ((w[q] & ~kCountMask) == 0u) break;
                exclusive += w[q] & kCountMask;
                if (w[q] & kFlagInclusive) {
                    done = true;
                    break;
                }
            }
            if (done) break;
            t -= q;
            if (q < kWindow) {  // tile t has not published yet
                if (++spins > a.spinLimit || ld_relaxed(a.status) != 0u) {
                    atomicOr(a.status, 1u);
                    break;
                }
                __nanosleep(20);
            }
        }
        st_relaxed(mine, kFlagInclusive | ((exclusive + count) & kCountMask));
    }

    // digit starts within the tile (block-wide exclusive scan of the counts)
    {
        unsigned incl = count;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        __shared__ unsigned s_scanWarp[kWarps];
        if (lane == 31) s_scanWarp[warp] = incl;
        __syncthreads();
        unsigned base = 0;
        for (int w = 0; w < warp; ++w) base += s_scanWarp[w];
        const unsigned localStart = base + incl - count;
        s_localStart[b] = localStart;
        s_globalBase[b] = a.digitStart[b] + exclusive - localStart;
    }
    __syncthreads();

    // stage the tile in digit order, then write it out (runs of one digit are contiguous)
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        const unsigned d = digit[i];
        if (d < (unsigned)kBins) {
            const unsigned pos = s_localStart[d] + s_warpHist[warp][d] + rank[i];
            s_keys[pos] = key[i];
            s_values[pos] = val[i];
        }
    }
    __syncthreads();
    const int tileCount = min(kTile, a.n - tileBase);
    for (int j = threadIdx.x; j < tileCount; j += kThreads) {
        const uint64_t k = s_keys[j];
        const unsigned d = (unsigned)(k >> a.shift) & mask;
        const unsigned dst = s_globalBase[d] + (unsigned)j;
        if (dst < (unsigned)a.n) {  // always, unless an earlier wait gave up (then status is set)
            a.keysOut[dst] = k;
            a.valuesOut[dst] = s_values[j];
        } else {
            atomicOr(a.status, 4u);
        }
    }
}

__global__ void k_iota(uint32_t* __restrict__ v, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = (uint32_t)i;
}

static int num_passes(int beginBit, int endBit) { return (endBit - beginBit + 7) / 8; }
static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct SortLayout {
    size_t hist, counters, lookback, keysAlt, valuesAlt, total, zeroBytes;
};

static SortLayout sort_layout(int n, int beginBit, int endBit) {
    const int passes = num_passes(beginBit, endBit);
    const size_t tiles = ((size_t)n + kTile - 1) / kTile;
    SortLayout l;
    size_t off = 0;
    l.hist = off;
    off = align256(off + sizeof(unsigned) * passes * kBins);
    l.counters = off;  // passes tile counters + status
    off = align256(off + sizeof(unsigned) * (passes + 1));
    l.lookback = off;
    off = align256(off + sizeof(unsigned) * passes * tiles * kBins);
    l.zeroBytes = off;
    l.keysAlt = off;
    off = align256(off + sizeof(uint64_t) * (size_t)n);
    l.valuesAlt = off;
    off = align256(off + sizeof(uint32_t) * (size_t)n);
    l.total = off;
    return l;
}

size_t sort_temp_bytes(int n, int beginBit, int endBit) {
    if (n < 0 || beginBit < 0 || endBit > 64 || beginBit > endBit) return 0;
    return sort_layout(n, beginBit, endBit).total;
}

int sort_launches(int n, int beginBit, int endBit) {
    if (n <= 0) return 0;
    const int passes = num_passes(beginBit, endBit);
    return passes == 0 ? 1 : 2 + passes;
}

cudaError_t radix_sort(void* temp, size_t tempBytes, const uint64_t* keysIn, uint64_t* keysOut,
                       const uint32_t* valuesIn, uint32_t* valuesOut, int n, int beginBit, int endBit,
                       cudaStream_t s, unsigned** statusOut) {
    if (n < 0 || beginBit < 0 || endBit > 64 || beginBit > endBit) return cudaErrorInvalidValue;
    const SortLayout l = sort_layout(n, beginBit, endBit);
    if (!temp || tempBytes < l.total) return cudaErrorInvalidValue;
    char* base = static_cast<char*>(temp);
    unsigned* hist = reinterpret_cast<unsigned*>(base + l.hist);
    unsigned* counters = reinterpret_cast<unsigned*>(base + l.counters);
    const int passes = num_passes(beginBit, endBit);
    unsigned* status = counters + passes;
    if (statusOut) *statusOut = status;
    cudaError_t e = cudaMemsetAsync(temp, 0, l.zeroBytes, s);
    if (e != cudaSuccess || n == 0) return e;
    if (passes == 0) {
        e = cudaMemcpyAsync(keysOut, keysIn, sizeof(uint64_t) * (size_t)n, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return e;
        if (valuesIn) return cudaMemcpyAsync(valuesOut, valuesIn, sizeof(uint32_t) * (size_t)n,
                                             cudaMemcpyDeviceToDevice, s);
        k_iota<<<blocks_for(n, 256), 256, 0, s>>>(valuesOut, n);
        return cudaGetLastError();
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (kSweepSmem > 0) {
        e = cudaFuncSetAttribute(k_onesweep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSweepSmem);
        if (e != cudaSuccess) return e;
    }
    const int histBlocks = min(blocks_for(n, kThreads), 2 * (sms > 0 ? sms : 1));
    k_histogram<<<histBlocks, kThreads, 0, s>>>(keysIn, n, beginBit, endBit, passes, hist);
    k_digit_starts<<<passes, kBins, 0, s>>>(hist);
    const size_t tiles = ((size_t)n + kTile - 1) / kTile;
    uint64_t* keysAlt = reinterpret_cast<uint64_t*>(base + l.keysAlt);
    uint32_t* valuesAlt = reinterpret_cast<uint32_t*>(base + l.valuesAlt);
    const uint64_t* srcK = keysIn;
    const uint32_t* srcV = valuesIn;
    for (int p = 0; p < passes; ++p) {
        // the last pass writes the caller's output
        const bool toOut = ((passes - 1 - p) % 2) == 0;
        SweepArgs a;
        a.keysIn = srcK;
        a.valuesIn = srcV;
        a.keysOut = toOut ? keysOut : keysAlt;
        a.valuesOut = toOut ? valuesOut : valuesAlt;
        a.n = n;
        a.shift = beginBit + 8 * p;
        a.bits = min(8, endBit - a.shift);
        a.digitStart = hist + p * kBins;
        a.lookback = reinterpret_cast<unsigned*>(base + l.lookback) + (size_t)p * tiles * kBins;
        a.tileCounter = counters + p;
        a.status = status;
        a.spinLimit = g_sortSpinLimit > 0 ? g_sortSpinLimit : kSpinLimit;
        k_onesweep<<<(unsigned)tiles, kThreads, kSweepSmem, s>>>(a);
        srcK = a.keysOut;
        srcV = a.valuesOut;
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// Karras radix tree (T. Karras, "Maximizing Parallelism in the Construction of
// BVHs, Octrees, and k-d Trees", HPG 2012): one thread per internal node finds
// its key range from common-prefix lengths and splits it at the highest
// differing bit.  Equal keys are told apart by their positions (the prefix
// length of two equal keys is 64 + the common prefix of their positions).
// ---------------------------------------------------------------------------------

__device__ __forceinline__ int prefix_len(const uint64_t* __restrict__ k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint64_t a = k[i], b = k[j];
    if (a == b) return 64 + __clz((unsigned)(i ^ j));
    return __clzll((long long)(a ^ b));
}

__global__ void k_karras(const uint64_t* __restrict__ k, int n, int2* __restrict__ children, int* __restrict__ parents) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
        const int d = prefix_len(k, n, i, i + 1) - prefix_len(k, n, i, i - 1) >= 0 ? 1 : -1;
        const int dmin = prefix_len(k, n, i, i - d);
        int lmax = 2;
        while (prefix_len(k, n, i, i + lmax * d) > dmin) lmax <<= 1;  // ends: past the array the length is -1
        int l = 0;
        for (int t = lmax >> 1; t >= 1; t >>= 1)
            if (prefix_len(k, n, i, i + (l + t) * d) > dmin) l += t;
        const int j = i + l * d;
        const int dnode = prefix_len(k, n, i, j);
        int s = 0;
        for (int t = (l + 1) >> 1;; t = (t + 1) >> 1) {
            if (prefix_len(k, n, i, i + (s + t) * d) > dnode) s += t;
            if (t <= 1) break;
        }
        const int gamma = i + s * d + min(d, 0);
        const int lo = min(i, j), hi = max(i, j);
        const int left = lo == gamma ? ~gamma : gamma;
        const int right = hi == gamma + 1 ? ~(gamma + 1) : gamma + 1;
        children[i] = make_int2(left, right);
        parents[left >= 0 ? left : (n - 1) + ~left] = i;
        parents[right >= 0 ? right : (n - 1) + ~right] = i;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) parents[0] = -1;  // the root (internal node 0, or the only leaf)
}

cudaError_t karras_build(const uint64_t* sortedKeys, int n, int2* children, int* parents, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_karras<<<blocks_for(n, 256), 256, 0, s>>>(sortedKeys, n, children, parents);
    return cudaGetLastError();
}

constexpr int kMaxDepth = 128;  // > the deepest possible tree (64 key bits + 32 position bits)

__device__ __forceinline__ unsigned atomic_add_acq_rel(unsigned* p, unsigned v) {
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// Bottom-up boxes: a thread starts at each leaf and climbs; at each node the
// first of the two children to arrive stops, the second (which then finds both
// child boxes written) computes the union and goes on.
// READONLY: the boxes are final (point location) and go through L1; during the
// refit another thread writes them, so they are read through L2.
template <int D, bool READONLY = false>
__device__ __forceinline__ void child_box(const MdasDeviceGrid& g, const uint32_t* __restrict__ order, const float* boxes,
                                          int c, float (&mn)[D], float (&mx)[D]) {
    if (c < 0) {
        float h[(4 + 2 * D + 3) / 4 * 4];  // the leaf record's node and box (the record extends past them)
        ld_head64<4 + 2 * D>(g.nb + (size_t)order[~c] * g.nbFloats, h);
#pragma unroll
        for (int j = 0; j < D; ++j) {
            mn[j] = h[4 + j];
            mx[j] = h[4 + D + j];
        }
    } else {
        const float* b = boxes + (size_t)c * 2 * D;
#pragma unroll
        for (int j = 0; j < D; ++j) {
            mn[j] = READONLY ? __ldg(b + j) : __ldcg(b + j);
            mx[j] = READONLY ? __ldg(b + D + j) : __ldcg(b + D + j);
        }
    }
}

template <int D>
__global__ void k_refit(MdasDeviceGrid g, const uint32_t* __restrict__ order, int n, const int2* __restrict__ children,
                        const int* __restrict__ parents, unsigned* __restrict__ visits, float* boxes) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        int node = parents[(n - 1) + p];
        for (int depth = 0; node >= 0 && depth < kMaxDepth; ++depth) {
            // release: the box this thread wrote last is visible to the second arrival;
            // acquire: the second arrival sees its sibling's box
            if (atomic_add_acq_rel(&visits[node], 1u) == 0u) break;
            const int2 ch = children[node];
            float amn[D], amx[D], bmn[D], bmx[D];
            child_box<D>(g, order, boxes, ch.x, amn, amx);
            child_box<D>(g, order, boxes, ch.y, bmn, bmx);
            float* out = boxes + (size_t)node * 2 * D;
#pragma unroll
            for (int j = 0; j < D; ++j) {
                __stcg(out + j, fminf(amn[j], bmn[j]));
                __stcg(out + D + j, fmaxf(amx[j], bmx[j]));
            }
            node = parents[node];
        }
    }
}

cudaError_t karras_refit(const MdasDeviceGrid& g, const uint32_t* order, int n, const int2* children,
                         const int* parents, unsigned* visits, float* boxes, cudaStream_t s) {
    if (n <= 1) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(visits, 0, sizeof(unsigned) * (size_t)(n - 1), s);
    if (e != cudaSuccess) return e;
    ORDER_SWITCH_D(g.D, (k_refit<DD><<<blocks_for(n, 256), 256, 0, s>>>(g, order, n, children, parents, visits, boxes)));
    return cudaGetLastError();
}

// Point location: depth-first, left child first, pruning with closed boxes;
// a leaf holds p if mn <= p < mx in every dimension (p <= mx where the leaf's
// face is on the domain's upper face).  Left-first depth-first order visits
// leaves in key order, so the answer is the first holding leaf in key order.
constexpr int kStack = kMaxDepth;

// perm (may be null): the queries in the order the threads take them (points
// sorted by a coarse Morton key, so that a warp walks one region of the tree).
template <int D>
__global__ void k_locate(MdasDeviceGrid g, const uint32_t* __restrict__ order, int n, const int2* __restrict__ children,
                         const float* __restrict__ boxes, const float* __restrict__ points, int m,
                         const uint32_t* __restrict__ perm, int* __restrict__ leaves, unsigned* status) {
    float domMx[D];
    {
        float dmn[D];
        if (n == 1) child_box<D, true>(g, order, boxes, ~0, dmn, domMx);
        else child_box<D, true>(g, order, boxes, 0, dmn, domMx);
    }
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < m; t += gridDim.x * blockDim.x) {
        const int q = perm ? (int)perm[t] : t;
        if (q < 0 || q >= m) {  // a permutation from a sort that gave up
            atomicOr(status, 4u);
            continue;
        }
        float p[D];
#pragma unroll
        for (int j = 0; j < D; ++j) p[j] = points[(size_t)q * D + j];
        int stack[kStack];
        int sp = 0;
        stack[sp++] = n == 1 ? ~0 : 0;
        int found = -1;
        while (sp > 0) {
            const int c = stack[--sp];
            float mn[D], mx[D];
            child_box<D, true>(g, order, boxes, c, mn, mx);
            bool in = true;
            if (c < 0) {
#pragma unroll
                for (int j = 0; j < D; ++j)
                    in = in && mn[j] <= p[j] && (p[j] < mx[j] || (p[j] == mx[j] && mx[j] >= domMx[j]));
                if (in) {
                    found = (int)order[~c];
                    break;
                }
            } else {
#pragma unroll
                for (int j = 0; j < D; ++j) in = in && mn[j] <= p[j] && p[j] <= mx[j];
                if (in) {
                    if (sp + 2 > kStack) {
                        atomicOr(status, 2u);
                        break;
                    }
                    const int2 ch = children[c];
                    stack[sp++] = ch.y;
                    stack[sp++] = ch.x;
                }
            }
        }
        leaves[q] = found;
    }
}

cudaError_t locate(const MdasDeviceGrid& g, const uint32_t* order, int n, const int2* children, const float* boxes,
                   const float* points, int m, const uint32_t* perm, int* leaves, unsigned* status, cudaStream_t s) {
    if (m <= 0) return cudaSuccess;
    if (n <= 0) return cudaMemsetAsync(leaves, 0xff, sizeof(int) * (size_t)m, s);
    ORDER_SWITCH_D(g.D, (k_locate<DD><<<blocks_for(m, 128), 128, 0, s>>>(g, order, n, children, boxes, points, m,
                                                                         perm, leaves, status)));
    return cudaGetLastError();
}

int query_fine_bits(int D, int bitsPerDim, int extraImgBits) {
    const int base = D * bitsPerDim + 2 * extraImgBits;
    int fine = base >= 32 ? 0 : (32 - base) / D;
    if (fine > 31 - bitsPerDim - extraImgBits) fine = 31 - bitsPerDim - extraImgBits;
    return fine > 0 ? fine : 0;
}

void set_test_wait_limit(int polls) { g_sortSpinLimit = polls > 0 ? polls : 0; }

}  // namespace mdas_order
