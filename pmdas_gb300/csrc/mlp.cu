// mlp.cu — the learned leaf priority on the tcgen05 tensor cores.
//
// One CTA of 128 threads works on tiles of 128 rows (leaves).  Per tile:
//   features (FP32 -> BF16) into a shared-memory A tile;
//   layer 1: one tcgen05.mma (M 128, N 64, K 16) into 64 TMEM columns;
//   tcgen05.ld of the accumulators (thread t = row t), + b1, ReLU, BF16 into
//   the shared-memory A tile of layer 2;
//   layer 2: four tcgen05.mma (K 64 in steps of 16) into the same columns;
//   tcgen05.ld, + b2, ReLU, dot with w3 (+ b3) on the CUDA cores.
// The MMAs are issued by one thread and tracked by an mbarrier
// (tcgen05.commit); every wait on it is bounded and records a timeout in
// `status`.  Operands use the no-swizzle K-major layout: 8x8 BF16 core
// matrices of 128 contiguous bytes, K-blocks of one row group adjacent.
//
// Training (gradients) runs the same forward, then on the tensor cores
// dH1 = dZ2 . W2 (M 128, N 64, K 64, W2 transposed as the K-major B operand)
// and the weight gradients dW2 = dZ2^T H1, dW1 = dZ1^T X as one GEMM per tile
// (M 128, N 80, K 128 over the tile's rows) accumulated in tensor memory over
// all tiles of a persistent CTA, added to the global gradient once per CTA.
#include "mlp.h"
#include "leaf_raw.h"
#include "ld_hint.h"

#include <cuda_bf16.h>
#include <float.h>

namespace mdas_mlp {

namespace {

constexpr int kRows = 128;
constexpr int kThreads = 128;
constexpr int kH = MDAS_MLP_HIDDEN;
constexpr int kIn = MDAS_MLP_IN;
constexpr uint32_t kTmemCols = 64;
constexpr int kWaitLimit = 1 << 20;

// shared-memory map (bytes from the 1024-aligned base)
constexpr int SM_X = 0;          // 128 x 16 BF16, core matrices, 2 K-blocks per row group
constexpr int SM_H = 4096;       // 128 x 64 BF16, 8 K-blocks per row group
constexpr int SM_W1 = 20480;     // 64 x 16 BF16
constexpr int SM_W2 = 22528;     // 64 x 64 BF16 (B of layer 2: n = output, k = input)
constexpr int SM_W2T = 30720;    // 64 x 64 BF16 (B of dH1: n = input, k = output)
constexpr int SM_VEC = 38912;    // b1, b2, w3 (64 floats each), b3
constexpr int SM_BAR = 39744;    // mbarrier (8 B), TMEM address slot (4 B)
// b1 and b2 as 16 chunks of 4 columns each, every chunk one core matrix of
// 8 identical 16-byte rows: the sources of the accumulators' bias copies
constexpr int SM_BIAS = 39808;
constexpr int SM_FWD = SM_BIAS + 2 * 16 * 128;  // end of what the forward needs
// training only
constexpr int SM_Z2F = 44032;                    // dZ2, FP32 [128][65]
constexpr int SM_D = SM_Z2F + kRows * 65 * 4;    // dZ2, BF16 core matrices (A of dH1)
constexpr int SM_Z1F = SM_D + kRows * kH * 2;    // dZ1, FP32 [128][65]
constexpr int SM_G = SM_Z1F + kRows * 65 * 4;    // per-CTA gradient, FP32 [MDAS_MLP_PARAMS]
constexpr int SM_RED = SM_G + ((MDAS_MLP_PARAMS * 4 + 127) / 128) * 128;  // [3][4 warps][64] partial sums
constexpr int SM_TRAIN = SM_RED + 3 * 4 * kH * 4;
constexpr int kFwdSmem = SM_FWD + 1024;          // (+ alignment of the base) <= 5 CTAs x 64 TMEM columns per SM
constexpr int kTrainSmem = SM_TRAIN + 1024;

static_assert(SM_W2T + kH * kH * 2 == SM_VEC, "map");
static_assert(SM_VEC + (3 * kH + 4) * 4 <= SM_BAR, "map");
static_assert(SM_FWD <= SM_Z2F && SM_BIAS >= SM_BAR + 16 && SM_BIAS % 128 == 0, "map");

// ---- PTX wrappers ---------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Shared-memory matrix descriptor, K-major without swizzle: start address,
// leading byte offset (next core matrix along K), stride byte offset (next
// 8-row group), the fixed constant 0b001 at bits 46-48, swizzle mode 0.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3fffu) | ((uint64_t)((lbo >> 4) & 0x3fffu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3fffu) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A
// and B (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
constexpr uint32_t kIdesc = idesc_bf16(kRows, kH);

__device__ __forceinline__ void mma_bf16_id(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t accumulate) {
    mma_bf16_id(d, a, b, kIdesc, accumulate);
}
// A 32-row x 128-bit matrix from shared memory into the tensor-memory columns
// taddr .. taddr + 3 of all four 32-lane quarters (asynchronous; ordered with
// the issuing thread's MMAs).
__device__ __forceinline__ void tmem_cp_32x128b_x4(uint32_t taddr, uint64_t sdesc) {
    asm volatile("tcgen05.cp.cta_group::1.32x128b.warpx4 [%0], %1;" ::"r"(taddr), "l"(sdesc) : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 16 FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
        "[%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// element (r, k) of a BF16 tile with KB K-blocks per row group, in elements
__host__ __device__ __forceinline__ int core_off(int r, int k, int KB) {
    return (((r >> 3) * KB + (k >> 3)) << 6) + ((r & 7) << 3) + (k & 7);
}

__device__ __forceinline__ uint16_t bf16_bits(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float bf16_val(uint16_t b) { return __bfloat162float(__ushort_as_bfloat16(b)); }

// two floats as BF16 (round to nearest even), the first in the low half
__device__ __forceinline__ uint32_t bf16x2_bits(float lo, float hi) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// 8 consecutive K-elements of row r (one core-matrix row, 16 bytes)
__device__ __forceinline__ void st_row8(uint8_t* tile, int r, int kb, int KB, const float* v) {
    uint4 q;
    q.x = bf16x2_bits(v[0], v[1]);
    q.y = bf16x2_bits(v[2], v[3]);
    q.z = bf16x2_bits(v[4], v[5]);
    q.w = bf16x2_bits(v[6], v[7]);
    *reinterpret_cast<uint4*>(tile + 2 * core_off(r, kb * 8, KB)) = q;
}
__device__ __forceinline__ void ld_row8(const uint8_t* tile, int r, int kb, int KB, float* v) {
    const uint4 q = *reinterpret_cast<const uint4*>(tile + 2 * core_off(r, kb * 8, KB));
    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        v[2 * i] = bf16_val((uint16_t)(w[i] & 0xffffu));
        v[2 * i + 1] = bf16_val((uint16_t)(w[i] >> 16));
    }
}

// Sum of v[64] over the warp's lanes, stored to out[64]: a reduce-scatter by
// halving (62 shuffles); lane l ends with the sums of elements 2l and 2l + 1.
__device__ __forceinline__ void warp_sum64(float (&v)[kH], float* out) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int off = 16, n = 32; off >= 1; off >>= 1, n >>= 1) {
        const bool upper = (lane & off) != 0;
#pragma unroll
        for (int i = 0; i < n; ++i) {
            const float send = upper ? v[i] : v[i + n];
            const float keep = upper ? v[i + n] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
    }
    out[2 * lane] = v[0];
    out[2 * lane + 1] = v[1];
}

// ---- per-CTA setup / teardown -------------------------------------------------------
struct Ctx {
    uint8_t* sm;
    uint32_t base, bar, tmem, phase, cols;
    unsigned* status;
};

__device__ __forceinline__ uint8_t* aligned_smem() {
    extern __shared__ uint8_t dyn[];
    return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(dyn) + 1023) & ~(uintptr_t)1023);
}

// weights: W1, W2, W2^T tiles and the vectors (Packed keeps them contiguous),
// and the bias chunks (row r of chunk j of b: b[4j .. 4j + 3], every r)
__device__ __forceinline__ void copy_weights(uint8_t* sm, const Packed* w) {
    const uint4* src = reinterpret_cast<const uint4*>(w);
    uint4* dst = reinterpret_cast<uint4*>(sm + SM_W1);
    constexpr int n16 = (int)(sizeof(Packed) / 16);
    static_assert(sizeof(Packed) % 16 == 0, "Packed is copied in 16-byte pieces");
    static_assert(SM_W1 + (int)sizeof(Packed) <= SM_BAR, "Packed fits before the barrier");
    for (int i = threadIdx.x; i < n16; i += kThreads) dst[i] = src[i];
    uint4* bias = reinterpret_cast<uint4*>(sm + SM_BIAS);
    for (int i = threadIdx.x; i < 2 * 16 * 8; i += kThreads) {  // (layer, chunk, row)
        const float* b = (i >> 7) ? w->b2 : w->b1;
        bias[i] = reinterpret_cast<const uint4*>(b)[(i >> 3) & 15];
    }
}

// cols: tensor-memory columns of the CTA (a power of 2, >= 32)
__device__ void ctx_open(Ctx& c, const Packed* w, unsigned* status, uint32_t cols = kTmemCols) {
    c.sm = aligned_smem();
    c.base = smem_u32(c.sm);
    c.bar = c.base + SM_BAR;
    c.phase = 0;
    c.cols = cols;
    c.status = status;
    if (w) copy_weights(c.sm, w);
    if (threadIdx.x == 0) {
        mbar_init(c.bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (threadIdx.x < 32) {
        tmem_alloc(c.base + SM_BAR + 8, cols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    c.tmem = *reinterpret_cast<volatile uint32_t*>(c.sm + SM_BAR + 8);
}

__device__ void ctx_close(Ctx& c) {
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x < 32) {
        tc_fence_after();
        tmem_dealloc(c.tmem, c.cols);
    }
}

// Polls after which an MMA wait reports a timeout (0: kWaitLimit).  A test sets
// it small to drive the timeout path: the wait then polls without suspending
// (a suspending poll could sit out the MMA), records the timeout in the status
// word and waits on with kWaitLimit, so that the accumulator is complete before
// it is read and no MMA is in flight when the tensor memory is freed.
__device__ int test_wait_limit = 0;

__device__ __forceinline__ bool mbar_test_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void mma_wait(Ctx& c) {
    const int polls = test_wait_limit;
    bool ok = false;
    if (polls > 0)
        for (int i = 0; i < polls && !ok; ++i) ok = mbar_test_wait(c.bar, c.phase);
    else
        for (int i = 0; i < kWaitLimit && !ok; ++i) ok = mbar_try_wait(c.bar, c.phase);
    if (!ok) {
        atomicOr(c.status, 1u);
        for (int i = 0; i < kWaitLimit && !ok; ++i) ok = mbar_try_wait(c.bar, c.phase);
    }
    c.phase ^= 1u;
    tc_fence_after();
}

// this thread's row of the 64 accumulator columns
__device__ __forceinline__ void tmem_row(const Ctx& c, float (&acc)[kH]) {
    const uint32_t lane = (threadIdx.x & ~31u) << 16;
#pragma unroll
    for (int q = 0; q < kH / 16; ++q) tmem_ld16(c.tmem + lane + 16 * q, acc + 16 * q);
    tmem_wait_ld();
}

// Issue `steps` MMAs over K (16 each) of A at aOff (KB K-blocks) x B at bOff
// (after the CTA's shared-memory writes); mma_wait completes them.  biasOff >=
// 0: the accumulators start from that bias (its 16 chunks copied into the 64
// columns first; a chunk's descriptor has zero strides, so its one 8-row core
// matrix stands for all 32 rows), else from zero.
__device__ __forceinline__ void mma_issue(Ctx& c, int aOff, int bOff, int KB, int steps, int biasOff = -1) {
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
        tc_fence_after();
        if (biasOff >= 0)
            for (int j = 0; j < kH / 4; ++j) tmem_cp_32x128b_x4(c.tmem + 4 * j, smem_desc(c.base + biasOff + 128 * j, 0, 0));
        const uint32_t sbo = (uint32_t)KB * 128u;
        for (int s = 0; s < steps; ++s)
            mma_bf16(c.tmem, smem_desc(c.base + aOff + 256 * s, 128, sbo), smem_desc(c.base + bOff + 256 * s, 128, sbo),
                     s > 0 || biasOff >= 0 ? 1u : 0u);
        mma_commit(c.bar);
    }
}

__device__ __forceinline__ void run_mma(Ctx& c, int aOff, int bOff, int KB, int steps) {
    mma_issue(c, aOff, bOff, KB, steps);
    mma_wait(c);
}

// Forward of the tile whose features this thread wrote as row threadIdx.x of SM_X:
// z2 = the layer-2 pre-activations (b2 added).  during1() and during2() run
// while layer 1's and layer 2's MMAs execute (global loads for the next tile
// into registers; they touch neither the operand tiles nor tensor memory).
// The biases enter as the accumulators' initial values (copied into tensor
// memory ahead of each layer's MMAs).
template <typename During1, typename During2>
__device__ __forceinline__ void tile_forward(Ctx& c, float (&z2)[kH], During1 during1, During2 during2) {
    mma_issue(c, SM_X, SM_W1, 2, 1, SM_BIAS);
    during1();
    mma_wait(c);
    float acc[kH];
    tmem_row(c, acc);
#pragma unroll
    for (int i = 0; i < kH; ++i) acc[i] = fmaxf(acc[i], 0.0f);
#pragma unroll
    for (int kb = 0; kb < kH / 8; ++kb) st_row8(c.sm + SM_H, threadIdx.x, kb, 8, acc + 8 * kb);
    mma_issue(c, SM_H, SM_W2, 8, kH / 16, SM_BIAS + 16 * 128);
    during2();
    mma_wait(c);
    tmem_row(c, z2);
}

__device__ __forceinline__ void tile_forward(Ctx& c, float (&z2)[kH]) {
    tile_forward(c, z2, [] {}, [] {});
}

__device__ __forceinline__ float head(const Ctx& c, const float (&z2)[kH]) {
    const float* w3 = reinterpret_cast<const float*>(c.sm + SM_VEC) + 2 * kH;
    float p = w3[kH];  // b3
#pragma unroll
    for (int i = 0; i < kH; ++i) p += fmaxf(z2[i], 0.0f) * w3[i];
    return p;
}

__device__ __forceinline__ void put_features(const Ctx& c, const float (&f)[kIn]) {
    st_row8(c.sm + SM_X, threadIdx.x, 0, 2, f);
    st_row8(c.sm + SM_X, threadIdx.x, 1, 2, f + 8);
}

// ---- features --------------------------------------------------------------------
// Per leaf (16): log2 box extents of the first five dimensions (image axes
// relative to the image; 0 past D) / 16; the sample count / 4; log2(1 + x) of
// the samples' luminance mean, standard deviation, minimum and maximum; the
// plain error log2(error) / 32; the depth (splits below the initial cell,
// sum over dimensions of log2(initial extent / extent)) / 32; and the plain
// errors of the four neighbouring leaf slots (slot +-1, +-2: initial cells in
// Morton order, split children next to the children of neighbouring parents),
// log2(error) / 32.
// (The features use the hardware base-2 logarithm, MUFU.LG2 via __log2f: its
// arguments here are normal numbers >= 1e-30, and its relative error of about
// 2^-22 is far below what the BF16 inputs of the network resolve.)
__device__ __forceinline__ float log2_err(float e) { return __log2f(fmaxf(e, 1e-30f)) * (1.0f / MDAS_MLP_TARGET_SCALE); }

// The raw inputs of a leaf's features (leaf_raw.h), gathered from its record
// and sample values.
template <int D>
__device__ __forceinline__ void leaf_raw(const MdasDeviceGrid& g, int leaf, float (&raw)[MDAS_RAW_FLOATS]) {
    float h[(4 + 2 * D + 3) / 4 * 4];  // node and box (the record extends past them)
    ld_head64<4 + 2 * D>(g.nb + (size_t)leaf * g.nbFloats, h);
    const int4 node = make_int4(__float_as_int(h[0]), __float_as_int(h[1]), __float_as_int(h[2]), __float_as_int(h[3]));
    float mn[D], mx[D];
#pragma unroll
    for (int j = 0; j < D; ++j) {
        mn[j] = h[4 + j];
        mx[j] = h[4 + D + j];
    }
    const int idx[4] = {node.x, node.y, node.z, node.w};
    MdasLumStats s = mdas_lum_empty();
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (idx[i] >= 0) {
            const float* p = g.values + 3 * (size_t)idx[i];
            mdas_lum_add(s, mdas_luminance(__ldg(p), __ldg(p + 1), __ldg(p + 2)));
        }
    }
#pragma unroll
    for (int j = 0; j < 6; ++j) raw[j] = j < D ? __fsub_rn(mx[j < D ? j : 0], mn[j < D ? j : 0]) : 0.0f;
    raw[6] = s.n;
    raw[7] = s.sum;
    raw[8] = s.sq;
    raw[9] = s.mn;
    raw[10] = s.mx;
    raw[11] = g.errors[leaf];
}

// A row written by the errors pass (16-byte loads).
__device__ __forceinline__ void load_raw(const float* __restrict__ row, float (&raw)[MDAS_RAW_FLOATS]) {
    const float4* r4 = reinterpret_cast<const float4*>(row);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const float4 v = r4[q];
        raw[4 * q] = v.x;
        raw[4 * q + 1] = v.y;
        raw[4 * q + 2] = v.z;
        raw[4 * q + 3] = v.w;
    }
}

// The errors of the leaf's slot neighbours (slot -2, -1, +1, +2; a NaN where a
// neighbour does not exist: feats_of_raw then takes the leaf's own error).
__device__ __forceinline__ void nbr_errors(const MdasDeviceGrid& g, int leaf, int L, float (&ne)[4]) {
    const int nbr[4] = {leaf - 2, leaf - 1, leaf + 1, leaf + 2};
#pragma unroll
    for (int q = 0; q < 4; ++q) ne[q] = nbr[q] >= 0 && nbr[q] < L ? g.errors[nbr[q]] : __int_as_float(0x7fffffff);
}

// Features from the raw inputs and the neighbours' errors.
template <int D>
__device__ void feats_of_raw(const MdasDeviceGrid& g, const float (&raw)[MDAS_RAW_FLOATS], const float (&ne)[4],
                             float (&f)[kIn]) {
    float depth = 0.0f;
#pragma unroll
    for (int j = 0; j < D; ++j) {
        float e = raw[j];
        if (j == 0) e = __fdividef(e, g.scaleX);
        if (j == 1) e = __fdividef(e, g.scaleY);
        const float l = __log2f(fmaxf(e, 1e-30f));
        if (j < 5) f[j] = l * (1.0f / 16.0f);
        depth += -(float)(g.bitsPerDim + (j < 2 ? g.extraImgBits : 0)) - l;
    }
#pragma unroll
    for (int j = D; j < 5; ++j) f[j] = 0.0f;
    const float n = raw[6];
    const float inv = n > 0.0f ? __frcp_rn(n) : 0.0f;
    const float mean = raw[7] * inv;
    const float var = fmaxf(raw[8] * inv - mean * mean, 0.0f);
    f[5] = n * 0.25f;
    f[6] = __log2f(1.0f + fabsf(mean));
    f[7] = __log2f(1.0f + sqrtf(var));
    f[8] = n > 0.0f ? __log2f(1.0f + fabsf(raw[9])) : 0.0f;
    f[9] = n > 0.0f ? __log2f(1.0f + fabsf(raw[10])) : 0.0f;
    f[10] = log2_err(raw[11]);
    f[11] = depth * (1.0f / 32.0f);
#pragma unroll
    for (int q = 0; q < 4; ++q) f[12 + q] = log2_err(ne[q] != ne[q] ? raw[11] : ne[q]);
}

template <int D>
__device__ void leaf_feats(const MdasDeviceGrid& g, int leaf, int L, float (&f)[kIn], float* err) {
    float raw[MDAS_RAW_FLOATS], ne[4];
    leaf_raw<D>(g, leaf, raw);
    nbr_errors(g, leaf, L, ne);
    feats_of_raw<D>(g, raw, ne, f);
    if (err) *err = raw[11];
}

__device__ __forceinline__ float target_of(float err) {
    return log2f(fmaxf(err, 1e-30f)) * (1.0f / MDAS_MLP_TARGET_SCALE);
}

// ---- kernels ---------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_forward_rows(const Packed* __restrict__ w, const float* __restrict__ feats,
                                                           int m, float* __restrict__ pred, unsigned* status) {
    Ctx c;
    ctx_open(c, w, status);
    const int tiles = (m + kRows - 1) / kRows;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int r = tile * kRows + threadIdx.x;
        float f[kIn];
#pragma unroll
        for (int i = 0; i < kIn; ++i) f[i] = r < m ? feats[(size_t)r * kIn + i] : 0.0f;
        put_features(c, f);
        float z2[kH];
        tile_forward(c, z2);
        const float p = head(c, z2);
        if (r < m) pred[r] = p;
    }
    ctx_close(c);
}

// Priority of leaves: the plain log2 error (feature 10) plus the network's
// correction.  MODE 0: every leaf; 1: the leaves whose error the last errors
// pass recomputed (the split children of the last adaptive pass: its split
// list and the appended right children); 3: as 1, from the raw rows that
// errors pass wrote (g.featRaw); 2: as 3 (as 1 without rows), or every leaf
// before the first adaptive pass.  Lhost < 0: the leaf count in the device
// counters.
// predMax (may be null): receives the largest priority over all leaves: the
// largest of the rows predicted here, and for the split children only, that
// of the leaves the last adaptive pass kept (*keptMax).
template <int D>
__global__ void __launch_bounds__(kThreads, 4) k_predict_leaves(MdasDeviceGrid g, int Lhost, int mode,
                                                             const Packed* __restrict__ w, float* __restrict__ pred,
                                                             unsigned* predMax, const unsigned* keptMax,
                                                             unsigned* status) {
    Ctx c;
    ctx_open(c, w, status);
    const int L = Lhost >= 0 ? Lhost : g.counts->L;
    const bool dirty = mode == 1 || mode == 3 || (mode == 2 && g.counts->passes > 0);
    unsigned best = 0u;  // order bits of this thread's largest prediction
    if (predMax && dirty && keptMax && blockIdx.x == 0 && threadIdx.x == 0 && *keptMax) atomicMax(predMax, *keptMax);
    const bool rows_raw = dirty && g.featRaw && mode != 1;
    const int newL = g.counts->newL;
    const int rows = dirty ? 2 * newL : L;
    const int tiles = (rows + kRows - 1) / kRows;
    auto leaf_of = [&](int r) { return !dirty ? r : (r < newL ? g.dirty[r] : (L - newL) + (r - newL)); };
    if (rows_raw) {
        // The rows of the errors pass.  While a tile's layer-1 MMA runs, the
        // next tile's row and its neighbours' errors are loaded (that leaf's
        // index came a tile earlier) and the index of the tile after it, so
        // every load has a whole tile's work to arrive.
        const int G = gridDim.x;
        int tile = blockIdx.x;
        int r = tile * kRows + threadIdx.x;
        float raw[MDAS_RAW_FLOATS], ne[4];
        int leaf = 0, leafNext = 0;
        if (tile < tiles && r < rows) {
            load_raw(g.featRaw + (size_t)r * MDAS_RAW_FLOATS, raw);
            leaf = leaf_of(r);
            nbr_errors(g, leaf, L, ne);
        }
        if (tile + G < tiles && r + G * kRows < rows) leafNext = leaf_of(r + G * kRows);
        for (; tile < tiles; tile += G) {
            float f[kIn];
            if (r < rows) feats_of_raw<D>(g, raw, ne, f);
            else
#pragma unroll
                for (int i = 0; i < kIn; ++i) f[i] = 0.0f;
            put_features(c, f);
            const int rNext = r + G * kRows, rNext2 = rNext + G * kRows;
            const bool more = tile + G < tiles && rNext < rows;
            const bool more2 = tile + 2 * G < tiles && rNext2 < rows;
            float rawNext[MDAS_RAW_FLOATS], neNext[4];
            int leafNext2 = 0;
            float z2[kH];
            tile_forward(
                c, z2,
                [&] {
                    if (more) {
                        load_raw(g.featRaw + (size_t)rNext * MDAS_RAW_FLOATS, rawNext);
                        nbr_errors(g, leafNext, L, neNext);
                    }
                    if (more2) leafNext2 = leaf_of(rNext2);
                },
                [] {});
            const float p = head(c, z2);
            if (r < rows) {
                pred[leaf] = f[10] + p;
                best = max(best, mdas_float_order(f[10] + p));
            }
            if (more) {
#pragma unroll
                for (int i = 0; i < MDAS_RAW_FLOATS; ++i) raw[i] = rawNext[i];
#pragma unroll
                for (int q = 0; q < 4; ++q) ne[q] = neNext[q];
                leaf = leafNext;
                leafNext = leafNext2;
            }
            r = rNext;
        }
        if (predMax) {
            best = __reduce_max_sync(0xffffffffu, best);
            if ((threadIdx.x & 31) == 0 && best) atomicMax(predMax, best);
        }
        ctx_close(c);
        return;
    }
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int r = tile * kRows + threadIdx.x;
        const int leaf = leaf_of(r);
        float f[kIn];
        if (r < rows) {
            float raw[MDAS_RAW_FLOATS], ne[4];
            leaf_raw<D>(g, leaf, raw);
            nbr_errors(g, leaf, L, ne);
            feats_of_raw<D>(g, raw, ne, f);
        } else
#pragma unroll
            for (int i = 0; i < kIn; ++i) f[i] = 0.0f;
        put_features(c, f);
        float z2[kH];
        tile_forward(c, z2);
        const float p = head(c, z2);
        if (r < rows) {
            pred[leaf] = f[10] + p;
            best = max(best, mdas_float_order(f[10] + p));
        }
    }
    if (predMax) {
        best = __reduce_max_sync(0xffffffffu, best);
        if ((threadIdx.x & 31) == 0 && best) atomicMax(predMax, best);
    }
    ctx_close(c);
}

// Batched: the learned images' priorities in one launch (one dimension), and
// into each image's predMax the largest (which k_batch_reset started from the
// leaves the last pass kept).
// Tiles of 128 rows are enumerated across the images (each image's rows as in
// mode 2 above); a CTA reloads the weights when its tile belongs to an image
// with other weights.
template <int D>
__global__ void __launch_bounds__(kThreads, 4) k_batch_predict(const MdasBatchImage* __restrict__ imgs, int n,
                                                            unsigned* status) {
    __shared__ int s_pre[257];
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int i = 0; i < n; ++i) {
            s_pre[i] = acc;
            const MdasCounts* cn = imgs[i].g.counts;
            if (imgs[i].mlp && cn->active) acc += ((cn->passes > 0 ? 2 * cn->newL : cn->L) + kRows - 1) / kRows;
        }
        s_pre[n] = acc;
    }
    __syncthreads();
    const int total = s_pre[n];
    const Packed* loaded = nullptr;
    Ctx c;
    ctx_open(c, nullptr, status);
    // A tile: its image, its row of that image's rows, and whether those rows
    // come from the errors pass (split children after the first pass).
    struct TileRows {
        int img, r, rows, L, leaf;
        bool fromRows;
    };
    auto tile_rows = [&](int t) {
        int lo = 0, hi = n - 1;  // the image whose tile range holds t
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_pre[mid] <= t) lo = mid;
            else hi = mid - 1;
        }
        const MdasDeviceGrid& g = imgs[lo].g;
        TileRows tr;
        tr.img = lo;
        tr.L = g.counts->L;
        const bool dirty = g.counts->passes > 0;
        const int newL = g.counts->newL;
        tr.rows = dirty ? 2 * newL : tr.L;
        tr.r = (t - s_pre[lo]) * kRows + threadIdx.x;
        tr.leaf = tr.r >= tr.rows ? 0 : !dirty ? tr.r : (tr.r < newL ? g.dirty[tr.r] : (tr.L - newL) + (tr.r - newL));
        tr.fromRows = dirty && g.featRaw != nullptr;
        return tr;
    };
    // the inputs of the CTA's current tile: rows are loaded while the previous
    // tile's MMAs run (the leaf index and row under layer 1, the neighbours'
    // errors under layer 2); gathered rows (an image's first pass) at the tile
    float raw[MDAS_RAW_FLOATS], ne[4];
    TileRows cur;
    if ((int)blockIdx.x < total) {
        cur = tile_rows(blockIdx.x);
        const MdasDeviceGrid& g = imgs[cur.img].g;
        if (cur.fromRows && cur.r < cur.rows) {
            load_raw(g.featRaw + (size_t)cur.r * MDAS_RAW_FLOATS, raw);
            nbr_errors(g, cur.leaf, cur.L, ne);
        }
    }
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const MdasBatchImage& im = imgs[cur.img];
        const Packed* w = reinterpret_cast<const Packed*>(im.mlp);
        if (w != loaded) {  // no MMA is in flight between tiles
            __syncthreads();
            copy_weights(c.sm, w);
            __syncthreads();
            loaded = w;
        }
        const MdasDeviceGrid& g = im.g;
        float f[kIn];
        if (cur.r < cur.rows) {
            if (!cur.fromRows) {
                leaf_raw<D>(g, cur.leaf, raw);
                nbr_errors(g, cur.leaf, cur.L, ne);
            }
            feats_of_raw<D>(g, raw, ne, f);
        } else
#pragma unroll
            for (int i = 0; i < kIn; ++i) f[i] = 0.0f;
        put_features(c, f);
        const bool more = t + (int)gridDim.x < total;
        TileRows nxt = cur;
        float rawNext[MDAS_RAW_FLOATS], neNext[4];
        float z2[kH];
        tile_forward(
            c, z2,
            [&] {
                if (more) {
                    nxt = tile_rows(t + gridDim.x);
                    if (nxt.fromRows && nxt.r < nxt.rows)
                        load_raw(imgs[nxt.img].g.featRaw + (size_t)nxt.r * MDAS_RAW_FLOATS, rawNext);
                }
            },
            [&] {
                if (more && nxt.fromRows && nxt.r < nxt.rows) nbr_errors(imgs[nxt.img].g, nxt.leaf, nxt.L, neNext);
            });
        const float p = head(c, z2);
        unsigned best = 0u;
        if (cur.r < cur.rows) {
            const_cast<float*>(g.priority)[cur.leaf] = f[10] + p;
            best = mdas_float_order(f[10] + p);
        }
        best = __reduce_max_sync(0xffffffffu, best);  // the tile is one image's
        if ((threadIdx.x & 31) == 0 && best) atomicMax(&g.learned->predMax, best);
        if (more) {
            if (nxt.fromRows && nxt.r < nxt.rows) {
#pragma unroll
                for (int i = 0; i < MDAS_RAW_FLOATS; ++i) raw[i] = rawNext[i];
#pragma unroll
                for (int q = 0; q < 4; ++q) ne[q] = neNext[q];
            }
            cur = nxt;
        }
    }
    ctx_close(c);
}

template <int D>
__global__ void k_leaf_features(MdasDeviceGrid g, int L, float* __restrict__ out) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < L; r += gridDim.x * blockDim.x) {
        float f[kIn];
        leaf_feats<D>(g, r, L, f, nullptr);
#pragma unroll
        for (int i = 0; i < kIn; ++i) out[(size_t)r * kIn + i] = f[i];
    }
}

// Training: persistent CTAs over tiles of 128 rows.  Per tile: forward, then
// dZ2 (CUDA cores), dH1 = dZ2 . W2 on the tensor cores, dZ1; the weight
// gradients of both layers as one more tensor-core GEMM per tile,
//   [dZ2^T ; dZ1^T] (128 x 128 rows) . [H1 | X] (128 rows x 80)
// whose 64 x 64 top-left block is dW2 and 64 x 16 bottom-right block is dW1
// (the other blocks are not used), accumulated in tensor memory over all the
// CTA's tiles; the bias-like gradients as warp reductions into shared memory.
// At the end each CTA adds its gradient to the global one (a few thousand
// atomics per CTA, not per tile).  BF16 operands (dZ rounded like the other
// GEMM inputs), FP32 accumulation.
constexpr int SM_AG = SM_Z2F;            // [dZ2^T ; dZ1^T]: 128 x 128 BF16, K-major, 16 K-blocks per row group
constexpr int SM_BG = SM_Z1F;            // [H1 | X]^T: 80 x 128 BF16, K-major, 16 K-blocks per row group
constexpr int kGradN = kH + kIn;         // 80 columns of the weight-gradient accumulator
constexpr uint32_t kGradCol = 128;       // its first tensor-memory column
constexpr uint32_t kTrainCols = 256;     // tensor-memory columns of a training CTA
constexpr uint32_t kGradIdesc = idesc_bf16(kRows, kGradN);
static_assert(kRows * kRows * 2 <= SM_D - SM_Z2F, "the A tile of the weight gradients fits");
static_assert(kGradN * kRows * 2 <= SM_G - SM_Z1F, "the B tile of the weight gradients fits");
static_assert(kGradCol + kGradN <= kTrainCols, "tensor-memory columns");

template <int D>
__global__ void __launch_bounds__(kThreads) k_gradients(const Packed* __restrict__ w, const float* __restrict__ feats,
                                                        const float* __restrict__ targets, MdasDeviceGrid g, int L,
                                                        int offset, int stride, int m, float* __restrict__ grads,
                                                        float* __restrict__ lossSum, unsigned* status) {
    Ctx c;
    ctx_open(c, w, status, kTrainCols);
    float* sg = reinterpret_cast<float*>(c.sm + SM_G);
    for (int i = threadIdx.x; i < MDAS_MLP_PARAMS; i += kThreads) sg[i] = 0.0f;
    const float* vec = reinterpret_cast<const float*>(c.sm + SM_VEC);
    const float* w3 = vec + 2 * kH;
    uint8_t* ag = c.sm + SM_AG;
    uint8_t* bg = c.sm + SM_BG;
    float* red = reinterpret_cast<float*>(c.sm + SM_RED);
    const int t = threadIdx.x;
    const int warp = t >> 5;
    const int tiles = (m + kRows - 1) / kRows;
    float lossPart = 0.0f;
    bool first = true;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int r = tile * kRows + t;
        const bool valid = r < m;
        float f[kIn];
        float y = 0.0f;
        if (!valid) {
#pragma unroll
            for (int i = 0; i < kIn; ++i) f[i] = 0.0f;
        } else if (feats) {
#pragma unroll
            for (int i = 0; i < kIn; ++i) f[i] = feats[(size_t)r * kIn + i];
            y = targets[r];
        } else {
            const int leaf = (int)(((long long)offset + (long long)r * stride) % L);
            float err;
            leaf_feats<D>(g, leaf, L, f, &err);
            y = target_of(err);
        }
        put_features(c, f);
        float z2[kH];
        tile_forward(c, z2);
        const float e = valid ? head(c, z2) - y : 0.0f;
        const float dpred = 2.0f * e / (float)m;  // 0 on rows past m
        float dz[kH];
        {
            float v[kH];
#pragma unroll
            for (int j = 0; j < kH; ++j) {
                v[j] = dpred * fmaxf(z2[j], 0.0f);
                dz[j] = z2[j] > 0.0f ? dpred * w3[j] : 0.0f;
            }
            warp_sum64(v, red + (0 * 4 + warp) * kH);  // dw3
#pragma unroll
            for (int j = 0; j < kH; ++j) v[j] = dz[j];
            warp_sum64(v, red + (1 * 4 + warp) * kH);  // db2
            float d3 = dpred;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) d3 += __shfl_xor_sync(0xffffffffu, d3, o);
            __syncthreads();  // sg zeroed (first tile); red written
            if ((t & 31) == 0) atomicAdd(&sg[MDAS_MLP_OFF_B3], d3);
        }
#pragma unroll
        for (int kb = 0; kb < kH / 8; ++kb) st_row8(c.sm + SM_D, t, kb, 8, dz + 8 * kb);
        // dH1 = dZ2 . W2 on the tensor cores (B = W2 transposed, K-major)
        run_mma(c, SM_D, SM_W2T, 8, kH / 16);
        float dh[kH];
        tmem_row(c, dh);
        float h1[kH];
#pragma unroll
        for (int kb = 0; kb < kH / 8; ++kb) ld_row8(c.sm + SM_H, t, kb, 8, h1 + 8 * kb);
#pragma unroll
        for (int i = 0; i < kH; ++i) dh[i] = h1[i] > 0.0f ? dh[i] : 0.0f;  // dZ1 (0 on rows past m)
        // the operands of the weight-gradient GEMM, this thread's row r as column r
        // (K) of [dZ2^T ; dZ1^T] and of [H1 | X]^T (the previous tile's GEMM has
        // completed: its wait came before this tile's dH1 GEMM)
        uint16_t* a16 = reinterpret_cast<uint16_t*>(ag);
        uint16_t* b16 = reinterpret_cast<uint16_t*>(bg);
#pragma unroll
        for (int j = 0; j < kH; ++j) {
            a16[core_off(j, t, kRows / 8)] = bf16_bits(dz[j]);
            a16[core_off(kH + j, t, kRows / 8)] = bf16_bits(dh[j]);
            b16[core_off(j, t, kRows / 8)] = bf16_bits(h1[j]);
        }
#pragma unroll
        for (int k = 0; k < kIn; ++k) b16[core_off(kH + k, t, kRows / 8)] = bf16_bits(f[k]);
        warp_sum64(dh, red + (2 * 4 + warp) * kH);  // db1
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (t < kH) {
            float a = 0.0f, b2 = 0.0f, d1 = 0.0f;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                a += red[(0 * 4 + q) * kH + t];
                b2 += red[(1 * 4 + q) * kH + t];
                d1 += red[(2 * 4 + q) * kH + t];
            }
            sg[MDAS_MLP_OFF_W3 + t] += a;
            sg[MDAS_MLP_OFF_B2 + t] += b2;
            sg[MDAS_MLP_OFF_B1 + t] += d1;
        }
        if (t == 0) {
            tc_fence_after();
            const uint32_t sbo = (uint32_t)(kRows / 8) * 128u;
            for (int ks = 0; ks < kRows / 16; ++ks)
                mma_bf16_id(c.tmem + kGradCol, smem_desc(c.base + SM_AG + 256 * ks, 128, sbo),
                            smem_desc(c.base + SM_BG + 256 * ks, 128, sbo), kGradIdesc,
                            (first && ks == 0) ? 0u : 1u);
            mma_commit(c.bar);
        }
        mma_wait(c);
        lossPart += e * e;
        first = false;
    }
    // this CTA's sums into the global gradient
    float l = lossPart;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((t & 31) == 0 && l != 0.0f) atomicAdd(lossSum, l);
    if (!first) {
        // the weight gradients: lane t of the accumulator is row t of [dZ2^T ; dZ1^T] . [H1 | X]
        float acc[kGradN];
        const uint32_t lane = (threadIdx.x & ~31u) << 16;
#pragma unroll
        for (int q = 0; q < kGradN / 16; ++q) tmem_ld16(c.tmem + lane + kGradCol + 16 * q, acc + 16 * q);
        tmem_wait_ld();
        if (t < kH) {
#pragma unroll
            for (int i = 0; i < kH; ++i)
                if (acc[i] != 0.0f) atomicAdd(&grads[MDAS_MLP_OFF_W2 + t * kH + i], acc[i]);
        } else {
#pragma unroll
            for (int k = 0; k < kIn; ++k)
                if (acc[kH + k] != 0.0f) atomicAdd(&grads[MDAS_MLP_OFF_W1 + (t - kH) * kIn + k], acc[kH + k]);
        }
    }
    __syncthreads();
    for (int i = t; i < MDAS_MLP_PARAMS; i += kThreads) {
        const float v = sg[i];
        if (v != 0.0f) atomicAdd(&grads[i], v);
    }
    ctx_close(c);
}

__global__ void k_pack(const float* __restrict__ p, Packed* __restrict__ out) {
    for (int idx = threadIdx.x; idx < kH * kH; idx += blockDim.x) {
        const int j = idx / kH, i = idx % kH;  // W2[j][i]: output j, input i
        const uint16_t b = bf16_bits(p[MDAS_MLP_OFF_W2 + idx]);
        out->w2[core_off(j, i, 8)] = b;
        out->w2t[core_off(i, j, 8)] = b;
        if (idx < kH * kIn) out->w1[core_off(idx / kIn, idx % kIn, 2)] = bf16_bits(p[MDAS_MLP_OFF_W1 + idx]);
        if (idx < kH) {
            out->b1[idx] = p[MDAS_MLP_OFF_B1 + idx];
            out->b2[idx] = p[MDAS_MLP_OFF_B2 + idx];
            out->w3[idx] = p[MDAS_MLP_OFF_W3 + idx];
        }
        if (idx < 4) out->b3[idx] = idx == 0 ? p[MDAS_MLP_OFF_B3] : 0.0f;
    }
}

__global__ void k_adam(float* __restrict__ p, float* __restrict__ m1, float* __restrict__ m2, float* __restrict__ g,
                       int step, float lr) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < MDAS_MLP_PARAMS; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float a = b1 * m1[i] + (1.0f - b1) * gi;
        const float b = b2 * m2[i] + (1.0f - b2) * gi * gi;
        m1[i] = a;
        m2[i] = b;
        p[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
        g[i] = 0.0f;
    }
}

int sm_count() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

template <class K>
cudaError_t set_smem(K kernel, int bytes) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

#define MLP_SWITCH_D(D, CALL)                           \
    switch (D) {                                        \
        case 3: { constexpr int DD = 3; CALL; } break;  \
        case 4: { constexpr int DD = 4; CALL; } break;  \
        case 5: { constexpr int DD = 5; CALL; } break;  \
        case 6: { constexpr int DD = 6; CALL; } break;  \
        default: return cudaErrorInvalidValue;          \
    }

}  // namespace

cudaError_t pack(const float* params, Packed* packed, cudaStream_t s) {
    k_pack<<<1, 1024, 0, s>>>(params, packed);
    return cudaGetLastError();
}

cudaError_t set_test_wait_limit(int polls) {
    const int v = polls > 0 ? polls : 0;
    return cudaMemcpyToSymbol(test_wait_limit, &v, sizeof(int));
}

cudaError_t forward(const Packed* w, const float* features, int m, float* pred, unsigned* status, cudaStream_t s) {
    if (m <= 0) return cudaSuccess;
    cudaError_t e = set_smem(k_forward_rows, kFwdSmem);
    if (e != cudaSuccess) return e;
    const int tiles = (m + kRows - 1) / kRows;
    const int grid = tiles < sm_count() * 4 ? tiles : sm_count() * 4;
    k_forward_rows<<<grid, kThreads, kFwdSmem, s>>>(w, features, m, pred, status);
    return cudaGetLastError();
}

cudaError_t predict_leaves(const MdasDeviceGrid& g, int L, int mode, const Packed* w, float* pred, unsigned* predMax,
                           unsigned* status, cudaStream_t s) {
    if (L == 0) return cudaSuccess;
    const int tiles = L > 0 && mode == 0 ? (L + kRows - 1) / kRows : sm_count() * 4;
    const int grid = tiles < sm_count() * 4 ? tiles : sm_count() * 4;
    cudaError_t e = predMax ? cudaMemsetAsync(predMax, 0, sizeof(unsigned), s) : cudaSuccess;
    if (e != cudaSuccess) return e;
    const unsigned* kept = g.learned ? &g.learned->keptMax : nullptr;
    MLP_SWITCH_D(g.D, (e = set_smem(k_predict_leaves<DD>, kFwdSmem),
                       e == cudaSuccess ? (k_predict_leaves<DD><<<grid, kThreads, kFwdSmem, s>>>(g, L, mode, w, pred,
                                                                                               predMax, kept, status),
                                           0)
                                        : 0));
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

cudaError_t batch_predict(const MdasBatchImage* imgs, int n, int D, unsigned* status, cudaStream_t s) {
    const int grid = sm_count() * 4;
    cudaError_t e = cudaSuccess;
    MLP_SWITCH_D(D, (e = set_smem(k_batch_predict<DD>, kFwdSmem),
                     e == cudaSuccess ? (k_batch_predict<DD><<<grid, kThreads, kFwdSmem, s>>>(imgs, n, status), 0)
                                      : 0));
    return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t leaf_features(const MdasDeviceGrid& g, int L, float* features, cudaStream_t s) {
    if (L <= 0) return cudaSuccess;
    const int grid = (L + 255) / 256 < 4096 ? (L + 255) / 256 : 4096;
    MLP_SWITCH_D(g.D, (k_leaf_features<DD><<<grid, 256, 0, s>>>(g, L, features)));
    return cudaGetLastError();
}

cudaError_t gradients(const Packed* w, const float* features, const float* targets, const MdasDeviceGrid* g, int L,
                      int offset, int stride, int m, float* grads, float* lossSum, unsigned* status, cudaStream_t s) {
    if (m <= 0) return cudaSuccess;
    if (!features && (!g || L <= 0)) return cudaErrorInvalidValue;
    const int tiles = (m + kRows - 1) / kRows;
    MdasDeviceGrid none{};
    none.D = 4;
    const MdasDeviceGrid& gg = g ? *g : none;
    cudaError_t e = cudaSuccess;
    const int grid = tiles < sm_count() ? tiles : sm_count();  // persistent: one CTA per SM (shared memory)
    MLP_SWITCH_D(gg.D, (e = set_smem(k_gradients<DD>, kTrainSmem),
                        e == cudaSuccess ? (k_gradients<DD><<<grid, kThreads, kTrainSmem, s>>>(
                                                w, features, targets, gg, L, offset, stride, m, grads, lossSum, status),
                                            0)
                                         : 0));
    return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t adam(float* params, float* m1, float* m2, float* grads, int step, float lr, Packed* packed,
                 cudaStream_t s) {
    k_adam<<<(MDAS_MLP_PARAMS + 255) / 256, 256, 0, s>>>(params, m1, m2, grads, step, lr);
    k_pack<<<1, 1024, 0, s>>>(params, packed);
    return cudaGetLastError();
}

}  // namespace mdas_mlp
