// order.h — Morton keys of points and leaves, LSD radix sort (one sweep per
// digit), Karras radix-tree hierarchy over the sorted leaves and point location.
//
// None of this has a counterpart in the reference; it must not change MDAS
// results (the kernels only read the grid).  The key numbering extends the
// reference's initial-cell numbering (uniformSamplingKernel, kdgrid.cu:144-160)
// to finer cells, so the top bits of a key are the index of the initial cell
// that holds the point.
#pragma once

#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime.h>
#include "grid_types.h"

namespace mdas_order {

// Bits of a key at `fineBits` extra bits per dimension, or -1 if that exceeds 64.
int key_bits(int D, int bitsPerDim, int extraImgBits, int fineBits);
// The largest fineBits whose keys fit in 64 bits (-1 if none).
int max_fine_bits(int D, int bitsPerDim, int extraImgBits);

cudaError_t morton_encode(const float* points, int n, int D, int bitsPerDim, int extraImgBits, int fineBits,
                          float scaleX, float scaleY, uint64_t* keys, cudaStream_t s);
cudaError_t morton_decode(const uint64_t* cells, int n, int D, int bitsPerDim, int extraImgBits, float scaleX,
                          float scaleY, float* boxes, cudaStream_t s);
// keys of the grid's leaves [0, L): the key of each leaf's box centre
cudaError_t leaf_keys(const MdasDeviceGrid& g, int L, int fineBits, uint64_t* keys, cudaStream_t s);

// Stable LSD radix sort of (key, value) pairs on bits [beginBit, endBit) of the
// keys; valuesIn == nullptr sorts the values 0..n-1.  `status` (device, one
// word in the temp block) is nonzero after the call if a look-back wait gave up.
size_t sort_temp_bytes(int n, int beginBit, int endBit);
cudaError_t radix_sort(void* temp, size_t tempBytes, const uint64_t* keysIn, uint64_t* keysOut,
                       const uint32_t* valuesIn, uint32_t* valuesOut, int n, int beginBit, int endBit,
                       cudaStream_t s, unsigned** status);
// Launches of one radix_sort call (for launch counts).
int sort_launches(int n, int beginBit, int endBit);

// Karras radix tree over n sorted keys: internal nodes [0, n-1), root 0;
// children[i] = (left, right), a child c >= 0 is internal node c and c < 0 is
// the leaf at sorted position ~c; parents[0, n-1) of internal nodes,
// parents[n-1 + p] of the leaf at sorted position p; parent of the root = -1.
cudaError_t karras_build(const uint64_t* sortedKeys, int n, int2* children, int* parents, cudaStream_t s);
// Boxes of the internal nodes (2D floats each: mn, mx), unions of their
// children's; leaf p's box is the box of grid leaf order[p].  visits: n-1
// counters (zeroed here).
cudaError_t karras_refit(const MdasDeviceGrid& g, const uint32_t* order, int n, const int2* children,
                         const int* parents, unsigned* visits, float* boxes, cudaStream_t s);
// For each point, the grid leaf whose box holds it (mn <= p < mx per
// dimension, p <= mx on the domain's upper faces); the first in key order if
// several do, -1 if none.  perm (may be null): the order in which threads take
// the points (a permutation of 0..m-1).  status: set nonzero if a traversal
// stack overflowed or perm held an index out of range.
cudaError_t locate(const MdasDeviceGrid& g, const uint32_t* order, int n, const int2* children,
                   const float* boxes, const float* points, int m, const uint32_t* perm, int* leaves,
                   unsigned* status, cudaStream_t s);
// Extra bits per dimension of the coarse keys that order the queries of a
// large point location (the keys then fit in 32 bits where the grid allows).
int query_fine_bits(int D, int bitsPerDim, int extraImgBits);

// Polls of the sort's look-back before it gives up (<= 0: its own limit); a test hook.
void set_test_wait_limit(int polls);

}  // namespace mdas_order
