// mlp.h — the learned leaf priority: a 16 -> 64 -> 64 -> 1 MLP over per-leaf
// features, run on the 5th-generation tensor cores (tcgen05.mma, BF16
// operands in shared memory, FP32 accumulators in tensor memory).
//
// No counterpart in the reference: the reference accepts a leaf with
// probability powf(error / g_error, alpha) (kdgrid.cu:326).  In learned mode
// the error is replaced by an estimate of the leaf's true reconstruction error:
// the plain error times 2^(32 x the MLP's output), the network being trained
// offline on log2(true error / plain error) / 32 against high-sample integrals
// of the leaves; the ratio is that estimate over the largest one.  Every pass
// a judge compares the plain errors each schedule would leave unrefined and
// sends the pass back to the plain acceptance when the learned one leaves more
// than (1 + tolerance) times the plain one's.
#pragma once

#include <stdint.h>
#include <cuda_runtime.h>
#include "grid_types.h"

#define MDAS_MLP_IN 16
#define MDAS_MLP_HIDDEN 64
// flat FP32 parameter vector: W1 [64][16], b1 [64], W2 [64][64], b2 [64], w3 [64], b3
#define MDAS_MLP_OFF_W1 0
#define MDAS_MLP_OFF_B1 (MDAS_MLP_OFF_W1 + MDAS_MLP_HIDDEN * MDAS_MLP_IN)
#define MDAS_MLP_OFF_W2 (MDAS_MLP_OFF_B1 + MDAS_MLP_HIDDEN)
#define MDAS_MLP_OFF_B2 (MDAS_MLP_OFF_W2 + MDAS_MLP_HIDDEN * MDAS_MLP_HIDDEN)
#define MDAS_MLP_OFF_W3 (MDAS_MLP_OFF_B2 + MDAS_MLP_HIDDEN)
#define MDAS_MLP_OFF_B3 (MDAS_MLP_OFF_W3 + MDAS_MLP_HIDDEN)
#ifndef MDAS_MLP_PARAMS
#define MDAS_MLP_PARAMS 5313  // as include/mdas.h declares it
#endif
static_assert(MDAS_MLP_OFF_B3 + 1 == MDAS_MLP_PARAMS, "the layout above fills the parameter vector");
// priorities, network outputs and training targets are log2 quantities / MDAS_MLP_TARGET_SCALE
#define MDAS_MLP_TARGET_SCALE 32.0f

namespace mdas_mlp {

// Weights in the layout the kernels copy to shared memory: BF16 core-matrix
// tiles (8 rows x 8 K-elements, 128 contiguous bytes) of W1 [64 x 16],
// W2 [64 x 64] and W2 transposed, then the FP32 biases and the output layer.
struct Packed {
    uint16_t w1[MDAS_MLP_HIDDEN * MDAS_MLP_IN];
    uint16_t w2[MDAS_MLP_HIDDEN * MDAS_MLP_HIDDEN];
    uint16_t w2t[MDAS_MLP_HIDDEN * MDAS_MLP_HIDDEN];
    float b1[MDAS_MLP_HIDDEN];
    float b2[MDAS_MLP_HIDDEN];
    float w3[MDAS_MLP_HIDDEN];
    float b3[4];
};

// FP32 parameters -> packed copy.
cudaError_t pack(const float* params, Packed* packed, cudaStream_t s);
// pred[i] = MLP(features[i]) for m rows of 16 features (FP32, converted to BF16).
cudaError_t forward(const Packed* w, const float* features, int m, float* pred, unsigned* status, cudaStream_t s);
// Priorities of the grid's leaves: log2(plain error) / 32 plus the network's
// correction, for every leaf (mode 0), the leaves whose error the last errors
// pass recomputed (1: features gathered; 3: from the raw rows that pass wrote
// to g.featRaw), or as 3 unless no adaptive pass ran yet (2; as 1 if
// g.featRaw is null); L < 0: the leaf count in the device counters.  The largest priority over all
// leaves goes to *predMax (order-preserving bits; skipped if null): the largest
// prediction made, and where only the split children were predicted, that of
// the leaves the last adaptive pass kept (g.learned->keptMax, from its decide).
cudaError_t predict_leaves(const MdasDeviceGrid& g, int L, int mode, const Packed* w, float* pred, unsigned* predMax,
                           unsigned* status, cudaStream_t s);
// Batched: the priorities of the active learned images of a batch (all of one
// dimension D), each image's rows as predict_leaves mode 2.
cudaError_t batch_predict(const MdasBatchImage* imgs, int n, int D, unsigned* status, cudaStream_t s);
// Features of the grid's leaves (training data, tests).
cudaError_t leaf_features(const MdasDeviceGrid& g, int L, float* features, cudaStream_t s);
// Adds the gradients of the mean squared error over m rows to grads (FP32,
// MDAS_MLP_PARAMS) and the sum of squared errors to *lossSum.  Rows come from
// features/targets if given, else from the grid's leaves (row r = leaf
// (offset + r * stride) % L, target = its plain log2(error) / MDAS_MLP_TARGET_SCALE).
cudaError_t gradients(const Packed* w, const float* features, const float* targets, const MdasDeviceGrid* g, int L,
                      int offset, int stride, int m, float* grads, float* lossSum, unsigned* status, cudaStream_t s);
// One Adam step (bias-corrected, step >= 1) on params with grads (zeroed
// afterwards), then repacks.
cudaError_t adam(float* params, float* m1, float* m2, float* grads, int step, float lr, Packed* packed,
                 cudaStream_t s);

// Polls after which the MMA waits report a timeout (<= 0: their own limit); a test hook.
cudaError_t set_test_wait_limit(int polls);

}  // namespace mdas_mlp
