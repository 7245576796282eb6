// mlp.h — the learned leaf priority: a 16 -> 64 -> 64 -> 1 MLP over per-leaf
// features, run on the 5th-generation tensor cores (tcgen05.mma, BF16
// operands in shared memory, FP32 accumulators in tensor memory).
//
// No counterpart in the reference: the reference accepts a leaf with
// probability powf(error / g_error, alpha) (kdgrid.cu:326).  In learned mode
// the ratio comes from the MLP's predicted error instead, except on a fixed
// hashed fraction of the leaves, which keep the plain error; the plain error is
// also the training target, so it judges the model every pass.
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
#define MDAS_MLP_PARAMS (MDAS_MLP_OFF_B3 + 1)  // 5313
// the target and the prediction are log2(error) / MDAS_MLP_TARGET_SCALE
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
// Predictions for the grid's leaves [0, L) from their own features.
cudaError_t predict_leaves(const MdasDeviceGrid& g, int L, const Packed* w, float* pred, unsigned* status,
                           cudaStream_t s);
// Features of the grid's leaves (for tests and callers that train elsewhere).
cudaError_t leaf_features(const MdasDeviceGrid& g, int L, float* features, cudaStream_t s);
// Adds the gradients of the mean squared error over m rows to grads (FP32,
// MDAS_MLP_PARAMS) and the sum of squared errors to *lossSum.  Rows come from
// features/targets if given, else from the grid's leaves (row r = leaf
// (offset + r * stride) % L, target = log2(error) / MDAS_MLP_TARGET_SCALE).
cudaError_t gradients(const Packed* w, const float* features, const float* targets, const MdasDeviceGrid* g, int L,
                      int offset, int stride, int m, float* grads, float* lossSum, unsigned* status, cudaStream_t s);
// One Adam step (bias-corrected, step >= 1) on params with grads (zeroed
// afterwards), then repacks.
cudaError_t adam(float* params, float* m1, float* m2, float* grads, int step, float lr, Packed* packed,
                 cudaStream_t s);

}  // namespace mdas_mlp
