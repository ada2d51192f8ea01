// Learned skeleton-rank predictor: a 12 -> 64 -> 64 -> 1 multilayer
// perceptron (ReLU hidden layers, logistic output) on per-box features,
// predicting the rank fraction k / n of a box's interpolative decomposition.
// Trained and evaluated in FP32 by this file's own CUDA kernels.
//
// Model blob (floats): feature mean (12) | feature scale (12) | W1 (64 x 12) |
// b1 (64) | W2 (64 x 64) | b2 (64) | W3 (64) | b3 (1).  Inputs are
// standardized as (x - mean) / scale before the first layer.
#pragma once

#include <cuda_runtime.h>

namespace ki {

constexpr int kMlpIn = 12;
constexpr int kMlpHidden = 64;
// offsets into the model blob
constexpr int kMlpMean = 0, kMlpScale = kMlpIn, kMlpW1 = 2 * kMlpIn,
              kMlpB1 = kMlpW1 + kMlpHidden * kMlpIn, kMlpW2 = kMlpB1 + kMlpHidden,
              kMlpB2 = kMlpW2 + kMlpHidden * kMlpHidden, kMlpW3 = kMlpB2 + kMlpHidden,
              kMlpB3 = kMlpW3 + kMlpHidden;
constexpr int kMlpModelFloats = kMlpB3 + 1;

// Forward pass of one sample (device; `m` may point to shared memory).
__device__ __forceinline__ float mlp_forward_one(const float* m, const float* x) {
  float xn[kMlpIn];
  for (int f = 0; f < kMlpIn; f++) xn[f] = (x[f] - m[kMlpMean + f]) / m[kMlpScale + f];
  float a1[kMlpHidden];
  for (int k = 0; k < kMlpHidden; k++) {
    float z = m[kMlpB1 + k];
    for (int f = 0; f < kMlpIn; f++) z += m[kMlpW1 + k * kMlpIn + f] * xn[f];
    a1[k] = z > 0.f ? z : 0.f;
  }
  float zo = m[kMlpB3];
  for (int j = 0; j < kMlpHidden; j++) {
    float z = m[kMlpB2 + j];
    for (int k = 0; k < kMlpHidden; k++) z += m[kMlpW2 + j * kMlpHidden + k] * a1[k];
    zo += m[kMlpW3 + j] * (z > 0.f ? z : 0.f);
  }
  return 1.f / (1.f + expf(-zo));
}

// Host drivers (device buffers unless noted).
// Mean-squared-error loss and its gradient over a batch: grad (kMlpModelFloats,
// the normalization entries stay zero), loss (host).
void mlp_loss_grad(const float* d_model, const float* d_x, const float* d_y, int n, float* d_grad,
                   float* loss, cudaStream_t s);
// Full-batch Adam training (model updated in place); returns the final loss.
float mlp_train(float* d_model, const float* d_x, const float* d_y, int n, int epochs, float lr,
                cudaStream_t s);
// Predictions for n samples.
void mlp_predict(const float* d_model, const float* d_x, int n, float* d_out, cudaStream_t s);
// The same in BF16 on the tensor cores (tcgen05, FP32 accumulation; the
// factorization's inference): 128 samples per CTA.  A bounded MMA wait that
// gives up sets *d_err to 3 and leaves those outputs unwritten.
void mlp_predict_bf16(const float* d_model, const float* d_x, int n, float* d_out, int* d_err,
                      cudaStream_t s);

}  // namespace ki
