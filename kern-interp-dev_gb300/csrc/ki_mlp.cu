// Rank-predictor MLP (see ki_mlp.h): forward, backward and Adam kernels.
// Every reduction over samples is a fixed-order two-pass sum, so training is
// deterministic for a given input.
#include "ki_launch.cuh"
#include "ki_mlp.h"

#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "ki_pool.h"

namespace ki {

namespace {

#define KI_MLP_CUDA(call)                                                                  \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      throw std::runtime_error(std::string("CUDA error (mlp): ") + cudaGetErrorString(e_)); \
  } while (0)

constexpr int H = kMlpHidden, F = kMlpIn;
constexpr int kMean = kMlpMean, kScale = kMlpScale, kW1 = kMlpW1, kB1 = kMlpB1, kW2 = kMlpW2,
              kB2 = kMlpB2, kW3 = kMlpW3, kB3 = kMlpB3;

constexpr int kParts = 64;   // sample chunks of the two-pass reductions

// Forward pass of every sample; keeps the hidden activations for backward.
__global__ void k_mlp_fwd(const float* model, const float* x, int n, float* h1, float* h2,
                          float* out) {
  __shared__ float sm[kMlpModelFloats];
  for (int e = threadIdx.x; e < kMlpModelFloats; e += blockDim.x) sm[e] = model[e];
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float xn[F];
  for (int f = 0; f < F; f++) xn[f] = (x[(size_t)i * F + f] - sm[kMean + f]) / sm[kScale + f];
  float a1[H];
  for (int k = 0; k < H; k++) {
    float z = sm[kB1 + k];
    for (int f = 0; f < F; f++) z += sm[kW1 + k * F + f] * xn[f];
    a1[k] = z > 0.f ? z : 0.f;
    if (h1) h1[(size_t)i * H + k] = a1[k];
  }
  float zo = sm[kB3];
  for (int j = 0; j < H; j++) {
    float z = sm[kB2 + j];
    for (int k = 0; k < H; k++) z += sm[kW2 + j * H + k] * a1[k];
    const float a = z > 0.f ? z : 0.f;
    if (h2) h2[(size_t)i * H + j] = a;
    zo += sm[kW3 + j] * a;
  }
  out[i] = 1.f / (1.f + expf(-zo));
}

// Per-sample backward: dO = dL/dz_out, G2 = dL/dz2, G1 = dL/dz1 (loss: mean
// squared error over n samples); also the squared errors for the loss.
__global__ void k_mlp_bwd_samples(const float* model, const float* y, int n, const float* h1,
                                  const float* h2, const float* out, float* dO, float* g2,
                                  float* g1, float* sqerr) {
  __shared__ float sm[kMlpModelFloats];
  for (int e = threadIdx.x; e < kMlpModelFloats; e += blockDim.x) sm[e] = model[e];
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float o = out[i], err = o - y[i];
  sqerr[i] = err * err;
  const float d = 2.f * err / (float)n * o * (1.f - o);
  dO[i] = d;
  float gz2[H];
  for (int j = 0; j < H; j++) {
    gz2[j] = h2[(size_t)i * H + j] > 0.f ? d * sm[kW3 + j] : 0.f;
    g2[(size_t)i * H + j] = gz2[j];
  }
  for (int k = 0; k < H; k++) {
    float s = 0.f;
    for (int j = 0; j < H; j++) s += gz2[j] * sm[kW2 + j * H + k];
    g1[(size_t)i * H + k] = h1[(size_t)i * H + k] > 0.f ? s : 0.f;
  }
}

// part[z][a * q + b] = sum over the samples of chunk z of A[i][a] * B[i][b]
// (B null: a column of ones).  A: n x p, B: n x q, row-major.
__global__ void k_outer_partial(const float* A, int p, const float* B, int q, int n, float* part) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  const int qq = B ? q : 1;
  if (o >= p * qq) return;
  const int a = o / qq, b = o % qq;
  const int z = blockIdx.y;
  const int chunk = (n + kParts - 1) / kParts;
  const int i0 = z * chunk, i1 = min(n, i0 + chunk);
  float s = 0.f;
  for (int i = i0; i < i1; i++) s += A[(size_t)i * p + a] * (B ? B[(size_t)i * q + b] : 1.f);
  part[(size_t)z * p * qq + o] = s;
}

__global__ void k_outer_final(const float* part, int count, float* g) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= count) return;
  float s = 0.f;
  for (int z = 0; z < kParts; z++) s += part[(size_t)z * count + o];
  g[o] = s;
}

__global__ void k_standardize(const float* model, const float* x, int n, float* xn) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * F) return;
  const int f = e % F;
  xn[e] = (x[e] - model[kMean + f]) / model[kScale + f];
}

// Adam on the trainable entries (the normalization stays fixed).
__global__ void k_adam(float* model, const float* g, float* m1, float* m2, float lr, float b1,
                       float b2, float c1, float c2) {
  const int e = kW1 + blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= kMlpModelFloats) return;
  const float gr = g[e];
  const float a = b1 * m1[e] + (1.f - b1) * gr;
  const float v = b2 * m2[e] + (1.f - b2) * gr * gr;
  m1[e] = a;
  m2[e] = v;
  model[e] -= lr * (a / c1) / (sqrtf(v / c2) + 1e-8f);
}

struct Work {
  float *h1, *h2, *out, *dO, *g2, *g1, *sq, *xn, *part, *grad;
  std::vector<void*> owned;
  cudaStream_t s;
  Work(int n, cudaStream_t st) : s(st) {
    auto take = [&](size_t floats) {
      void* p = nullptr;
      KI_MLP_CUDA(pool_malloc(&p, sizeof(float) * (floats ? floats : 1), s));
      owned.push_back(p);
      return (float*)p;
    };
    h1 = take((size_t)n * H);
    h2 = take((size_t)n * H);
    out = take(n);
    dO = take(n);
    g2 = take((size_t)n * H);
    g1 = take((size_t)n * H);
    sq = take(n);
    xn = take((size_t)n * F);
    part = take((size_t)kParts * H * H);
    grad = take(kMlpModelFloats);
  }
  ~Work() {
    for (void* p : owned) cudaFreeAsync(p, s);
  }
};

float loss_grad(Work& w, const float* model, const float* x, const float* y, int n) {
  cudaStream_t s = w.s;
  const int nb = (n + 127) / 128;
  ki::launch(k_mlp_fwd, nb, 128, 0, s, model, x, n, w.h1, w.h2, w.out);
  ki::launch(k_mlp_bwd_samples, nb, 128, 0, s, model, y, n, w.h1, w.h2, w.out, w.dO, w.g2, w.g1, w.sq);
  ki::launch(k_standardize, (n * F + 255) / 256, 256, 0, s, model, x, n, w.xn);
  KI_MLP_CUDA(cudaMemsetAsync(w.grad, 0, sizeof(float) * kMlpModelFloats, s));
  auto outer = [&](const float* A, int p, const float* B, int q, float* g) {
    const int cnt = p * (B ? q : 1);
    ki::launch(k_outer_partial, dim3((cnt + 127) / 128, kParts), 128, 0, s, A, p, B, q, n, w.part);
    ki::launch(k_outer_final, (cnt + 127) / 128, 128, 0, s, w.part, cnt, g);
  };
  outer(w.g1, H, w.xn, F, w.grad + kW1);     // dW1[k][f] = sum G1[i][k] xn[i][f]
  outer(w.g1, H, nullptr, 1, w.grad + kB1);  // db1
  outer(w.g2, H, w.h1, H, w.grad + kW2);     // dW2[j][k] = sum G2[i][j] h1[i][k]
  outer(w.g2, H, nullptr, 1, w.grad + kB2);  // db2
  outer(w.dO, 1, w.h2, H, w.grad + kW3);     // dW3[j] = sum dO[i] h2[i][j]
  outer(w.dO, 1, nullptr, 1, w.grad + kB3);  // db3
  outer(w.sq, 1, nullptr, 1, w.part + (size_t)kParts * H * H - 1);   // loss * n (scratch)
  KI_MLP_CUDA(cudaGetLastError());
  float lsum = 0.f;
  KI_MLP_CUDA(cudaMemcpyAsync(&lsum, w.part + (size_t)kParts * H * H - 1, sizeof(float),
                              cudaMemcpyDeviceToHost, s));
  KI_MLP_CUDA(cudaStreamSynchronize(s));
  return lsum / (float)n;
}

}  // namespace

void mlp_loss_grad(const float* d_model, const float* d_x, const float* d_y, int n, float* d_grad,
                   float* loss, cudaStream_t s) {
  if (n <= 0) throw std::invalid_argument("mlp: no samples");
  Work w(n, s);
  *loss = loss_grad(w, d_model, d_x, d_y, n);
  KI_MLP_CUDA(cudaMemcpyAsync(d_grad, w.grad, sizeof(float) * kMlpModelFloats,
                              cudaMemcpyDeviceToDevice, s));
  KI_MLP_CUDA(cudaStreamSynchronize(s));
}

float mlp_train(float* d_model, const float* d_x, const float* d_y, int n, int epochs, float lr,
                cudaStream_t s) {
  if (n <= 0) throw std::invalid_argument("mlp: no samples");
  Work w(n, s);
  float* mom = nullptr;
  KI_MLP_CUDA(pool_malloc((void**)&mom, sizeof(float) * 2 * kMlpModelFloats, s));
  KI_MLP_CUDA(cudaMemsetAsync(mom, 0, sizeof(float) * 2 * kMlpModelFloats, s));
  const float b1 = 0.9f, b2 = 0.999f;
  float c1 = 1.f, c2 = 1.f, loss = 0.f;
  for (int ep = 0; ep < epochs; ep++) {
    loss = loss_grad(w, d_model, d_x, d_y, n);
    c1 *= b1;
    c2 *= b2;
    ki::launch(k_adam, (kMlpModelFloats - kW1 + 255) / 256, 256, 0, s, d_model, w.grad, mom,
                                                               mom + kMlpModelFloats, lr, b1, b2,
                                                               1.f - c1, 1.f - c2);
    KI_MLP_CUDA(cudaGetLastError());
  }
  loss = loss_grad(w, d_model, d_x, d_y, n);
  KI_MLP_CUDA(cudaFreeAsync(mom, s));
  return loss;
}

void mlp_predict(const float* d_model, const float* d_x, int n, float* d_out, cudaStream_t s) {
  if (n <= 0) return;
  ki::launch(k_mlp_fwd, (n + 127) / 128, 128, 0, s, d_model, d_x, n, nullptr, nullptr, d_out);
  KI_MLP_CUDA(cudaGetLastError());
}

}  // namespace ki
