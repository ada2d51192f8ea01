// Rank-predictor MLP (see ki_mlp.h): forward, backward and Adam kernels.
// Every reduction over samples is a fixed-order two-pass sum, so training is
// deterministic for a given input.
#include "ki_launch.cuh"
#include "ki_mlp.h"
#include "ki_tc.cuh"

#include <cuda_bf16.h>

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

namespace {

// ------------------------------------------- BF16 inference on tensor cores --
// 128 samples per CTA, one per thread: the standardized features (12, padded
// to K = 16) and the hidden activations are BF16 operand tiles in shared
// memory, the weights BF16 tiles, the two layers tcgen05 MMAs (kind::f16,
// M = 128, N = 64) into FP32 TMEM accumulators; biases, ReLU and the output
// layer in FP32 on the CUDA cores.
constexpr int kTcSamples = 128;
constexpr uint32_t kSbo16 = 256;    // 8-row groups of a K = 16 tile (two core matrices)
constexpr uint32_t kSbo64 = 1024;   // K = 64 (eight core matrices)
constexpr uint32_t kOffX = 0, kOffW1 = kOffX + kTcSamples * 32, kOffH = kOffW1 + kMlpHidden * 32,
                   kOffW2 = kOffH + kTcSamples * 128, kOffPar = kOffW2 + kMlpHidden * 128,
                   kOffBar = kOffPar + 1024, kTcSmem = kOffBar + 16;
// bounded waits for the MMAs (SM cycles): far above their microseconds
constexpr long long kMlpWaitCycles = 200000000LL;

__device__ __forceinline__ void put_bf16(unsigned char* tile, int row, int k, uint32_t sbo, float v) {
  *reinterpret_cast<__nv_bfloat16*>(tile + tc::kmajor_offset_bf16(row, k, sbo)) = __float2bfloat16_rn(v);
}

__global__ void __launch_bounds__(kTcSamples) k_mlp_tc(const float* model, const float* x, int n,
                                                       float* out, int* err) {
  extern __shared__ __align__(128) unsigned char tsm[];
  unsigned char* Xs = tsm + kOffX;
  unsigned char* W1s = tsm + kOffW1;
  unsigned char* Hs = tsm + kOffH;
  unsigned char* W2s = tsm + kOffW2;
  float* b1 = reinterpret_cast<float*>(tsm + kOffPar);
  float* b2 = b1 + kMlpHidden;
  float* w3 = b2 + kMlpHidden;
  uint64_t* bar = reinterpret_cast<uint64_t*>(tsm + kOffBar);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(tsm + kOffBar + 8);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int i = blockIdx.x * kTcSamples + tid;
  for (int e = tid; e < kMlpHidden; e += blockDim.x) {
    b1[e] = model[kMlpB1 + e];
    b2[e] = model[kMlpB2 + e];
    w3[e] = model[kMlpW3 + e];
  }
  for (int k = 0; k < 16; k++) {
    float v = 0.f;
    if (i < n && k < kMlpIn) v = (x[(size_t)i * kMlpIn + k] - model[kMlpMean + k]) / model[kMlpScale + k];
    put_bf16(Xs, tid, k, kSbo16, v);
  }
  for (int e = tid; e < kMlpHidden * 16; e += blockDim.x) {
    const int j = e / 16, k = e % 16;
    put_bf16(W1s, j, k, kSbo16, k < kMlpIn ? model[kMlpW1 + j * kMlpIn + k] : 0.f);
  }
  for (int e = tid; e < kMlpHidden * kMlpHidden; e += blockDim.x) {
    const int j = e / kMlpHidden, k = e % kMlpHidden;
    put_bf16(W2s, j, k, kSbo64, model[kMlpW2 + j * kMlpHidden + k]);
  }
  if (warp == 0) tc::tmem_alloc(tslot, 128);
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    tc::fence_mbar_init();
  }
  tc::fence_proxy_async_smem();   // the operand tiles, visible to the tensor core
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = tc::idesc_bf16(kTcSamples, kMlpHidden);
  // layer 1: D1 (TMEM columns 0-63) = X W1^T
  if (tid == 0) {
    tc::mma_bf16(tmem, tc::smem_desc(tc::smem_u32(Xs), tc::kLbo, kSbo16),
                 tc::smem_desc(tc::smem_u32(W1s), tc::kLbo, kSbo16), idesc, 0);
    tc::mma_commit(bar);
  }
  bool ok = tc::mbar_wait(bar, 0, kMlpWaitCycles);
  tc::fence_after_sync();
  const uint32_t lane_base = (uint32_t)(32 * warp) << 16;
  float v[16];
  if (ok) {
    for (int c = 0; c < kMlpHidden; c += 16) {
      tc::tmem_ld16(tmem + lane_base + c, v);
      for (int q = 0; q < 16; q++) {
        const float z = v[q] + b1[c + q];
        put_bf16(Hs, tid, c + q, kSbo64, z > 0.f ? z : 0.f);
      }
    }
  }
  tc::fence_proxy_async_smem();
  tc::fence_before_sync();
  const bool ok1 = __syncthreads_and(ok);
  tc::fence_after_sync();
  // layer 2: D2 (columns 64-127) = H W2^T, four K = 16 steps
  if (ok1 && tid == 0) {
    for (int j = 0; j < kMlpHidden / 16; j++)
      tc::mma_bf16(tmem + 64, tc::smem_desc(tc::smem_u32(Hs) + 256u * j, tc::kLbo, kSbo64),
                   tc::smem_desc(tc::smem_u32(W2s) + 256u * j, tc::kLbo, kSbo64), idesc, j > 0);
    tc::mma_commit(bar);
  }
  ok = ok1 && tc::mbar_wait(bar, 1, kMlpWaitCycles);
  tc::fence_after_sync();
  float zo = model[kMlpB3];
  if (ok) {
    for (int c = 0; c < kMlpHidden; c += 16) {
      tc::tmem_ld16(tmem + lane_base + 64 + c, v);
      for (int q = 0; q < 16; q++) {
        const float z = v[q] + b2[c + q];
        zo += w3[c + q] * (z > 0.f ? z : 0.f);
      }
    }
  }
  ok = __syncthreads_and(ok);
  if (!ok) {
    // a wait gave up: wait (bounded again) for the last MMA group issued
    // before the accumulators are freed, and report
    if (tid == 0) atomicMax(err, 3);
    tc::mbar_wait(bar, ok1 ? 1 : 0, kMlpWaitCycles);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 128);
  if (ok && i < n) out[i] = 1.f / (1.f + expf(-zo));
}

}  // namespace

void mlp_predict_bf16(const float* d_model, const float* d_x, int n, float* d_out, int* d_err,
                      cudaStream_t s) {
  if (n <= 0) return;
  ki::launch(k_mlp_tc, (n + kTcSamples - 1) / kTcSamples, kTcSamples, kTcSmem, s, d_model, d_x, n,
             d_out, d_err);
  KI_MLP_CUDA(cudaGetLastError());
}

void mlp_predict(const float* d_model, const float* d_x, int n, float* d_out, cudaStream_t s) {
  if (n <= 0) return;
  ki::launch(k_mlp_fwd, (n + 127) / 128, 128, 0, s, d_model, d_x, n, nullptr, nullptr, d_out);
  KI_MLP_CUDA(cudaGetLastError());
}

}  // namespace ki
