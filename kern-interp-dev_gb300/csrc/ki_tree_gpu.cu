// GPU descent codes and their stable radix sort (see ki_tree_gpu.h).
//
// Codes: one thread per point walks `depth` levels, comparing the point
// with each box centre and moving the centre exactly as the host build's
// child construction does (c + side/4 or c - side/4, then side/2: the same
// IEEE operations, so the same boxes).
//
// Sort: least-significant-digit radix sort of the 64-bit codes with the
// point indices as values, 8-bit digits, one pass per digit of the
// dim * depth code bits.  Per pass: tile histograms (2048 keys per CTA),
// an exclusive scan of the (digit, tile) counts in digit-major order (each
// digit's row by one CTA, then the digit totals), and
// a stable scatter in which each warp ranks its keys among equal digits
// with __match_any_sync and the tile's warps and rounds are taken in key
// order.  Ties keep the input order, and the input starts in point order.
#include "ki_launch.cuh"
#include "ki_tree_gpu.h"

#include <algorithm>
#include <stdexcept>
#include <string>
#include <vector>

#include "ki_pool.h"

namespace ki {

namespace {

#define KI_TREE_CUDA(call)                                                                  \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      throw std::runtime_error(std::string("CUDA error (tree): ") + cudaGetErrorString(e_)); \
  } while (0)

constexpr int kRsThreads = 256;
constexpr int kRsWarps = kRsThreads / 32;
constexpr int kRsItems = 8;
constexpr int kRsTile = kRsThreads * kRsItems;
constexpr int kRsBins = 256;
constexpr int kScanThreads = 1024;

__global__ void k_tree_codes(const double* pts, int n, int dim, double c0, double side0,
                             int depth, unsigned long long* codes, int* order) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double p[3], c[3];
  for (int d = 0; d < 3; d++) {
    p[d] = d < dim ? pts[(size_t)dim * i + d] : 0.0;
    c[d] = c0;
  }
  double side = side0;
  unsigned long long code = 0;
  for (int l = 0; l < depth; l++) {
    int ci = 0;
    for (int d = 0; d < dim; d++)
      if (p[d] >= c[d]) ci += 1 << (dim - 1 - d);
    code = (code << dim) | (unsigned long long)ci;
    for (int d = 0; d < dim; d++)
      c[d] = __dadd_rn(c[d], ((ci >> (dim - 1 - d)) & 1) ? side / 4. : -side / 4.);
    side = side / 2.0;
  }
  codes[i] = code;
  order[i] = i;
}

// hist[b * ntile + tile] = keys of the tile whose digit is b
__global__ void k_rs_hist(const unsigned long long* keys, int n, int shift, int ntile,
                          unsigned* hist) {
  __shared__ unsigned h[kRsBins];
  for (int b = threadIdx.x; b < kRsBins; b += blockDim.x) h[b] = 0;
  __syncthreads();
  const int base = blockIdx.x * kRsTile;
  for (int k = 0; k < kRsItems; k++) {
    const int i = base + k * kRsThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(unsigned)(keys[i] >> shift) & (kRsBins - 1)], 1u);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < kRsBins; b += blockDim.x)
    hist[(size_t)b * ntile + blockIdx.x] = h[b];
}

// In-place exclusive scan of each digit's row of tile counts (one CTA per
// digit: per-thread serial sums of contiguous runs, a scan of the run sums,
// then the runs), the row total to tot[digit].
__global__ void k_rs_scan_rows(unsigned* hist, int ntile, unsigned* tot) {
  __shared__ unsigned part[kScanThreads];
  unsigned* a = hist + (size_t)blockIdx.x * ntile;
  const int per = (ntile + blockDim.x - 1) / blockDim.x;
  const int lo = min(ntile, (int)threadIdx.x * per), hi = min(ntile, lo + per);
  unsigned sum = 0;
  for (int i = lo; i < hi; i++) sum += a[i];
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < (int)blockDim.x; o <<= 1) {
    const unsigned v = (int)threadIdx.x >= o ? part[threadIdx.x - o] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  unsigned run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
  for (int i = lo; i < hi; i++) {
    const unsigned v = a[i];
    a[i] = run;
    run += v;
  }
  if (threadIdx.x == blockDim.x - 1) tot[blockIdx.x] = part[threadIdx.x];
}

// Exclusive scan of the kRsBins digit totals (one CTA of kRsBins threads).
__global__ void k_rs_scan_base(unsigned* tot) {
  __shared__ unsigned part[kRsBins];
  const unsigned v0 = tot[threadIdx.x];
  part[threadIdx.x] = v0;
  __syncthreads();
  for (int o = 1; o < kRsBins; o <<= 1) {
    const unsigned v = (int)threadIdx.x >= o ? part[threadIdx.x - o] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  tot[threadIdx.x] = part[threadIdx.x] - v0;
}

// Stable scatter of one tile: rounds of 256 keys in key order; in a round,
// warp w's keys follow warps 0..w-1's, and a lane's rank among its warp's
// equal digits comes from __match_any_sync.
__global__ void k_rs_scatter(const unsigned long long* keys, const int* vals, int n, int shift,
                             int ntile, const unsigned* offs, const unsigned* dbase,
                             unsigned long long* okeys, int* ovals) {
  __shared__ unsigned run[kRsBins];
  __shared__ unsigned wcnt[kRsWarps][kRsBins];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int b = threadIdx.x; b < kRsBins; b += blockDim.x)
    run[b] = dbase[b] + offs[(size_t)b * ntile + blockIdx.x];
  const int base = blockIdx.x * kRsTile;
  for (int k = 0; k < kRsItems; k++) {
    for (int e = threadIdx.x; e < kRsWarps * kRsBins; e += blockDim.x) (&wcnt[0][0])[e] = 0;
    __syncthreads();
    const int i = base + k * kRsThreads + threadIdx.x;
    const bool on = i < n;
    const unsigned long long key = on ? keys[i] : 0ull;
    // lanes past the end share a digit outside 0..255 and write nothing
    const unsigned d = on ? ((unsigned)(key >> shift) & (kRsBins - 1)) : (unsigned)kRsBins;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    if (on && rank == 0) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    for (int b = threadIdx.x; b < kRsBins; b += blockDim.x) {
      unsigned r = run[b];
      for (int w = 0; w < kRsWarps; w++) {
        const unsigned c = wcnt[w][b];
        wcnt[w][b] = r;
        r += c;
      }
      run[b] = r;
    }
    __syncthreads();
    if (on) {
      const unsigned pos = wcnt[warp][d] + (unsigned)rank;
      okeys[pos] = key;
      ovals[pos] = vals[i];
    }
    __syncthreads();
  }
}

}  // namespace

void tree_codes_sorted(const double* d_points, int n, int dim, double centre, double side,
                       int depth, uint64_t* h_codes, int* h_order, cudaStream_t s) {
  if (n <= 0) return;
  if ((dim != 2 && dim != 3) || depth < 1 || dim * depth > 64)
    throw std::invalid_argument("tree codes: bad dimension or depth");
  const int ntile = (n + kRsTile - 1) / kRsTile;
  unsigned long long* keys[2] = {nullptr, nullptr};
  int* vals[2] = {nullptr, nullptr};
  unsigned* hist = nullptr;
  std::vector<void*> owned;
  auto take = [&](size_t bytes) {
    void* p = nullptr;
    KI_TREE_CUDA(pool_malloc(&p, bytes, s));
    owned.push_back(p);
    return p;
  };
  try {
    for (int b = 0; b < 2; b++) {
      keys[b] = (unsigned long long*)take(sizeof(unsigned long long) * n);
      vals[b] = (int*)take(sizeof(int) * n);
    }
    hist = (unsigned*)take(sizeof(unsigned) * ((size_t)kRsBins * ntile + kRsBins));
    unsigned* tot = hist + (size_t)kRsBins * ntile;
    ki::launch(k_tree_codes, (n + 255) / 256, 256, 0, s, d_points, n, dim, centre, side, depth, keys[0],
                                                 vals[0]);
    KI_TREE_CUDA(cudaGetLastError());
    const int bits = dim * depth;
    int cur = 0;
    for (int shift = 0; shift < bits; shift += 8) {
      ki::launch(k_rs_hist, ntile, kRsThreads, 0, s, keys[cur], n, shift, ntile, hist);
      ki::launch(k_rs_scan_rows, kRsBins, 256, 0, s, hist, ntile, tot);
      ki::launch(k_rs_scan_base, 1, kRsBins, 0, s, tot);
      ki::launch(k_rs_scatter, ntile, kRsThreads, 0, s, keys[cur], vals[cur], n, shift, ntile, hist, tot,
                                                keys[1 - cur], vals[1 - cur]);
      KI_TREE_CUDA(cudaGetLastError());
      cur = 1 - cur;
    }
    KI_TREE_CUDA(cudaMemcpyAsync(h_codes, keys[cur], sizeof(uint64_t) * n,
                                 cudaMemcpyDeviceToHost, s));
    KI_TREE_CUDA(cudaMemcpyAsync(h_order, vals[cur], sizeof(int) * n, cudaMemcpyDeviceToHost, s));
    KI_TREE_CUDA(cudaStreamSynchronize(s));
  } catch (...) {
    for (void* p : owned) cudaFreeAsync(p, s);
    throw;
  }
  for (void* p : owned) KI_TREE_CUDA(cudaFreeAsync(p, s));
}

}  // namespace ki
