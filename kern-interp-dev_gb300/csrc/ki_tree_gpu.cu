// The tree on the GPU: descent codes, their stable radix sort, boxes level
// by level, neighbour lists and leaf DOF lists (see ki_tree_gpu.h).
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
#include "ki_tree.h"
#include "ki_parallel.h"

#include <algorithm>
#include <stdexcept>
#include <string>
#include <tuple>
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


// ----------------------------------------------------- the tree on the GPU --
// One level of boxes: point ranges [lo, hi) of the sorted codes, centres.
// Boxes of level l have global ids base_l + index (level-major, children of
// consecutive parents consecutive: the host build's numbering).

// flag[i] = box i of the level splits (holds more than max_leaf_dofs DOFs)
__global__ void k_tree_split_flags(const int* lo, const int* hi, int nbox, int sol_dim, int max_leaf,
                                   int* flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nbox) flag[i] = (hi[i] - lo[i]) * sol_dim > max_leaf ? 1 : 0;
}

// Exclusive scan of n ints by one CTA (rank[i]; rank[n] = total).
__global__ void __launch_bounds__(1024) k_tree_scan(const int* flag, int n, int* rank) {
  __shared__ int part[1024];
  const int t = threadIdx.x, T = blockDim.x;
  const int per = (n + T - 1) / T;
  const int b0 = t * per, b1 = min(n, b0 + per);
  int s = 0;
  for (int i = b0; i < b1; i++) s += flag[i];
  part[t] = s;
  __syncthreads();
  for (int o = 1; o < T; o <<= 1) {
    const int v = t >= o ? part[t - o] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int run = part[t] - s;
  for (int i = b0; i < b1; i++) {
    rank[i] = run;
    run += flag[i];
  }
  if (t == T - 1) rank[n] = part[t];
}

// Children of the splitting boxes of a level: child ranges by binary search
// on the level's code digit, centres c +- side/4 (QuadTree::node_subdivide,
// quadtree.cpp:377-388), the parents' child ids.
__global__ void k_tree_children(const unsigned long long* codes, const int* lo, const int* hi,
                                const double* cen, int nbox, const int* flag, const int* rank,
                                int dim, int shift, double side, int next_base, int* child,
                                int* nlo, int* nhi, double* ncen, int* nparent, int base) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbox || !flag[i]) return;
  const int nch = 1 << dim;
  const int r = rank[i];
  int st = lo[i];
  const int h = hi[i];
  for (int ci = 0; ci < nch; ci++) {
    // first position whose digit is above ci (the codes of [lo, hi) share
    // the digits above `shift` and ascend in this one)
    int a = st, b = h;
    if (ci < nch - 1) {
      while (a < b) {
        const int mid = (a + b) >> 1;
        if ((int)((codes[mid] >> shift) & (unsigned long long)(nch - 1)) <= ci) a = mid + 1;
        else b = mid;
      }
    } else {
      a = h;
    }
    const int j = nch * r + ci;
    nlo[j] = st;
    nhi[j] = a;
    nparent[j] = base + i;
    for (int d = 0; d < dim; d++)
      ncen[(size_t)dim * j + d] =
          __dadd_rn(cen[(size_t)dim * i + d], ((ci >> (dim - 1 - d)) & 1) ? side / 4. : -side / 4.);
    child[(size_t)(base + i) * nch + ci] = next_base + j;
    st = a;
  }
}

__device__ __forceinline__ bool tree_touching(const double* ca, double sa, const double* cb, double sb,
                                              int dim) {
  const double pred = (sa + sb) / 2.;
  for (int d = 0; d < dim; d++)
    if (__dsub_rn(fabs(__dsub_rn(ca[d], cb[d])), pred) > 1e-9) return false;
  return true;
}

// Neighbour lists of one level from its parents' (host order: siblings,
// then per parent neighbour either its touching-leaf entry or its children
// within side sqrt(dim), then the parent's touching coarser leaves).
__global__ void k_tree_neighbours(int base, int nbox, int dim, const int* parent, const int* child,
                                  const int* leaf, const double* cen, const double* side_of,
                                  const int* level_of, int cap, int* same, int* nsame, int* coarse,
                                  int* ncoarse, int* overflow) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbox) return;
  const int b = base + i;
  const int nch = 1 << dim;
  const int par = parent[b];
  const double sq = sqrt((double)dim);
  const double sb = side_of[level_of[b]];
  const double* cbx = cen + (size_t)dim * b;
  int* ls = same + (size_t)b * cap;
  int* lc = coarse + (size_t)b * cap;
  int ns = 0, nc = 0;
  bool over = false;
  for (int ci = 0; ci < nch; ci++) {
    const int o = child[(size_t)par * nch + ci];
    if (o != b) { if (ns < cap) ls[ns++] = o; else over = true; }
  }
  const int* ps = same + (size_t)par * cap;
  for (int q = 0; q < nsame[par]; q++) {
    const int pn = ps[q];
    if (leaf[pn]) {
      if (tree_touching(cbx, sb, cen + (size_t)dim * pn, side_of[level_of[pn]], dim)) {
        if (nc < cap) lc[nc++] = pn; else over = true;
      }
      continue;
    }
    for (int ci = 0; ci < nch; ci++) {
      const int cb = child[(size_t)pn * nch + ci];
      double d2 = 0;
      for (int d = 0; d < dim; d++) {
        const double df = __dsub_rn(cbx[d], cen[(size_t)dim * cb + d]);
        d2 = __dadd_rn(d2, __dmul_rn(df, df));
      }
      if (sqrt(d2) < __dadd_rn(__dmul_rn(sb, sq), 1e-9)) {
        if (ns < cap) ls[ns++] = cb; else over = true;
      }
    }
  }
  const int* pc = coarse + (size_t)par * cap;
  for (int q = 0; q < ncoarse[par]; q++) {
    const int pn = pc[q];
    if (tree_touching(cbx, sb, cen + (size_t)dim * pn, side_of[level_of[pn]], dim)) {
      if (nc < cap) lc[nc++] = pn; else over = true;
    }
  }
  nsame[b] = ns;
  ncoarse[b] = nc;
  if (over) atomicMax(overflow, 1);
}

// A leaf's points ascending by index (the codes ordered them by deeper
// digits): one CTA per leaf, ranks by counting (indices are distinct).
__global__ void k_tree_leaf_sort(const int* leaf_list, int nleaf, const int* lo, const int* hi, int* order,
                                 int* overflow) {
  __shared__ int s_v[1024];
  const int b = leaf_list[blockIdx.x];
  const int a0 = lo[b], n = hi[b] - a0;
  if (n > 1024) {
    if (threadIdx.x == 0) atomicMax(overflow, 2);
    return;
  }
  for (int e = threadIdx.x; e < n; e += blockDim.x) s_v[e] = order[a0 + e];
  __syncthreads();
  for (int e = threadIdx.x; e < n; e += blockDim.x) {
    const int v = s_v[e];
    int r = 0;
    for (int q = 0; q < n; q++) r += s_v[q] < v;
    order[a0 + r] = v;
  }
}

__global__ void k_tree_fill(int* a, int n, int v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = v;
}

__global__ void k_tree_dofs(const int* order, int n, int sol_dim, int* dofs) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n * sol_dim; i += gridDim.x * blockDim.x)
    dofs[i] = order[i / sol_dim] * sol_dim + i % sol_dim;
}
}  // namespace

bool tree_build_gpu(const double* d_points, int n, int dim, int sol_dim, int max_leaf_dofs,
                    double centre, double side, int depth, Tree* tree, cudaStream_t s) {
  if (n <= 0) throw std::invalid_argument("no boundary points");
  if ((dim != 2 && dim != 3) || depth < 1 || dim * depth > 64)
    throw std::invalid_argument("tree: bad dimension or depth");
  if (max_leaf_dofs < 1) throw std::invalid_argument("max_leaf_dofs must be positive");
  const int nch = 1 << dim, cap = tree_nbr_cap(dim);
  const int ntile = (n + kRsTile - 1) / kRsTile;
  std::vector<void*> owned;
  auto take = [&](size_t bytes) {
    void* p = nullptr;
    KI_TREE_CUDA(pool_malloc(&p, bytes + 16, s));
    owned.push_back(p);
    return p;
  };
  auto release = [&] {
    for (void* p : owned) cudaFreeAsync(p, s);
    owned.clear();
  };
  try {
    // ---- codes, stable radix sort
    unsigned long long* keys[2];
    int* vals[2];
    for (int b = 0; b < 2; b++) {
      keys[b] = (unsigned long long*)take(sizeof(unsigned long long) * n);
      vals[b] = (int*)take(sizeof(int) * n);
    }
    unsigned* hist = (unsigned*)take(sizeof(unsigned) * ((size_t)kRsBins * ntile + kRsBins));
    unsigned* tot = hist + (size_t)kRsBins * ntile;
    ki::launch(k_tree_codes, (n + 255) / 256, 256, 0, s, d_points, n, dim, centre, side, depth, keys[0],
               vals[0]);
    KI_TREE_CUDA(cudaGetLastError());
    int cur = 0;
    for (int shift = 0; shift < dim * depth; shift += 8) {
      ki::launch(k_rs_hist, ntile, kRsThreads, 0, s, keys[cur], n, shift, ntile, hist);
      ki::launch(k_rs_scan_rows, kRsBins, 256, 0, s, hist, ntile, tot);
      ki::launch(k_rs_scan_base, 1, kRsBins, 0, s, tot);
      ki::launch(k_rs_scatter, ntile, kRsThreads, 0, s, keys[cur], vals[cur], n, shift, ntile, hist, tot,
                 keys[1 - cur], vals[1 - cur]);
      KI_TREE_CUDA(cudaGetLastError());
      cur = 1 - cur;
    }
    const unsigned long long* codes = keys[cur];
    int* order = vals[cur];

    // ---- boxes level by level (per-box arrays indexed by global id)
    size_t bcap = (size_t)2 * nch * ((size_t)n * sol_dim / max_leaf_dofs + 1) + 1;
    int *lo = nullptr, *hi = nullptr, *parent = nullptr, *child = nullptr, *split = nullptr,
        *level_of = nullptr, *rank = nullptr;
    double* cen = nullptr;
    auto alloc_boxes = [&](size_t c) {
      int* nlo = (int*)take(sizeof(int) * c);
      int* nhi = (int*)take(sizeof(int) * c);
      int* npar = (int*)take(sizeof(int) * c);
      int* nchild = (int*)take(sizeof(int) * c * nch);
      int* nsplit = (int*)take(sizeof(int) * c);
      int* nlev = (int*)take(sizeof(int) * c);
      double* ncen = (double*)take(sizeof(double) * c * dim);
      return std::make_tuple(nlo, nhi, npar, nchild, nsplit, nlev, ncen);
    };
    std::tie(lo, hi, parent, child, split, level_of, cen) = alloc_boxes(bcap);
    rank = (int*)take(sizeof(int) * (bcap + 1));
    KI_TREE_CUDA(cudaMemsetAsync(child, 0xff, sizeof(int) * bcap * nch, s));
    {
      const int z = 0, nn = n, m1 = -1;
      std::vector<double> c0(dim, centre);
      KI_TREE_CUDA(cudaMemcpyAsync(lo, &z, sizeof(int), cudaMemcpyHostToDevice, s));
      KI_TREE_CUDA(cudaMemcpyAsync(hi, &nn, sizeof(int), cudaMemcpyHostToDevice, s));
      KI_TREE_CUDA(cudaMemcpyAsync(parent, &m1, sizeof(int), cudaMemcpyHostToDevice, s));
      KI_TREE_CUDA(cudaMemcpyAsync(level_of, &z, sizeof(int), cudaMemcpyHostToDevice, s));
      KI_TREE_CUDA(cudaMemcpyAsync(cen, c0.data(), sizeof(double) * dim, cudaMemcpyHostToDevice, s));
      KI_TREE_CUDA(cudaStreamSynchronize(s));   // the host values above leave scope
    }
    std::vector<int> lbase{0}, lcount{1};
    std::vector<double> side_of{side};
    int total = 1;
    for (int l = 0;; l++) {
      const int base = lbase[l], cnt = lcount[l];
      const int g = (cnt + 255) / 256;
      ki::launch(k_tree_split_flags, g, 256, 0, s, lo + base, hi + base, cnt, sol_dim, max_leaf_dofs,
                 split + base);
      ki::launch(k_tree_scan, 1, 1024, 0, s, split + base, cnt, rank);
      int S = 0;
      KI_TREE_CUDA(cudaMemcpyAsync(&S, rank + cnt, sizeof(int), cudaMemcpyDeviceToHost, s));
      KI_TREE_CUDA(cudaStreamSynchronize(s));
      if (S == 0) break;
      if (l >= depth) {   // the codes end here: the caller builds by partition
        release();
        return false;
      }
      const int next_base = base + cnt, next_cnt = nch * S;
      if ((size_t)next_base + next_cnt > bcap) {
        // grow every per-box array (rare: deep, strongly clustered trees)
        const size_t nc = 2 * ((size_t)next_base + next_cnt);
        int *a1, *a2, *a3, *a4, *a5, *a6;
        double* a7;
        std::tie(a1, a2, a3, a4, a5, a6, a7) = alloc_boxes(nc);
        KI_TREE_CUDA(cudaMemsetAsync(a4, 0xff, sizeof(int) * nc * nch, s));
        KI_TREE_CUDA(cudaMemcpyAsync(a1, lo, sizeof(int) * total, cudaMemcpyDeviceToDevice, s));
        KI_TREE_CUDA(cudaMemcpyAsync(a2, hi, sizeof(int) * total, cudaMemcpyDeviceToDevice, s));
        KI_TREE_CUDA(cudaMemcpyAsync(a3, parent, sizeof(int) * total, cudaMemcpyDeviceToDevice, s));
        KI_TREE_CUDA(cudaMemcpyAsync(a4, child, sizeof(int) * total * nch, cudaMemcpyDeviceToDevice, s));
        KI_TREE_CUDA(cudaMemcpyAsync(a5, split, sizeof(int) * total, cudaMemcpyDeviceToDevice, s));
        KI_TREE_CUDA(cudaMemcpyAsync(a6, level_of, sizeof(int) * total, cudaMemcpyDeviceToDevice, s));
        KI_TREE_CUDA(cudaMemcpyAsync(a7, cen, sizeof(double) * total * dim, cudaMemcpyDeviceToDevice, s));
        lo = a1; hi = a2; parent = a3; child = a4; split = a5; level_of = a6; cen = a7;
        bcap = nc;
        rank = (int*)take(sizeof(int) * (bcap + 1));
        ki::launch(k_tree_scan, 1, 1024, 0, s, split + base, cnt, rank);
      }
      const int shift = dim * (depth - 1 - l);
      ki::launch(k_tree_children, g, 256, 0, s, codes, lo + base, hi + base, cen + (size_t)dim * base, cnt,
                 split + base, rank, dim, shift, side_of[l], next_base, child, lo + next_base,
                 hi + next_base, cen + (size_t)dim * next_base, parent + next_base, base);
      KI_TREE_CUDA(cudaGetLastError());
      ki::launch(k_tree_fill, std::min(1024, (next_cnt + 255) / 256), 256, 0, s, level_of + next_base,
                 next_cnt, l + 1);
      lbase.push_back(next_base);
      lcount.push_back(next_cnt);
      side_of.push_back(side_of[l] / 2.0);
      total = next_base + next_cnt;
    }
    const int L = (int)lbase.size();
    // split flags of the last level were written by its flag launch; leaf = !split
    int* leaf = (int*)take(sizeof(int) * total);
    {
      std::vector<int> hs(total);
      KI_TREE_CUDA(cudaMemcpyAsync(hs.data(), split, sizeof(int) * total, cudaMemcpyDeviceToHost, s));
      KI_TREE_CUDA(cudaStreamSynchronize(s));
      for (auto& v : hs) v = !v;
      KI_TREE_CUDA(cudaMemcpyAsync(leaf, hs.data(), sizeof(int) * total, cudaMemcpyHostToDevice, s));
      KI_TREE_CUDA(cudaStreamSynchronize(s));
    }
    // ---- neighbour lists, top-down
    double* d_side = (double*)take(sizeof(double) * L);
    KI_TREE_CUDA(cudaMemcpyAsync(d_side, side_of.data(), sizeof(double) * L, cudaMemcpyHostToDevice, s));
    int* same = (int*)take(sizeof(int) * (size_t)total * cap);
    int* coarse = (int*)take(sizeof(int) * (size_t)total * cap);
    int* nsame = (int*)take(sizeof(int) * total);
    int* ncoarse = (int*)take(sizeof(int) * total);
    int* flagd = (int*)take(sizeof(int));
    KI_TREE_CUDA(cudaMemsetAsync(nsame, 0, sizeof(int) * total, s));
    KI_TREE_CUDA(cudaMemsetAsync(ncoarse, 0, sizeof(int) * total, s));
    KI_TREE_CUDA(cudaMemsetAsync(flagd, 0, sizeof(int), s));
    for (int l = 1; l < L; l++)
      ki::launch(k_tree_neighbours, (lcount[l] + 127) / 128, 128, 0, s, lbase[l], lcount[l], dim, parent,
                 child, leaf, cen, d_side, level_of, cap, same, nsame, coarse, ncoarse, flagd);
    // ---- leaves' points ascending, the DOF list
    std::vector<int> hleaf_ids;
    {
      std::vector<int> hl(total);
      KI_TREE_CUDA(cudaMemcpyAsync(hl.data(), leaf, sizeof(int) * total, cudaMemcpyDeviceToHost, s));
      KI_TREE_CUDA(cudaStreamSynchronize(s));
      for (int b = 0; b < total; b++)
        if (hl[b]) hleaf_ids.push_back(b);
    }
    int* d_leaves = (int*)take(sizeof(int) * hleaf_ids.size());
    KI_TREE_CUDA(cudaMemcpyAsync(d_leaves, hleaf_ids.data(), sizeof(int) * hleaf_ids.size(),
                                 cudaMemcpyHostToDevice, s));
    ki::launch(k_tree_leaf_sort, (unsigned)hleaf_ids.size(), 128, 0, s, d_leaves, (int)hleaf_ids.size(), lo,
               hi, order, flagd);
    const int N = n * sol_dim;
    int* dofs = (int*)take(sizeof(int) * N);
    ki::launch(k_tree_dofs, std::min(4096, (N + 255) / 256), 256, 0, s, order, n, sol_dim, dofs);
    KI_TREE_CUDA(cudaGetLastError());
    // ---- to the host
    std::vector<int> h_lo(total), h_hi(total), h_par(total), h_child((size_t)total * nch), h_lev(total);
    std::vector<double> h_cen((size_t)total * dim);
    int h_flag = 0;
    tree->dof_sorted.resize(N);
    tree->nbr_same.resize((size_t)total * cap);
    tree->nbr_coarse.resize((size_t)total * cap);
    tree->n_same.resize(total);
    tree->n_coarse.resize(total);
    KI_TREE_CUDA(cudaMemcpyAsync(h_lo.data(), lo, sizeof(int) * total, cudaMemcpyDeviceToHost, s));
    KI_TREE_CUDA(cudaMemcpyAsync(h_hi.data(), hi, sizeof(int) * total, cudaMemcpyDeviceToHost, s));
    KI_TREE_CUDA(cudaMemcpyAsync(h_par.data(), parent, sizeof(int) * total, cudaMemcpyDeviceToHost, s));
    KI_TREE_CUDA(cudaMemcpyAsync(h_child.data(), child, sizeof(int) * (size_t)total * nch,
                                 cudaMemcpyDeviceToHost, s));
    KI_TREE_CUDA(cudaMemcpyAsync(h_lev.data(), level_of, sizeof(int) * total, cudaMemcpyDeviceToHost, s));
    KI_TREE_CUDA(cudaMemcpyAsync(h_cen.data(), cen, sizeof(double) * total * dim, cudaMemcpyDeviceToHost, s));
    KI_TREE_CUDA(cudaMemcpyAsync(tree->dof_sorted.data(), dofs, sizeof(int) * N, cudaMemcpyDeviceToHost, s));
    KI_TREE_CUDA(cudaMemcpyAsync(tree->nbr_same.data(), same, sizeof(int) * (size_t)total * cap,
                                 cudaMemcpyDeviceToHost, s));
    KI_TREE_CUDA(cudaMemcpyAsync(tree->nbr_coarse.data(), coarse, sizeof(int) * (size_t)total * cap,
                                 cudaMemcpyDeviceToHost, s));
    KI_TREE_CUDA(cudaMemcpyAsync(tree->n_same.data(), nsame, sizeof(int) * total, cudaMemcpyDeviceToHost, s));
    KI_TREE_CUDA(cudaMemcpyAsync(tree->n_coarse.data(), ncoarse, sizeof(int) * total, cudaMemcpyDeviceToHost, s));
    KI_TREE_CUDA(cudaMemcpyAsync(&h_flag, flagd, sizeof(int), cudaMemcpyDeviceToHost, s));
    KI_TREE_CUDA(cudaStreamSynchronize(s));
    release();
    if (h_flag) {   // more neighbours than 3^dim - 1, or a leaf beyond 1,024 points
      tree->dof_sorted.clear();
      return false;
    }
    tree->dim = dim;
    tree->n_points = n;
    tree->sol_dim = sol_dim;
    tree->n_dofs = N;
    tree->max_leaf_dofs = max_leaf_dofs;
    tree->boxes.assign(total, Box());
    tree->levels.assign(L, {});
    for (int l = 0; l < L; l++) {
      tree->levels[l].resize(lcount[l]);
      for (int i = 0; i < lcount[l]; i++) tree->levels[l][i] = lbase[l] + i;
    }
    std::vector<char> is_leaf(total, 0);
    for (int b : hleaf_ids) is_leaf[b] = 1;
    parallel_ranges(total, [&](int b0, int b1) {
    for (int b = b0; b < b1; b++) {
      Box& bx = tree->boxes[b];
      const int l = h_lev[b];
      bx.level = l;
      bx.parent = h_par[b];
      for (int ci = 0; ci < nch; ci++) bx.child[ci] = h_child[(size_t)b * nch + ci];
      bx.leaf = is_leaf[b] != 0;
      for (int d = 0; d < dim; d++) bx.c[d] = h_cen[(size_t)b * dim + d];
      bx.side = side_of[l];
      bx.orig_count = (h_hi[b] - h_lo[b]) * sol_dim;
      bx.orig_start = bx.leaf ? h_lo[b] * sol_dim : 0;
      bx.level_pos = b - lbase[l];
    }
    });
    return true;
  } catch (...) {
    release();
    throw;
  }
}

}  // namespace ki
