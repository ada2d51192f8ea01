// Dense LU factorization and solves for the root skeleton block (and the
// bordered root system of multiply connected problems): the role of
// LAPACK dgetrf / dgetrs in the reference (ki_Mat::LU_factorize,
// left_multiply_inverse, kern_interp/ki_mat.cpp:445-513).
//
// Right-looking blocked LU with partial pivoting, panel width kNb:
//   k_lu_panel   one CTA factors the (n-p) x kNb panel (row pivoting)
//   k_lu_swap    the panel's row swaps applied to the other columns
//   k_lu_trsm    U12 = L11^-1 A12
//   k_lu_gemm    A22 -= L21 U12, 64 x 64 output tiles staged in shared memory
// Solves: pivots, then blocked forward/backward substitution whose
// off-diagonal updates run on the whole GPU.
#include "ki_launch.cuh"
#include "ki_dense.h"

#include <algorithm>
#include <stdexcept>
#include <string>

namespace ki {

namespace {

constexpr int kNb = 32;

#define KI_DENSE_CUDA(call)                                                                \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      throw std::runtime_error(std::string("CUDA error: ") + cudaGetErrorString(e_));     \
  } while (0)

// Unblocked LU of the panel A(p:n, p:p+w) with partial pivoting (dgetf2
// order: pivot = first index of the largest |A(i, j)|, i >= j), one CTA.
// Each column costs three barriers and one pass over the rows: the pass
// that scales column j and updates the panel's later columns also finds
// each thread's candidate pivot of column j + 1 in the rows it just updated
// (every row is read and written by one thread only, so no barrier is needed
// between the update and that search).
template <typename T>
__global__ void __launch_bounds__(1024) k_lu_panel(T* A, int n, int lda, int p, int w, int* piv,
                                                   int* err) {
  __shared__ T s_val[32];
  __shared__ int s_idx[32];
  __shared__ int s_p;
  __shared__ T s_pv;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int nth = blockDim.x;
  // this thread's candidate pivot of column p
  T best = T(-1);
  int bi = p;
  for (int i = p + (int)threadIdx.x; i < n; i += nth) {
    const T v = fabs(A[i + (size_t)lda * p]);
    if (v > best) { best = v; bi = i; }
  }
  for (int j = p; j < p + w; j++) {
    // pivot: argmax |A(i, j)|, i >= j (first index on ties)
    for (int o = 16; o > 0; o >>= 1) {
      const T ov = __shfl_down_sync(0xffffffff, best, o);
      const int oi = __shfl_down_sync(0xffffffff, bi, o);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
    }
    if (lane == 0) { s_val[warp] = best; s_idx[warp] = bi; }
    __syncthreads();
    if (warp == 0) {
      best = lane < nw ? s_val[lane] : T(-1);
      bi = lane < nw ? s_idx[lane] : n;
      for (int o = 16; o > 0; o >>= 1) {
        const T ov = __shfl_down_sync(0xffffffff, best, o);
        const int oi = __shfl_down_sync(0xffffffff, bi, o);
        if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
      }
      if (lane == 0) { s_p = bi; s_pv = best; piv[j] = bi; }
    }
    __syncthreads();
    const int pr = s_p;
    const bool next = j + 1 < p + w;
    best = T(-1);
    bi = j + 1;
    if (s_pv == T(0)) {
      // singular column: flagged, no elimination; the next column's candidates
      if (threadIdx.x == 0) atomicMax(err, 2);
      if (next)
        for (int i = j + 1 + (int)threadIdx.x; i < n; i += nth) {
          const T v = fabs(A[i + (size_t)lda * (j + 1)]);
          if (v > best) { best = v; bi = i; }
        }
      continue;
    }
    if (pr != j)
      for (int c = p + (int)threadIdx.x; c < p + w; c += nth) {
        const T t = A[j + (size_t)lda * c];
        A[j + (size_t)lda * c] = A[pr + (size_t)lda * c];
        A[pr + (size_t)lda * c] = t;
      }
    __syncthreads();
    const T d = A[j + (size_t)lda * j];
    // scale column j, update the later panel columns, and search column j + 1
    for (int i = j + 1 + (int)threadIdx.x; i < n; i += nth) {
      const T l = A[i + (size_t)lda * j] / d;
      A[i + (size_t)lda * j] = l;
      for (int c = j + 1; c < p + w; c++) A[i + (size_t)lda * c] -= l * A[j + (size_t)lda * c];
      if (next) {
        const T v = fabs(A[i + (size_t)lda * (j + 1)]);
        if (v > best) { best = v; bi = i; }
      }
    }
  }
}

template <typename T>
__global__ void k_lu_swap(T* A, int n, int lda, int p, int w, const int* piv) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n || (c >= p && c < p + w)) return;
  for (int j = p; j < p + w; j++) {
    int r = piv[j];
    if (r != j) {
      T t = A[j + (size_t)lda * c];
      A[j + (size_t)lda * c] = A[r + (size_t)lda * c];
      A[r + (size_t)lda * c] = t;
    }
  }
}

template <typename T>
__global__ void k_lu_trsm(T* A, int n, int lda, int p, int w) {
  __shared__ T L[kNb][kNb + 1];
  for (int e = threadIdx.x; e < w * w; e += blockDim.x) L[e % w][e / w] = A[p + e % w + (size_t)lda * (p + e / w)];
  __syncthreads();
  int c = p + w + blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  T x[kNb];
  for (int i = 0; i < w; i++) x[i] = A[p + i + (size_t)lda * c];
  for (int i = 0; i < w; i++)
    for (int l = 0; l < i; l++) x[i] -= L[i][l] * x[l];
  for (int i = 0; i < w; i++) A[p + i + (size_t)lda * c] = x[i];
}

// A(r0:n, c0:n) -= A(r0:n, p:p+w) * A(p:p+w, c0:n), r0 = c0 = p + w
template <typename T>
__global__ void __launch_bounds__(256) k_lu_gemm(T* A, int n, int lda, int p, int w) {
  __shared__ T Ls[64][kNb + 1];
  __shared__ T Us[kNb][64 + 1];
  const int r0 = p + w + blockIdx.x * 64, c0 = p + w + blockIdx.y * 64;
  for (int e = threadIdx.x; e < 64 * kNb; e += blockDim.x) {
    int i = e % 64, l = e / 64;
    Ls[i][l] = (r0 + i < n && l < w) ? A[r0 + i + (size_t)lda * (p + l)] : T(0);
    int l2 = e % kNb, j = e / kNb;
    Us[l2][j] = (c0 + j < n && l2 < w) ? A[p + l2 + (size_t)lda * (c0 + j)] : T(0);
  }
  __syncthreads();
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) acc[a][b] = T(0);
  for (int l = 0; l < kNb; l++) {
    T lv[4], uv[4];
#pragma unroll
    for (int a = 0; a < 4; a++) lv[a] = Ls[tx + 16 * a][l];
#pragma unroll
    for (int b = 0; b < 4; b++) uv[b] = Us[l][ty + 16 * b];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int b = 0; b < 4; b++) acc[a][b] += lv[a] * uv[b];
  }
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) {
      int i = r0 + tx + 16 * a, j = c0 + ty + 16 * b;
      if (i < n && j < n) A[i + (size_t)lda * j] -= acc[a][b];
    }
}

// ---- solves on B (n x nrhs, ld ldb)
template <typename T>
__global__ void k_apply_piv(T* B, int ldb, int nrhs, const int* piv, int n, bool reverse) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nrhs) return;
  T* b = B + (size_t)ldb * c;
  if (!reverse) {
    for (int i = 0; i < n; i++) {
      int r = piv[i];
      if (r != i) { T t = b[i]; b[i] = b[r]; b[r] = t; }
    }
  } else {
    for (int i = n - 1; i >= 0; i--) {
      int r = piv[i];
      if (r != i) { T t = b[i]; b[i] = b[r]; b[r] = t; }
    }
  }
}

// Diagonal block of the substitution: rows p..p+w-1, one thread per column.
// lower: unit lower L (forward); else upper U with its diagonal (backward).
// trans: use the transpose of the stored factor (solves with A^T).
template <typename T>
__global__ void k_tri_block(const T* LU, int lda, int p, int w, T* B, int ldb, int nrhs, bool lower,
                            bool trans) {
  __shared__ T D[kNb][kNb + 1];
  for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
    int i = e % w, l = e / w;
    D[i][l] = trans ? LU[p + l + (size_t)lda * (p + i)] : LU[p + i + (size_t)lda * (p + l)];
  }
  __syncthreads();
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nrhs) return;
  T x[kNb];
  T* b = B + (size_t)ldb * c + p;
  for (int i = 0; i < w; i++) x[i] = b[i];
  // effective matrix M = D (or D^T already transposed into D); lower/upper refer to M
  if (lower) {
    for (int i = 0; i < w; i++) {
      for (int l = 0; l < i; l++) x[i] -= D[i][l] * x[l];
      if (trans) x[i] /= D[i][i];   // U^T is lower with U's diagonal
    }
  } else {
    for (int i = w - 1; i >= 0; i--) {
      for (int l = i + 1; l < w; l++) x[i] -= D[i][l] * x[l];
      if (!trans) x[i] /= D[i][i];  // U (L^T is unit upper)
    }
  }
  for (int i = 0; i < w; i++) b[i] = x[i];
}

// B(rows, :) -= M(rows, p:p+w) B(p:p+w, :); rows = [r0, r1); M = LU or LU^T
template <typename T>
__global__ void k_tri_update(const T* LU, int lda, int p, int w, int r0, int r1, T* B, int ldb,
                             int nrhs, bool trans) {
  __shared__ T Xs[kNb][33];
  const int c0 = blockIdx.y * 32;
  for (int e = threadIdx.x; e < kNb * 32; e += blockDim.x) {
    int l = e % kNb, c = e / kNb;
    Xs[l][c] = (l < w && c0 + c < nrhs) ? B[p + l + (size_t)ldb * (c0 + c)] : T(0);
  }
  __syncthreads();
  int i = r0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= r1) return;
  T m[kNb];
  for (int l = 0; l < w; l++) m[l] = trans ? LU[p + l + (size_t)lda * i] : LU[i + (size_t)lda * (p + l)];
  for (int c = 0; c < 32 && c0 + c < nrhs; c++) {
    T acc = T(0);
    for (int l = 0; l < w; l++) acc += m[l] * Xs[l][c];
    B[i + (size_t)ldb * (c0 + c)] -= acc;
  }
}

// The whole solve L U x = P b for one cw-column chunk of B per CTA (cw <= 32),
// the chunk held in shared memory (n x cw, odd leading dimension): pivots, then the
// blocked forward and backward substitutions of the launches above in one
// kernel -- each kNb-row diagonal block staged and solved one thread per
// column, the rows below (above) it updated by every thread.  The same
// operations in the same order as the multi-launch path.
template <typename T>
size_t fused_solve_smem(int n, int cw = 32) {
  return sizeof(T) * ((size_t)(n | 1) * cw + (size_t)kNb * (kNb + 1));
}

// Columns per CTA of the fused solve: narrower chunks when the right-hand
// sides are few, so that about 16 CTAs share the substitutions (each reads
// the factors from L2) instead of one or two.
inline int fused_solve_cols(int nrhs) {
  int cw = 32;
  while (cw > 4 && (nrhs + cw - 1) / cw < 16) cw >>= 1;
  return cw;
}

template <typename T>
__global__ void __launch_bounds__(256) k_lu_solve_fused(const T* LU, int n, const int* piv, T* B,
                                                        int ldb, int nrhs, int cw) {
  extern __shared__ __align__(16) unsigned char fs_smem[];
  const int ldx = n | 1;
  T* X = reinterpret_cast<T*>(fs_smem);
  T (*D)[kNb + 1] = reinterpret_cast<T (*)[kNb + 1]>(X + (size_t)ldx * cw);
  const int tid = threadIdx.x, nth = blockDim.x;
  const int c0 = blockIdx.x * cw, nc = min(cw, nrhs - c0);
  for (int e = tid; e < n * nc; e += nth) {
    const int c = e / n, i = e % n;
    X[i + (size_t)ldx * c] = B[i + (size_t)ldb * (c0 + c)];
  }
  __syncthreads();
  if (tid < nc) {
    T* x = X + (size_t)ldx * tid;
    for (int i = 0; i < n; i++) {
      const int r = piv[i];
      if (r != i) { T t = x[i]; x[i] = x[r]; x[r] = t; }
    }
  }
  __syncthreads();
  auto stage = [&](int p, int w) {
    for (int e = tid; e < w * w; e += nth) {
      const int i = e % w, l = e / w;
      D[i][l] = LU[p + i + (size_t)n * (p + l)];
    }
    __syncthreads();
  };
  auto update = [&](int p, int w, int r0, int r1) {   // X(r0:r1, :) -= LU(r0:r1, p:p+w) X(p:p+w, :)
    const int rows = r1 - r0;
    for (int e = tid; e < rows * nc; e += nth) {
      const int i = r0 + e % rows, c = e / rows;
      const T* xc = X + (size_t)ldx * c + p;
      T acc = T(0);
      for (int l = 0; l < w; l++) acc += LU[i + (size_t)n * (p + l)] * xc[l];
      X[i + (size_t)ldx * c] -= acc;
    }
    __syncthreads();
  };
  for (int p = 0; p < n; p += kNb) {   // L y = b (unit lower)
    const int w = min(kNb, n - p);
    stage(p, w);
    if (tid < nc) {
      T* x = X + (size_t)ldx * tid + p;
      for (int i = 0; i < w; i++)
        for (int l = 0; l < i; l++) x[i] -= D[i][l] * x[l];
    }
    __syncthreads();
    if (p + w < n) update(p, w, p + w, n);
  }
  for (int p = ((n - 1) / kNb) * kNb; p >= 0; p -= kNb) {   // U x = y
    const int w = min(kNb, n - p);
    stage(p, w);
    if (tid < nc) {
      T* x = X + (size_t)ldx * tid + p;
      for (int i = w - 1; i >= 0; i--) {
        for (int l = i + 1; l < w; l++) x[i] -= D[i][l] * x[l];
        x[i] /= D[i][i];
      }
    }
    __syncthreads();
    if (p > 0) update(p, w, 0, p);
  }
  for (int e = tid; e < n * nc; e += nth) {
    const int c = e / n, i = e % n;
    B[i + (size_t)ldb * (c0 + c)] = X[i + (size_t)ldx * c];
  }
}

}  // namespace

template <typename T>
void dense_lu(T* A, int n, int* piv, int* err, cudaStream_t s) {
  for (int p = 0; p < n; p += kNb) {
    int w = std::min(kNb, n - p);
    ki::launch(k_lu_panel<T>, 1, 1024, 0, s, A, n, n, p, w, piv, err);
    ki::launch(k_lu_swap<T>, (n + 255) / 256, 256, 0, s, A, n, n, p, w, piv);
    int rest = n - p - w;
    if (rest > 0) {
      ki::launch(k_lu_trsm<T>, (rest + 127) / 128, 128, 0, s, A, n, n, p, w);
      dim3 g((rest + 63) / 64, (rest + 63) / 64);
      ki::launch(k_lu_gemm<T>, g, 256, 0, s, A, n, n, p, w);
    }
  }
  KI_DENSE_CUDA(cudaGetLastError());
}

template <typename T>
void dense_lu_solve(const T* LU, int n, const int* piv, T* B, int ldb, int nrhs, bool trans,
                    cudaStream_t s) {
  if (n == 0 || nrhs == 0) return;
  dim3 cb((nrhs + 127) / 128);
  const int cw = fused_solve_cols(nrhs);
  // the fused kernel streams all of L and U through each of its few CTAs:
  // for factors over 16 MB (n > 2,048 in FP32) the multi-launch path, whose
  // updates spread every block row over the GPU, is the faster one (a
  // 7,656-row root solve with one right-hand side: 91 ms fused)
  const bool small = (double)n * n * sizeof(T) <= 16.0 * 1024 * 1024;
  if (!trans && small && fused_solve_smem<T>(n, cw) <= 160 * 1024) {
    KI_DENSE_CUDA(cudaFuncSetAttribute(k_lu_solve_fused<T>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024));
    ki::launch(k_lu_solve_fused<T>, (nrhs + cw - 1) / cw, 256, fused_solve_smem<T>(n, cw), s, LU, n, piv,
               B, ldb, nrhs, cw);
    KI_DENSE_CUDA(cudaGetLastError());
    return;
  }
  if (!trans) {
    ki::launch(k_apply_piv<T>, cb, 128, 0, s, B, ldb, nrhs, piv, n, false);
    for (int p = 0; p < n; p += kNb) {       // L y = b (unit lower)
      int w = std::min(kNb, n - p);
      ki::launch(k_tri_block<T>, cb, 128, 0, s, LU, n, p, w, B, ldb, nrhs, true, false);
      if (p + w < n) {
        dim3 g((n - p - w + 127) / 128, (nrhs + 31) / 32);
        ki::launch(k_tri_update<T>, g, 128, 0, s, LU, n, p, w, p + w, n, B, ldb, nrhs, false);
      }
    }
    for (int p = ((n - 1) / kNb) * kNb; p >= 0; p -= kNb) {   // U x = y
      int w = std::min(kNb, n - p);
      ki::launch(k_tri_block<T>, cb, 128, 0, s, LU, n, p, w, B, ldb, nrhs, false, false);
      if (p > 0) {
        dim3 g((p + 127) / 128, (nrhs + 31) / 32);
        ki::launch(k_tri_update<T>, g, 128, 0, s, LU, n, p, w, 0, p, B, ldb, nrhs, false);
      }
    }
  } else {
    for (int p = 0; p < n; p += kNb) {       // U^T y = b (lower, U's diagonal)
      int w = std::min(kNb, n - p);
      ki::launch(k_tri_block<T>, cb, 128, 0, s, LU, n, p, w, B, ldb, nrhs, true, true);
      if (p + w < n) {
        dim3 g((n - p - w + 127) / 128, (nrhs + 31) / 32);
        ki::launch(k_tri_update<T>, g, 128, 0, s, LU, n, p, w, p + w, n, B, ldb, nrhs, true);
      }
    }
    for (int p = ((n - 1) / kNb) * kNb; p >= 0; p -= kNb) {   // L^T x = y (unit upper)
      int w = std::min(kNb, n - p);
      ki::launch(k_tri_block<T>, cb, 128, 0, s, LU, n, p, w, B, ldb, nrhs, false, true);
      if (p > 0) {
        dim3 g((p + 127) / 128, (nrhs + 31) / 32);
        ki::launch(k_tri_update<T>, g, 128, 0, s, LU, n, p, w, 0, p, B, ldb, nrhs, true);
      }
    }
    ki::launch(k_apply_piv<T>, cb, 128, 0, s, B, ldb, nrhs, piv, n, true);
  }
  KI_DENSE_CUDA(cudaGetLastError());
}

template void dense_lu<double>(double*, int, int*, int*, cudaStream_t);
template void dense_lu<float>(float*, int, int*, int*, cudaStream_t);
template void dense_lu_solve<double>(const double*, int, const int*, double*, int, int, bool, cudaStream_t);
template void dense_lu_solve<float>(const float*, int, const int*, float*, int, int, bool, cudaStream_t);

}  // namespace ki
