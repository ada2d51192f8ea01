// GPU recursive-skeletonization factor and solve (sm_103a).
//
// The level loop restates SkelFactorization::skeletonize
// (kern_interp/skel_factorization/skel_factorization.cpp:173-551): for each
// tree level, bottom-up, every box with enough active DOFs is compressed by
// an interpolative decomposition of its proxy/near-field matrix and its
// redundant DOFs are eliminated by a Schur complement.  All boxes of a level
// are processed by one launch per stage (one CTA per box):
//
//   k_build_active   active DOF lists (QuadTree::remove_inactive_dofs_at_box)
//   k_id             ID matrix generated on the fly (Kernel::get_id_mat), folded
//                    into an n x n triangle by Householder TSQR, then column-
//                    pivoted QR on the triangle, rank cut and T = R11^-1 R12
//                    (ki_Mat::id)
//   k_assemble       box self-block K_BN: children's accumulated self-blocks on
//                    the diagonal, kernel entries elsewhere (replaces the
//                    reference's descendant-update gather, quadtree.cpp:1545-1632)
//   k_schur          SkelFactorization::decouple: X_rr, LU(X_rr), L, U and the
//                    box's accumulated self-block K_ss - L K~_rs
//
// The host reads back only the ranks of each level (to size the next level).
#include "ki_factor.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <string>

#include "ki_common.cuh"

namespace ki {

#define KI_CUDA(call)                                                                      \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      throw std::runtime_error(std::string("CUDA error: ") + cudaGetErrorString(e_) +     \
                               " at " + __FILE__ + ":" + std::to_string(__LINE__));        \
  } while (0)

template <typename T>
void* Factorization<T>::alloc(size_t bytes) {
  void* p = nullptr;
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMallocAsync(&p, bytes, stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw std::runtime_error(std::string("device allocation failed: ") + cudaGetErrorString(e));
  }
  owned.push_back(p);
  device_bytes += bytes;
  return p;
}

template <typename T>
Factorization<T>::~Factorization() {
  for (void* p : owned) cudaFreeAsync(p, stream);
  if (stream) cudaStreamSynchronize(stream);
}

namespace {

constexpr int kThreads = 256;
constexpr int kFoldRows = 32;   // rows of the ID matrix generated per TSQR fold

template <typename T> __device__ __forceinline__ T tol3z();
template <> __device__ __forceinline__ double tol3z<double>() { return 1.0536712127723509e-08; }  // sqrt(2^-53)
template <> __device__ __forceinline__ float tol3z<float>() { return 2.44140625e-04f; }          // sqrt(2^-24)

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffff, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffff, v, o);
  return v;
}

// ---------------------------------------------------------------- tasks --
struct ActiveTask {
  int64_t dst;        // ipool offset of the box's active list
  int nseg;
  int64_t src[4];     // ipool offsets of the pieces (leaf: 1 piece)
  int len[4];
};

struct IdTask {
  int64_t act;        // ipool offset of the active list (n)
  int n;
  int seg_begin, seg_end;
  int mode;           // 0: inner-circle filter + proxy rows; 1: all candidates, no proxy
  double cx, cy, rad_filter, rad_proxy;
  int64_t rows;       // iscratch offset of the row list (capacity = candidates)
  int64_t ws;         // T-scratch offset: R (n*n) | B (32*n) | vn1 (n) | vn2 (n) | Tout (n*n/4+1)
  int64_t perm;       // iscratch offset of the pivot order (n)
  int64_t pact;       // ipool offset of the permuted active list (n), kept for the solve
};

template <typename T>
struct AsmTask {
  int64_t act;
  int n;
  T* out;             // n x n
  int nchild;         // 0 for a leaf
  int coff[4], clen[4];
  const T* ctile[4];  // child accumulated self-blocks (clen x clen)
};

template <typename T>
struct SchurTask {
  const T* K;         // n x n self block K_BN
  int n, k;
  const int* perm;    // n
  const T* Tin;       // k x r (from the ID scratch)
  T* Tout;            // k x r persistent
  T* L;               // k x r
  T* U;               // r x k
  T* X;               // r x r LU
  int* piv;           // r
  T* Atil;            // k x k accumulated self-block
  T* ws;              // scratch: P (n*n) | Wrs (r*k) | Wsr (k*r) | Lt (r*k)
};

// ---------------------------------------------------------------- kernels --
__global__ void k_build_active(const ActiveTask* tasks, int* ipool) {
  const ActiveTask t = tasks[blockIdx.x];
  int64_t dst = t.dst;
  for (int s = 0; s < t.nseg; s++) {
    for (int i = threadIdx.x; i < t.len[s]; i += blockDim.x) ipool[dst + i] = ipool[t.src[s] + i];
    dst += t.len[s];
  }
}

// One ID-matrix entry, row `row` of the stacked matrix
// [K(I,A); K(A,I)^T; box->proxy; proxy->box] (Kernel::get_id_mat,
// kern_interp/kernel/kernel.cpp:565-640; proxy rows Kernel::get_proxy_mat,
// :646-717), column = active DOF `adof`.
template <typename T>
__device__ __forceinline__ T id_entry(const Points<T>& P, int sol_dim, int row, int nI,
                                      const int* rows, int adof, int nprox, const double* pcos,
                                      const double* psin, double cx, double cy, double rad) {
  if (row < nI) return kernel_entry<T>(P, sol_dim, rows[row], adof);
  if (row < 2 * nI) return kernel_entry<T>(P, sol_dim, adof, rows[row - nI]);
  int q = row - 2 * nI;
  int ap = sol_dim == 1 ? adof : (adof >> 1);
  T bx = P.x[ap], by = P.y[ap], bnx = P.nx[ap], bny = P.ny[ap], bw = P.w[ap];
  T pw = T(2.0 * kPi * rad / nprox);
  if (sol_dim == 1) {
    int i = q < nprox ? q : q - nprox;
    T px = T(cx + rad * pcos[i]), py = T(cy + rad * psin[i]);
    T pnx = T(pcos[i]), pny = T(psin[i]);
    if (q < nprox) return laplace_entry<T>(px, py, bx, by, bnx, bny, bw, T(0));
    return laplace_entry<T>(bx, by, px, py, pnx, pny, pw, T(0));
  }
  int half = 2 * nprox;
  int qq = q < half ? q : q - half;
  int i = qq >> 1, par = qq & 1;
  T px = T(cx + rad * pcos[i]), py = T(cy + rad * psin[i]);
  T pnx = T(pcos[i]), pny = T(psin[i]);
  if (q < half) return stokes_entry<T>(par, adof & 1, px, py, pnx, pny, bx, by, bnx, bny, bw, T(0));
  return stokes_entry<T>(adof & 1, par, bx, by, bnx, bny, px, py, pnx, pny, pw, T(0));
}

// Interpolative decomposition of one box per CTA.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_id(const IdTask* tasks, const int64_t* seg_off,
                                                  const int* seg_len, int* ipool, int* iscratch, T* tws,
                                                  Points<T> P, int sol_dim, int nprox,
                                                  const double* pcos, const double* psin,
                                                  double tol, int* k_out, int* err) {
  const IdTask t = tasks[blockIdx.x];
  const int n = t.n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  __shared__ int s_cnt;
  __shared__ int s_scan[kThreads];
  __shared__ T s_tau, s_beta, s_red;
  __shared__ int s_piv, s_k, s_stop;

  int* rows = iscratch + t.rows;
  const int* act = ipool + t.act;
  int* perm = iscratch + t.perm;
  T* R = tws + t.ws;
  T* B = R + (size_t)n * n;
  T* vn1 = B + (size_t)kFoldRows * n;
  T* vn2 = vn1 + n;
  T* Tout = vn2 + n;

  // 1. candidate rows, optionally filtered to the proxy circle, order kept
  if (threadIdx.x == 0) s_cnt = 0;
  __syncthreads();
  for (int s = t.seg_begin; s < t.seg_end; s++) {
    const int* src = ipool + seg_off[s];
    int len = seg_len[s];
    for (int base = 0; base < len; base += blockDim.x) {
      int i = base + threadIdx.x;
      int keep = 0, dof = 0;
      if (i < len) {
        dof = src[i];
        if (t.mode == 1) {
          keep = 1;
        } else {
          int p = sol_dim == 1 ? dof : dof >> 1;
          double dx = t.cx - (double)P.x[p], dy = t.cy - (double)P.y[p];
          double dist = sqrt(dx * dx + dy * dy);
          keep = dist < t.rad_filter;
        }
      }
      s_scan[threadIdx.x] = keep;
      __syncthreads();
      for (int o = 1; o < blockDim.x; o <<= 1) {
        int v = threadIdx.x >= o ? s_scan[threadIdx.x - o] : 0;
        __syncthreads();
        s_scan[threadIdx.x] += v;
        __syncthreads();
      }
      if (keep) rows[s_cnt + s_scan[threadIdx.x] - 1] = dof;
      __syncthreads();
      if (threadIdx.x == blockDim.x - 1) s_cnt += s_scan[threadIdx.x];
      __syncthreads();
    }
  }
  const int nI = s_cnt;
  const int nprox_rows = t.mode == 0 ? 2 * nprox * sol_dim : 0;
  const int m = 2 * nI + nprox_rows;

  // 2. TSQR: R <- qr([R; B]) for successive row blocks B of the ID matrix
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) R[idx] = T(0);
  __syncthreads();
  for (int r0 = 0; r0 < m; r0 += kFoldRows) {
    for (int idx = threadIdx.x; idx < kFoldRows * n; idx += blockDim.x) {
      int i = idx % kFoldRows, j = idx / kFoldRows;
      int row = r0 + i;
      T v = T(0);
      if (row < m)
        v = id_entry<T>(P, sol_dim, row, nI, rows, act[j], nprox, pcos, psin, t.cx, t.cy,
                        t.rad_proxy);
      B[i + (size_t)kFoldRows * j] = v;
    }
    __syncthreads();
    for (int j = 0; j < n; j++) {
      if (warp == 0) {
        T b = B[lane + (size_t)kFoldRows * j];
        T sigma = warp_sum(b * b);
        T alpha = R[j + (size_t)n * j];
        T tau = T(0), beta = alpha, scale = T(0);
        if (sigma != T(0)) {
          T nrm = sqrt(alpha * alpha + sigma);
          beta = alpha >= T(0) ? -nrm : nrm;
          tau = (beta - alpha) / beta;
          scale = T(1) / (alpha - beta);
        }
        B[lane + (size_t)kFoldRows * j] = b * scale;   // u (v = [1; u])
        if (lane == 0) { s_tau = tau; s_beta = beta; }
      }
      __syncthreads();
      T tau = s_tau;
      if (tau != T(0)) {
        T u = B[lane + (size_t)kFoldRows * j];
        for (int c = j + 1 + warp; c < n; c += nwarps) {
          T bc = B[lane + (size_t)kFoldRows * c];
          T rjc = R[j + (size_t)n * c];
          T w = (warp_sum(u * bc) + rjc) * tau;
          B[lane + (size_t)kFoldRows * c] = bc - w * u;
          if (lane == 0) R[j + (size_t)n * c] = rjc - w;
        }
      }
      if (threadIdx.x == 0) R[j + (size_t)n * j] = s_beta;
      __syncthreads();
    }
  }

  // 3. column-pivoted QR of the n x n triangle (LAPACK xGEQP3/xLAQP2 norm
  //    downdating with recomputation after cancellation), stopping at the
  //    first |R_jj| < tol |R_00| for j >= 1
  for (int c = warp; c < n; c += nwarps) {
    T s = T(0);
    for (int i = lane; i <= c; i += 32) s += R[i + (size_t)n * c] * R[i + (size_t)n * c];
    s = warp_sum(s);
    if (lane == 0) { vn1[c] = sqrt(s); vn2[c] = vn1[c]; perm[c] = c; }
  }
  if (threadIdx.x == 0) { s_k = 0; s_stop = 0; }
  __syncthreads();
  T thresh = T(0);
  const int jmax = min(n, m);
  for (int j = 0; j < jmax; j++) {
    if (warp == 0) {
      T best = T(-1);
      int bi = j;
      for (int c = j + lane; c < n; c += 32) {
        T v = vn1[c];
        if (v > best) { best = v; bi = c; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        T ov = __shfl_down_sync(0xffffffff, best, o);
        int oi = __shfl_down_sync(0xffffffff, bi, o);
        if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
      }
      if (lane == 0) s_piv = bi;
    }
    __syncthreads();
    int p = s_piv;
    if (p != j) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        T a = R[i + (size_t)n * j];
        R[i + (size_t)n * j] = R[i + (size_t)n * p];
        R[i + (size_t)n * p] = a;
      }
      if (threadIdx.x == 0) {
        int a = perm[j]; perm[j] = perm[p]; perm[p] = a;
        T v = vn1[j]; vn1[j] = vn1[p]; vn1[p] = v;
        v = vn2[j]; vn2[j] = vn2[p]; vn2[p] = v;
      }
    }
    __syncthreads();
    // Householder for R(j:n, j)
    if (warp == 0) {
      T sigma = T(0);
      for (int i = j + 1 + lane; i < n; i += 32) sigma += R[i + (size_t)n * j] * R[i + (size_t)n * j];
      sigma = warp_sum(sigma);
      T alpha = R[j + (size_t)n * j];
      T tau = T(0), beta = alpha, scale = T(0);
      if (sigma != T(0)) {
        T nrm = sqrt(alpha * alpha + sigma);
        beta = alpha >= T(0) ? -nrm : nrm;
        tau = (beta - alpha) / beta;
        scale = T(1) / (alpha - beta);
      }
      for (int i = j + 1 + lane; i < n; i += 32) R[i + (size_t)n * j] *= scale;
      if (lane == 0) {
        s_tau = tau;
        s_beta = beta;
        R[j + (size_t)n * j] = beta;
      }
    }
    __syncthreads();
    T beta = s_beta;
    if (j == 0) thresh = fabs(T(tol) * beta);
    if (j >= 1 && fabs(beta) < thresh) {
      if (threadIdx.x == 0) s_k = j;
      break;
    }
    T tau = s_tau;
    for (int c = j + 1 + warp; c < n; c += nwarps) {
      if (tau != T(0)) {
        T rjc0 = R[j + (size_t)n * c];
        T part = T(0);
        for (int i = j + 1 + lane; i < n; i += 32) part += R[i + (size_t)n * j] * R[i + (size_t)n * c];
        T w = (warp_sum(part) + rjc0) * tau;
        for (int i = j + 1 + lane; i < n; i += 32) R[i + (size_t)n * c] -= w * R[i + (size_t)n * j];
        if (lane == 0) R[j + (size_t)n * c] = rjc0 - w;
        __syncwarp();
      }
      // norm downdate of column c (xLAQP2), recomputed after cancellation
      T rjc = R[j + (size_t)n * c];
      T v1 = vn1[c];
      int recompute = 0;
      T newv = v1;
      if (v1 != T(0)) {
        T temp = fabs(rjc) / v1;
        temp = T(1) - temp * temp;
        temp = temp < T(0) ? T(0) : temp;
        T q = v1 / vn2[c];
        T temp2 = temp * q * q;
        if (temp2 <= tol3z<T>()) recompute = 1;
        else newv = v1 * sqrt(temp);
      }
      if (recompute) {
        T s2 = T(0);
        for (int i = j + 1 + lane; i < n; i += 32) s2 += R[i + (size_t)n * c] * R[i + (size_t)n * c];
        newv = sqrt(warp_sum(s2));
      }
      __syncwarp();
      if (lane == 0) {
        vn1[c] = newv;
        if (recompute) vn2[c] = newv;
      }
      __syncwarp();
    }
    __syncthreads();
  }
  __syncthreads();
  const int k = s_k;
  if (threadIdx.x == 0) k_out[blockIdx.x] = k;
  if (k == 0) return;
  const int r = n - k;

  // 4. T = R11^-1 R12 (k x r), one thread per column, and the permuted list
  for (int c = threadIdx.x; c < r; c += blockDim.x) {
    T* tc = Tout + (size_t)k * c;
    const T* rc = R + (size_t)n * (k + c);
    for (int i = k - 1; i >= 0; i--) {
      T s = rc[i];
      for (int l = i + 1; l < k; l++) s -= R[i + (size_t)n * l] * tc[l];
      tc[i] = s / R[i + (size_t)n * i];
    }
  }
  int* pact = ipool + t.pact;
  for (int i = threadIdx.x; i < n; i += blockDim.x) pact[i] = act[perm[i]];
  (void)err;
}

// Self block K_BN of a box (kernel entries plus children's accumulated
// self-blocks on the diagonal).
template <typename T>
__global__ void k_assemble(const AsmTask<T>* tasks, const int* ipool, Points<T> P, int sol_dim) {
  const AsmTask<T> t = tasks[blockIdx.x];
  const int n = t.n;
  const int* act = ipool + t.act;
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    int i = idx % n, j = idx / n;
    T v;
    int ci = -1, cj = -1;
    for (int c = 0; c < t.nchild; c++) {
      if (i >= t.coff[c] && i < t.coff[c] + t.clen[c]) ci = c;
      if (j >= t.coff[c] && j < t.coff[c] + t.clen[c]) cj = c;
    }
    if (ci >= 0 && ci == cj) {
      int l = t.clen[ci];
      v = t.ctile[ci][(i - t.coff[ci]) + (size_t)l * (j - t.coff[ci])];
    } else {
      v = kernel_entry<T>(P, sol_dim, act[i], act[j]);
    }
    t.out[i + (size_t)n * j] = v;
  }
}

// Schur-complement elimination of a compressed box
// (SkelFactorization::decouple, skel_factorization.cpp:91-127).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_schur(const SchurTask<T>* tasks, int* err) {
  const SchurTask<T> t = tasks[blockIdx.x];
  const int n = t.n, k = t.k, r = n - k;
  __shared__ T s_red;
  __shared__ int s_idx, s_flag;
  T* Pm = t.ws;                       // permuted K_BN
  T* Wrs = Pm + (size_t)n * n;        // r x k
  T* Wsr = Wrs + (size_t)r * k;       // k x r
  T* Lt = Wsr + (size_t)k * r;        // r x k
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    int i = idx % n, j = idx / n;
    Pm[idx] = t.K[t.perm[i] + (size_t)n * t.perm[j]];
  }
  for (int idx = threadIdx.x; idx < k * r; idx += blockDim.x) t.Tout[idx] = t.Tin[idx];
  __syncthreads();
  const T* Kss = Pm;
  const T* Ksr = Pm + (size_t)n * k;
  const T* Krs = Pm + k;
  const T* Krr = Pm + k + (size_t)n * k;
  const T* Tm = t.Tin;
  // K~_rs = K_rs - T^T K_ss  (r x k)
  for (int idx = threadIdx.x; idx < r * k; idx += blockDim.x) {
    int i = idx % r, j = idx / r;
    Wrs[idx] = Krs[i + (size_t)n * j];
  }
  __syncthreads();
  cta_gemm<T>(r, k, k, T(-1), Tm, k, true, Kss, n, false, T(1), Wrs, r);
  // X = K_rr - T^T K_sr - K~_rs T  (r x r)
  for (int idx = threadIdx.x; idx < r * r; idx += blockDim.x) {
    int i = idx % r, j = idx / r;
    t.X[idx] = Krr[i + (size_t)n * j];
  }
  // K~_sr = K_sr - K_ss T  (k x r)
  for (int idx = threadIdx.x; idx < k * r; idx += blockDim.x) {
    int i = idx % k, j = idx / k;
    Wsr[idx] = Ksr[i + (size_t)n * j];
  }
  __syncthreads();
  cta_gemm<T>(r, r, k, T(-1), Tm, k, true, Ksr, n, false, T(1), t.X, r);
  __syncthreads();
  cta_gemm<T>(r, r, k, T(-1), Wrs, r, false, Tm, k, false, T(1), t.X, r);
  cta_gemm<T>(k, r, k, T(-1), Kss, n, false, Tm, k, false, T(1), Wsr, k);
  __syncthreads();
  int info = cta_lu<T>(r, t.X, r, t.piv, &s_flag, &s_red, &s_idx);
  if (info != 0 && threadIdx.x == 0) atomicMax(err, (int)kDevSingular);
  // U = X^-1 K~_rs (r x k)
  for (int idx = threadIdx.x; idx < r * k; idx += blockDim.x) t.U[idx] = Wrs[idx];
  // L^T = X^-T K~_sr^T (r x k)
  for (int idx = threadIdx.x; idx < r * k; idx += blockDim.x) {
    int i = idx % r, j = idx / r;
    Lt[idx] = Wsr[j + (size_t)k * i];
  }
  __syncthreads();
  cta_lu_solve<T>(r, t.X, r, t.piv, false, t.U, r, k);
  cta_lu_solve<T>(r, t.X, r, t.piv, true, Lt, r, k);
  for (int idx = threadIdx.x; idx < k * r; idx += blockDim.x) {
    int i = idx % k, j = idx / k;
    t.L[idx] = Lt[j + (size_t)r * i];
  }
  __syncthreads();
  // A~ = K_ss - L K~_rs  (k x k)
  for (int idx = threadIdx.x; idx < k * k; idx += blockDim.x) {
    int i = idx % k, j = idx / k;
    t.Atil[idx] = Kss[i + (size_t)n * j];
  }
  __syncthreads();
  cta_gemm<T>(k, k, r, T(-1), t.L, k, false, Wrs, r, false, T(1), t.Atil, k);
}

// Dense LU of the root block on one CTA.
template <typename T>
__global__ void k_root_lu(T* A, int n, int* piv, int* err) {
  __shared__ T s_red;
  __shared__ int s_idx, s_flag;
  int info = cta_lu<T>(n, A, n, piv, &s_flag, &s_red, &s_idx);
  if (info != 0 && threadIdx.x == 0) atomicMax(err, (int)kDevSingular);
}

template <typename T>
__global__ void k_check_finite(const T* a, size_t n, int* err) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    if (!isfinite(a[i])) atomicMax(err, (int)kDevNonFinite);
}

// ---------------------------------------------------------------- solve --
template <typename T>
struct SweepTask {
  int n, k;
  const int* pact;
  const T* Tm;   // k x r
  const T* L;    // k x r
  const T* U;    // r x k
  const T* X;    // r x r LU
  const int* piv;
};

enum SweepMode : int {
  kUpDiag = 0,     // x_r -= T^T x_s; x_s -= L x_r; x_r <- X^-1 x_r
  kUp = 1,         // without the diagonal solve
  kPsi = 2,        // x_r -= T^T x_s; x_s -= U^T x_r   (transposed down sweep)
  kDown = 3,       // x_r -= U x_s; x_s -= T x_r
  kDiag = 4,       // x_r <- X^-1 x_r
};

// x is DOF-major: row = DOF, ld = ldx; a CTA handles one box and a chunk of
// `cw` columns starting at blockIdx.y * cw.
template <typename T>
__global__ void k_sweep(const SweepTask<T>* tasks, T* x, int ldx, int ncols, int cw, int mode) {
  extern __shared__ unsigned char smem_raw[];
  T* sx = reinterpret_cast<T*>(smem_raw);
  const SweepTask<T> t = tasks[blockIdx.x];
  const int n = t.n, k = t.k, r = n - k;
  const int c0 = blockIdx.y * cw;
  const int nc = min(cw, ncols - c0);
  if (nc <= 0) return;
  // sx: n x nc column-major (rows 0..k-1 skeleton, k..n-1 redundant)
  for (int idx = threadIdx.x; idx < n * nc; idx += blockDim.x) {
    int i = idx % n, c = idx / n;
    sx[idx] = x[(size_t)t.pact[i] * ldx + c0 + c];
  }
  __syncthreads();
  T* xs = sx;
  T* xr = sx + k;
  if (mode == kUpDiag || mode == kUp || mode == kPsi) {
    // x_r -= T^T x_s
    for (int idx = threadIdx.x; idx < r * nc; idx += blockDim.x) {
      int i = idx % r, c = idx / r;
      T acc = T(0);
      const T* tc = t.Tm + (size_t)k * i;
      for (int l = 0; l < k; l++) acc += tc[l] * xs[l + (size_t)n * c];
      xr[i + (size_t)n * c] -= acc;
    }
    __syncthreads();
    // x_s -= L x_r   or   x_s -= U^T x_r
    for (int idx = threadIdx.x; idx < k * nc; idx += blockDim.x) {
      int l = idx % k, c = idx / k;
      T acc = T(0);
      if (mode == kPsi) {
        const T* uc = t.U + (size_t)r * l;
        for (int i = 0; i < r; i++) acc += uc[i] * xr[i + (size_t)n * c];
      } else {
        for (int i = 0; i < r; i++) acc += t.L[l + (size_t)k * i] * xr[i + (size_t)n * c];
      }
      xs[l + (size_t)n * c] -= acc;
    }
    __syncthreads();
    if (mode == kUpDiag) cta_lu_solve<T>(r, t.X, r, t.piv, false, xr, n, nc);
  } else if (mode == kDown) {
    // x_r -= U x_s
    for (int idx = threadIdx.x; idx < r * nc; idx += blockDim.x) {
      int i = idx % r, c = idx / r;
      T acc = T(0);
      for (int l = 0; l < k; l++) acc += t.U[i + (size_t)r * l] * xs[l + (size_t)n * c];
      xr[i + (size_t)n * c] -= acc;
    }
    __syncthreads();
    // x_s -= T x_r
    for (int idx = threadIdx.x; idx < k * nc; idx += blockDim.x) {
      int l = idx % k, c = idx / k;
      T acc = T(0);
      for (int i = 0; i < r; i++) acc += t.Tm[l + (size_t)k * i] * xr[i + (size_t)n * c];
      xs[l + (size_t)n * c] -= acc;
    }
    __syncthreads();
  } else if (mode == kDiag) {
    cta_lu_solve<T>(r, t.X, r, t.piv, false, xr, n, nc);
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < n * nc; idx += blockDim.x) {
    int i = idx % n, c = idx / n;
    x[(size_t)t.pact[i] * ldx + c0 + c] = sx[idx];
  }
}

// Root solve: y = A^-1 x[idx] (dense LU), scattered back.
template <typename T>
__global__ void k_root_solve(const T* LU, const int* piv, const int* idx, int n, T* x, int ldx,
                             int ncols, T* ws) {
  for (int e = threadIdx.x; e < n * ncols; e += blockDim.x) {
    int i = e % n, c = e / n;
    ws[e] = x[(size_t)idx[i] * ldx + c];
  }
  __syncthreads();
  cta_lu_solve<T>(n, LU, n, piv, false, ws, n, ncols);
  for (int e = threadIdx.x; e < n * ncols; e += blockDim.x) {
    int i = e % n, c = e / n;
    x[(size_t)idx[i] * ldx + c] = ws[e];
  }
}

template <typename T>
__global__ void k_fill_points(const double* pts, const double* nrm, const double* w,
                              const double* kap, int n, T* x, T* y, T* nx, T* ny, T* ww, T* kk) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] = T(pts[2 * i]);
    y[i] = T(pts[2 * i + 1]);
    nx[i] = T(nrm[2 * i]);
    ny[i] = T(nrm[2 * i + 1]);
    ww[i] = T(w[i]);
    kk[i] = kap ? T(kap[i]) : T(0);
  }
}

template <typename T>
void upload(T* dst, const std::vector<T>& v, cudaStream_t s) {
  if (!v.empty())
    KI_CUDA(cudaMemcpyAsync(dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s));
}

struct HostBox {
  int n = 0;           // active DOFs
  int k = 0;           // rank if compressed
  bool compressed = false;
  int64_t act = 0;     // ipool offset of the active list
  int64_t pact = 0;    // ipool offset of the permuted list (compressed)
  const void* tile = nullptr;  // accumulated self-block on the device
};

}  // namespace

template <typename T>
std::unique_ptr<Factorization<T>> factorize(const Params& prm, int n_points, const double* points,
                                            const double* normals, const double* weights,
                                            const double* curvatures, const HoleDesc& holes,
                                            cudaStream_t stream) {
  auto t_start = std::chrono::steady_clock::now();
  auto F = std::make_unique<Factorization<T>>();
  F->prm = prm;
  F->stream = stream;
  F->n_points = n_points;
  Tree& tree = F->tree;
  tree.build(points, n_points, prm.sol_dim, prm.max_leaf_dofs);
  const int sd = prm.sol_dim;
  const int N = tree.n_dofs;
  F->N = N;
  const int L = tree.num_levels();
  cudaStream_t s = stream;

  // point data
  {
    double* d_in = (double*)F->alloc(sizeof(double) * (size_t)n_points * 6);
    KI_CUDA(cudaMemcpyAsync(d_in, points, sizeof(double) * 2 * n_points, cudaMemcpyHostToDevice, s));
    KI_CUDA(cudaMemcpyAsync(d_in + 2 * (size_t)n_points, normals, sizeof(double) * 2 * n_points,
                            cudaMemcpyHostToDevice, s));
    KI_CUDA(cudaMemcpyAsync(d_in + 4 * (size_t)n_points, weights, sizeof(double) * n_points,
                            cudaMemcpyHostToDevice, s));
    if (curvatures)
      KI_CUDA(cudaMemcpyAsync(d_in + 5 * (size_t)n_points, curvatures, sizeof(double) * n_points,
                              cudaMemcpyHostToDevice, s));
    T* d = (T*)F->alloc(sizeof(T) * (size_t)n_points * 6);
    F->d_x = d; F->d_y = d + n_points; F->d_nx = d + 2 * (size_t)n_points;
    F->d_ny = d + 3 * (size_t)n_points; F->d_w = d + 4 * (size_t)n_points;
    F->d_kappa = d + 5 * (size_t)n_points;
    k_fill_points<T><<<std::min(1024, (n_points + 255) / 256), 256, 0, s>>>(
        d_in, d_in + 2 * (size_t)n_points, d_in + 4 * (size_t)n_points,
        curvatures ? d_in + 5 * (size_t)n_points : nullptr, n_points, F->d_x, F->d_y, F->d_nx,
        F->d_ny, F->d_w, F->d_kappa);
    KI_CUDA(cudaGetLastError());
  }
  Points<T> P{F->d_x, F->d_y, F->d_nx, F->d_ny, F->d_w, F->d_kappa};
  F->d_err = (int*)F->alloc(sizeof(int));
  KI_CUDA(cudaMemsetAsync(F->d_err, 0, sizeof(int), s));

  // proxy angles (Kernel::get_proxy_mat: ang = 2 pi i / P)
  const int np = prm.num_proxy_points;
  double* d_pcs = (double*)F->alloc(sizeof(double) * 2 * std::max(np, 1));
  {
    std::vector<double> pc(2 * std::max(np, 1));
    for (int i = 0; i < np; i++) {
      double ang = 2 * M_PI * i * (1.0 / np);
      pc[i] = std::cos(ang);
      pc[np + i] = std::sin(ang);
    }
    upload(d_pcs, pc, s);
  }

  // integer pool: dof_sorted | per-level active lists | permuted lists
  const int64_t ipool_size = (int64_t)N * (2 * (int64_t)L + 1) + 16;
  int* ipool = (int*)F->alloc(sizeof(int) * ipool_size);
  upload(ipool, tree.dof_sorted, s);
  int64_t ipool_top = N;   // bump pointer for active lists
  int64_t pact_top = (int64_t)N * (L + 1);

  std::vector<HostBox> hb(tree.boxes.size());
  for (size_t b = 0; b < tree.boxes.size(); b++)
    if (tree.boxes[b].leaf) hb[b].n = tree.boxes[b].orig_count;

  F->levels.resize(L);
  std::vector<void*> level_scratch;
  const size_t Tsz = sizeof(T);

  for (int l = L - 1; l >= 0; l--) {
    const std::vector<int>& lv = tree.levels[l];
    // ---- active lists of the level
    std::vector<ActiveTask> atasks;
    for (int b : lv) {
      const Box& bx = tree.boxes[b];
      HostBox& h = hb[b];
      ActiveTask at{};
      if (bx.leaf) {
        h.n = bx.orig_count;
        at.nseg = 1;
        at.src[0] = bx.orig_start;
        at.len[0] = h.n;
      } else {
        h.n = 0;
        at.nseg = 4;
        for (int ci = 0; ci < 4; ci++) {
          const HostBox& c = hb[bx.child[ci]];
          at.src[ci] = c.compressed ? c.pact : c.act;
          at.len[ci] = c.compressed ? c.k : c.n;
          h.n += at.len[ci];
        }
      }
      h.act = ipool_top;
      at.dst = ipool_top;
      ipool_top += h.n;
      if (h.n > 0) atasks.push_back(at);
    }
    if (!atasks.empty()) {
      ActiveTask* d_at = (ActiveTask*)F->alloc(sizeof(ActiveTask) * atasks.size());
      upload(d_at, atasks, s);
      k_build_active<<<(unsigned)atasks.size(), 128, 0, s>>>(d_at, ipool);
      KI_CUDA(cudaGetLastError());
    }
    if (l == 0) break;

    // ---- self blocks of every box with active DOFs
    std::vector<AsmTask<T>> asm_tasks;
    int64_t kbn_total = 0;
    for (int b : lv) kbn_total += (int64_t)hb[b].n * hb[b].n;
    T* d_kbn = (T*)F->alloc(Tsz * (kbn_total + 1));
    std::vector<T*> kbn_of(lv.size(), nullptr);
    {
      int64_t off = 0;
      for (size_t i = 0; i < lv.size(); i++) {
        int b = lv[i];
        const Box& bx = tree.boxes[b];
        HostBox& h = hb[b];
        if (h.n == 0) continue;
        AsmTask<T> at{};
        at.act = h.act;
        at.n = h.n;
        at.out = d_kbn + off;
        kbn_of[i] = at.out;
        off += (int64_t)h.n * h.n;
        if (!bx.leaf) {
          int o = 0;
          for (int ci = 0; ci < 4; ci++) {
            const HostBox& c = hb[bx.child[ci]];
            int len = c.compressed ? c.k : c.n;
            if (len == 0) continue;
            at.coff[at.nchild] = o;
            at.clen[at.nchild] = len;
            at.ctile[at.nchild] = (const T*)c.tile;
            at.nchild++;
            o += len;
          }
        }
        h.tile = at.out;   // uncompressed boxes pass K_BN up as their self-block
        asm_tasks.push_back(at);
      }
    }
    if (!asm_tasks.empty()) {
      AsmTask<T>* d_as = (AsmTask<T>*)F->alloc(sizeof(AsmTask<T>) * asm_tasks.size());
      upload(d_as, asm_tasks, s);
      k_assemble<T><<<(unsigned)asm_tasks.size(), kThreads, 0, s>>>(d_as, ipool, P, sd);
      KI_CUDA(cudaGetLastError());
    }

    // ---- ID tasks
    std::vector<int> comp;  // boxes to compress
    for (int b : lv)
      if (hb[b].n >= prm.min_dofs_to_compress && hb[b].n > 0) comp.push_back(b);
    std::vector<IdTask> itasks;
    std::vector<int64_t> seg_off;
    std::vector<int> seg_len;
    int64_t rows_cap = 0, ws_cap = 0, perm_cap = 0;
    auto add_seg = [&](int64_t off, int len) {
      if (len > 0) { seg_off.push_back(off); seg_len.push_back(len); }
    };
    for (int b : comp) {
      const Box& bx = tree.boxes[b];
      const HostBox& h = hb[b];
      IdTask it{};
      it.act = h.act;
      it.n = h.n;
      it.cx = bx.cx;
      it.cy = bx.cy;
      it.seg_begin = (int)seg_off.size();
      if (l == 1 || l == 2) {
        // Kernel::get_id_mat levels 1/2 (kernel.cpp:441-563): every other box of
        // the level, plus (level 2) the leaves of the levels above; no proxy.
        it.mode = 1;
        for (int o : lv)
          if (o != b) add_seg(hb[o].act, hb[o].n);
        if (l == 2)
          for (int ll = l - 1; ll >= 0; ll--)
            for (int o : tree.levels[ll])
              if (tree.boxes[o].leaf) add_seg(tree.boxes[o].orig_start, tree.boxes[o].orig_count);
      } else {
        it.mode = 0;
        it.rad_filter = std::sqrt(2.0) * prm.radius_ratio * (bx.side / 2);
        it.rad_proxy = (bx.side / 2) * std::sqrt(2.0) * prm.radius_ratio;
        for (int o : bx.coarse_nbrs) add_seg(tree.boxes[o].orig_start, tree.boxes[o].orig_count);
        for (int o : bx.same_nbrs) {
          const Box& ob = tree.boxes[o];
          if (ob.leaf) add_seg(ob.orig_start, ob.orig_count);
          else add_seg(hb[o].act, hb[o].n);
        }
      }
      it.seg_end = (int)seg_off.size();
      int64_t cand = 0;
      for (int q = it.seg_begin; q < it.seg_end; q++) cand += seg_len[q];
      it.rows = rows_cap;
      rows_cap += cand + 1;
      int64_t n = h.n;
      it.ws = ws_cap;
      ws_cap += n * n + kFoldRows * n + 2 * n + n * n / 4 + 1;
      it.perm = perm_cap;
      perm_cap += n;
      itasks.push_back(it);
    }
    LevelFactor& LF = F->levels[l];
    if (itasks.empty()) continue;
    // scratch
    int* d_irows = (int*)F->alloc(sizeof(int) * (rows_cap + perm_cap + 16));
    T* d_tws = (T*)F->alloc(Tsz * (ws_cap + 16));
    for (auto& it : itasks) {
      it.perm += rows_cap;
      it.pact = pact_top;
      pact_top += it.n;
    }
    for (size_t i = 0; i < comp.size(); i++) hb[comp[i]].pact = itasks[i].pact;
    IdTask* d_it = (IdTask*)F->alloc(sizeof(IdTask) * itasks.size());
    int64_t* d_soff = (int64_t*)F->alloc(sizeof(int64_t) * (seg_off.size() + 1));
    int* d_slen = (int*)F->alloc(sizeof(int) * (seg_len.size() + 1));
    int* d_k = (int*)F->alloc(sizeof(int) * itasks.size());
    upload(d_it, itasks, s);
    upload(d_soff, seg_off, s);
    upload(d_slen, seg_len, s);
    k_id<T><<<(unsigned)itasks.size(), kThreads, 0, s>>>(d_it, d_soff, d_slen, ipool, d_irows, d_tws, P, sd,
                                                         np, d_pcs, d_pcs + np, prm.id_tol, d_k,
                                                         F->d_err);
    KI_CUDA(cudaGetLastError());
    std::vector<int> kh(itasks.size());
    KI_CUDA(cudaMemcpyAsync(kh.data(), d_k, sizeof(int) * kh.size(), cudaMemcpyDeviceToHost, s));
    KI_CUDA(cudaStreamSynchronize(s));

    // ---- Schur elimination of the compressed boxes
    std::vector<int> ci_list;
    int64_t tr_tot = 0, x_tot = 0, r_tot = 0, kk_tot = 0, ws_tot = 0;
    for (size_t i = 0; i < comp.size(); i++) {
      if (kh[i] == 0) continue;
      int64_t n = itasks[i].n, k = kh[i], r = n - k;
      ci_list.push_back((int)i);
      tr_tot += k * r;
      x_tot += r * r;
      r_tot += r;
      kk_tot += k * k;
      ws_tot += n * n + 3 * r * k;
    }
    LF.n_comp = (int)ci_list.size();
    if (ci_list.empty()) continue;
    T* d_Tp = (T*)F->alloc(Tsz * (tr_tot + 1));
    T* d_LUp = (T*)F->alloc(Tsz * (2 * tr_tot + 1));
    T* d_Xp = (T*)F->alloc(Tsz * (x_tot + 1));
    int* d_pivp = (int*)F->alloc(sizeof(int) * (r_tot + 1));
    T* d_At = (T*)F->alloc(Tsz * (kk_tot + 1));
    T* d_sws = (T*)F->alloc(Tsz * (ws_tot + 1));
    std::vector<SchurTask<T>> st;
    std::vector<SweepTask<T>> sw;
    int64_t o_tr = 0, o_x = 0, o_r = 0, o_kk = 0, o_ws = 0;
    for (int i : ci_list) {
      int b = comp[i];
      int n = itasks[i].n, k = kh[i], r = n - k;
      size_t pos = tree.boxes[b].level_pos;
      SchurTask<T> t{};
      t.K = kbn_of[pos];
      t.n = n;
      t.k = k;
      t.perm = d_irows + itasks[i].perm;
      t.Tin = d_tws + itasks[i].ws + (int64_t)n * n + kFoldRows * (int64_t)n + 2 * (int64_t)n;
      t.Tout = d_Tp + o_tr;
      t.L = d_LUp + 2 * o_tr;
      t.U = d_LUp + 2 * o_tr + (int64_t)k * r;
      t.X = d_Xp + o_x;
      t.piv = d_pivp + o_r;
      t.Atil = d_At + o_kk;
      t.ws = d_sws + o_ws;
      o_tr += (int64_t)k * r;
      o_x += (int64_t)r * r;
      o_r += r;
      o_kk += (int64_t)k * k;
      o_ws += (int64_t)n * n + 3 * (int64_t)r * k;
      st.push_back(t);
      SweepTask<T> w{};
      w.n = n;
      w.k = k;
      w.pact = ipool + itasks[i].pact;
      w.Tm = t.Tout;
      w.L = t.L;
      w.U = t.U;
      w.X = t.X;
      w.piv = t.piv;
      sw.push_back(w);
      HostBox& h = hb[b];
      h.compressed = true;
      h.k = k;
      h.tile = t.Atil;
      F->n_compressed++;
      F->n_redundant += r;
      LF.max_n = std::max(LF.max_n, n);
    }
    SchurTask<T>* d_st = (SchurTask<T>*)F->alloc(sizeof(SchurTask<T>) * st.size());
    upload(d_st, st, s);
    k_schur<T><<<(unsigned)st.size(), kThreads, 0, s>>>(d_st, F->d_err);
    KI_CUDA(cudaGetLastError());
    SweepTask<T>* d_sw = (SweepTask<T>*)F->alloc(sizeof(SweepTask<T>) * sw.size());
    upload(d_sw, sw, s);
    LF.d_tasks = d_sw;
    for (int i : ci_list) F->rank_hist.push_back(kh[i]);
  }

  // ---- root block
  {
    int root = tree.levels[0][0];
    HostBox& h = hb[root];
    F->n_root = h.n;
    const Box& bx = tree.boxes[root];
    if (h.n > 0) {
      F->d_root_idx = ipool + h.act;
      T* A = (T*)F->alloc(Tsz * (size_t)h.n * h.n);
      AsmTask<T> at{};
      at.act = h.act;
      at.n = h.n;
      at.out = A;
      if (!bx.leaf) {
        int o = 0;
        for (int ci = 0; ci < 4; ci++) {
          const HostBox& c = hb[bx.child[ci]];
          int len = c.compressed ? c.k : c.n;
          if (len == 0) continue;
          at.coff[at.nchild] = o;
          at.clen[at.nchild] = len;
          at.ctile[at.nchild] = (const T*)c.tile;
          at.nchild++;
          o += len;
        }
      }
      AsmTask<T>* d_as = (AsmTask<T>*)F->alloc(sizeof(AsmTask<T>));
      KI_CUDA(cudaMemcpyAsync(d_as, &at, sizeof(at), cudaMemcpyHostToDevice, s));
      k_assemble<T><<<1, kThreads, 0, s>>>(d_as, ipool, P, sd);
      KI_CUDA(cudaGetLastError());
      if (holes.n_holes > 0) throw std::runtime_error("multiply connected problems: not yet supported");
      F->d_root_lu = A;
      F->d_root_piv = (int*)F->alloc(sizeof(int) * h.n);
      k_root_lu<T><<<1, 1024, 0, s>>>(A, h.n, F->d_root_piv, F->d_err);
      KI_CUDA(cudaGetLastError());
      F->n_root_sys = h.n;
    }
  }
  int herr = 0;
  KI_CUDA(cudaMemcpyAsync(&herr, F->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  KI_CUDA(cudaStreamSynchronize(s));
  if (herr == kDevSingular) throw std::runtime_error("singular pivot in a Schur or root LU factorization");
  if (herr == kDevNonFinite) throw std::runtime_error("non-finite values in the factorization");
  F->factor_seconds =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  return F;
}

template <typename T>
void solve_device(Factorization<T>& F, T* d_x, int ncols, T* d_alpha) {
  cudaStream_t s = F.stream;
  const int L = (int)F.levels.size();
  auto launch = [&](int l, int mode) {
    LevelFactor& LF = F.levels[l];
    if (LF.n_comp == 0) return;
    int cw = std::max(1, std::min(ncols, (int)(96 * 1024 / (sizeof(T) * std::max(1, LF.max_n)))));
    cw = std::min(cw, 32);
    dim3 grid(LF.n_comp, (ncols + cw - 1) / cw);
    size_t sm = sizeof(T) * (size_t)LF.max_n * cw;
    if (sm > 200 * 1024) throw std::runtime_error("box too large for the sweep kernel");
    if (sm > 48 * 1024)
      KI_CUDA(cudaFuncSetAttribute(k_sweep<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_sweep<T><<<grid, kThreads, sm, s>>>(reinterpret_cast<SweepTask<T>*>(LF.d_tasks), d_x, ncols, ncols,
                                          cw, mode);
    KI_CUDA(cudaGetLastError());
  };
  for (int l = L - 1; l >= 1; l--) launch(l, kUpDiag);
  if (F.n_root > 0) {
    T* ws = (T*)F.alloc(sizeof(T) * (size_t)F.n_root * ncols);
    k_root_solve<T><<<1, 1024, 0, s>>>(F.d_root_lu, F.d_root_piv, F.d_root_idx, F.n_root, d_x,
                                       ncols, ncols, ws);
    KI_CUDA(cudaGetLastError());
  }
  for (int l = 1; l < L; l++) launch(l, kDown);
  (void)d_alpha;
}

template std::unique_ptr<Factorization<double>> factorize<double>(
    const Params&, int, const double*, const double*, const double*, const double*,
    const HoleDesc&, cudaStream_t);
template std::unique_ptr<Factorization<float>> factorize<float>(
    const Params&, int, const double*, const double*, const double*, const double*,
    const HoleDesc&, cudaStream_t);
template void solve_device<double>(Factorization<double>&, double*, int, double*);
template void solve_device<float>(Factorization<float>&, float*, int, float*);
template struct Factorization<double>;
template struct Factorization<float>;

}  // namespace ki
