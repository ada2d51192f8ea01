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
#include "ki_launch.cuh"
#include "ki_pool.h"
#include "ki_factor.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "ki_common.cuh"
#include "ki_dense.h"
#include "ki_mlp.h"
#include "ki_tc.cuh"
#include "ki_tree_gpu.h"
#include "ki_tune.h"

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
  cudaError_t e = pool_malloc(&p, bytes, stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw std::runtime_error(std::string("device allocation failed: ") + cudaGetErrorString(e));
  }
  owned.push_back(p);
  device_bytes += bytes;
  return p;
}

template <typename T>
void Factorization<T>::stage_begin(const char* name, double flops, double bytes, cudaStream_t on) {
  StageRec r;
  r.stage = name;
  r.flops = flops;
  r.bytes = bytes;
  KI_CUDA(cudaEventCreate(&r.a));
  KI_CUDA(cudaEventCreate(&r.b));
  KI_CUDA(cudaEventRecord(r.a, on ? on : stream));
  prof_stack.push_back(prof_open.size());
  prof_open.push_back(r);
}

template <typename T>
void Factorization<T>::stage_end(cudaStream_t on) {
  if (prof_stack.empty()) throw std::logic_error("stage_end without stage_begin");
  size_t idx = prof_stack.back();
  prof_stack.pop_back();
  KI_CUDA(cudaEventRecord(prof_open[idx].b, on ? on : stream));
}

template <typename T>
std::vector<StageSum> Factorization<T>::collect() {
  std::vector<StageSum> out;
  for (auto& r : prof_open) {
    float ms = 0;
    KI_CUDA(cudaEventSynchronize(r.b));
    KI_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
    StageSum* d = nullptr;
    for (auto& o : out)
      if (o.stage == r.stage) d = &o;
    if (!d) {
      out.push_back(StageSum{r.stage});
      d = &out.back();
    }
    d->launches++;
    d->ms += ms;
    d->flops += r.flops;
    d->bytes += r.bytes;
  }
  prof_open.clear();
  return out;
}

template <typename T>
void Factorization<T>::fork() {
  if (serial) {
    for (int i = 0; i < kAux; i++) aux[i] = stream;
    return;
  }
  if (!fork_ev) {
    KI_CUDA(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
    for (int i = 0; i < kAux; i++) {
      KI_CUDA(cudaStreamCreateWithFlags(&aux[i], cudaStreamNonBlocking));
      KI_CUDA(cudaEventCreateWithFlags(&join_ev[i], cudaEventDisableTiming));
    }
  }
  KI_CUDA(cudaEventRecord(fork_ev, stream));
  for (int i = 0; i < kAux; i++) KI_CUDA(cudaStreamWaitEvent(aux[i], fork_ev, 0));
}

template <typename T>
void Factorization<T>::join(int used) {
  if (serial) return;
  for (int i = 0; i < used && i < kAux; i++) {
    KI_CUDA(cudaEventRecord(join_ev[i], aux[i]));
    KI_CUDA(cudaStreamWaitEvent(stream, join_ev[i], 0));
  }
}

template <typename T>
Factorization<T>::~Factorization() {
  if (stream) cudaStreamSynchronize(stream);
  for (int i = 0; i < kAux; i++) {
    if (aux[i] && aux[i] != stream) {   // serial factorizations alias `stream`
      cudaStreamSynchronize(aux[i]);
      cudaStreamDestroy(aux[i]);
    }
    if (join_ev[i]) cudaEventDestroy(join_ev[i]);
  }
  if (fork_ev) cudaEventDestroy(fork_ev);
  for (auto& r : prof_open) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (void* p : owned) cudaFreeAsync(p, stream);
  if (stream) cudaStreamSynchronize(stream);
}

namespace {

constexpr int kThreads = 256;
// A sketched ID's rank counts only when the sketch revealed it with at least
// this many sketch rows to spare: a rank found in the sketch's last rows can
// be an artefact of the sketch's own smallest singular values (the
// oversampling of a randomized range finder, Halko, Martinsson and Tropp
// 2011, section 4.2), and the box is recompressed by the plain ID instead.
constexpr int kSketchGuard = 5;
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
  int64_t src[kMaxChildren];   // ipool offsets of the pieces (leaf: 1 piece)
  int len[kMaxChildren];
};

struct IdTask {
  int64_t act;        // ipool offset of the active list (n)
  int n;
  int seg_begin, seg_end;
  int mode;           // 0: inner-circle filter + proxy rows; 1: all candidates, no proxy
  double cx, cy, cz, rad_filter, rad_proxy;
  double side;        // box side length
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
  int coff[kMaxChildren], clen[kMaxChildren];
  const T* ctile[kMaxChildren];  // child accumulated self-blocks (clen x clen)
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
  T* Xi;              // r x r explicit inverse of X (FP32 forms), or null
  int gj;             // Gauss-Jordan path in shared memory (forms Xi); else LU
};

// Shared-memory bytes of k_schur for a task on its path.
template <typename T>
size_t schur_bytes(int n, int k, bool inv);
template <typename T>
size_t schur_task_bytes(const SchurTask<T>& q) {
  return schur_bytes<T>(q.n, q.k, q.gj != 0);
}

// ---------------------------------------------------------------- kernels --
__global__ void k_build_active(const ActiveTask* tasks, int* ipool) {
  const ActiveTask t = tasks[blockIdx.x];
  int64_t dst = t.dst;
  for (int s = 0; s < t.nseg; s++) {
    for (int i = threadIdx.x; i < t.len[s]; i += blockDim.x) ipool[dst + i] = ipool[t.src[s] + i];
    dst += t.len[s];
  }
}

// Proxy surface of unit radius (Kernel::get_proxy_mat, kern_interp/kernel/
// kernel.cpp:646-717: 2D, n points equispaced on a circle; get_proxy_mat3d,
// :720-790: 3D, a theta x phi grid with theta outer).  A box's proxy point i
// is c + rad * u_i with outward normal u_i and weight 2 pi rad / n (2D) or
// rad^2 * wu_i (3D, wu = Gauss-Legendre phi weight * sin(phi) * theta weight).
// Tables in the factor precision.
template <typename T>
struct ProxyTab {
  const T* ux;
  const T* uy;
  const T* uz;   // 3D only
  const T* wu;   // 3D only
  int n;
  // 2D concentric proxy rings per direction: 1, or 3 for the Gaussian kernel
  // (radii rad - 1, rad, rad + 1; Kernel::get_proxy_mat, kernel.cpp:661-672)
  int rings = 1;
};

// Rows of the proxy blocks (box -> proxy, then proxy -> box) of a box's ID
// matrix.
template <typename T>
__host__ __device__ __forceinline__ int proxy_rows(const ProxyTab<T>& px, int sol_dim) {
  return 2 * px.n * px.rings * sol_dim;
}

// A box's proxy geometry in the factor precision: the centre split as
// hi + lo (so that box-point offsets b - c keep full relative accuracy in
// FP32), the radius and the 2D proxy weight 2 pi rad / n.
template <typename T>
struct ProxyBox {
  T hx, hy, hz, lx, ly, lz;
  T rad, pw2;
};

template <typename T>
__device__ __forceinline__ ProxyBox<T> proxy_box(double cx, double cy, double cz, double rad,
                                                 int nprox) {
  ProxyBox<T> b;
  b.hx = T(cx); b.lx = T(cx - (double)b.hx);
  b.hy = T(cy); b.ly = T(cy - (double)b.hy);
  b.hz = T(cz); b.lz = T(cz - (double)b.hz);
  b.rad = T(rad);
  b.pw2 = T(2.0 * kPi * rad / nprox);
  return b;
}

// One ID-matrix entry, row `row` of the stacked matrix
// [K(I,A); K(A,I)^T; box->proxy; proxy->box] (Kernel::get_id_mat,
// kern_interp/kernel/kernel.cpp:565-640; proxy rows Kernel::get_proxy_mat,
// :646-790), column = active DOF `adof`.  Proxy offsets are formed as
// rad u - (b - c).
template <typename T>
__device__ __forceinline__ T id_entry(const Points<T>& P, int sol_dim, int row, int nI,
                                      const int* rows, int adof, const ProxyTab<T>& px,
                                      const ProxyBox<T>& c) {
  if (row < nI) return kernel_entry<T>(P, sol_dim, rows[row], adof);
  if (row < 2 * nI) return kernel_entry<T>(P, sol_dim, adof, rows[row - nI]);
  const int q = row - 2 * nI;
  const int nprox = px.n;
  const int ap = dof_point(adof, sol_dim);
  const T bcx = (P.x[ap] - c.hx) + ((P.xl ? P.xl[ap] : T(0)) - c.lx);
  const T bcy = (P.y[ap] - c.hy) + ((P.yl ? P.yl[ap] : T(0)) - c.ly);
  const T bnx = P.nx[ap], bny = P.ny[ap], bw = P.w[ap];
  const int half = sol_dim * nprox * px.rings;
  const int qq = q < half ? q : q - half;
  if (px.rings > 1) {
    // Gaussian kernel: proxy point (ring, direction) = qq as ring-minor
    const int i = qq / px.rings, ring = qq - px.rings * i;
    const T rr = c.rad + T(ring - 1);
    return gauss_entry_r<T>(rr * px.ux[i] - bcx, rr * px.uy[i] - bcy);
  }
  const int i = sol_dim == 1 ? qq : qq / sol_dim, par = qq - sol_dim * i;
  const T ux = px.ux[i], uy = px.uy[i];
  const T rx = c.rad * ux - bcx, ry = c.rad * uy - bcy;   // proxy - box
  if (P.dim == 3) {
    const T bcz = (P.z[ap] - c.hz) + ((P.zl ? P.zl[ap] : T(0)) - c.lz);
    const T uz = px.uz[i];
    const T rz = c.rad * uz - bcz;
    const T bnz = P.nz[ap];
    const T pw = c.rad * c.rad * px.wu[i];
    if (sol_dim == 1) {
      if (q < half) return laplace3_entry<T>(rx, ry, rz, bnx, bny, bnz, bw, T(0));
      return laplace3_entry<T>(-rx, -ry, -rz, ux, uy, uz, pw, T(0));
    }
    const int apar = adof - 3 * ap;
    if (q < half)
      return stokes3_entry<T>(par, apar, rx, ry, rz, ux, uy, uz, bnx, bny, bnz, bw, nullptr);
    return stokes3_entry<T>(apar, par, -rx, -ry, -rz, bnx, bny, bnz, ux, uy, uz, pw, nullptr);
  }
  if (sol_dim == 1) {
    if (q < half) return scalar2_entry_r<T>(P.pde, rx, ry, ux, uy, bnx, bny, bw, T(0));
    return scalar2_entry_r<T>(P.pde, -rx, -ry, bnx, bny, ux, uy, c.pw2, T(0));
  }
  const int apar = adof & 1;
  if (q < half) return stokes_entry_r<T>(par, apar, rx, ry, ux, uy, bnx, bny, bw, T(0));
  return stokes_entry_r<T>(apar, par, -rx, -ry, bnx, bny, ux, uy, c.pw2, T(0));
}

// Order-preserving integer key of a non-negative norm (FP32 keys avoid an
// FP64 conversion in the FP32 kernels).
__device__ __forceinline__ long long norm_key(double v) { return __double_as_longlong(v); }
__device__ __forceinline__ long long norm_key(float v) { return (long long)__float_as_int(v); }

// Resident CTAs per SM k_id is compiled for: three in FP32 (the register
// budget of the register-tiled sketch fold would otherwise allow two), two
// in FP64 (no register spills).
template <typename T> constexpr int kIdMinBlocks = sizeof(T) == 4 ? 3 : 2;
// Block size of the FP32 launches whose boxes are too few to give every SM a
// CTA (the upper levels' large boxes): twice the warps to hide the latency of
// each CTA's serial pivot / reflector steps.
constexpr int kIdBigThreads = 512;

// Interpolative decomposition of one box per CTA.
//
// Thread-per-column formulation: every dot product and update runs inside
// one thread over a column (no cross-lane reductions), which keeps the FP64
// instruction count at the algorithmic 2 FMAs per matrix entry and step.
// R (n x n triangle) and the 32-row block B are row-major, so the threads of
// a warp touch consecutive columns.  Shared-memory layout (dynamic):
//   B (32 x ldB) | hu (2 x 32 Householder tails) | vn1 (n) | vn2 (n) | perm (n) |
//   R (n x ldR) when it fits (mode 0); mode 1 keeps R in the global scratch.
template <typename T, int FR, int NT = kThreads>
__global__ void __launch_bounds__(NT, NT == kThreads ? kIdMinBlocks<T> : 1) k_id(const IdTask* tasks, int task_base,
                                                  const int64_t* seg_off, const int* seg_len,
                                                  int* ipool, int* iscratch, T* tws, Points<T> P,
                                                  int sol_dim, ProxyTab<T> px, double tol, int* k_out,
                                                  int* m_out, int mode, int flags,
                                                  const int* sketch_l) {
  // flags: 1 gather the rows (writes m), 2 fold the ID matrix into R,
  //        4 R already formed (row-major n x n in the global scratch)
  // sketch_l (optional, per task): with 0 < l < n and the triangle in shared
  // memory (mode 0), the ID matrix M is compressed to the l x n sketch
  // Y = Omega M (Omega: random signs) instead of being folded into R, and the
  // column-pivoted QR runs on Y (randomized ID).  When Y does not reveal the
  // rank within l pivots the box is flagged (k = -1) for the plain ID.
  extern __shared__ __align__(16) unsigned char id_smem[];
  const int task = task_base + blockIdx.x;
  const IdTask t = tasks[task];
  const int n = t.n;
  const int tid = threadIdx.x, nth = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = nth >> 5;
  __shared__ int s_cnt;
  __shared__ int s_scan[64];
  __shared__ int s_piv, s_k;
  __shared__ T s_tau[2], s_beta;

  // the box's centre split hi + lo with the proxy and filter radii, formed
  // once (FP64 arithmetic, slow in the FP32 kernels when every thread does it)
  __shared__ ProxyBox<T> s_boxes[2];
  if (tid == 0) {
    s_boxes[0] = proxy_box<T>(t.cx, t.cy, t.cz, t.rad_proxy, px.n);
    s_boxes[1] = proxy_box<T>(t.cx, t.cy, t.cz, t.rad_filter, 1);
  }
  __syncthreads();

  int* rows = iscratch + t.rows;
  const int* act = ipool + t.act;
  T* gws = tws + t.ws;   // global scratch: R (n*n) | Tout (n*n/4+1)
  const int ldB = n | 1;
  size_t off = 0;
  T* B = reinterpret_cast<T*>(id_smem);
  if (flags & 2) off += sizeof(T) * (size_t)FR * ldB;   // the fold block exists only when folding
  T* hu = reinterpret_cast<T*>(id_smem + off);   // [2][n] reflector tails (fold: 32, CPQR: n)
  off += sizeof(T) * 2 * (size_t)max(n, FR);
  T* vn1 = reinterpret_cast<T*>(id_smem + off);
  off += sizeof(T) * (size_t)n;
  T* vn2 = reinterpret_cast<T*>(id_smem + off);
  off += sizeof(T) * (size_t)n;
  int* perm = reinterpret_cast<int*>(id_smem + off);
  off += sizeof(int) * (size_t)n;
  off = (off + 15) & ~size_t(15);
  // mode 2: the fold keeps the triangle packed by rows in shared memory
  // (row i holds columns i..n-1), the pivoting then runs on a full copy in
  // the global scratch
  const bool packed = mode == 2;
  int ldR = mode == 0 ? (n | 1) : n;
  T* R = mode == 0 ? reinterpret_cast<T*>(id_smem + off) : gws;
  T* RF = packed ? reinterpret_cast<T*>(id_smem + off) : R;   // fold storage
  auto rowbase = [&](int i) -> size_t {
    return packed ? (size_t)i * n - (size_t)i * (i - 1) / 2 - i : (size_t)i * ldR;
  };
  T* Tout = gws + (size_t)n * n;

  // 1. candidate rows, optionally filtered to the proxy circle, order kept
  const int nprox_rows = t.mode == 0 ? proxy_rows(px, sol_dim) : 0;
  if (flags & 1) {
  if (tid == 0) s_cnt = 0;
  // the box centre split hi + lo and the filter radius, for the FP32 filter
  const ProxyBox<T> cb = s_boxes[1];
  __syncthreads();
  for (int s = t.seg_begin; s < t.seg_end; s++) {
    const int* src = ipool + seg_off[s];
    int len = seg_len[s];
    for (int base = 0; base < len; base += nth) {
      int i = base + tid;
      int keep = 0, dof = 0;
      if (i < len) {
        dof = src[i];
        if (t.mode == 1) {
          keep = 1;
        } else {
          const int p = dof_point(dof, sol_dim);
          if (sizeof(T) < sizeof(double)) {
            // FP32 forms: the offset from the split centre in FP32 and the
            // squared comparison (no FP64 arithmetic in the FP32 kernels)
            const T dx = (cb.hx - P.x[p]) + (cb.lx - (P.xl ? P.xl[p] : T(0)));
            const T dy = (cb.hy - P.y[p]) + (cb.ly - (P.yl ? P.yl[p] : T(0)));
            T d2 = dx * dx + dy * dy;
            if (P.dim == 3) {
              const T dz = (cb.hz - P.z[p]) + (cb.lz - (P.zl ? P.zl[p] : T(0)));
              d2 += dz * dz;
            }
            keep = d2 < cb.rad * cb.rad;
          } else {
            double dx = t.cx - ((double)P.x[p] + (P.xl ? (double)P.xl[p] : 0.0));
            double dy = t.cy - ((double)P.y[p] + (P.yl ? (double)P.yl[p] : 0.0));
            double d2 = dx * dx + dy * dy;
            if (P.dim == 3) {
              double dz = t.cz - ((double)P.z[p] + (P.zl ? (double)P.zl[p] : 0.0));
              d2 += dz * dz;
            }
            double dist = sqrt(d2);
            keep = dist < t.rad_filter;
          }
        }
      }
      int v = keep;
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffff, v, o);
        if (lane >= o) v += y;
      }
      if (lane == 31) s_scan[warp] = v;
      __syncthreads();
      if (warp == 0) {
        int wv = lane < nwarps ? s_scan[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
          int y = __shfl_up_sync(0xffffffff, wv, o);
          if (lane >= o) wv += y;
        }
        if (lane < nwarps) s_scan[32 + lane] = wv;
      }
      __syncthreads();
      int before = warp > 0 ? s_scan[32 + warp - 1] : 0;
      if (keep) rows[s_cnt + before + v - 1] = dof;
      int total = s_scan[32 + nwarps - 1];
      __syncthreads();
      if (tid == 0) s_cnt += total;
      __syncthreads();
    }
  }
  if (tid == 0) m_out[task] = 2 * s_cnt + nprox_rows;
  }
  if (!(flags & 6)) return;
  __syncthreads();
  const int m = m_out[task];
  const int nI = (m - nprox_rows) / 2;
  // a sketch is folded here only with the triangle in shared memory; an R
  // formed beforehand (flags 4) may be an lsk x n sketch in either mode
  const int lsk_in = sketch_l ? sketch_l[task] : 0;
  const int lsk = (flags & 2) ? (mode == 0 ? lsk_in : 0) : ((flags & 4) ? lsk_in : 0);
  // folded sketches need l < n (else the triangle is cheaper); a formed
  // sketch may have l = n rows (a full-size randomized ID, no fallback)
  const bool sketch = (flags & 2) ? (lsk > 0 && lsk < n) : (lsk > 0 && lsk <= n);
  const bool sketch_fold = sketch && (flags & 2);
  const int rowsR = sketch ? lsk : n;   // rows of the matrix the pivoted QR runs on

  // 2a. Sketch: Y (lsk x n, in R's place) = sum over 32/64-row blocks B of
  //     S_B B, S_B[q][i] = +-1 from a hash of (box, row, q).
  if (sketch && !sketch_fold) {
    // a sketch formed by k_wide_sketch: row-major lsk x n in the global scratch
    if (mode == 0)
      for (int idx = tid; idx < lsk * n; idx += nth) R[(idx / n) * (size_t)ldR + idx % n] = gws[idx];
    __syncthreads();
  }
  if (sketch_fold) {
    for (int idx = tid; idx < lsk * n; idx += nth) R[(idx / n) * (size_t)ldR + idx % n] = T(0);
    const ProxyBox<T> pb = s_boxes[0];
    uint32_t* sgn = reinterpret_cast<uint32_t*>(hu);   // FR rows x ceil(lsk/32) words
    const int words = (lsk + 31) >> 5;
    for (int r0 = 0; r0 < m; r0 += FR) {
      __syncthreads();
      for (int idx = tid; idx < FR * n; idx += nth) {
        int j = idx % n, i = idx / n;
        int row = r0 + i;
        B[(size_t)i * ldB + j] =
            row < m ? id_entry<T>(P, sol_dim, row, nI, rows, act[j], px, pb) : T(0);
      }
      for (int idx = tid; idx < FR * words; idx += nth) {
        // lowbias32 integer hash (C. Wellons) of (box's active offset, row, word)
        uint32_t x = (uint32_t)(t.act * 2654435761u) ^ (uint32_t)((r0 + idx / words) * 40503u) ^
                     (uint32_t)((idx % words) * 2246822519u);
        x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
        sgn[idx] = x;
      }
      __syncthreads();
      // Y += S_B B with threads on (8 sketch rows, 1 column) tiles: one load
      // of B(i, c) serves 8 rows.  The signs as +-1 entries (FMAs) in rows
      // lsk.. of R, unused while sketching, when they fit; else bit tests.
      const int lq = (lsk + 7) & ~7;
      // 16-byte aligned start (R is), so a thread's 8 signs load as two vectors
      const size_t s0 = ((size_t)lsk * ldR + 3) & ~size_t(3);
      T* Sf = ((size_t)n * ldR >= s0 + (size_t)FR * lq) ? R + s0 : nullptr;
      if (Sf) {
        for (int e = tid; e < FR * lq; e += nth) {
          const int i = e / lq, q = e % lq;
          Sf[e] = (q < lsk && ((sgn[i * words + (q >> 5)] >> (q & 31)) & 1u)) ? T(-1) : T(1);
        }
        __syncthreads();
      }
      for (int it = tid; it < (lq / 8) * n; it += nth) {
        const int c = it % n, q0 = (it / n) * 8;
        T acc[8];
#pragma unroll
        for (int u = 0; u < 8; u++) acc[u] = T(0);
        if (Sf) {
          for (int i = 0; i < FR; i++) {
            const T b = B[(size_t)i * ldB + c];
            const T* srow = Sf + (size_t)i * lq + q0;
            T sv[8];
            if (sizeof(T) == 4) {
              const float4 v0 = *reinterpret_cast<const float4*>(srow);
              const float4 v1 = *reinterpret_cast<const float4*>(srow + 4);
              sv[0] = v0.x; sv[1] = v0.y; sv[2] = v0.z; sv[3] = v0.w;
              sv[4] = v1.x; sv[5] = v1.y; sv[6] = v1.z; sv[7] = v1.w;
            } else {
#pragma unroll
              for (int u = 0; u < 8; u++) sv[u] = srow[u];
            }
#pragma unroll
            for (int u = 0; u < 8; u++) acc[u] = fma(sv[u], b, acc[u]);
          }
        } else {
          for (int i = 0; i < FR; i++) {
            const T b = B[(size_t)i * ldB + c];
            const uint32_t bits = sgn[i * words + (q0 >> 5)] >> (q0 & 31);
#pragma unroll
            for (int u = 0; u < 8; u++) acc[u] += ((bits >> u) & 1u) ? -b : b;
          }
        }
#pragma unroll
        for (int u = 0; u < 8; u++)
          if (q0 + u < lsk) R[(size_t)(q0 + u) * ldR + c] += acc[u];
      }
    }
    __syncthreads();
  }

  if (!sketch) {
  // 2. TSQR: R <- qr([R; B]) for successive 32-row blocks B of the ID
  //    matrix.  The thread that owns column j+1 forms reflector j+1 right
  //    after updating that column (look-ahead), so one barrier per column.
  if (flags & 4) {
    if (mode == 0)
      for (int idx = tid; idx < n * n; idx += nth) R[(idx / n) * (size_t)ldR + idx % n] = gws[idx];
  } else if (packed) {
    for (int idx = tid; idx < n * (n + 1) / 2; idx += nth) RF[idx] = T(0);
  } else {
    for (int idx = tid; idx < n * n; idx += nth) R[(idx / n) * (size_t)ldR + idx % n] = T(0);
  }
  __syncthreads();
  // reflector of [R(j,j); B(:,j)] formed by warp 0 (lane i <-> row i of the
  // block); tail -> hu[buf], tau -> s_tau[buf], beta -> R(j,j)
  auto reflect = [&](int j, int buf) {
    T alpha = RF[rowbase(j) + j];
    T b[FR / 32];
    T sq = T(0);
#pragma unroll
    for (int q = 0; q < FR / 32; q++) {
      b[q] = B[(size_t)(lane + 32 * q) * ldB + j];
      sq += b[q] * b[q];
    }
    T sigma = warp_sum(sq);
    T tau = T(0), beta = alpha, scale = T(0);
    if (sigma != T(0)) {
      T nrm = sqrt(alpha * alpha + sigma);
      beta = alpha >= T(0) ? -nrm : nrm;
      tau = (beta - alpha) / beta;
      scale = T(1) / (alpha - beta);
    }
#pragma unroll
    for (int q = 0; q < FR / 32; q++) hu[buf * FR + lane + 32 * q] = b[q] * scale;
    if (lane == 0) {
      s_tau[buf] = tau;
      RF[rowbase(j) + j] = beta;
    }
  };
  const ProxyBox<T> pbox = s_boxes[0];
  for (int r0 = 0; (flags & 2) && r0 < m; r0 += FR) {
    for (int idx = tid; idx < FR * n; idx += nth) {
      int j = idx % n, i = idx / n;
      int row = r0 + i;
      T v = T(0);
      if (row < m)
        v = id_entry<T>(P, sol_dim, row, nI, rows, act[j], px, pbox);
      B[(size_t)i * ldB + j] = v;
    }
    __syncthreads();
    if (warp == 0) reflect(0, 0);
    __syncthreads();
    for (int j = 0; j < n; j++) {
      const int buf = j & 1;
      const T tau = s_tau[buf];
      if (tau != T(0)) {
        // four threads per column (adjacent lanes), each over 8 interleaved
        // rows of the block: every step spreads over up to 64 columns x 4
        // lanes, i.e. all warps, and the column sum is two lane shuffles
        const T* u = hu + buf * FR;
        T* Rj = RF + rowbase(j);
        const int cq = tid >> 2, rg = tid & 3;
        for (int cb = j + 1; cb < n; cb += nth >> 2) {
          const int c = cb + cq;
          const bool on = c < n;
          T p0 = T(0), p1 = T(0);
          T rjc = T(0);
          if (on) {
#pragma unroll
            for (int t = 0; t < FR / 4; t += 2) {
              p0 += u[rg + 4 * t] * B[(size_t)(rg + 4 * t) * ldB + c];
              p1 += u[rg + 4 * t + 4] * B[(size_t)(rg + 4 * t + 4) * ldB + c];
            }
            rjc = Rj[c];
          }
          T dot = p0 + p1;
          dot += __shfl_xor_sync(0xffffffff, dot, 1);
          dot += __shfl_xor_sync(0xffffffff, dot, 2);
          if (on) {
            const T w = (dot + rjc) * tau;
            if (rg == 0) Rj[c] = rjc - w;
#pragma unroll
            for (int t = 0; t < FR / 4; t++)
              B[(size_t)(rg + 4 * t) * ldB + c] -= w * u[rg + 4 * t];
          }
        }
      }
      // column j+1 is owned by thread 0: warp 0 forms the next reflector
      if (warp == 0 && j + 1 < n) {
        __syncwarp();
        reflect(j + 1, buf ^ 1);
      }
      __syncthreads();
    }
  }

  if (packed && (flags & 2)) {
    for (int idx = tid; idx < n * n; idx += nth) {
      int i = idx / n, c = idx % n;
      gws[idx] = c >= i ? RF[rowbase(i) + c] : T(0);
    }
    __syncthreads();
  }
  }   // !sketch

  // 3. column-pivoted QR of the n x n triangle (LAPACK xGEQP3/xLAQP2 norm
  //    downdating with recomputation after cancellation), stopping at the
  //    first |R_jj| < tol |R_00| for j >= 1.  Thread per column again.
  for (int c = tid; c < n; c += nth) {
    T s = T(0);
    const int ilast = sketch ? rowsR - 1 : c;   // the triangle is zero below the diagonal
    for (int i = 0; i <= ilast; i++) s += R[(size_t)i * ldR + c] * R[(size_t)i * ldR + c];
    vn1[c] = sqrt(s);
    vn2[c] = vn1[c];
    perm[c] = c;
  }
  if (tid == 0) s_k = 0;
  __syncthreads();
  T thresh = T(0);
  const int jmax = min(min(n, m), rowsR);
  for (int j = 0; j < jmax; j++) {
    // pivot: first index of the largest partial norm (norms are >= 0, so
    // their bit patterns order like the values)
    if (warp == 0) {
      long long best = -1;
      int bi = j;
      for (int c = j + lane; c < n; c += 32) {
        long long v = norm_key(vn1[c]);
        if (v > best) { best = v; bi = c; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        long long ov = __shfl_down_sync(0xffffffff, best, o);
        int oi = __shfl_down_sync(0xffffffff, bi, o);
        if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
      }
      if (lane == 0) s_piv = bi;
    }
    __syncthreads();
    const int p = s_piv;
    if (p != j) {
      for (int i = tid; i < rowsR; i += nth) {
        T a = R[(size_t)i * ldR + j];
        R[(size_t)i * ldR + j] = R[(size_t)i * ldR + p];
        R[(size_t)i * ldR + p] = a;
      }
      if (tid == 0) {
        int a = perm[j]; perm[j] = perm[p]; perm[p] = a;
        T v = vn1[j]; vn1[j] = vn1[p]; vn1[p] = v;
        v = vn2[j]; vn2[j] = vn2[p]; vn2[p] = v;
      }
      __syncthreads();
    }
    // reflector of R(j:n, j) by warp 0; tail -> hu[0..], scalars -> shared
    if (warp == 0) {
      T sg = T(0);
      for (int i = j + 1 + lane; i < rowsR; i += 32) sg += R[(size_t)i * ldR + j] * R[(size_t)i * ldR + j];
      T sigma = warp_sum(sg);
      T alpha = R[(size_t)j * ldR + j];
      T tau = T(0), beta = alpha, scale = T(0);
      if (sigma != T(0)) {
        T nrm = sqrt(alpha * alpha + sigma);
        beta = alpha >= T(0) ? -nrm : nrm;
        tau = (beta - alpha) / beta;
        scale = T(1) / (alpha - beta);
      }
      for (int i = j + 1 + lane; i < rowsR; i += 32) hu[i] = R[(size_t)i * ldR + j] * scale;
      if (lane == 0) { s_tau[0] = tau; s_beta = beta; }
    }
    __syncthreads();
    const T beta = s_beta, tau = s_tau[0];
    if (j == 0) thresh = fabs(T(tol) * beta);
    if (j >= 1 && fabs(beta) < thresh) {
      if (tid == 0) s_k = j;
      break;
    }
    for (int c = j + 1 + tid; c < n; c += nth) {
      if (tau != T(0)) {
        T w0 = R[(size_t)j * ldR + c], w1 = T(0), w2 = T(0), w3 = T(0);
        int i = j + 1;
        for (; i + 3 < rowsR; i += 4) {
          w0 += hu[i] * R[(size_t)i * ldR + c];
          w1 += hu[i + 1] * R[(size_t)(i + 1) * ldR + c];
          w2 += hu[i + 2] * R[(size_t)(i + 2) * ldR + c];
          w3 += hu[i + 3] * R[(size_t)(i + 3) * ldR + c];
        }
        for (; i < rowsR; i++) w0 += hu[i] * R[(size_t)i * ldR + c];
        T w = ((w0 + w1) + (w2 + w3)) * tau;
        R[(size_t)j * ldR + c] -= w;
        // four rows per step with the loads issued together (the global-
        // memory modes would otherwise wait one round trip per row)
        int q = j + 1;
        for (; q + 3 < rowsR; q += 4) {
          T* r0 = R + (size_t)q * ldR + c;
          const T a0 = r0[0], a1 = r0[ldR], a2 = r0[2 * (size_t)ldR], a3 = r0[3 * (size_t)ldR];
          r0[0] = a0 - w * hu[q];
          r0[ldR] = a1 - w * hu[q + 1];
          r0[2 * (size_t)ldR] = a2 - w * hu[q + 2];
          r0[3 * (size_t)ldR] = a3 - w * hu[q + 3];
        }
        for (; q < rowsR; q++) R[(size_t)q * ldR + c] -= w * hu[q];
      }
      // norm downdate of column c (xLAQP2), recomputed after cancellation
      T rjc = R[(size_t)j * ldR + c];
      T v1 = vn1[c];
      if (v1 != T(0)) {
        T temp = fabs(rjc) / v1;
        temp = T(1) - temp * temp;
        temp = temp < T(0) ? T(0) : temp;
        T q = v1 / vn2[c];
        T temp2 = temp * q * q;
        if (temp2 <= tol3z<T>()) {
          T s2 = T(0);
          for (int i = j + 1; i < rowsR; i++) s2 += R[(size_t)i * ldR + c] * R[(size_t)i * ldR + c];
          vn1[c] = sqrt(s2);
          vn2[c] = vn1[c];
        } else {
          vn1[c] = v1 * sqrt(temp);
        }
      }
    }
    if (tid == 0) R[(size_t)j * ldR + j] = beta;
    __syncthreads();
  }
  __syncthreads();
  const int k = s_k;
  if (sketch && rowsR < n && (k == 0 ? jmax == rowsR : k > rowsR - kSketchGuard)) {
    // the sketch did not reveal the rank with kSketchGuard rows to spare:
    // recompress with the plain ID
    if (tid == 0) k_out[task] = -1;
    return;
  }
  if (tid == 0) k_out[task] = k;
  int* gperm = iscratch + t.perm;
  for (int i = tid; i < n; i += nth) gperm[i] = perm[i];
  if (k == 0) return;
  const int r = n - k;

  // 4. T = R11^-1 R12 in place over R12 (one thread per column), then out
  for (int c = k + tid; c < n; c += nth) {
    for (int i = k - 1; i >= 0; i--) {
      T s = R[(size_t)i * ldR + c];
#pragma unroll 8
      for (int l = i + 1; l < k; l++) s -= R[(size_t)i * ldR + l] * R[(size_t)l * ldR + c];
      R[(size_t)i * ldR + c] = s / R[(size_t)i * ldR + i];
    }
  }
  __syncthreads();
  for (int e = tid; e < k * r; e += nth) {
    int i = e % k, c = e / k;
    Tout[e] = R[(size_t)i * ldR + k + c];
  }
  int* pact = ipool + t.pact;
  for (int i = tid; i < n; i += nth) pact[i] = act[perm[i]];
}

// ------------------------------------------------ tensor-core ID sketch --
// Y = Omega M (l x n) for the narrow boxes of a sketched (randomized) ID, on
// the tensor cores: M's rows are generated 32 at a time into shared memory
// (the A operand, box columns x block rows, K-major), Omega's matching
// columns (the same +-1 signs as k_id's fold) form the B operand, and
// tcgen05 kind::tf32 MMAs accumulate Y^T (box columns x sketch rows) in
// TMEM.  Each entry enters as hi + lo, both rounded to TF32, so it is
// represented to 2^-22 relative; the signs are exact.  The tensor core's
// FP32 accumulation does not round to nearest: over the few hundred ID rows
// of a box it loses about a decimal digit against the CUDA-core fold, which
// is why this path is opt-in.  Y goes row-major into the task's global
// scratch, where k_id's pivoted QR (flags 4) picks it up.  Boxes of up to
// 128 columns use one M = 128 accumulator tile, up to 256 columns two.
constexpr int kTcRows = 32;         // ID-matrix rows per MMA block (K of 4 MMAs)
constexpr int kTcThreads = 256;
constexpr long long kTcWaitCycles = 2000000000LL;   // ~1 s at 2 GHz: bounded waits

__host__ __device__ constexpr size_t tc_sketch_smem(int tiles, int nq) {
  return (size_t)tiles * 2 * 128 * kTcRows * sizeof(float) + (size_t)nq * kTcRows * sizeof(float);
}

__device__ __forceinline__ uint32_t tc_tmem_cols(int used) {
  uint32_t c = 32;
  while ((int)c < used) c <<= 1;
  return c;
}

// Sign of Omega(q, row) for a box (k_id's fold uses the same hash): bit q % 32
// of word q / 32 of the row's lowbias32 hash (C. Wellons).
__device__ __forceinline__ float sketch_sign(int64_t act, int row, int q) {
  uint32_t x = (uint32_t)(act * 2654435761u) ^ (uint32_t)(row * 40503u) ^
               (uint32_t)((q >> 5) * 2246822519u);
  x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
  return ((x >> (q & 31)) & 1u) ? -1.f : 1.f;
}

// Issue the MMAs of one 32-row block (one thread): D_t (+)= A_t B for the
// tiles t, with A_t = A_hi,t + A_lo,t.
__device__ __forceinline__ void tc_issue_block(uint32_t tmem, const float* a_hi, const float* a_lo,
                                               const float* b, int tiles, int nq, bool first) {
  const uint32_t sbo = 32 * kTcRows;   // bytes between 8-row groups: kTcRows / 4 core matrices
  const uint32_t idesc = tc::idesc_tf32(128, nq);
  const uint32_t tile_bytes = 128 * kTcRows * sizeof(float);
  for (int tt = 0; tt < tiles; tt++)
    for (int s = 0; s < kTcRows / 8; s++) {
      const uint64_t bd = tc::smem_desc(tc::smem_u32(b) + 256 * s, tc::kLbo, sbo);
      const uint64_t ah = tc::smem_desc(tc::smem_u32(a_hi) + tt * tile_bytes + 256 * s, tc::kLbo, sbo);
      const uint64_t al = tc::smem_desc(tc::smem_u32(a_lo) + tt * tile_bytes + 256 * s, tc::kLbo, sbo);
      tc::mma_tf32(tmem + tt * nq, ah, bd, idesc, (first && s == 0) ? 0u : 1u);
      tc::mma_tf32(tmem + tt * nq, al, bd, idesc, 1u);
    }
}

// The A and B operands of one block.  Warps fill whole core matrices (8 rows
// x 4 block rows; lane -> (row 8 rb + lane / 4, block row 4 kb + lane % 4)).
// entry(c, i) gives A's value at box column c, block row i (0 outside).
template <typename Entry>
__device__ __forceinline__ void tc_fill_block(float* a_hi, float* a_lo, float* b, int tiles, int nq,
                                              Entry entry, int64_t act, int r0, int l) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const uint32_t sbo = 32 * kTcRows, tile_bytes = 128 * kTcRows * sizeof(float);
  constexpr int kb_n = kTcRows / 4;
  for (int u = warp; u < tiles * 16 * kb_n; u += nw) {
    const int rb = u / kb_n, kb = u % kb_n;
    const float v = entry(rb * 8 + (lane >> 2), kb * 4 + (lane & 3));
    const float hi = tc::to_tf32(v);
    const float lo = tc::to_tf32(v - hi);
    const uint32_t off = (uint32_t)(rb >> 4) * tile_bytes + tc::core_offset(rb & 15, kb, sbo) + 4 * lane;
    *reinterpret_cast<float*>(reinterpret_cast<char*>(a_hi) + off) = hi;
    *reinterpret_cast<float*>(reinterpret_cast<char*>(a_lo) + off) = lo;
  }
  for (int u = warp; u < (nq / 8) * kb_n; u += nw) {
    const int qb = u / kb_n, kb = u % kb_n;
    const int q = qb * 8 + (lane >> 2), i = kb * 4 + (lane & 3);
    const float sv = q < l ? sketch_sign(act, r0 + i, q) : 0.f;
    *reinterpret_cast<float*>(reinterpret_cast<char*>(b) + tc::core_offset(qb, kb, sbo) + 4 * lane) = sv;
  }
}

// The product D = A B^T (A: rows x m, B: l x m, generated blockwise by
// fill) of one CTA on the tensor cores.  Blocks of kTcRows columns of A and
// B alternate between two operand stages and two TMEM accumulators, so that
// the fill of a block overlaps the MMAs of the one before; each block's
// partial sums are read back from TMEM and added in FP32 registers (round to
// nearest), so TMEM accumulates only the 8 MMAs of one block.  Thread (warp
// w, lane) owns row 32 (w % 4) + lane of each 128-row tile and the 16-column
// chunks w / 4, w / 4 + 2, ..: CH of them (tiles x nq <= 32 CH).  The caller
// provides 2 tc_sketch_smem(TILES, nq) bytes of dynamic shared memory.
// Returns false when a bounded wait gave up.
template <int TILES, int CH, typename Entry>
__device__ __forceinline__ bool tc_sketch_core(unsigned char* smem, uint64_t* bar, uint32_t* tmem_slot,
                                               int m, int l, int64_t act, Entry entry,
                                               float (&acc)[CH][16]) {
  const int nq = (l + 15) & ~15;
  const int tid = threadIdx.x, warp = tid >> 5;
  const size_t stage_floats = tc_sketch_smem(TILES, nq) / sizeof(float);
  const int acc_cols = TILES * nq;   // TMEM columns of one accumulator
  const uint32_t ncols = tc_tmem_cols(2 * acc_cols);
  if (warp == 0) tc::tmem_alloc(tmem_slot, ncols);
  if (tid == 0) {
    tc::mbar_init(&bar[0], 1);
    tc::mbar_init(&bar[1], 1);
    tc::fence_mbar_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  const int chunks = TILES * (nq / 16);
#pragma unroll
  for (int q = 0; q < CH; q++)
#pragma unroll
    for (int j = 0; j < 16; j++) acc[q][j] = 0.f;
  uint32_t parity = 0;   // bit st: phase parity awaited on bar[st]
  bool ok = true;
  auto drain = [&](int st) {
    ok = tc::mbar_wait(&bar[st], (parity >> st) & 1u, kTcWaitCycles) && ok;
    parity ^= 1u << st;
    tc::fence_after_sync();
#pragma unroll
    for (int q = 0; q < CH; q++) {
      const int ch = (warp >> 2) + 2 * q;
      if (ch < chunks) {   // uniform per warp
        const int tt = ch / (nq / 16), q0 = (ch % (nq / 16)) * 16;
        float v[16];
        tc::tmem_ld16(tmem + ((uint32_t)(32 * (warp & 3)) << 16) +
                          (uint32_t)(st * acc_cols + tt * nq + q0), v);
#pragma unroll
        for (int j = 0; j < 16; j++) acc[q][j] += v[j];
      }
    }
    tc::fence_before_sync();
  };
  int blk = 0;
  for (int r0 = 0; r0 < m; r0 += kTcRows, blk++) {
    const int st = blk & 1;
    if (blk >= 2) drain(st);   // block blk - 2: its operands and accumulator are free
    float* a_hi = reinterpret_cast<float*>(smem) + st * stage_floats;
    float* a_lo = a_hi + TILES * 128 * kTcRows;
    float* bs = a_lo + TILES * 128 * kTcRows;
    tc_fill_block(a_hi, a_lo, bs, TILES, nq, [&](int c, int i) { return entry(c, r0 + i); }, act, r0, l);
    tc::fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      tc_issue_block(tmem + st * acc_cols, a_hi, a_lo, bs, TILES, nq, true);
      tc::mma_commit(&bar[st]);
    }
  }
  // the last one or two blocks, in issue order
  if (blk >= 2) drain(blk & 1);
  if (blk >= 1) drain((blk + 1) & 1);
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, ncols);
  return ok;
}

// Y = Omega M of one box per CTA (the boxes of `list`), written row-major
// (l x n) into the task's global scratch.
template <int TILES, int CH>
__global__ void __launch_bounds__(kTcThreads) k_sketch_tc(const IdTask* tasks, const int* list,
                                                          const int* m_arr, const int* sketch_l,
                                                          const int* ipool, const int* iscratch,
                                                          float* tws, Points<float> P, int sol_dim,
                                                          ProxyTab<float> px, int* err) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  __shared__ uint64_t bar[2];
  __shared__ uint32_t tmem_slot;
  __shared__ ProxyBox<float> s_box;
  const int ti = list[blockIdx.x];
  const IdTask t = tasks[ti];
  const int n = t.n, m = m_arr[ti], l = sketch_l[ti];
  const int nq = (l + 15) & ~15;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nI = (m - (t.mode == 0 ? proxy_rows(px, sol_dim) : 0)) / 2;
  const int* rows = iscratch + t.rows;
  const int* act = ipool + t.act;
  if (threadIdx.x == 0) s_box = proxy_box<float>(t.cx, t.cy, t.cz, t.rad_proxy, px.n);
  __syncthreads();
  const ProxyBox<float> pb = s_box;
  float acc[CH][16];
  const bool ok = tc_sketch_core<TILES, CH>(
      tc_smem, bar, &tmem_slot, m, l, t.act,
      [&](int c, int row) {
        return (c < n && row < m) ? id_entry<float>(P, sol_dim, row, nI, rows, act[c], px, pb) : 0.f;
      },
      acc);
  // Y^T: lane = box column, chunk column = sketch row
  float* gws = tws + t.ws;
  const int chunks = TILES * (nq / 16);
#pragma unroll
  for (int q = 0; q < CH; q++) {
    const int ch = (warp >> 2) + 2 * q;
    if (ch >= chunks) continue;
    const int tt = ch / (nq / 16), q0 = (ch % (nq / 16)) * 16;
    const int c = tt * 128 + 32 * (warp & 3) + lane;
    if (ok && c < n) {
#pragma unroll
      for (int j = 0; j < 16; j++)
        if (q0 + j < l) gws[(size_t)(q0 + j) * n + c] = acc[q][j];
    }
  }
  if (!ok && threadIdx.x == 0) atomicMax(err, (int)kDevTimeout);
}

// Column-pivoted Householder QR of a box's sketch Y (l x n, row-major at the
// start of the task's global scratch; l <= LMAX, n <= 256) and its
// interpolation matrix, with k_id's semantics: xGEQP3 / xLAQP2 pivot order
// (first logical column of largest partial norm) and norm downdating with
// recomputation after cancellation, rank k = first j >= 1 with
// |R_jj| < tol |R_00|, and a sketch that does not reveal the rank within l
// pivots flagged k = -1 (the plain ID then recompresses the box).  One CTA
// per box, lane = column of its warp's 32-column slab, the column in
// registers.  Columns do not move: each keeps its logical position, which
// is swapped as xGEQP3 swaps columns; perm (logical -> column) lives in
// shared memory.  Two barriers per pivot among the box's warps.  Then
// T = R11^-1 R12 by back substitution, every redundant column in its own
// lane, R's first k rows staged in shared memory (dynamic: l x n floats).
template <int LMAX>
__global__ void __launch_bounds__(256) k_cpqr(const IdTask* tasks, const int* list, const int* sketch_l,
                                              int* ipool, int* iscratch, float* tws, double tol,
                                              int* k_out) {
  extern __shared__ __align__(16) float cq_smem[];   // Rs: l x n (row a, column c)
  __shared__ float s_wbest[8];
  __shared__ int s_wpos[8];
  __shared__ float s_u[LMAX];
  __shared__ float s_tau, s_beta;
  __shared__ int s_perm[256];
  __shared__ int s_k;
  const int ti = list[blockIdx.x];
  const IdTask t = tasks[ti];
  const int n = t.n, l = sketch_l[ti];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, W = blockDim.x >> 5;
  const int c = 32 * w + lane;            // this lane's column
  const bool has = c < n;
  float* gws = tws + t.ws;
  float y[LMAX];
#pragma unroll
  for (int i = 0; i < LMAX; i++) y[i] = (has && i < l) ? gws[(size_t)i * n + c] : 0.f;
  float vn1 = 0.f;
#pragma unroll
  for (int i = 0; i < LMAX; i++) vn1 = fmaf(y[i], y[i], vn1);
  vn1 = sqrtf(vn1);
  float vn2 = vn1;
  int pos = c;                            // logical position of this column
  for (int e = threadIdx.x; e < n; e += blockDim.x) s_perm[e] = e;
  if (threadIdx.x == 0) s_k = 0;
  __syncthreads();
  const float ftol = (float)tol;
  float thresh = 0.f;
  const int jmax = min(n, l);
  int k = 0;
  bool done = false;
  for (int j = 0; j < jmax && !done; j++) {
    // 1. pivot: largest vn1 over logical positions >= j, ties to the lowest
    float best = -1.f;
    int bpos = n;
    if (has && pos >= j) { best = vn1; bpos = pos; }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int op = __shfl_xor_sync(0xffffffffu, bpos, o);
      if (ob > best || (ob == best && op < bpos)) { best = ob; bpos = op; }
    }
    if (lane == 0) { s_wbest[w] = best; s_wpos[w] = bpos; }
    __syncthreads();
    best = s_wbest[0];
    bpos = s_wpos[0];
    for (int q = 1; q < W; q++) {
      const float ob = s_wbest[q];
      const int op = s_wpos[q];
      if (ob > best || (ob == best && op < bpos)) { best = ob; bpos = op; }
    }
    const int pc = s_perm[bpos], qc = s_perm[j];   // pivot column, column at position j
    // xGEQP3's interchange of logical positions j and bpos
    if (c == pc) pos = j;
    else if (c == qc) pos = bpos;
    // 2. the pivot column's reflector (rows j..l-1), by its lane
    if (c == pc) {
      float sg = 0.f, alpha = 0.f;
#pragma unroll
      for (int i = 0; i < LMAX; i++) {
        if (i > j && i < l) sg = fmaf(y[i], y[i], sg);
        if (i == j) alpha = y[i];
      }
      float tau = 0.f, beta = alpha, scale = 0.f;
      if (sg != 0.f) {
        const float nrm = sqrtf(alpha * alpha + sg);
        beta = alpha >= 0.f ? -nrm : nrm;
        tau = (beta - alpha) / beta;
        scale = 1.f / (alpha - beta);
      }
#pragma unroll
      for (int i = 0; i < LMAX; i++) {
        if (i > j && i < l) s_u[i] = y[i] * scale;
        if (i == j) y[i] = beta;
      }
      s_tau = tau;
      s_beta = beta;
    }
    __syncthreads();
    // every thread has read perm[j], perm[bpos]: apply the interchange (read
    // after the next step's first barrier)
    if (c == pc) {
      s_perm[j] = pc;
      s_perm[bpos] = qc;
    }
    const float beta = s_beta, tau = s_tau;
    if (j == 0) thresh = fabsf(ftol * beta);
    if (j >= 1 && fabsf(beta) < thresh) {
      k = j;
      done = true;
      break;
    }
    // 3. the remaining columns: y -= tau (u . y) u on rows j..l-1, then
    // their norms downdated (xLAQP2)
    if (has && pos > j && tau != 0.f) {
      float wsum = 0.f;
#pragma unroll
      for (int i = 0; i < LMAX; i++) {
        if (i == j) wsum += y[i];
        else if (i > j && i < l) wsum = fmaf(s_u[i], y[i], wsum);
      }
      wsum *= tau;
#pragma unroll
      for (int i = 0; i < LMAX; i++) {
        if (i == j) y[i] -= wsum;
        else if (i > j && i < l) y[i] = fmaf(-wsum, s_u[i], y[i]);
      }
    }
    if (has && pos > j && vn1 != 0.f) {
      float rjc = 0.f;
#pragma unroll
      for (int i = 0; i < LMAX; i++) rjc = (i == j) ? y[i] : rjc;
      float temp = fabsf(rjc) / vn1;
      temp = 1.f - temp * temp;
      temp = temp < 0.f ? 0.f : temp;
      const float qv = vn1 / vn2;
      const float temp2 = temp * qv * qv;
      if (temp2 <= tol3z<float>()) {
        float s2 = 0.f;
#pragma unroll
        for (int i = 0; i < LMAX; i++)
          if (i > j && i < l) s2 = fmaf(y[i], y[i], s2);
        vn1 = sqrtf(s2);
        vn2 = vn1;
      } else {
        vn1 = vn1 * sqrtf(temp);
      }
    }
  }
  int* gperm = iscratch + t.perm;
  if (l < n && (done ? k > l - kSketchGuard : jmax == l)) {
    // the sketch did not reveal the rank with kSketchGuard rows to spare:
    // recompress with the plain ID
    if (threadIdx.x == 0) k_out[ti] = -1;
    return;
  }
  __syncthreads();   // final perm
  if (threadIdx.x == 0) k_out[ti] = k;
  for (int e = threadIdx.x; e < n; e += blockDim.x) gperm[e] = s_perm[e];
  if (k == 0) return;
  // R's first k rows (columns in place) into shared memory
  float* Rs = cq_smem;
  if (has) {
#pragma unroll
    for (int i = 0; i < LMAX; i++)
      if (i < k) Rs[(size_t)i * n + c] = y[i];
  }
  __syncthreads();
  // T(:, q - k) = R11^-1 R(0:k, column at position q), q >= k: back
  // substitution over the column's own entries in Rs, R11(a, b) =
  // Rs[a][perm[b]] (broadcast reads)
  float* Tout = gws + (size_t)n * n;
  if (has && pos >= k) {
    for (int a = k - 1; a >= 0; a--) {
      float s = Rs[(size_t)a * n + c];
      for (int b = a + 1; b < k; b++) s = fmaf(-Rs[(size_t)a * n + s_perm[b]], Rs[(size_t)b * n + c], s);
      s = s / Rs[(size_t)a * n + s_perm[a]];
      Rs[(size_t)a * n + c] = s;
      Tout[a + (size_t)k * (pos - k)] = s;
    }
  }
  int* pact = ipool + t.pact;
  const int* act = ipool + t.act;
  for (int e = threadIdx.x; e < n; e += blockDim.x) pact[e] = act[s_perm[e]];
}

// Self-check of the tensor-core sketch routine on fixed data: two tiles
// (256 rows), l = 45 sketch rows (nq = 48), 200 columns of A (7 blocks,
// both stages and accumulators, a ragged last block); d (256 x 48,
// row-major) receives the result, ref the same product summed in FP64 on the
// CUDA cores.
constexpr int kTcCheckRows = 256, kTcCheckQ = 48, kTcCheckL = 45, kTcCheckK = 200;
__device__ __forceinline__ float tc_check_entry(int c, int i) {
  return __sinf(0.05f * c + 0.31f * i) * (1.0f + 0.001f * c) + 1e-3f * (float)((c * 7 + i * 13) % 17);
}
__global__ void __launch_bounds__(kTcThreads) k_tc_selfcheck(float* d, double* ref, int* err) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  __shared__ uint64_t bar[2];
  __shared__ uint32_t tmem_slot;
  constexpr int TILES = 2, nq = kTcCheckQ, CH = (TILES * nq + 31) / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t act = 12345;
  float acc[CH][16];
  const bool ok = tc_sketch_core<TILES, CH>(
      tc_smem, bar, &tmem_slot, kTcCheckK, kTcCheckL, act,
      [&](int c, int i) { return i < kTcCheckK ? tc_check_entry(c, i) : 0.f; }, acc);
  const int chunks = TILES * (nq / 16);
#pragma unroll
  for (int q = 0; q < CH; q++) {
    const int ch = (warp >> 2) + 2 * q;
    if (ch >= chunks) continue;
    const int tt = ch / (nq / 16), q0 = (ch % (nq / 16)) * 16;
    const int c = tt * 128 + 32 * (warp & 3) + lane;
#pragma unroll
    for (int j = 0; j < 16; j++) d[(size_t)c * nq + q0 + j] = acc[q][j];
  }
  // the same product in FP64 on the CUDA cores
  for (int e = threadIdx.x; e < kTcCheckRows * nq; e += blockDim.x) {
    const int c = e / nq, q = e % nq;
    double a2 = 0.0;
    if (q < kTcCheckL)
      for (int i = 0; i < kTcCheckK; i++) a2 += (double)tc_check_entry(c, i) * sketch_sign(act, i, q);
    ref[e] = a2;
  }
  if (!ok && threadIdx.x == 0) atomicMax(err, (int)kDevTimeout);
}

// Features of the learned rank predictor for every ID box of a level (one
// warp per box, four per CTA), and with a model the predicted sketch size
// l = min(n, ceil((1 + margin) k^) + oversample), k^ = n * MLP(features):
//   0 log2 n            1 level / (levels - 1)   2 log2(m + 1)   3 log2(nI + 1)
//   4 dim == 3          5 solution dim / 3       6 -log10(tol) / 10
//   7 proxy-free box (levels 1-2)   8-10 eigenvalues of the covariance of
//   the box's active points / side^2 (descending)   11 |mean - centre| / side.
template <typename T>
__global__ void __launch_bounds__(128) k_box_features(const IdTask* tasks, int ntask,
                                                      const int* ipool, Points<T> P, int sol_dim,
                                                      const int* m_arr, int nprox_rows,
                                                      float level_frac, float tol_feat,
                                                      const float* model, float margin,
                                                      int oversample, float* feat, int* l_out,
                                                      float* khat_out) {
  __shared__ float sm[kMlpModelFloats];
  if (model)
    for (int e = threadIdx.x; e < kMlpModelFloats; e += blockDim.x) sm[e] = model[e];
  __syncthreads();
  // one warp per box: lanes take the box's nodes and combine their sums by
  // shuffles; the network's hidden units are split over the lanes
  __shared__ float s_a1[4][kMlpHidden];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int task = blockIdx.x * (blockDim.x >> 5) + wib;
  if (task >= ntask) return;
  const IdTask t = tasks[task];
  const int n = t.n, m = m_arr[task];
  const int* act = ipool + t.act;
  const double c[3] = {t.cx, t.cy, t.cz};
  double s1[3] = {0, 0, 0}, s2[6] = {0, 0, 0, 0, 0, 0};
  const int dim = P.dim;
  int cnt = 0;
  for (int j = lane; j < n; j += 32) {
    const int p = dof_point(act[j], sol_dim);
    if (j > 0 && dof_point(act[j - 1], sol_dim) == p) continue;   // a node's DOFs are adjacent
    double x[3] = {(double)P.x[p] + (P.xl ? (double)P.xl[p] : 0.0),
                   (double)P.y[p] + (P.yl ? (double)P.yl[p] : 0.0),
                   dim == 3 ? (double)P.z[p] + (P.zl ? (double)P.zl[p] : 0.0) : c[2]};
    for (int d = 0; d < 3; d++) x[d] -= c[d];
    for (int d = 0; d < 3; d++) s1[d] += x[d];
    s2[0] += x[0] * x[0]; s2[1] += x[1] * x[1]; s2[2] += x[2] * x[2];
    s2[3] += x[0] * x[1]; s2[4] += x[0] * x[2]; s2[5] += x[1] * x[2];
    cnt++;
  }
  for (int o = 16; o > 0; o >>= 1) {
    for (int d = 0; d < 3; d++) s1[d] += __shfl_xor_sync(0xffffffffu, s1[d], o);
    for (int d = 0; d < 6; d++) s2[d] += __shfl_xor_sync(0xffffffffu, s2[d], o);
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  }
  const double inv = cnt ? 1.0 / cnt : 0.0, side2 = t.side * t.side;
  double mu[3] = {s1[0] * inv, s1[1] * inv, s1[2] * inv};
  // covariance a11 a22 a33 a12 a13 a23
  double a[6] = {s2[0] * inv - mu[0] * mu[0], s2[1] * inv - mu[1] * mu[1],
                 s2[2] * inv - mu[2] * mu[2], s2[3] * inv - mu[0] * mu[1],
                 s2[4] * inv - mu[0] * mu[2], s2[5] * inv - mu[1] * mu[2]};
  double ev[3] = {0, 0, 0};
  if (dim == 2) {
    const double h = 0.5 * (a[0] + a[1]), d = sqrt(0.25 * (a[0] - a[1]) * (a[0] - a[1]) + a[3] * a[3]);
    ev[0] = h + d;
    ev[1] = h - d;
  } else {
    // symmetric 3 x 3 eigenvalues by the trigonometric method (O. K. Smith, 1961)
    const double p1 = a[3] * a[3] + a[4] * a[4] + a[5] * a[5];
    const double q = (a[0] + a[1] + a[2]) / 3.0;
    if (p1 == 0.0) {
      ev[0] = a[0]; ev[1] = a[1]; ev[2] = a[2];
    } else {
      const double p2 = (a[0] - q) * (a[0] - q) + (a[1] - q) * (a[1] - q) + (a[2] - q) * (a[2] - q) + 2 * p1;
      const double pp = sqrt(p2 / 6.0);
      const double b0 = (a[0] - q) / pp, b1 = (a[1] - q) / pp, b2 = (a[2] - q) / pp;
      const double b3 = a[3] / pp, b4 = a[4] / pp, b5 = a[5] / pp;
      double r = 0.5 * (b0 * (b1 * b2 - b5 * b5) - b3 * (b3 * b2 - b5 * b4) + b4 * (b3 * b5 - b1 * b4));
      r = fmin(1.0, fmax(-1.0, r));
      const double phi = acos(r) / 3.0;
      ev[0] = q + 2 * pp * cos(phi);
      ev[2] = q + 2 * pp * cos(phi + 2.0943951023931957);
      ev[1] = 3 * q - ev[0] - ev[2];
    }
  }
  for (int i = 0; i < 2; i++)   // descending
    for (int j = 0; j < 2 - i; j++)
      if (ev[j] < ev[j + 1]) { double tmp = ev[j]; ev[j] = ev[j + 1]; ev[j + 1] = tmp; }
  const int nI = (m - (t.mode == 0 ? nprox_rows : 0)) / 2;
  float f[kMlpIn];
  f[0] = log2f((float)n);
  f[1] = level_frac;
  f[2] = log2f((float)m + 1.f);
  f[3] = log2f((float)nI + 1.f);
  f[4] = dim == 3 ? 1.f : 0.f;
  f[5] = sol_dim / 3.f;
  f[6] = tol_feat;
  f[7] = t.mode == 1 ? 1.f : 0.f;
  f[8] = (float)(fmax(ev[0], 0.0) / side2);
  f[9] = (float)(fmax(ev[1], 0.0) / side2);
  f[10] = (float)(fmax(ev[2], 0.0) / side2);
  f[11] = (float)(sqrt(mu[0] * mu[0] + mu[1] * mu[1] + mu[2] * mu[2]) / t.side);
  if (lane < kMlpIn) feat[(size_t)task * kMlpIn + lane] = f[lane];
  int l = 0;
  float khat = 0.f;
  if (model) {
    // the forward pass of mlp_forward_one with lanes on hidden units
    float xn[kMlpIn];
    for (int q = 0; q < kMlpIn; q++) xn[q] = (f[q] - sm[kMlpMean + q]) / sm[kMlpScale + q];
    for (int k = lane; k < kMlpHidden; k += 32) {
      float z = sm[kMlpB1 + k];
      for (int q = 0; q < kMlpIn; q++) z += sm[kMlpW1 + k * kMlpIn + q] * xn[q];
      s_a1[wib][k] = z > 0.f ? z : 0.f;
    }
    __syncwarp();
    float zo = 0.f;
    for (int j = lane; j < kMlpHidden; j += 32) {
      float z = sm[kMlpB2 + j];
      for (int k = 0; k < kMlpHidden; k++) z += sm[kMlpW2 + j * kMlpHidden + k] * s_a1[wib][k];
      zo += sm[kMlpW3 + j] * (z > 0.f ? z : 0.f);
    }
    for (int o = 16; o > 0; o >>= 1) zo += __shfl_xor_sync(0xffffffffu, zo, o);
    zo += sm[kMlpB3];
    khat = (float)n * (1.f / (1.f + expf(-zo)));
    l = min(n, (int)ceilf((1.f + margin) * khat) + oversample);
  }
  if (lane == 0) {
    l_out[task] = l;
    khat_out[task] = khat;
  }
}

// Sketch sizes from the predicted rank fractions (the tensor-core
// inference): k^ = n ratio, l = min(n, ceil((1 + margin) k^) + oversample),
// as k_box_features forms them; a ratio outside [0, 1] (an inference whose
// wait gave up) takes the whole box, l = n.
__global__ void k_sketch_sizes(const IdTask* tasks, int ntask, const float* ratio, float margin,
                               int oversample, int* l_out, float* khat_out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ntask) return;
  const int n = tasks[i].n;
  float r = ratio[i];
  if (!(r >= 0.f && r <= 1.f)) r = 1.f;
  const float khat = (float)n * r;
  l_out[i] = min(n, (int)ceilf((1.f + margin) * khat) + oversample);
  khat_out[i] = khat;
}

// Streaming multiprocessors of the current device.
inline int device_sm_count() {
  int dev = 0, n = 0;
  KI_CUDA(cudaGetDevice(&dev));
  KI_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
  return n;
}

// k_id with fr-row fold blocks over `grid` boxes.  threads: kThreads or (FP32)
// kIdBigThreads, 0 for the heuristic: FP32 launches of fewer boxes than SMs
// use kIdBigThreads threads per CTA.
template <typename T, typename... A>
void launch_k_id(int fr, int threads, unsigned grid, size_t smem, cudaStream_t st, A&&... args) {
  static const int n_sm = device_sm_count();
  if constexpr (sizeof(T) == 4) {
    if (threads == 0 ? (int)grid < n_sm : threads == kIdBigThreads) {
      if (fr == 64)
        ki::launch(k_id<T, 64, kIdBigThreads>, grid, kIdBigThreads, smem, st, std::forward<A>(args)...);
      else
        ki::launch(k_id<T, 32, kIdBigThreads>, grid, kIdBigThreads, smem, st, std::forward<A>(args)...);
      return;
    }
  }
  if (fr == 64)
    ki::launch(k_id<T, 64>, grid, kThreads, smem, st, std::forward<A>(args)...);
  else
    ki::launch(k_id<T, 32>, grid, kThreads, smem, st, std::forward<A>(args)...);
}

// Shared-memory bytes of k_id for a box of n active DOFs: mode 0 keeps the
// triangle in shared memory, mode 1 in the global scratch.
template <typename T>
size_t id_smem_bytes(int n, int mode, int fr = kFoldRows, int flags = 2) {
  size_t b = ((flags & 2) ? sizeof(T) * (size_t)fr * (n | 1) : 0) + sizeof(T) * 2 * (size_t)std::max(n, fr) +
             sizeof(T) * 2 * (size_t)n + sizeof(int) * (size_t)n;
  b = (b + 15) & ~size_t(15);
  if (mode == 0) b += sizeof(T) * (size_t)n * (n | 1);
  if (mode == 2) b += sizeof(T) * (size_t)n * (n + 1) / 2;
  return b;
}

// ---------------------------------------------------------------- wide boxes --
// Boxes whose ID matrix is tall (many rows, levels 1-2 in particular) or whose
// triangle does not fit in shared memory: the ID matrix is formed explicitly
// and reduced to its n x n triangle by a blocked Householder QR whose trailing
// updates (compact WY) run on many CTAs; k_id then pivots the triangle.
struct WideTask {
  int task;            // index into the level's IdTask array
  int n, m, nI;
  int64_t M;           // T-pool offset of M (m x n, column-major, ld = m)
  int64_t Tf;          // T-pool offset of the current panel's WY factor (kQrNb x kQrNb)
  int64_t act, rows;   // ipool / iscratch offsets
  double cx, cy, cz, rad;
  int64_t R;           // T-scratch offset (tws) of the row-major triangle for k_id
  int l;               // sketch rows (k_wide_sketch), 0 for the blocked QR
  int chunks;          // row chunks of the sketch
  int64_t part;        // T-pool offset of the sketch partials (chunks x l x n)
};

constexpr int kQrNb = 32;     // panel width

template <typename T>
__global__ void k_wide_assemble(const WideTask* tasks, T* wpool, const int* ipool, const int* iscratch,
                                Points<T> P, int sol_dim, ProxyTab<T> px) {
  const WideTask t = tasks[blockIdx.x];
  const int j0 = blockIdx.y * 8;
  if (j0 >= t.n) return;
  const int j1 = min(t.n, j0 + 8);
  const int* act = ipool + t.act;
  const int* rows = iscratch + t.rows;
  T* M = wpool + t.M;
  const ProxyBox<T> pbox = proxy_box<T>(t.cx, t.cy, t.cz, t.rad, px.n);
  for (int j = j0; j < j1; j++) {
    int a = act[j];
    for (int row = threadIdx.x; row < t.m; row += blockDim.x)
      M[row + (size_t)t.m * j] = id_entry<T>(P, sol_dim, row, t.nI, rows, a, px, pbox);
  }
}

// Sketched ID of a wide box: Y = Omega M (l x n) with M the box's ID matrix
// (generated on the fly) and Omega random signs.  Grid (box, row chunk of
// kSketchRows, column block of kSketchCols): each CTA sums its chunk into
// its own partial, k_wide_sketch_reduce adds the partials in a fixed order
// into the row-major sketch the ID kernel then pivots (flags 4).
constexpr int kSketchRows = 256;
constexpr int kSketchCols = 64;
constexpr int kSketchSub = 32;   // rows generated per pass

template <typename T>
__global__ void __launch_bounds__(256) k_wide_sketch(const WideTask* tasks, T* wpool,
                                                     const int* ipool, const int* iscratch,
                                                     Points<T> P, int sol_dim, ProxyTab<T> px) {
  extern __shared__ __align__(16) unsigned char sk_smem[];
  const WideTask t = tasks[blockIdx.x];
  if (t.l <= 0) return;
  const int r0 = blockIdx.y * kSketchRows, c0 = blockIdx.z * kSketchCols;
  if (r0 >= t.m || c0 >= t.n) return;
  const int r1 = min(t.m, r0 + kSketchRows), nc = min(kSketchCols, t.n - c0);
  const int l = t.l, words = (l + 31) >> 5;
  T* Y = reinterpret_cast<T*>(sk_smem);                  // l x kSketchCols
  T* B = Y + (size_t)l * kSketchCols;                    // kSketchSub x kSketchCols
  uint32_t* sgn = reinterpret_cast<uint32_t*>(B + kSketchSub * kSketchCols);
  const int* act = ipool + t.act;
  const int* rows = iscratch + t.rows;
  const ProxyBox<T> pb = proxy_box<T>(t.cx, t.cy, t.cz, t.rad, px.n);
  for (int e = threadIdx.x; e < l * kSketchCols; e += blockDim.x) Y[e] = T(0);
  for (int rb = r0; rb < r1; rb += kSketchSub) {
    __syncthreads();
    for (int e = threadIdx.x; e < kSketchSub * kSketchCols; e += blockDim.x) {
      const int i = e / kSketchCols, c = e % kSketchCols, row = rb + i;
      B[e] = (row < r1 && c < nc) ? id_entry<T>(P, sol_dim, row, t.nI, rows, act[c0 + c], px, pb)
                                  : T(0);
    }
    for (int e = threadIdx.x; e < kSketchSub * words; e += blockDim.x) {
      // lowbias32 integer hash (C. Wellons) of (box's active offset, row, word)
      uint32_t x = (uint32_t)(t.act * 2654435761u) ^ (uint32_t)((rb + e / words) * 40503u) ^
                   (uint32_t)((e % words) * 2246822519u);
      x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
      sgn[e] = x;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < l * kSketchCols; e += blockDim.x) {
      const int q = e / kSketchCols, c = e % kSketchCols;
      T acc = T(0);
#pragma unroll 8
      for (int i = 0; i < kSketchSub; i++) {
        const T b = B[i * kSketchCols + c];
        acc += ((sgn[i * words + (q >> 5)] >> (q & 31)) & 1u) ? -b : b;
      }
      Y[e] += acc;
    }
  }
  __syncthreads();
  T* part = wpool + t.part + (size_t)blockIdx.y * l * t.n;
  for (int e = threadIdx.x; e < l * nc; e += blockDim.x) {
    const int q = e / nc, c = e % nc;
    part[(size_t)q * t.n + c0 + c] = Y[q * kSketchCols + c];
  }
}

template <typename T>
__global__ void k_wide_sketch_reduce(const WideTask* tasks, const T* wpool, T* tws) {
  const WideTask t = tasks[blockIdx.x];
  if (t.l <= 0) return;
  const size_t ln = (size_t)t.l * t.n;
  T* Y = tws + t.R;
  for (size_t e = threadIdx.x; e < ln; e += blockDim.x) {
    T s = T(0);
    for (int z = 0; z < t.chunks; z++) s += wpool[t.part + (size_t)z * ln + e];
    Y[e] = s;
  }
}

// Block-wide sums of kQrNb per-thread values at once: a butterfly inside each
// warp leaves lane q with the warp's sum of value q (31 shuffles for 32
// values), then lane q of every warp is added.  Result in out[0..kQrNb).
template <typename T>
__device__ void block_sum_vec(T (&vals)[kQrNb], T* red /* [nwarps][kQrNb] */, T* out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int half = 16; half >= 1; half >>= 1) {
    // keep values whose bit `half` matches the lane's, send the others
    const bool upper = (lane & half) != 0;
#pragma unroll
    for (int q = 0; q < half; q++) {
      T send = upper ? vals[q] : vals[q + half];
      T keep = upper ? vals[q + half] : vals[q];
      vals[q] = keep + __shfl_xor_sync(0xffffffff, send, half);
    }
  }
  // lane holds the warp sum of value index = bit-reversed bookkeeping: lane
  // ends with value (lane) because each step kept the half selected by the
  // lane's bit in order 16, 8, 4, 2, 1
  red[warp * kQrNb + lane] = vals[0];
  __syncthreads();
  if (threadIdx.x < kQrNb) {
    T s = T(0);
    for (int w = 0; w < nw; w++) s += red[w * kQrNb + threadIdx.x];
    out[threadIdx.x] = s;
  }
  __syncthreads();
}

// Grid barrier of a cooperative launch (every CTA resident by construction):
// the CTA arrives on a counter, the last arriver resets it and advances the
// generation, the others wait for the advance -- for at most `limit` SM
// cycles.  A wait that gives up sets the abort flag and the device status
// (kDevTimeout); from then on every CTA's barrier returns false at once and
// the CTAs leave the kernel.
struct GridBar {
  unsigned int count;
  unsigned int gen;
  int abort;
};
constexpr long long kGridBarCycles = 4000000000LL;   // ~2 s at 2 GHz, far above a barrier

__device__ bool grid_sync_bounded(GridBar* bar, unsigned nblocks, int* err) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vgen = &bar->gen;
    volatile int* vab = &bar->abort;
    int ok = *vab == 0;
    if (ok) {
      const unsigned g = *vgen;
      __threadfence();
      if (atomicAdd(&bar->count, 1u) == nblocks - 1) {
        atomicExch(&bar->count, 0u);
        __threadfence();
        atomicAdd(&bar->gen, 1u);
      } else {
        const long long t0 = clock64();
        while (*vgen == g) {
          if (*vab) { ok = 0; break; }
          if (clock64() - t0 > kGridBarCycles) {
            atomicExch(&bar->abort, 1);
            atomicMax(err, (int)kDevTimeout);
            ok = 0;
            break;
          }
        }
      }
      __threadfence();
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Householder QR of the panel M(p:m, p:p+w) in place (LAPACK xGEQR2 layout:
// reflector tails below the diagonal, R on and above), plus the forward
// column-wise WY factor T (xLARFT) of the panel, for every wide box of a
// level at once: one cooperative launch, the rows of each box's panel split
// over consecutive CTAs (`rows` rows each, chunk 0 from row p).  Per
// reflector j: each CTA forms its rows' share of ||column j below the
// diagonal||^2; after a grid barrier every CTA of the box sums the shares in
// chunk order (the same value everywhere), forms beta, tau and v, and its
// share of v^T against the panel's other columns; after a second barrier it
// sums those, updates its rows, and chunk 0 (which holds rows p .. p+31)
// updates row j and the WY factor.  Values written by other CTAs are read
// past L1 (__ldcg).
constexpr int kPanelRed = 40;   // per-CTA stride of the partial sums: 1 norm + 32 products

template <typename T>
__global__ void __launch_bounds__(256) k_qr_panel_coop(const WideTask* tasks, int ntask, T* wpool,
                                                      int p, int rows, T* red, GridBar* bar,
                                                      int* err) {
  int box = 0, first = 0, cnt = 0;
  for (int acc = 0; box < ntask; box++) {
    const WideTask& tb = tasks[box];
    cnt = p < min(tb.n, tb.m) ? (tb.m - p + rows - 1) / rows : 0;
    if ((int)blockIdx.x < acc + cnt) {
      first = acc;
      break;
    }
    acc += cnt;
  }
  // (the grid is the sum of the counts, so every CTA has a box; one without
  // would take part in the barriers only)
  WideTask t{};
  if (box < ntask) t = tasks[box];
  const int m = t.m, n = t.n, w = box < ntask ? min(kQrNb, min(n, m) - p) : 0;
  const int chunk = blockIdx.x - first;
  const int r0 = p + chunk * rows, r1 = min(m, r0 + rows);
  T* A = wpool + t.M;
  T* Tf = wpool + t.Tf;
  T* my = red + (size_t)blockIdx.x * kPanelRed;
  const T* box_red = red + (size_t)first * kPanelRed;
  __shared__ T sred[8 * kQrNb];
  __shared__ T s_sum[kQrNb];
  __shared__ T s_row[kQrNb];   // row j of the panel (read before anyone updates it)
  __shared__ T s_w[kQrNb];
  __shared__ T s_tau, s_beta, s_scale;
  const int nwarp = blockDim.x >> 5;
  T vals[kQrNb];
  for (int jj = 0; jj < kQrNb; jj++) {
    const bool live = jj < w;
    const int j = p + jj;
    const int i0 = max(r0, j + 1);   // this CTA's rows below the diagonal
    // (A) this CTA's share of the column's squared norm below the diagonal
    if (live) {
      T sq = T(0);
      for (int i = i0 + threadIdx.x; i < r1; i += blockDim.x) {
        const T x = A[i + (size_t)m * j];
        sq += x * x;
      }
      sq = warp_sum(sq);
      if ((threadIdx.x & 31) == 0) sred[threadIdx.x >> 5] = sq;
      __syncthreads();
      if (threadIdx.x == 0) {
        T s2 = T(0);
        for (int q = 0; q < nwarp; q++) s2 += sred[q];
        my[0] = s2;
      }
    }
    if (!grid_sync_bounded(bar, gridDim.x, err)) return;
    // (B) beta, tau, v on this CTA's rows, and its share of v^T (panel columns)
    if (live) {
      if (threadIdx.x < w) s_row[threadIdx.x] = __ldcg(A + j + (size_t)m * (p + threadIdx.x));
      if (threadIdx.x == 0) {
        T sigma = T(0);
        for (int c = 0; c < cnt; c++) sigma += __ldcg(box_red + (size_t)c * kPanelRed);
        const T alpha = __ldcg(A + j + (size_t)m * j);
        T tau = T(0), beta = alpha, scale = T(0);
        if (sigma != T(0)) {
          const T nrm = sqrt(alpha * alpha + sigma);
          beta = alpha >= T(0) ? -nrm : nrm;
          tau = (beta - alpha) / beta;
          scale = T(1) / (alpha - beta);
        }
        s_tau = tau;
        s_beta = beta;
        s_scale = scale;
      }
      __syncthreads();
      const T scale = s_scale;
      // products: z_l = V(:, l)^T v for the earlier reflectors (l < jj),
      // d = c^T v for the later panel columns, packed as q < jj then q - jj
      const int nz = jj, nd = w - jj - 1;
#pragma unroll
      for (int q = 0; q < kQrNb; q++) vals[q] = T(0);
      for (int i = i0 + threadIdx.x; i < r1; i += blockDim.x) {
        const T v = A[i + (size_t)m * j] * scale;
        A[i + (size_t)m * j] = v;
#pragma unroll
        for (int q = 0; q < kQrNb; q++) {
          const int col = q < nz ? p + q : j + 1 + (q - nz);
          if (q < nz + nd) vals[q] += A[i + (size_t)m * col] * v;
        }
      }
      block_sum_vec<T>(vals, sred, s_sum);
      if (threadIdx.x < kQrNb) my[1 + threadIdx.x] = s_sum[threadIdx.x];
    }
    if (!grid_sync_bounded(bar, gridDim.x, err)) return;
    // (C) the box's sums, this CTA's rows of the later panel columns, and
    // (chunk 0) row j and the WY factor's column jj
    if (live) {
      const T tau = s_tau;
      const int nz = jj, nd = w - jj - 1;
      if (threadIdx.x < kQrNb) {
        T tot = T(0);
        for (int c = 0; c < cnt; c++) tot += __ldcg(box_red + (size_t)c * kPanelRed + 1 + threadIdx.x);
        s_sum[threadIdx.x] = tot;
      }
      __syncthreads();
      if (threadIdx.x < nd) s_w[threadIdx.x] = (s_row[jj + 1 + threadIdx.x] + s_sum[nz + threadIdx.x]) * tau;
      __syncthreads();
      for (int i = i0 + threadIdx.x; i < r1; i += blockDim.x) {
        const T v = A[i + (size_t)m * j];
        for (int q = 0; q < nd; q++) A[i + (size_t)m * (j + 1 + q)] -= s_w[q] * v;
      }
      if (chunk == 0) {
        if (threadIdx.x < nd) A[j + (size_t)m * (j + 1 + threadIdx.x)] = s_row[jj + 1 + threadIdx.x] - s_w[threadIdx.x];
        if (threadIdx.x == 32) A[j + (size_t)m * j] = s_beta;
        if (threadIdx.x == 64) {
          // T(0:jj, jj) = -tau T(0:jj, 0:jj) z, z_l = V(j, l) + V(j+1:, l)^T v
          T z[kQrNb];
          for (int l = 0; l < nz; l++) z[l] = s_sum[l] + s_row[l];
          for (int l = 0; l < nz; l++) {
            T acc = T(0);
            for (int q = l; q < nz; q++) acc += Tf[l + kQrNb * q] * z[q];
            Tf[l + kQrNb * jj] = -tau * acc;
          }
          Tf[jj + kQrNb * jj] = tau;
        }
      }
      __syncthreads();
    }
  }
}

// Trailing update of the blocked QR, A(p:m, p+w:n) <- (I - V T V^T)^T
// A(p:m, p+w:n), in three register-tiled launches over many CTAs per box:
//   k_qr_wpart  partial products V^T A over chunks of kQrChunk rows;
//   k_qr_wsum   W = the partials summed in a fixed order, then W <- T^T W;
//   k_qr_apply  A -= V W in tiles of kQrTileRows x kQrTileCols.
// V (the panel's reflectors) is unit lower trapezoidal: V(row, l) is the
// stored tail below the diagonal (row > p + l), 1 on it, 0 above.
constexpr int kQrChunk = 2048;     // rows per partial product
constexpr int kQrWCols = 64;       // trailing columns per CTA of k_qr_wpart / k_qr_wsum
constexpr int kQrSub = 32;         // rows staged per step of k_qr_wpart
constexpr int kQrTileRows = 64;    // k_qr_apply tile
constexpr int kQrTileCols = 64;

template <typename T>
__device__ __forceinline__ T qr_v(const T* A, int m, int p, int row, int l) {
  return row > p + l ? A[row + (size_t)m * (p + l)] : (row == p + l ? T(1) : T(0));
}

// Grid (box, column block of kQrWCols, row chunk).  Thread (4 reflectors x
// 4 columns) of the 32 x 64 block; rows staged kQrSub at a time.
template <typename T>
__global__ void __launch_bounds__(128) k_qr_wpart(const WideTask* tasks, const T* wpool, T* parts,
                                                  int p) {
  const WideTask t = tasks[blockIdx.x];
  const int m = t.m, n = t.n;
  if (p >= min(n, m)) return;
  const int w = min(kQrNb, min(n, m) - p);   // reflectors of the panel (rows below p permitting)
  const int c0 = p + w + blockIdx.y * kQrWCols;
  const int r0 = p + blockIdx.z * kQrChunk;
  if (c0 >= n || r0 >= m) return;
  const int r1 = min(m, r0 + kQrChunk), nc = min(kQrWCols, n - c0);
  const T* A = wpool + t.M;
  __shared__ T Vs[kQrSub][kQrNb + 1];
  __shared__ T As[kQrSub][kQrWCols + 1];
  const int tid = threadIdx.x, lr = (tid >> 4) * 4, lc = (tid & 15) * 4;
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) acc[a][b] = T(0);
  for (int rb = r0; rb < r1; rb += kQrSub) {
    __syncthreads();
    for (int e = tid; e < kQrSub * kQrNb; e += blockDim.x) {
      const int i = e % kQrSub, l = e / kQrSub, row = rb + i;   // rows fastest: coalesced
      Vs[i][l] = (row < r1 && l < w) ? qr_v(A, m, p, row, l) : T(0);
    }
    for (int e = tid; e < kQrSub * kQrWCols; e += blockDim.x) {
      const int i = e % kQrSub, c = e / kQrSub, row = rb + i;
      As[i][c] = (row < r1 && c < nc) ? A[row + (size_t)m * (c0 + c)] : T(0);
    }
    __syncthreads();
#pragma unroll 4
    for (int i = 0; i < kQrSub; i++) {
      T v[4], x[4];
#pragma unroll
      for (int a = 0; a < 4; a++) v[a] = Vs[i][lr + a];
#pragma unroll
      for (int b = 0; b < 4; b++) x[b] = As[i][lc + b];
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] += v[a] * x[b];
    }
  }
  // partial z of the box: kQrNb x n, row-major (reflector l, column c)
  T* out = parts + t.part + (size_t)blockIdx.z * kQrNb * n;
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++)
      if (lr + a < w && lc + b < nc) out[(size_t)(lr + a) * n + c0 + lc + b] = acc[a][b];
}

// Grid (box, column block): one thread per trailing column sums the row
// chunks' partials in chunk order, applies T^T (T upper triangular:
// (T^T W)_l = sum_(r <= l) T(r, l) W_r) and writes W into partial 0.
template <typename T>
__global__ void __launch_bounds__(kQrWCols) k_qr_wsum(const WideTask* tasks, const T* wpool, T* parts,
                                                      int p) {
  const WideTask t = tasks[blockIdx.x];
  const int m = t.m, n = t.n;
  if (p >= min(n, m)) return;
  const int w = min(kQrNb, min(n, m) - p);   // reflectors of the panel (rows below p permitting)
  const int c = p + w + blockIdx.y * kQrWCols + threadIdx.x;
  if (c >= n) return;
  const int chunks = (m - p + kQrChunk - 1) / kQrChunk;
  const T* Tf = wpool + t.Tf;
  T* W = parts + t.part;
  T s[kQrNb];
#pragma unroll
  for (int l = 0; l < kQrNb; l++) s[l] = T(0);
  for (int z = 0; z < chunks; z++) {
    const T* pz = W + (size_t)z * kQrNb * n;
#pragma unroll
    for (int l = 0; l < kQrNb; l++)
      if (l < w) s[l] += pz[(size_t)l * n + c];
  }
#pragma unroll
  for (int l = 0; l < kQrNb; l++) {
    if (l >= w) break;
    T acc = T(0);
#pragma unroll
    for (int r = 0; r < kQrNb; r++)
      if (r <= l) acc += Tf[r + kQrNb * l] * s[r];
    W[(size_t)l * n + c] = acc;
  }
}

// Grid (box, row tile, column tile): A(rows, cols) -= V(rows, :) W(:, cols).
// Thread: 4 consecutive rows x 8 columns (16 threads cover a tile column's
// 64 rows, coalesced); V^T and W staged in shared memory.
template <typename T>
__global__ void __launch_bounds__(128) k_qr_apply(const WideTask* tasks, T* wpool, const T* parts, int p) {
  const WideTask t = tasks[blockIdx.x];
  const int m = t.m, n = t.n;
  if (p >= min(n, m)) return;
  const int w = min(kQrNb, min(n, m) - p);   // reflectors of the panel (rows below p permitting)
  const int rt = p + blockIdx.y * kQrTileRows, ct = p + w + blockIdx.z * kQrTileCols;
  if (rt >= m || ct >= n) return;
  const int nr = min(kQrTileRows, m - rt), nc = min(kQrTileCols, n - ct);
  T* A = wpool + t.M;
  const T* W = parts + t.part;
  __shared__ T Vt[kQrNb][kQrTileRows];
  __shared__ T Ws[kQrNb][kQrTileCols];
  const int tid = threadIdx.x;
  for (int e = tid; e < kQrNb * kQrTileRows; e += blockDim.x) {
    const int i = e % kQrTileRows, l = e / kQrTileRows;
    Vt[l][i] = (i < nr && l < w) ? qr_v(A, m, p, rt + i, l) : T(0);
  }
  for (int e = tid; e < kQrNb * kQrTileCols; e += blockDim.x) {
    const int c = e % kQrTileCols, l = e / kQrTileCols;
    Ws[l][c] = (c < nc && l < w) ? W[(size_t)l * n + ct + c] : T(0);
  }
  __syncthreads();
  const int r4 = (tid & 15) * 4, c8 = (tid >> 4) * 8;
  T acc[4][8];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 8; b++) acc[a][b] = T(0);
  for (int l = 0; l < w; l++) {
    T v[4], x[8];
#pragma unroll
    for (int a = 0; a < 4; a++) v[a] = Vt[l][r4 + a];
#pragma unroll
    for (int b = 0; b < 8; b++) x[b] = Ws[l][c8 + b];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int b = 0; b < 8; b++) acc[a][b] += v[a] * x[b];
  }
#pragma unroll
  for (int b = 0; b < 8; b++) {
    if (c8 + b >= nc) continue;
    T* col = A + (size_t)m * (ct + c8 + b) + rt;
#pragma unroll
    for (int a = 0; a < 4; a++)
      if (r4 + a < nr) col[r4 + a] -= acc[a][b];
  }
}

// Column-pivoted QR of wide boxes' triangles (or formed sketches) over many
// CTAs per box: the rank decision, permutation, T = R11^-1 R12 and permuted
// active list k_id writes with flags 4, for boxes too large for one CTA to
// pivot quickly.  R (rows x n, row-major, ld n) sits in the task's scratch,
// T is written after it.  One cooperative launch for all such boxes of a
// level; each CTA owns kCpqrCols consecutive columns of its box, one thread
// per column.  Columns do not move: pivoting marks a column done and
// records it as the next logical position.  Per step j: each CTA's largest
// partial norm among its active columns (the first column on ties); after a
// grid barrier every CTA of the box picks the box's pivot from those in CTA
// order, and the pivot's owner forms the reflector of its column below row j
// (xLARFG) into the box's shared vector; after a second barrier every CTA
// checks the rank rule (|R_jj| < tol |R_00| at j >= 1 stops, before the
// reflector is applied) and applies the reflector to its active columns with
// xLAQP2's norm downdating.  The remaining columns follow the pivots in
// column order.  Boxes that stopped wait in the barriers; when every box has
// stopped all CTAs leave the loop together.  Values other CTAs wrote are
// read past L1.
constexpr int kCpqrCols = 64;
// Wide boxes of at least this many columns take the cooperative pivoted QR.
constexpr int kCoopCpqrMinN = 384;

struct CpqrTask {
  int task;          // the level's IdTask index (rank out)
  int n, rows;       // columns; rows of R (n for a triangle, l for a sketch)
  int jmax;          // pivot steps available: min(n, m, rows)
  int sketch;        // R is a sketch with fewer rows than columns (rank guard)
  int first, ctas;   // the box's CTAs in the grid
  int64_t R;         // scratch offset of R; T at R + n n
  int64_t perm, pact, act;   // iscratch / ipool offsets
  int64_t v;         // offset in the launch's vector pool: rows + 2 values
};

template <typename T>
__global__ void __launch_bounds__(kCpqrCols) k_cpqr_coop(const CpqrTask* tasks, int ntask, T* tws,
                                                         int* iscratch, int* ipool, T* vpool,
                                                         long long* ckey,
                                                         int* ccol, int* boxes_done, double tol,
                                                         int* k_out, GridBar* bar, int* err) {
  extern __shared__ __align__(16) unsigned char cc_smem[];
  int b = 0;
  while (b < ntask && (int)blockIdx.x >= tasks[b].first + tasks[b].ctas) b++;
  CpqrTask t{};
  if (b < ntask) t = tasks[b];
  const int n = t.n, rows = t.rows;
  const int cta = blockIdx.x - t.first;
  const int c = cta * kCpqrCols + threadIdx.x;
  const bool mine = b < ntask && c < n;
  T* R = tws + t.R;
  T* vb = vpool + t.v;
  int* perm = iscratch + t.perm;
  T* vs = reinterpret_cast<T*>(cc_smem);   // the reflector, rows values
  __shared__ long long s_key[kCpqrCols / 32];
  __shared__ int s_col[kCpqrCols / 32];
  __shared__ int s_p;
  __shared__ T s_red[kCpqrCols / 32];
  __shared__ T s_beta, s_tau;
  // partial norms of my column (the triangle is zero below the diagonal)
  T vn1 = T(0), vn2 = T(0);
  bool active = mine;
  if (mine) {
    const int ilast = t.sketch ? rows - 1 : min(c, rows - 1);
    T s2 = T(0);
    for (int i = 0; i <= ilast; i++) s2 += R[(size_t)i * n + c] * R[(size_t)i * n + c];
    vn1 = sqrt(s2);
    vn2 = vn1;
  }
  T thresh = T(0);
  int k = 0;
  bool stopped = b >= ntask;   // a CTA without a box only joins the barriers
  int jmax_all = 0;
  for (int q = 0; q < ntask; q++) jmax_all = max(jmax_all, tasks[q].jmax);
  for (int j = 0; j < jmax_all; j++) {
    // (A) this CTA's candidate
    if (!stopped) {
      long long key = active ? norm_key(vn1) : -1;
      int col = c;
      for (int o = 16; o > 0; o >>= 1) {
        const long long ok = __shfl_down_sync(0xffffffffu, key, o);
        const int oc = __shfl_down_sync(0xffffffffu, col, o);
        if (ok > key || (ok == key && oc < col)) { key = ok; col = oc; }
      }
      if ((threadIdx.x & 31) == 0) {
        s_key[threadIdx.x >> 5] = key;
        s_col[threadIdx.x >> 5] = col;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        long long bk = s_key[0];
        int bc = s_col[0];
        for (int w = 1; w < kCpqrCols / 32; w++)
          if (s_key[w] > bk || (s_key[w] == bk && s_col[w] < bc)) { bk = s_key[w]; bc = s_col[w]; }
        ckey[blockIdx.x] = bk;
        ccol[blockIdx.x] = bc;
      }
    }
    if (!grid_sync_bounded(bar, gridDim.x, err)) return;
    if (__ldcg(boxes_done) == ntask) break;   // every box has stopped (uniform)
    // (B) the box's pivot; its owner forms the reflector
    if (!stopped) {
      if (threadIdx.x == 0) {
        long long bk = -2;
        int bc = n;
        for (int q = 0; q < t.ctas; q++) {
          const long long kq = __ldcg(ckey + t.first + q);
          const int cq = __ldcg(ccol + t.first + q);
          if (kq > bk || (kq == bk && cq < bc)) { bk = kq; bc = cq; }
        }
        s_p = bc;
      }
      __syncthreads();
      const int p = s_p;
      if (p / kCpqrCols == cta) {
        T sg = T(0);
        for (int i = j + 1 + threadIdx.x; i < rows; i += blockDim.x) sg += R[(size_t)i * n + p] * R[(size_t)i * n + p];
        sg = warp_sum(sg);
        if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = sg;
        __syncthreads();
        if (threadIdx.x == 0) {
          T sigma = T(0);
          for (int w = 0; w < kCpqrCols / 32; w++) sigma += s_red[w];
          const T alpha = R[(size_t)j * n + p];
          T tau = T(0), beta = alpha, scale = T(0);
          if (sigma != T(0)) {
            const T nrm = sqrt(alpha * alpha + sigma);
            beta = alpha >= T(0) ? -nrm : nrm;
            tau = (beta - alpha) / beta;
            scale = T(1) / (alpha - beta);
          }
          vb[rows] = beta;
          vb[rows + 1] = tau;
          s_tau = scale;   // the owner's scale, below
          perm[j] = p;
        }
        __syncthreads();
        const T scale = s_tau;
        for (int i = j + 1 + threadIdx.x; i < rows; i += blockDim.x) vb[i] = R[(size_t)i * n + p] * scale;
        if (c == p) active = false;
      }
    }
    if (!grid_sync_bounded(bar, gridDim.x, err)) return;
    // (C) rank rule, then the reflector on this CTA's active columns
    if (!stopped) {
      if (threadIdx.x == 0) {
        s_beta = __ldcg(vb + rows);
        s_tau = __ldcg(vb + rows + 1);
      }
      __syncthreads();
      const T beta = s_beta, tau = s_tau;
      if (j == 0) thresh = fabs(T(tol) * beta);
      if (j >= 1 && fabs(beta) < thresh) {
        k = j;
        stopped = true;
        if (cta == 0 && threadIdx.x == 0) atomicAdd(boxes_done, 1);
      } else {
        const int p = s_p;
        if (c == p) R[(size_t)j * n + p] = beta;
        for (int i = j + 1 + threadIdx.x; i < rows; i += blockDim.x) vs[i] = __ldcg(vb + i);
        __syncthreads();
        if (active && tau != T(0)) {
          T w0 = R[(size_t)j * n + c], w1 = T(0);
          int i = j + 1;
          for (; i + 1 < rows; i += 2) {
            w0 += vs[i] * R[(size_t)i * n + c];
            w1 += vs[i + 1] * R[(size_t)(i + 1) * n + c];
          }
          for (; i < rows; i++) w0 += vs[i] * R[(size_t)i * n + c];
          const T w = (w0 + w1) * tau;
          R[(size_t)j * n + c] -= w;
          for (int q = j + 1; q < rows; q++) R[(size_t)q * n + c] -= w * vs[q];
        }
        if (active) {
          const T rjc = R[(size_t)j * n + c];
          if (vn1 != T(0)) {
            T temp = fabs(rjc) / vn1;
            temp = T(1) - temp * temp;
            temp = temp < T(0) ? T(0) : temp;
            const T qq = vn1 / vn2;
            if (temp * qq * qq <= tol3z<T>()) {
              T s2 = T(0);
              for (int q = j + 1; q < rows; q++) s2 += R[(size_t)q * n + c] * R[(size_t)q * n + c];
              vn1 = sqrt(s2);
              vn2 = vn1;
            } else {
              vn1 = vn1 * sqrt(temp);
            }
          }
        }
        if (j == t.jmax - 1) {   // pivots exhausted without the rule firing
          stopped = true;
          if (cta == 0 && threadIdx.x == 0) atomicAdd(boxes_done, 1);
        }
      }
    }
  }
  // k = 0: the rule never fired (no compression); a sketch must reveal the
  // rank with kSketchGuard rows to spare
  const bool fallback =
      b < ntask && t.sketch && rows < n && (k == 0 ? t.jmax == rows : k > rows - kSketchGuard);
  const bool need = b < ntask && !fallback && k > 0;
  if (b < ntask && cta == 0 && threadIdx.x == 0) k_out[t.task] = fallback ? -1 : k;
  // the redundant columns, in column order, after the k skeleton columns
  // perm[0 .. k) (the pivot of step k, chosen before the rule fired, is
  // redundant): the box's first CTA marks those in shared memory and one
  // thread lists the rest (~n steps)
  if (need && cta == 0) {
    unsigned char* skel = cc_smem;   // n bytes
    for (int q = threadIdx.x; q < n; q += blockDim.x) skel[q] = 0;
    __syncthreads();
    for (int a = threadIdx.x; a < k; a += blockDim.x) skel[__ldcg(perm + a)] = 1;
    __syncthreads();
    if (threadIdx.x == 0) {
      int pos = k;
      for (int q = 0; q < n; q++)
        if (!skel[q]) perm[pos++] = q;
    }
  }
  // every CTA (of every box, and the ones without a box) passes this barrier
  // once: the box's CTAs then read the tail of perm
  if (!grid_sync_bounded(bar, gridDim.x, err)) return;
  if (!need) return;
  int* sp = reinterpret_cast<int*>(cc_smem);   // perm, n ints
  for (int e = threadIdx.x; e < n; e += blockDim.x) sp[e] = __ldcg(perm + e);
  __syncthreads();
  const int r = n - k;
  T* Tout = R + (size_t)n * n;
  const int* act = ipool + t.act;
  int* pact = ipool + t.pact;
  for (int e = cta * kCpqrCols + threadIdx.x; e < n; e += t.ctas * kCpqrCols) pact[e] = act[sp[e]];
  // T = R11^-1 R12: one redundant column per thread, back substitution with
  // the pivot columns' upper triangle
  for (int cr = cta * kCpqrCols + threadIdx.x; cr < r; cr += t.ctas * kCpqrCols) {
    const int pc = sp[k + cr];
    for (int a = k - 1; a >= 0; a--) {
      T s = __ldcg(R + (size_t)a * n + pc);
      for (int l = a + 1; l < k; l++) s -= __ldcg(R + (size_t)a * n + sp[l]) * Tout[l + (size_t)k * cr];
      Tout[a + (size_t)k * cr] = s / __ldcg(R + (size_t)a * n + sp[a]);
    }
  }
}

// Upper triangle of M (column-major) -> row-major n x n scratch for k_id.
template <typename T>
__global__ void k_wide_triangle(const WideTask* tasks, const T* wpool, T* tws) {
  const WideTask t = tasks[blockIdx.x];
  const T* M = wpool + t.M;
  T* R = tws + t.R;
  for (int e = threadIdx.x; e < t.n * t.n; e += blockDim.x) {
    int i = e / t.n, c = e % t.n;
    R[e] = (i <= c && i < t.m) ? M[i + (size_t)t.m * c] : T(0);
  }
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
// (SkelFactorization::decouple, skel_factorization.cpp:91-127).  Working set
// K_ss (k x k) | T (k x r) | Wrs (r x k) | Lt (r x k) | X (r x r) | r scratch
// entries (and, inverse path, X's copy, U0, L0) in shared memory when it fits
// (smem != 0), else in the global scratch t.ws
// (X in place in the output).  The blocks are gathered from the box's self
// block through the skeleton-first permutation; K_sr is held only
// transposed (Lt), and K_rr only as X.  With t.Xi (FP32 forms, shared-
// memory boxes) X is inverted in place by Gauss-Jordan elimination and L, U
// are products with the inverse; otherwise X is LU-factored (the
// reference's dgetrf / dgetrs) and L, U come from triangular solves.
// Block sizes k_schur is compiled for: FP32 up to 1024 threads (64 registers,
// so four 256-thread CTAs or one 1024-thread CTA per SM), FP64 256 threads
// with two CTAs per SM.  Boxes whose shared working set leaves room for only
// one or two CTAs per SM get the larger blocks (schur_threads).
template <typename T> constexpr int kSchurMaxThreads = sizeof(T) == 4 ? 1024 : kThreads;
// Register tile of the Gauss-Jordan inverse: up to kGjCols columns per warp
// (X up to 64 rows and kGjCols W columns with W warps).
constexpr int kGjCols = 8;
template <typename T> constexpr int kSchurMinBlocks = sizeof(T) == 4 ? 1 : 2;
// phase (Gauss-Jordan path in shared memory only): 0 the whole elimination;
// 1 up to X = K_rr - T^T K_sr - K~_rs T, which is stored in t.X (r x r) with
// K_ss, K~_rs and K~_sr^T in t.ws (k x k | r x k | r x k), for k_gj to
// invert into t.Xi; 2 the products with the inverse, from those stores.
template <typename T>
__global__ void __launch_bounds__(kSchurMaxThreads<T>, kSchurMinBlocks<T>) k_schur(const SchurTask<T>* tasks, int task_base,
                                                     int smem, int* err, int phase) {
  extern __shared__ __align__(16) unsigned char sc_smem[];
  const SchurTask<T> t = tasks[task_base + blockIdx.x];
  const int n = t.n, k = t.k, r = n - k;
  // r-row blocks in shared memory use an odd leading dimension, so that
  // threads stepping along a row (transposed operands) hit distinct banks
  const int ld = smem ? (r | 1) : r;
  __shared__ T s_red, s_val[2];
  __shared__ int s_idx, s_flag;
  T* base = smem ? reinterpret_cast<T*>(sc_smem) : t.ws;
  T* Kss = base;                      // k x k
  // shared-memory boxes: T (k x r) staged with the odd leading dimension kt
  const int kt = smem ? (k | 1) : k;
  T* Ts = Kss + (size_t)k * k;
  T* Wrs = smem ? Ts + (size_t)kt * r : Ts;   // r x k : K_rs, then K~_rs, then U
  T* Lt = Wrs + (size_t)ld * k;       // r x k : K_sr^T, then K~_sr^T, then L^T
  T* X = smem ? Lt + (size_t)ld * k : t.X;   // r x r
  const int* pm = t.perm;
  if (phase == 2) {
    // K_ss | K~_rs | K~_sr^T from t.ws, X^-1 from t.Xi, X itself from t.X
    T* X0 = X + (size_t)ld * r + 5 * (size_t)r;
    const T* g = t.ws;
    for (int idx = threadIdx.x; idx < k * k; idx += blockDim.x) Kss[idx] = g[idx];
    for (int idx = threadIdx.x; idx < r * k; idx += blockDim.x) {
      const int i = idx % r, j = idx / r;
      Wrs[i + (size_t)ld * j] = g[k * k + idx];
      Lt[i + (size_t)ld * j] = g[k * k + r * k + idx];
    }
    for (int idx = threadIdx.x; idx < r * r; idx += blockDim.x) {
      const int i = idx % r, j = idx / r;
      X[i + (size_t)ld * j] = t.Xi[idx];
      X0[i + (size_t)ld * j] = t.X[idx];
    }
    __syncthreads();
  } else {
  for (int idx = threadIdx.x; idx < k * k; idx += blockDim.x) {
    const int i = idx % k, j = idx / k;
    Kss[idx] = t.K[pm[i] + (size_t)n * pm[j]];
  }
  for (int idx = threadIdx.x; idx < r * k; idx += blockDim.x) {
    const int i = idx % r, j = idx / r;
    Wrs[i + (size_t)ld * j] = t.K[pm[k + i] + (size_t)n * pm[j]];   // K_rs(i, j)
    Lt[i + (size_t)ld * j] = t.K[pm[j] + (size_t)n * pm[k + i]];    // K_sr(j, i)
  }
  for (int idx = threadIdx.x; idx < r * r; idx += blockDim.x) {
    const int i = idx % r, j = idx / r;
    X[i + (size_t)ld * j] = t.K[pm[k + i] + (size_t)n * pm[k + j]];
  }
  for (int idx = threadIdx.x; idx < k * r; idx += blockDim.x) {
    const T v = t.Tin[idx];
    t.Tout[idx] = v;
    if (smem) Ts[idx % k + (size_t)kt * (idx / k)] = v;
  }
  __syncthreads();
  const T* Tm = smem ? Ts : t.Tin;
  // X -= T^T K_sr  (K_sr(l, j) = Lt[j + ld l])
  cta_gemm<T>(r, r, k, T(-1), Tm, kt, true, Lt, ld, true, T(1), X, ld);
  __syncthreads();
  // K~_rs = K_rs - T^T K_ss ;  K~_sr^T = K_sr^T - T^T K_ss^T
  cta_gemm<T>(r, k, k, T(-1), Tm, kt, true, Kss, k, false, T(1), Wrs, ld);
  cta_gemm<T>(r, k, k, T(-1), Tm, kt, true, Kss, k, true, T(1), Lt, ld);
  __syncthreads();
  // X -= K~_rs T
  cta_gemm<T>(r, r, k, T(-1), Wrs, ld, false, Tm, kt, false, T(1), X, ld);
  __syncthreads();
  if (phase == 1) {
    T* g = t.ws;
    for (int idx = threadIdx.x; idx < k * k; idx += blockDim.x) g[idx] = Kss[idx];
    for (int idx = threadIdx.x; idx < r * k; idx += blockDim.x) {
      const int i = idx % r, j = idx / r;
      g[k * k + idx] = Wrs[i + (size_t)ld * j];
      g[k * k + r * k + idx] = Lt[i + (size_t)ld * j];
    }
    for (int idx = threadIdx.x; idx < r * r; idx += blockDim.x)
      t.X[idx] = X[idx % r + (size_t)ld * (idx / r)];
    return;
  }
  }   // phase != 2
  if (smem && t.gj) {
    // shared memory after X: scratch (5r) | X0 (r x r) | U0 (r x k) | L0 (k x r)
    T* colj = X + (size_t)ld * r;
    T* X0 = colj + 5 * (size_t)r;
    T* U0 = X0 + (size_t)ld * r;
    T* L0 = U0 + (size_t)ld * k;
    if (phase == 0) {
      for (int idx = threadIdx.x; idx < ld * r; idx += blockDim.x) X0[idx] = X[idx];
      __syncthreads();
      // X <- X^-1: in registers where the block's tile covers X, else in shared memory
      const int W = blockDim.x >> 5;
      const int info = (r <= 64 && r <= W * kGjCols)
                           ? cta_gj_inverse_reg<T, 2, kGjCols>(r, X, ld, t.piv, colj)
                           : cta_gj_inverse<T>(r, X, ld, t.piv, colj, s_val, &s_idx);
      if (info != 0 && threadIdx.x == 0) atomicMax(err, (int)kDevSingular);
    }
    // U0 = X^-1 K~_rs (r x k), L0 = K~_sr X^-1 (k x r)
    cta_gemm<T>(r, k, r, T(1), X, ld, false, Wrs, ld, false, T(0), U0, ld);
    cta_gemm<T>(k, r, r, T(1), Lt, ld, true, X, ld, false, T(0), L0, k);
    __syncthreads();
    // A~ = K_ss - L0 K~_rs (the correction's share follows below)
    cta_gemm_to<T>(k, k, r, T(-1), L0, k, false, Wrs, ld, false, T(1), Kss, k, t.Atil, k);
    __syncthreads();
    // one step of refinement in the same precision (products with an explicit
    // inverse are not backward stable; the corrected ones are): the residuals
    // RU = K~_rs - X U0 and RL = K~_sr - L0 X, in place of K~_rs and K~_sr^T
    // (RL^T = K~_sr^T - X^T L0^T)
    cta_gemm<T>(r, k, r, T(-1), X0, ld, false, U0, ld, false, T(1), Wrs, ld);
    cta_gemm<T>(r, k, r, T(-1), X0, ld, true, L0, k, true, T(1), Lt, ld);
    __syncthreads();
    // U = U0 + X^-1 RU, L = L0 + RL X^-1, A~ -= RL U0 (RL X^-1 K~_rs)
    cta_gemm_to<T>(r, k, r, T(1), X, ld, false, Wrs, ld, false, T(1), U0, ld, t.U, r);
    cta_gemm_to<T>(k, r, r, T(1), Lt, ld, true, X, ld, false, T(1), L0, k, t.L, k);
    cta_gemm<T>(k, k, r, T(-1), Lt, ld, true, U0, ld, false, T(1), t.Atil, k);
    if (phase == 0)
      for (int idx = threadIdx.x; idx < r * r; idx += blockDim.x)
        t.Xi[idx] = X[idx % r + (size_t)ld * (idx / r)];
    return;
  }
  int info = cta_lu<T>(r, X, ld, t.piv, &s_flag, &s_red, &s_idx);
  if (info != 0 && threadIdx.x == 0) atomicMax(err, (int)kDevSingular);
  // L^T = X^-T K~_sr^T
  cta_lu_solve_par<T>(r, X, ld, t.piv, true, Lt, ld, k);
  // A~ = K_ss - L K~_rs  (k x k), L = Lt^T
  for (int idx = threadIdx.x; idx < k * k; idx += blockDim.x) t.Atil[idx] = Kss[idx];
  __syncthreads();
  cta_gemm<T>(k, k, r, T(-1), Lt, ld, true, Wrs, ld, false, T(1), t.Atil, k);
  __syncthreads();
  // U = X^-1 K~_rs (in place on Wrs)
  cta_lu_solve_par<T>(r, X, ld, t.piv, false, Wrs, ld, k);
  for (int idx = threadIdx.x; idx < r * k; idx += blockDim.x)
    t.U[idx] = Wrs[idx % r + (size_t)ld * (idx / r)];
  for (int idx = threadIdx.x; idx < k * r; idx += blockDim.x) {
    int i = idx % k, j = idx / k;
    t.L[idx] = Lt[j + (size_t)ld * i];
  }
  if (smem)
    for (int idx = threadIdx.x; idx < r * r; idx += blockDim.x)
      t.X[idx] = X[idx % r + (size_t)ld * (idx / r)];
}

// Gauss-Jordan inverse of one FP32 redundant block X (r x r, column-major in
// t.X, r <= 32 MA) per CTA into t.Xi, with partial pivoting by rows that are
// not swapped but recorded (X^-1(spinv[i], spiv[c]) = a(i, c) at the end):
// the arithmetic of cta_gj_inverse_reg, with the block in registers (lane =
// rows lane, lane + 32, ..; warp w = columns CW w .. CW w + CW - 1) and only
// the warps that own columns doing work.  Per column j the warp owning it
// picks the pivot among the unused rows and publishes the column (the
// multipliers) and the pivot index in shared memory; one barrier; each warp
// takes its slab of the pivot row from the owning lane by shuffles and
// eliminates.  A zero pivot is reported (kDevSingular) and skipped.
constexpr int kGjLeanCols = 16;
template <int MA, int CW>
__global__ void __launch_bounds__(32 * (32 * MA / CW)) k_gj(const SchurTask<float>* tasks, int task_base,
                                                            int* err) {
  __shared__ float s_col[2][32 * MA];
  __shared__ int s_p[2];
  __shared__ int s_spiv[32 * MA], s_spinv[32 * MA];
  const SchurTask<float> t = tasks[task_base + blockIdx.x];
  const int r = t.n - t.k;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // warps without columns only keep the barriers company
  const bool active = w * CW < r;
  float a[MA][CW];
#pragma unroll
  for (int ia = 0; ia < MA; ia++)
#pragma unroll
    for (int c = 0; c < CW; c++) {
      const int i = lane + 32 * ia, gc = CW * w + c;
      a[ia][c] = (active && i < r && gc < r) ? t.X[i + (size_t)r * gc] : 0.f;
    }
  // column jn of the owner warp's registers into f (dynamic column index:
  // a select over the unrolled slab)
  auto column = [&](int jn, float (&f)[MA]) {
    const int jj = jn - CW * w;
#pragma unroll
    for (int ia = 0; ia < MA; ia++) {
      float v = 0.f;
#pragma unroll
      for (int c = 0; c < CW; c++) v = (c == jj) ? a[ia][c] : v;
      f[ia] = v;
    }
  };
  float fcol[MA];
  if (w == 0) column(0, fcol);
  unsigned used = 0;   // bit ia: row lane + 32 ia already a pivot row
  int info = 0;
  for (int j = 0; j < r; j++) {
    const int buf = j & 1;
    const int ow = j / CW;
    if (w == ow) {
      float best = -1.f;
      int bi = r;
#pragma unroll
      for (int ia = 0; ia < MA; ia++) {
        const int i = lane + 32 * ia;
        if (i < r && !((used >> ia) & 1u)) {
          float v = fabsf(fcol[ia]);
          if (!(v == v)) v = 3e38f;   // a NaN orders first, so the choice stays a valid row
          if (v > best) { best = v; bi = i; }
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
      }
#pragma unroll
      for (int ia = 0; ia < MA; ia++) s_col[buf][lane + 32 * ia] = fcol[ia];
      if (lane == 0) {
        s_p[buf] = bi;
        s_spiv[j] = bi;
        s_spinv[bi] = j;
        t.piv[j] = bi;
      }
    }
    __syncthreads();
    const int p = s_p[buf];
    const int pa = p >> 5, pl = p & 31;
    if (pl == lane) used |= 1u << pa;
    const float pv = s_col[buf][p];
    const int jn = j + 1;
    const bool own_next = jn < r && w == jn / CW;
    if (pv == 0.f) {   // the same branch in every thread
      if (info == 0) info = j + 1;
      if (own_next) column(jn, fcol);
      continue;
    }
    if (!active) continue;
    const float inv = 1.f / pv;
    float m[MA];
    bool isp[MA];
#pragma unroll
    for (int ia = 0; ia < MA; ia++) {
      isp[ia] = (ia == pa) && (pl == lane);
      m[ia] = isp[ia] ? 1.f : -s_col[buf][lane + 32 * ia];
    }
    // every row: a(i, c) -= f_i rp_c; the pivot row: rp_c (rp = scaled pivot row)
#pragma unroll
    for (int c = 0; c < CW; c++) {
      float src = a[0][c];
#pragma unroll
      for (int ia = 1; ia < MA; ia++) src = (pa == ia) ? a[ia][c] : src;
      const float rp = __shfl_sync(0xffffffffu, src, pl) * inv;
#pragma unroll
      for (int ia = 0; ia < MA; ia++) a[ia][c] = fmaf(m[ia], rp, isp[ia] ? 0.f : a[ia][c]);
    }
    if (w == ow) {
      // column j of the inverse: inv in the pivot row, -f_i inv elsewhere
      const int jj = j - CW * w;
#pragma unroll
      for (int ia = 0; ia < MA; ia++) {
        const float v = isp[ia] ? inv : m[ia] * inv;
#pragma unroll
        for (int c = 0; c < CW; c++) a[ia][c] = (c == jj) ? v : a[ia][c];
      }
    }
    if (own_next) column(jn, fcol);
  }
  __syncthreads();   // every step's pivots recorded
  if (!active) return;
  float* Xi = t.Xi;
#pragma unroll
  for (int ia = 0; ia < MA; ia++) {
    const int i = lane + 32 * ia;
    if (i >= r) continue;
    const int ri = s_spinv[i];
#pragma unroll
    for (int c = 0; c < CW; c++) {
      const int gc = CW * w + c;
      if (gc < r) Xi[ri + (size_t)r * s_spiv[gc]] = a[ia][c];
    }
  }
  if (info != 0 && lane == 0) atomicMax(err, (int)kDevSingular);
}

// ------------------------------------------------- multi-CTA dense helpers --
// C (m x n, ldc) = beta C + alpha op(A) op(B), op(A) m x kk: 64 x 64 output
// tiles, 16-deep shared-memory stages, 4 x 4 outputs per thread.
template <typename T>
__global__ void __launch_bounds__(256) k_gemm(int m, int n, int kk, T alpha, const T* A, int lda,
                                              int ta, const T* B, int ldb, int tb, T beta, T* C,
                                              int ldc, int kchunk, int64_t sA, int64_t sB,
                                              int64_t sC) {
  // split-K: slice z multiplies the k-range [z*kchunk, ...) into its own C
  const int z = blockIdx.z;
  A += z * sA;
  B += z * sB;
  C += z * sC;
  kk = min(kchunk, kk - z * kchunk);
  __shared__ T As[16][64 + 1];
  __shared__ T Bs[16][64 + 1];
  const int r0 = blockIdx.x * 64, c0 = blockIdx.y * 64;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) acc[a][b] = T(0);
  for (int l0 = 0; l0 < kk; l0 += 16) {
    for (int e = threadIdx.x; e < 16 * 64; e += blockDim.x) {
      int l = e % 16, i = e / 16;
      int gi = r0 + i, gl = l0 + l;
      T av = T(0);
      if (gi < m && gl < kk) av = ta ? A[gl + (size_t)lda * gi] : A[gi + (size_t)lda * gl];
      As[l][i] = av;
      int gj = c0 + i;
      T bv = T(0);
      if (gj < n && gl < kk) bv = tb ? B[gj + (size_t)ldb * gl] : B[gl + (size_t)ldb * gj];
      Bs[l][i] = bv;
    }
    __syncthreads();
#pragma unroll
    for (int l = 0; l < 16; l++) {
      T av[4], bv[4];
#pragma unroll
      for (int a = 0; a < 4; a++) av[a] = As[l][tx + 16 * a];
#pragma unroll
      for (int b = 0; b < 4; b++) bv[b] = Bs[l][ty + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] += av[a] * bv[b];
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) {
      int i = r0 + tx + 16 * a, j = c0 + ty + 16 * b;
      if (i < m && j < n) {
        T* c = C + i + (size_t)ldc * j;
        *c = (beta == T(0) ? T(0) : beta * *c) + alpha * acc[a][b];
      }
    }
}

template <typename T>
void gemm(cudaStream_t s, int m, int n, int kk, T alpha, const T* A, int lda, bool ta, const T* B,
          int ldb, bool tb, T beta, T* C, int ldc) {
  if (m <= 0 || n <= 0) return;
  dim3 g((m + 63) / 64, (n + 63) / 64);
  ki::launch(k_gemm<T>, g, 256, 0, s, m, n, kk, alpha, A, lda, ta, B, ldb, tb, beta, C, ldc,
                              std::max(kk, 1), 0, 0, 0);
}

// dst (rows x cols, ldd) = src block or its transpose (src rows/cols swapped)
template <typename T>
__global__ void k_copy_block(const T* src, int lds, int rows, int cols, int trans, T* dst, int ldd) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)rows * cols;
       e += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(e % rows), j = (int)(e / rows);
    dst[i + (size_t)ldd * j] = trans ? src[j + (size_t)lds * i] : src[i + (size_t)lds * j];
  }
}

template <typename T>
__global__ void k_perm_gather(const T* K, int n, const int* perm, T* P) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * n;
       e += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(e % n), j = (int)(e / n);
    P[e] = K[perm[i] + (size_t)n * perm[j]];
  }
}

template <typename T>
void copy_block(cudaStream_t s, const T* src, int lds, int rows, int cols, bool trans, T* dst, int ldd) {
  size_t ne = (size_t)rows * cols;
  if (ne == 0) return;
  ki::launch(k_copy_block<T>, (int)std::min<size_t>(2048, (ne + 255) / 256), 256, 0, s, src, lds, rows, cols,
                                                                              trans, dst, ldd);
}

// Shared-memory bytes of k_schur for a box: K_ss, T, K~_rs, K~_sr^T, X and r
// scratch entries, plus (inverse path) 4r more scratch, X's copy, U0 and L0.
template <typename T>
size_t schur_bytes(int n, int k, bool inv) {
  const size_t r = n - k, ld = (size_t)((n - k) | 1);   // k_schur's odd leading dimensions
  const size_t kt = (size_t)(k | 1);
  return sizeof(T) * ((size_t)k * k + kt * r + 2 * ld * k + ld * r + r +
                      (inv ? 4 * r + ld * r + ld * k + k * r : 0));
}

// Threads of a k_schur CTA when `per_sm` CTAs run per SM: 256 when four or
// more do (occupancy from CTAs), else enough to fill the SM's warps.
template <typename T>
int schur_threads(int per_sm) {
  if (kSchurMaxThreads<T> <= kThreads || per_sm >= 4) return kThreads;
  return per_sm == 3 ? 320 : (per_sm == 2 ? 512 : kSchurMaxThreads<T>);
}

// SkelFactorization::decouple for a box whose working set does not fit in one
// SM's shared memory: the same steps as k_schur as device-wide launches
// (tiled GEMMs, blocked LU and triangular solves) on stream st.
template <typename T>
void schur_wide(const SchurTask<T>& t, int* d_err, cudaStream_t st) {
  const int n = t.n, k = t.k, r = n - k;
  T* Pm = t.ws;
  T* Wrs = Pm + (size_t)n * n;
  T* Lt = Wrs + (size_t)r * k;
  T* X = t.X;
  const T* Tm = t.Tin;
  size_t ne = (size_t)n * n;
  ki::launch(k_perm_gather<T>, (int)std::min<size_t>(4096, (ne + 255) / 256), 256, 0, st, t.K, n, t.perm, Pm);
  KI_CUDA(cudaMemcpyAsync(t.Tout, t.Tin, sizeof(T) * (size_t)k * r, cudaMemcpyDeviceToDevice, st));
  const T* Kss = Pm;
  const T* Ksr = Pm + (size_t)n * k;
  copy_block<T>(st, Pm + k, n, r, k, false, Wrs, r);              // K_rs
  copy_block<T>(st, Ksr, n, r, k, true, Lt, r);                   // K_sr^T
  copy_block<T>(st, Pm + k + (size_t)n * k, n, r, r, false, X, r);  // K_rr
  gemm<T>(st, r, k, k, T(-1), Tm, k, true, Kss, n, false, T(1), Wrs, r);
  gemm<T>(st, r, k, k, T(-1), Tm, k, true, Kss, n, true, T(1), Lt, r);
  gemm<T>(st, r, r, k, T(-1), Tm, k, true, Ksr, n, false, T(1), X, r);
  gemm<T>(st, r, r, k, T(-1), Wrs, r, false, Tm, k, false, T(1), X, r);
  dense_lu<T>(X, r, t.piv, d_err, st);
  dense_lu_solve<T>(X, r, t.piv, Lt, r, k, true, st);              // L^T
  copy_block<T>(st, Kss, n, k, k, false, t.Atil, k);
  gemm<T>(st, k, k, r, T(-1), Lt, r, true, Wrs, r, false, T(1), t.Atil, k);
  dense_lu_solve<T>(X, r, t.piv, Wrs, r, k, false, st);            // U
  KI_CUDA(cudaMemcpyAsync(t.U, Wrs, sizeof(T) * (size_t)r * k, cudaMemcpyDeviceToDevice, st));
  copy_block<T>(st, Lt, r, k, r, true, t.L, k);                    // L = (L^T)^T
  KI_CUDA(cudaGetLastError());
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
  const T* Xi;   // r x r explicit inverse (FP32 factorizations, r <= kInvMax) or null
  int Xi_formed; // (host bookkeeping) Xi written by k_schur's Gauss-Jordan path
};

// Largest redundant block whose inverse is formed explicitly for the sweeps.
constexpr int kInvMax = 256;

enum SweepMode : int {
  kUpDiag = 0,     // x_r -= T^T x_s; x_s -= L x_r; x_r <- X^-1 x_r
  kUp = 1,         // without the diagonal solve
  kPsi = 2,        // x_r -= T^T x_s; x_s -= U^T x_r   (transposed down sweep)
  kDown = 3,       // x_r -= U x_s; x_s -= T x_r
  kDiag = 4,       // x_r <- X^-1 x_r
};

// Asynchronous global -> shared copy of one 4- or 8-byte element (cp.async,
// L1-allocating: the only form for copies under 16 bytes); completed by
// cp_async_wait_all, then a barrier makes the data visible to the CTA.
template <typename T>
__device__ __forceinline__ void cp_async_elem(T* dst, const T* src) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "4- or 8-byte elements");
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(tc::smem_u32(dst)), "l"(src),
               "n"((int)sizeof(T))
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

// x is DOF-major: row = DOF, ld = ldx; a CTA handles one box and a chunk of
// `cw` columns starting at blockIdx.y * cw.
// x_r <- X_rr^-1 x_r for one box's redundant rows (n x nc column-major block
// in shared memory, leading dimension n): with the explicit inverse one
// product (every thread an independent dot product, tmp: r x nc), else the
// LU substitution.
template <typename T>
__device__ void diag_solve(const SweepTask<T>& t, T* xr, int n, int nc, T* tmp,
                           const T* Xi = nullptr) {
  const int r = t.n - t.k;
  if (t.Xi) {
    if (!Xi) Xi = t.Xi;
    cta_for_2d(r, nc, [&](int i, int c) {
      T acc = T(0);
      for (int j = 0; j < r; j++) acc += Xi[i + (size_t)r * j] * xr[j + (size_t)n * c];
      tmp[i + (size_t)r * c] = acc;
    });
    __syncthreads();
    cta_for_2d(r, nc, [&](int i, int c) { xr[i + (size_t)n * c] = tmp[i + (size_t)r * c]; });
    __syncthreads();
  } else {
    cta_lu_solve_par<T>(r, t.X, r, t.piv, false, xr, n, nc);
  }
}

// A (n x n, column-major) = I.
template <typename T>
__global__ void k_set_identity(T* A, int n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * n;
       e += (size_t)gridDim.x * blockDim.x)
    A[e] = (e % n == e / n) ? T(1) : T(0);
}


template <typename T>
__global__ void k_sweep(const SweepTask<T>* tasks, T* x, int ldx, int ncols, int cw, int mode,
                        int stage_mats) {
  extern __shared__ unsigned char smem_raw[];
  T* sx = reinterpret_cast<T*>(smem_raw);
  const SweepTask<T> t = tasks[blockIdx.x];
  const int n = t.n, k = t.k, r = n - k;
  const int c0 = blockIdx.y * cw;
  const int nc = min(cw, ncols - c0);
  if (nc <= 0) return;
  // sx: n x nc column-major with an odd leading dimension (rows 0..k-1
  // skeleton, k..n-1 redundant); gathered and scattered a row of columns
  // per warp step (coalesced in x, conflict-free in sx).  With stage_mats
  // (uniform over the launch) each factor matrix is copied into shared
  // memory (after sx and the product temporary) before the phase that uses
  // it, so its entries are read from global memory once instead of once per
  // column.
  const int ld = n | 1;
  T* ms = sx + 2 * (size_t)ld * cw;
  // stage_mats 2: every factor matrix the mode uses is copied in up front,
  // together with the box's rows, by asynchronous copies that are all in
  // flight at once (one global-memory latency per box instead of one per
  // phase); stage_mats 1: one matrix at a time, before its phase
  const T* pre[3] = {nullptr, nullptr, nullptr};   // staged Tm / L-or-U / Xi
  if (stage_mats == 2) {
    cta_for_2d(nc, n, [&](int c, int i) {
      cp_async_elem(sx + i + (size_t)ld * c, x + (size_t)t.pact[i] * ldx + c0 + c);
    });
    const T* src[3] = {nullptr, nullptr, nullptr};
    int cnt[3] = {0, 0, 0};
    if (mode != kDiag) {
      src[0] = t.Tm;
      cnt[0] = k * r;
      src[1] = (mode == kPsi || mode == kDown) ? t.U : t.L;
      cnt[1] = k * r;
    }
    if ((mode == kUpDiag || mode == kDiag) && t.Xi) {
      src[2] = t.Xi;
      cnt[2] = r * r;
    }
    T* dst = ms;
    for (int q = 0; q < 3; q++) {
      if (!src[q]) continue;
      for (int e = threadIdx.x; e < cnt[q]; e += blockDim.x) cp_async_elem(dst + e, src[q] + e);
      pre[q] = dst;
      dst += cnt[q];
    }
    cp_async_wait_all();
  } else {
    cta_for_2d(nc, n, [&](int c, int i) {
      sx[i + (size_t)ld * c] = x[(size_t)t.pact[i] * ldx + c0 + c];
    });
  }
  __syncthreads();
  auto stage = [&](const T* g, int count, int q) -> const T* {
    if (stage_mats == 2) return pre[q];
    if (!stage_mats) return g;
    for (int e = threadIdx.x; e < count; e += blockDim.x) ms[e] = g[e];
    __syncthreads();
    return ms;
  };
  T* xs = sx;
  T* xr = sx + k;
  if (mode == kUpDiag || mode == kUp || mode == kPsi) {
    // x_r -= T^T x_s
    const T* Tm = stage(t.Tm, k * r, 0);
    cta_for_2d(r, nc, [&](int i, int c) {
      T acc = T(0);
      const T* tc = Tm + (size_t)k * i;
      for (int l = 0; l < k; l++) acc += tc[l] * xs[l + (size_t)ld * c];
      xr[i + (size_t)ld * c] -= acc;
    });
    __syncthreads();
    // x_s -= L x_r   or   x_s -= U^T x_r
    const T* M = stage(mode == kPsi ? t.U : t.L, k * r, 1);
    cta_for_2d(k, nc, [&](int l, int c) {
      T acc = T(0);
      if (mode == kPsi) {
        const T* uc = M + (size_t)r * l;
        for (int i = 0; i < r; i++) acc += uc[i] * xr[i + (size_t)ld * c];
      } else {
        for (int i = 0; i < r; i++) acc += M[l + (size_t)k * i] * xr[i + (size_t)ld * c];
      }
      xs[l + (size_t)ld * c] -= acc;
    });
    __syncthreads();
    if (mode == kUpDiag)
      diag_solve(t, xr, ld, nc, sx + (size_t)ld * nc, t.Xi ? stage(t.Xi, r * r, 2) : nullptr);
  } else if (mode == kDown) {
    // x_r -= U x_s
    const T* U = stage(t.U, r * k, 1);
    cta_for_2d(r, nc, [&](int i, int c) {
      T acc = T(0);
      for (int l = 0; l < k; l++) acc += U[i + (size_t)r * l] * xs[l + (size_t)ld * c];
      xr[i + (size_t)ld * c] -= acc;
    });
    __syncthreads();
    // x_s -= T x_r
    const T* Tm = stage(t.Tm, k * r, 0);
    cta_for_2d(k, nc, [&](int l, int c) {
      T acc = T(0);
      for (int i = 0; i < r; i++) acc += Tm[l + (size_t)k * i] * xr[i + (size_t)ld * c];
      xs[l + (size_t)ld * c] -= acc;
    });
    __syncthreads();
  } else if (mode == kDiag) {
    diag_solve(t, xr, ld, nc, sx + (size_t)ld * nc, t.Xi ? stage(t.Xi, r * r, 2) : nullptr);
  }
  __syncthreads();
  const int lo = mode == kDiag ? k : 0;   // the diagonal solve changes x_r only
  cta_for_2d(nc, n - lo, [&](int c, int ii) {
    const int i = lo + ii;
    x[(size_t)t.pact[i] * ldx + c0 + c] = sx[i + (size_t)ld * c];
  });
}

// ws (n x ncols, column-major) <-> rows idx of the DOF-major x
template <typename T>
__global__ void k_gather_rows(const T* x, int ldx, const int* idx, int n, int ncols, T* ws) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * ncols; e += gridDim.x * blockDim.x) {
    int i = e % n, c = e / n;
    ws[e] = x[(size_t)idx[i] * ldx + c];
  }
}

template <typename T>
__global__ void k_scatter_rows(T* x, int ldx, const int* idx, int n, int ncols, const T* ws) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * ncols; e += gridDim.x * blockDim.x) {
    int i = e % n, c = e / n;
    x[(size_t)idx[i] * ldx + c] = ws[e];
  }
}

// ------------------------------------------------------- bordered system --
// Border matrices of a multiply connected problem, DOF-major (row = DOF,
// nb columns): U (initialize_U_mat, kern_interp/linear_solve.cpp:19-107) and
// Psi^T (initialize_Psi_mat, :110-199, membership from node ranges).  Input
// coordinates are the interleaved FP64 arrays (dim per point).
template <typename T>
__global__ void k_border_init(const double* pts, const double* pw, int n_points, int dim,
                              int sol_dim, const double* hc, int nh, const int* hole_of, T* U,
                              T* PsiT) {
  const int c = border_cols_per_hole(dim, sol_dim);
  const int nb = c * nh;
  extern __shared__ float bi_smem[];
  float* s_ch = bi_smem;             // hole centres, FP32 high parts (FP32 Laplace path)
  float* s_cl = bi_smem + dim * nh;  // and low parts
  if (sol_dim == 1 && sizeof(T) < sizeof(double)) {
    for (int e = threadIdx.x; e < dim * nh; e += blockDim.x) {
      s_ch[e] = (float)hc[e];
      s_cl[e] = (float)(hc[e] - (double)s_ch[e]);
    }
    __syncthreads();
  }
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n_points; p += gridDim.x * blockDim.x) {
    const double* xp = pts + (size_t)dim * p;
    const int hp = hole_of[p];
    if (sol_dim == 1 && sizeof(T) < sizeof(double)) {
      // FP32 forms: offsets from hi/lo splits of the point and of the hole
      // centres (the latter formed once per CTA in shared memory), the log or
      // reciprocal in FP32
      float xh[3], xl[3];
      for (int d = 0; d < dim; d++) {
        xh[d] = (float)xp[d];
        xl[d] = (float)(xp[d] - (double)xh[d]);
      }
      for (int h = 0; h < nh; h++) {
        float r2 = 0.f;
        for (int d = 0; d < dim; d++) {
          const float dd = (xh[d] - s_ch[dim * h + d]) + (xl[d] - s_cl[dim * h + d]);
          r2 += dd * dd;
        }
        U[(size_t)p * nb + h] = T(dim == 2 ? 0.5f * logf(r2) : 1.f / sqrtf(r2));
        PsiT[(size_t)p * nb + h] = T(h == hp ? pw[p] : 0.0);
      }
    } else if (sol_dim == 1) {
      for (int h = 0; h < nh; h++) {
        double r2 = 0;
        for (int d = 0; d < dim; d++) r2 += (xp[d] - hc[dim * h + d]) * (xp[d] - hc[dim * h + d]);
        double rn = sqrt(r2);
        U[(size_t)p * nb + h] = T(dim == 2 ? log(rn) : 1.0 / rn);
        PsiT[(size_t)p * nb + h] = T(h == hp ? pw[p] : 0.0);
      }
    } else if (dim == 2) {
      const double x = xp[0], y = xp[1];
      T* u0 = U + (size_t)(2 * p) * nb;
      T* u1 = U + (size_t)(2 * p + 1) * nb;
      T* q0 = PsiT + (size_t)(2 * p) * nb;
      T* q1 = PsiT + (size_t)(2 * p + 1) * nb;
      for (int h = 0; h < nh; h++) {
        double rx = x - hc[2 * h], ry = y - hc[2 * h + 1];
        double rn = sqrt(rx * rx + ry * ry), r2 = rn * rn, sc = 1.0 / (4 * kPi);
        u0[3 * h] = T(sc * (log(1 / rn) + rx * rx / r2));
        u1[3 * h] = T(sc * (ry * rx / r2));
        u0[3 * h + 1] = T(sc * (rx * ry / r2));
        u1[3 * h + 1] = T(sc * (log(1 / rn) + ry * ry / r2));
        u0[3 * h + 2] = T(ry * (sc / r2));
        u1[3 * h + 2] = T(-rx * (sc / r2));
        double w = h == hp ? pw[p] : 0.0;
        q0[3 * h] = T(w);
        q1[3 * h] = T(0);
        q0[3 * h + 1] = T(0);
        q1[3 * h + 1] = T(w);
        q0[3 * h + 2] = T(w * y);
        q1[3 * h + 2] = T(-w * x);
      }
    } else {
      // 3D Stokes: Stokeslet (1/8pi)(delta/|r| + r_i r_j/|r|^3) in columns
      // 6h..6h+2, rotlet -(1/8pi|r|^3) [r]_x in 6h+3..6h+5 (linear_solve.cpp:49-76);
      // Psi: weights on the diagonal, -w [r]_x^T for the rotation rows
      // (r relative to the hole centre, :146-163)
      for (int h = 0; h < nh; h++) {
        const double r[3] = {xp[0] - hc[3 * h], xp[1] - hc[3 * h + 1], xp[2] - hc[3 * h + 2]};
        const double rn = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        const double rn3 = rn * rn * rn;
        const double rot = -1.0 / (8.0 * kPi * rn3);
        const double w = h == hp ? pw[p] : 0.0;
        for (int a = 0; a < 3; a++) {
          T* u = U + (size_t)(3 * p + a) * nb + 6 * h;
          T* q = PsiT + (size_t)(3 * p + a) * nb + 6 * h;
          for (int b = 0; b < 3; b++)
            u[b] = T((1.0 / (8.0 * kPi)) * ((a == b ? 1.0 : 0.0) / rn + r[a] * r[b] / rn3));
          for (int b = 0; b < 3; b++) q[b] = T(a == b ? w : 0.0);
        }
        T* u0 = U + (size_t)(3 * p) * nb + 6 * h;
        T* u1 = U + (size_t)(3 * p + 1) * nb + 6 * h;
        T* u2 = U + (size_t)(3 * p + 2) * nb + 6 * h;
        u0[3] = T(0);            u0[4] = T(rot * -r[2]); u0[5] = T(rot * r[1]);
        u1[3] = T(rot * r[2]);   u1[4] = T(0);           u1[5] = T(rot * -r[0]);
        u2[3] = T(rot * -r[1]);  u2[4] = T(rot * r[0]);  u2[5] = T(0);
        T* q0 = PsiT + (size_t)(3 * p) * nb + 6 * h;
        T* q1 = PsiT + (size_t)(3 * p + 1) * nb + 6 * h;
        T* q2 = PsiT + (size_t)(3 * p + 2) * nb + 6 * h;
        q0[3] = T(0);            q0[4] = T(-w * -r[2]);  q0[5] = T(-w * r[1]);
        q1[3] = T(-w * r[2]);    q1[4] = T(0);           q1[5] = T(-w * -r[0]);
        q2[3] = T(-w * -r[1]);   q2[4] = T(-w * r[0]);   q2[5] = T(0);
      }
    }
  }
}

// Diagonal entries of the 3D Nystrom matrices (Kernel::compute_diag_entries_
// 3dlaplace / _3dstokes, kern_interp/kernel/kernel.cpp:124-301): row sums of
// the off-diagonal kernel over the point's own surface (the outer surface
// [0, n_outer) or its hole's node range), then 1 - sum (Laplace) / I - sum
// (Stokes, every 3 x 3 block including the n_t n_s^T completion term) on the
// outer surface and -sum on holes.  FP64, one thread per target point,
// sources staged through shared memory; every thread adds its terms in
// source order.
constexpr int kDiagThreads = 128;
constexpr int kDiagTile = 256;

__global__ void __launch_bounds__(kDiagThreads) k_diag3(const double* pts, const double* nrm,
                                                        const double* w, int n_points,
                                                        const int* grp_lo, const int* grp_hi,
                                                        int n_outer, int sol_dim, double* out) {
  __shared__ double s[7][kDiagTile];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const bool on = t < n_points;
  const int tc = on ? t : n_points - 1;
  const int lo = grp_lo[tc], hi = grp_hi[tc];
  // source range of the block: union of its targets' ranges
  const int t0 = blockIdx.x * blockDim.x, t1 = min(n_points, t0 + (int)blockDim.x) - 1;
  const int blo = grp_lo[t0], bhi = max(grp_hi[t0], grp_hi[t1]);
  const double tx = pts[3 * (size_t)tc], ty = pts[3 * (size_t)tc + 1], tz = pts[3 * (size_t)tc + 2];
  const double tn[3] = {nrm[3 * (size_t)tc], nrm[3 * (size_t)tc + 1], nrm[3 * (size_t)tc + 2]};
  double acc[9];
  for (int q = 0; q < 9; q++) acc[q] = 0.0;
  for (int base = blo; base < bhi; base += kDiagTile) {
    __syncthreads();
    for (int i = threadIdx.x; i < kDiagTile; i += blockDim.x) {
      int p = base + i;
      if (p < bhi) {
        s[0][i] = pts[3 * (size_t)p]; s[1][i] = pts[3 * (size_t)p + 1]; s[2][i] = pts[3 * (size_t)p + 2];
        s[3][i] = nrm[3 * (size_t)p]; s[4][i] = nrm[3 * (size_t)p + 1]; s[5][i] = nrm[3 * (size_t)p + 2];
        s[6][i] = w[p];
      }
    }
    __syncthreads();
    const int i0 = max(0, lo - base), i1 = min(kDiagTile, hi - base);
    for (int i = i0; i < i1; i++) {
      if (base + i == t) continue;
      const double r1 = tx - s[0][i], r2 = ty - s[1][i], r3 = tz - s[2][i];
      const double rr = r1 * r1 + r2 * r2 + r3 * r3;
      const double rn = r1 * s[3][i] + r2 * s[4][i] + r3 * s[5][i];
      const double sw = s[6][i];
      if (sol_dim == 1) {
        acc[0] += -sw * (1.0 / (4 * kPi)) * rn / (rr * sqrt(rr));
      } else {
        const double r[3] = {r1, r2, r3};
        const double sn[3] = {s[3][i], s[4][i], s[5][i]};
        const double f = sw * (-3.0 / (4.0 * kPi)) * rn / (rr * rr * sqrt(rr));
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
          for (int b = 0; b < 3; b++) acc[3 * a + b] += f * r[a] * r[b] + sw * tn[a] * sn[b];
      }
    }
  }
  if (!on) return;
  const double one = t < n_outer ? 1.0 : 0.0;
  if (sol_dim == 1) {
    out[t] = one - acc[0];
  } else {
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) out[9 * (size_t)t + 3 * a + b] = (a == b ? one : 0.0) - acc[3 * a + b];
  }
}

// The 3D Laplace row sums of k_diag3 in FP32-pair arithmetic (the pair term
// of ki::pair_dipole3, ~1e-13 relative each; the FP32 pipes run at 64 x the
// FP64 rate on this part).  blockIdx.y takes the sources of one chunk of
// `chunk_pts` indices; each target's partial sum goes to part[y][t], and
// k_diag3_finish adds the chunks in order.  A source that coincides with the
// target is skipped.
__global__ void __launch_bounds__(kDiagThreads) k_diag3_pair(const double* pts, const double* nrm,
                                                             const double* w, int n_points,
                                                             const int* grp_lo, const int* grp_hi,
                                                             int chunk_pts, double* part) {
  __shared__ float4 s_ph[kDiagTile], s_pl[kDiagTile], s_nh[kDiagTile], s_nl[kDiagTile];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const bool on = t < n_points;
  const int tc = on ? t : n_points - 1;
  const int z0 = blockIdx.y * chunk_pts, z1 = min(n_points, z0 + chunk_pts);
  const int lo = max(grp_lo[tc], z0), hi = min(grp_hi[tc], z1);
  const int t0 = blockIdx.x * blockDim.x, t1 = min(n_points, t0 + (int)blockDim.x) - 1;
  const int blo = max(grp_lo[t0], z0), bhi = min(max(grp_hi[t0], grp_hi[t1]), z1);
  const float2 tx = split_pair(pts[3 * (size_t)tc]), ty = split_pair(pts[3 * (size_t)tc + 1]),
               tz = split_pair(pts[3 * (size_t)tc + 2]);
  constexpr double kC = -1.0 / (4.0 * kPi);
  float ah = 0.f, al = 0.f;
  for (int base = blo; base < bhi; base += kDiagTile) {
    __syncthreads();
    for (int i = threadIdx.x; i < kDiagTile; i += blockDim.x) {
      const int p = base + i;
      if (p < bhi) {
        const float2 a = split_pair(pts[3 * (size_t)p]), b = split_pair(pts[3 * (size_t)p + 1]),
                     c = split_pair(pts[3 * (size_t)p + 2]);
        s_ph[i] = make_float4(a.x, b.x, c.x, 0.f);
        s_pl[i] = make_float4(a.y, b.y, c.y, 0.f);
        const double cw = kC * w[p];
        const float2 u = split_pair(cw * nrm[3 * (size_t)p]),
                     v = split_pair(cw * nrm[3 * (size_t)p + 1]),
                     q = split_pair(cw * nrm[3 * (size_t)p + 2]);
        s_nh[i] = make_float4(u.x, v.x, q.x, 0.f);
        s_nl[i] = make_float4(u.y, v.y, q.y, 0.f);
      }
    }
    __syncthreads();
    const int i0 = max(0, lo - base), i1 = min(kDiagTile, hi - base);
    for (int i = i0; i < i1; i++) {
      if (base + i == t) continue;
      float kh, kl;
      if (!pair_dipole3(tx, ty, tz, s_ph[i], s_pl[i], s_nh[i], s_nl[i], kh, kl)) continue;
      float sh, sl;
      two_sum(ah, kh, sh, sl);
      al = __fadd_rn(al, __fadd_rn(sl, kl));
      ah = sh;
    }
  }
  if (on) part[(size_t)blockIdx.y * n_points + t] = (double)ah + (double)al;
}

// out[t] = (1 on the outer surface, 0 on holes) - the chunks' row sums, added in order.
__global__ void k_diag3_finish(const double* part, int nchunks, int n_points, int n_outer,
                               double* out) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n_points; t += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int z = 0; z < nchunks; z++) acc += part[(size_t)z * n_points + t];
    out[t] = (t < n_outer ? 1.0 : 0.0) - acc;
  }
}

template <typename T>
__global__ void k_convert(const double* a, size_t n, T* b) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = T(a[i]);
}

__global__ void k_mark(const int* idx, int n, unsigned char* mask) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) mask[idx[i]] = 1;
}

// Partial sums over row chunks of  out(a, c) = sum_{i not skeleton} A(i, a) B(i, c)
// (A: N x na, B: N x nc, both DOF-major); deterministic two-stage reduction.
constexpr int kRedRows = 1024;
template <typename T>
__global__ void k_reduce_partial(const T* A, int na, const T* B, int nc, int N,
                                 const unsigned char* mask, T* partial) {
  extern __shared__ unsigned char red_smem[];
  T* As = reinterpret_cast<T*>(red_smem);           // 32 x na
  T* Bs = As + 32 * (size_t)na;                      // 32 x nc
  const int r0 = blockIdx.x * kRedRows;
  const int r1 = min(N, r0 + kRedRows);
  const int nout = na * nc;
  T acc[16];
  for (int q = 0; q < 16; q++) acc[q] = T(0);
  for (int t0 = r0; t0 < r1; t0 += 32) {
    __syncthreads();
    for (int e = threadIdx.x; e < 32 * na; e += blockDim.x) {
      int i = t0 + e / na;
      As[e] = (i < r1 && !mask[i]) ? A[(size_t)i * na + e % na] : T(0);
    }
    for (int e = threadIdx.x; e < 32 * nc; e += blockDim.x) {
      int i = t0 + e / nc;
      Bs[e] = i < r1 ? B[(size_t)i * nc + e % nc] : T(0);
    }
    __syncthreads();
    for (int q = 0; q < 16; q++) {
      int o = threadIdx.x + q * blockDim.x;
      if (o >= nout) break;
      int a = o % na, c = o / na;
      T sum = T(0);
      for (int i = 0; i < 32; i++) sum += As[i * na + a] * Bs[i * nc + c];
      acc[q] += sum;
    }
  }
  T* out = partial + (size_t)blockIdx.x * nout;
  for (int q = 0; q < 16; q++) {
    int o = threadIdx.x + q * blockDim.x;
    if (o >= nout) break;
    out[o] = acc[q];
  }
}

// The same partial sums register-tiled: each thread owns up to two 4 x 2
// output tiles (a, c), so a row of the staged operands costs 6 shared-memory
// loads per 8 FMAs instead of 16.  Operands padded to multiples of 4 (A) and
// 2 (B) columns with zeros; used when ceil(na/4) ceil(nc/2) <= 2 blockDim.
template <typename T>
__global__ void __launch_bounds__(256) k_reduce_tiled(const T* A, int na, const T* B, int nc, int N,
                                                      const unsigned char* mask, T* partial) {
  extern __shared__ unsigned char red_smem[];
  const int lda = (na + 3) & ~3, ldb = (nc + 1) & ~1;
  T* As = reinterpret_cast<T*>(red_smem);   // 32 x lda
  T* Bs = As + 32 * (size_t)lda;            // 32 x ldb
  const int nga = lda / 4, ntile = nga * (ldb / 2);
  const int r0 = blockIdx.x * kRedRows;
  const int r1 = min(N, r0 + kRedRows);
  T acc[2][4][2];
  for (int q = 0; q < 2; q++)
    for (int u = 0; u < 4; u++) acc[q][u][0] = acc[q][u][1] = T(0);
  for (int t0 = r0; t0 < r1; t0 += 32) {
    __syncthreads();
    for (int e = threadIdx.x; e < 32 * lda; e += blockDim.x) {
      const int i = t0 + e / lda, a = e % lda;
      As[e] = (i < r1 && a < na && !mask[i]) ? A[(size_t)i * na + a] : T(0);
    }
    for (int e = threadIdx.x; e < 32 * ldb; e += blockDim.x) {
      const int i = t0 + e / ldb, c = e % ldb;
      Bs[e] = (i < r1 && c < nc) ? B[(size_t)i * nc + c] : T(0);
    }
    __syncthreads();
    for (int q = 0; q < 2; q++) {
      const int tile = threadIdx.x + q * blockDim.x;
      if (tile >= ntile) break;
      const int a0 = 4 * (tile % nga), c0 = 2 * (tile / nga);
      for (int i = 0; i < 32; i++) {
        const T* ar = As + i * lda + a0;
        const T b0 = Bs[i * ldb + c0], b1 = Bs[i * ldb + c0 + 1];
        for (int u = 0; u < 4; u++) {
          acc[q][u][0] += ar[u] * b0;
          acc[q][u][1] += ar[u] * b1;
        }
      }
    }
  }
  T* out = partial + (size_t)blockIdx.x * na * nc;
  for (int q = 0; q < 2; q++) {
    const int tile = threadIdx.x + q * blockDim.x;
    if (tile >= ntile) break;
    const int a0 = 4 * (tile % nga), c0 = 2 * (tile / nga);
    for (int u = 0; u < 4; u++)
      for (int v = 0; v < 2; v++)
        if (a0 + u < na && c0 + v < nc) out[(a0 + u) + (size_t)na * (c0 + v)] = acc[q][u][v];
  }
}

template <typename T>
__global__ void k_reduce_final(const T* partial, int nparts, int nout, T* out) {
  for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < nout; o += gridDim.x * blockDim.x) {
    T acc = T(0);
    for (int p = 0; p < nparts; p++) acc += partial[(size_t)p * nout + o];
    out[o] = acc;
  }
}

// Bordered root system S = [A_root, U~_s; Psi~_s, -I - Psi~_r D^-1 U~_r]
// (skel_factorization.cpp:524-542).
template <typename T>
__global__ void k_assemble_S(const T* A, int nr, const int* idx, const T* Um, const T* PsiTm,
                             const T* corr, int nb, T* S) {
  const int ns = nr + nb;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)ns * ns;
       e += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(e % ns), j = (int)(e / ns);
    T v;
    if (i < nr && j < nr) v = A[i + (size_t)nr * j];
    else if (i >= nr && j < nr) v = PsiTm[(size_t)idx[j] * nb + (i - nr)];
    else if (i < nr && j >= nr) v = Um[(size_t)idx[i] * nb + (j - nr)];
    else v = -(i == j ? T(1) : T(0)) - corr[(i - nr) + (size_t)nb * (j - nr)];
    S[e] = v;
  }
}

// M = [x(allskel, :); -t]  ((nr + nb) x nc, column-major)
template <typename T>
__global__ void k_mc_rhs(const T* x, int ldx, const int* idx, int nr, const T* t, int nb, int nc,
                         T* M, const T* g = nullptr) {
  // g: right-hand side of the border rows (Psi mu - alpha = g), row-major
  // nb x nc; absent for the reference's problem (g = 0)
  const int ns = nr + nb;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ns * nc; e += gridDim.x * blockDim.x) {
    int i = e % ns, c = e / ns;
    M[e] = i < nr ? x[(size_t)idx[i] * ldx + c]
                  : (g ? g[(size_t)(i - nr) * nc + c] : T(0)) - t[(i - nr) + (size_t)nb * c];
  }
}

// The redundant rows of the bordered solve's result, D^-1 (w - U~ alpha)
// formed as D^-1 w - (D^-1 U~) alpha (D^-1 is block diagonal on the
// redundant rows, so the two agree; the second form needs no second pass of
// diagonal solves): x(i, :) = Dw(i, :) - DU(i, :) alpha on the rows whose
// mask is clear (DU: N x nb row-major, nb <= 64; alpha = rows nr.. of M,
// ns x nc column-major).  Lanes are columns (blockIdx.y: a 32-column chunk);
// a warp takes one row at a time, its DU row loaded by the lanes and
// broadcast by shuffles; alpha staged in shared memory; each CTA owns a
// contiguous range of rows.
template <typename T>
__global__ void __launch_bounds__(256) k_mc_final(T* x, int nc, const T* Dw, const T* DU, int nb,
                                                  const T* M, int nr, int N,
                                                  const unsigned char* mask) {
  __shared__ T A[64 * 32];
  const int ns = nr + nb;
  const int c0 = blockIdx.y * 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int c = c0 + lane;
  const int per = (N + gridDim.x - 1) / gridDim.x;
  const int i0 = blockIdx.x * per, i1 = min(N, i0 + per);
  for (int e = threadIdx.x; e < 64 * 32; e += blockDim.x) {
    const int b = e / 32, cc = e % 32;
    A[e] = (b < nb && c0 + cc < nc) ? M[nr + b + (size_t)ns * (c0 + cc)] : T(0);
  }
  __syncthreads();
  for (int i = i0 + warp; i < i1; i += nw) {
    if (mask[i]) continue;
    const T* u = DU + (size_t)i * nb;
    const T u0 = lane < nb ? u[lane] : T(0);
    const T u1 = 32 + lane < nb ? u[32 + lane] : T(0);
    T acc = T(0);
    for (int b = 0; b < min(nb, 32); b++) acc += __shfl_sync(0xffffffffu, u0, b) * A[b * 32 + lane];
    for (int b = 32; b < nb; b++) acc += __shfl_sync(0xffffffffu, u1, b - 32) * A[b * 32 + lane];
    if (c < nc) x[(size_t)i * nc + c] = Dw[(size_t)i * nc + c] - acc;
  }
}

template <typename T>
void mc_final(T* x, int nc, const T* Dw, const T* DU, int nb, const T* M, int nr, int N,
              const unsigned char* mask, cudaStream_t s) {
  if (N <= 0 || nc <= 0 || nb <= 0) return;
  dim3 g((unsigned)std::max(1, std::min(4096, (N + 255) / 256)), (unsigned)((nc + 31) / 32));
  ki::launch(k_mc_final<T>, g, 256, 0, s, x, nc, Dw, DU, nb, M, nr, N, mask);
}

// x(allskel, :) = M(0:nr, :), alpha (row-major nb x nc) = M(nr:, :)
template <typename T>
__global__ void k_mc_finish(T* x, int nc, const int* idx, const T* M, int nr, int nb, T* alpha) {
  const int ns = nr + nb;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ns * nc; e += gridDim.x * blockDim.x) {
    int i = e % ns, c = e / ns;
    if (i < nr) x[(size_t)idx[i] * nc + c] = M[e];
    else if (alpha) alpha[(size_t)(i - nr) * nc + c] = M[e];
  }
}

// Interleaved FP64 input (dim per point) -> structure-of-arrays in the
// factor precision.
template <typename T>
__global__ void k_fill_points(const double* pts, const double* nrm, const double* w,
                              const double* kap, int n, int dim, T* x, T* y, T* z, T* nx, T* ny,
                              T* nz, T* ww, T* kk, T* lo) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] = T(pts[(size_t)dim * i]);
    y[i] = T(pts[(size_t)dim * i + 1]);
    if (lo) {   // x = x_hi + x_lo
      lo[i] = T(pts[(size_t)dim * i] - (double)x[i]);
      lo[n + i] = T(pts[(size_t)dim * i + 1] - (double)y[i]);
      if (dim == 3) lo[2 * (size_t)n + i] = T(pts[3 * (size_t)i + 2] - (double)T(pts[3 * (size_t)i + 2]));
    }
    nx[i] = T(nrm[(size_t)dim * i]);
    ny[i] = T(nrm[(size_t)dim * i + 1]);
    if (dim == 3) {
      z[i] = T(pts[3 * (size_t)i + 2]);
      nz[i] = T(nrm[3 * (size_t)i + 2]);
    }
    ww[i] = T(w[i]);
    kk[i] = kap ? T(kap[i]) : T(0);
  }
}

template <typename T>
void upload(T* dst, const std::vector<T>& v, cudaStream_t s) {
  if (!v.empty())
    KI_CUDA(cudaMemcpyAsync(dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s));
}

// Gauss-Legendre rule with n nodes on [a, b], ascending: Newton iteration on
// the three-term recurrence of P_n from the Chebyshev-like initial guesses
// cos(pi (i + 3/4) / (n + 1/2)).  (The reference calls the LGPL routine cgqf
// for its proxy-sphere latitudes, kern_interp/kernel/kernel.h:48-54.)
void gauss_legendre(int n, double a, double b, std::vector<double>* x, std::vector<double>* w) {
  x->assign(n, 0.0);
  w->assign(n, 0.0);
  for (int i = 0; i < n; i++) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; k++) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) { p1 = z; p0 = 1.0; }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    // recompute the derivative at the converged node
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= n; k++) {
      double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    dp = n == 1 ? 1.0 : n * (z * p1 - p0) / (z * z - 1.0);
    // node i of the descending order -> index n-1-i of the ascending one
    (*x)[n - 1 - i] = 0.5 * (b - a) * z + 0.5 * (b + a);
    (*w)[n - 1 - i] = (b - a) / ((1.0 - z * z) * dp * dp);
  }
}

// Latitude count of a 3D proxy sphere of P = 2 q^2 points (theta x phi grid
// with twice as many longitudes as latitudes, the reference's 8 x 4 = 32).
int proxy_phi_count(int P) {
  int q = (int)std::lround(std::sqrt(P / 2.0));
  if (q < 1 || 2 * q * q != P)
    throw std::invalid_argument("3D num_proxy_points must be 2 q^2 (8, 32, 72, 128, ..., 512)");
  return q;
}

struct HostBox {
  int n = 0;           // active DOFs
  int k = 0;           // rank if compressed
  bool compressed = false;
  int64_t act = 0;     // ipool offset of the active list
  int64_t pact = 0;    // ipool offset of the permuted list (compressed)
  const void* tile = nullptr;  // accumulated self-block on the device
};

// ------------------------------------------------ re-factorization support --
// The per-point arrays two factorizations compare: `per` values per point in
// each (the 3D diagonal has 1 or 9).
template <typename T>
struct PointArrays {
  static constexpr int kMax = 12;
  const T* a[kMax];
  const T* b[kMax];
  int per[kMax];
  int count;
};

// changed[p] = 1 when any listed array differs bitwise at point p.
template <typename T>
__global__ void k_points_changed(PointArrays<T> pa, int n, unsigned char* changed) {
  using W = typename std::conditional<sizeof(T) == 8, unsigned long long, unsigned int>::type;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    bool d = false;
    for (int q = 0; q < pa.count; q++)
      for (int e = 0; e < pa.per[q]; e++) {
        const size_t i = (size_t)p * pa.per[q] + e;
        d = d || reinterpret_cast<const W*>(pa.a[q])[i] != reinterpret_cast<const W*>(pa.b[q])[i];
      }
    changed[p] = d;
  }
}

// One device-to-device copy of `words` 4-byte words.
struct CopySeg {
  const void* src;
  void* dst;
  int64_t words;
};

// One CTA per segment.
__global__ void k_copy_segments(const CopySeg* segs) {
  const CopySeg sg = segs[blockIdx.x];
  const uint32_t* a = static_cast<const uint32_t*>(sg.src);
  uint32_t* d = static_cast<uint32_t*>(sg.dst);
  for (int64_t i = threadIdx.x; i < sg.words; i += blockDim.x) d[i] = a[i];
}

bool same_params(const Params& a, const Params& b) {
  return a.dim == b.dim && a.sol_dim == b.sol_dim && a.max_leaf_dofs == b.max_leaf_dofs &&
         a.num_proxy_points == b.num_proxy_points && a.radius_ratio == b.radius_ratio &&
         a.min_dofs_to_compress == b.min_dofs_to_compress && a.id_tol == b.id_tol &&
         a.pde == b.pde &&
         (a.rank_model != nullptr) == (b.rank_model != nullptr) &&
         a.sketch_margin == b.sketch_margin && a.sketch_oversample == b.sketch_oversample;
}

// Boxes of `tree` (the perturbed boundary's) whose ID and Schur elimination
// would see exactly the inputs they saw in `prev`, so that prev's factors
// serve unchanged: per box, prev's box to copy from, or -1.  The reference
// marks the boxes to recompute from the changed leaves up (every ancestor,
// and each marked box's same-level or finer neighbours:
// QuadTree::mark_neighbors_and_parents, kern_interp/quadtree/quadtree.cpp:
// 483-497); here the rule is stated per box from what its factors read.
//  - Boxes correspond by position: the roots when their centres and sides
//    are equal, then child for child while both are split.
//  - A leaf is unchanged when prev's box is a leaf with the same DOF list and
//    none of its points' data changed (changed[p]).
//  - A box's active list (and the self block assembled from its children)
//    is unchanged when it is an unchanged leaf, or it is split in both trees
//    and every child passes up the same list and block: a child that was
//    reused, or one too small to compress (fewer than min_dofs DOFs) whose
//    own active list is unchanged.
//  - Its ID's rows are the proxy surface and the near field, the active DOFs
//    of the same-level neighbours and the DOFs of the touching coarser leaves
//    (Kernel::get_id_mat, kernel/kernel.cpp:441-563): unchanged when both
//    neighbour lists correspond one to one and every neighbour's DOFs are
//    unchanged.  Levels whose ID reads every box of the level (1, and 2 in
//    2D) are always recomputed.
template <typename T>
std::vector<int> plan_reuse(const Factorization<T>& prev, const Tree& tree,
                            const std::vector<unsigned char>& changed, int min_dofs) {
  const Tree& ot = prev.tree;
  const int nb = (int)tree.boxes.size(), dim = tree.dim, sd = tree.sol_dim;
  std::vector<int> out(nb, -1);
  if (ot.dim != dim || ot.sol_dim != sd || ot.n_dofs != tree.n_dofs || ot.levels.empty() ||
      tree.levels.empty() || prev.box_factors.size() != ot.boxes.size())
    return out;
  std::vector<int> old_of(nb, -1);
  {
    const Box& r = tree.boxes[tree.levels[0][0]];
    const Box& o = ot.boxes[ot.levels[0][0]];
    if (r.side == o.side && r.c[0] == o.c[0] && r.c[1] == o.c[1] && r.c[2] == o.c[2])
      old_of[tree.levels[0][0]] = ot.levels[0][0];
  }
  const int nch = tree.n_children();
  for (const auto& lv : tree.levels)
    for (int b : lv) {
      const int ob = old_of[b];
      if (ob < 0 || tree.boxes[b].leaf || ot.boxes[ob].leaf) continue;
      for (int ci = 0; ci < nch; ci++) old_of[tree.boxes[b].child[ci]] = ot.boxes[ob].child[ci];
    }
  std::vector<char> leaf_same(nb, 0), act_same(nb, 0), out_same(nb, 0);
  for (int b = 0; b < nb; b++) {
    const Box& bx = tree.boxes[b];
    const int ob = old_of[b];
    if (!bx.leaf || ob < 0 || !ot.boxes[ob].leaf || ot.boxes[ob].orig_count != bx.orig_count) continue;
    bool s = true;
    for (int i = 0; i < bx.orig_count && s; i++) {
      const int d = tree.dof_sorted[bx.orig_start + i];
      s = d == ot.dof_sorted[ot.boxes[ob].orig_start + i] && !changed[d / sd];
    }
    leaf_same[b] = s;
  }
  // neighbour lists that correspond one to one (as sets of prev's boxes)
  auto same_list = [&](IdList a, IdList o) {
    if (a.size() != o.size()) return false;
    std::vector<int> x, y(o.begin(), o.end());
    for (int q : a) {
      if (old_of[q] < 0) return false;
      x.push_back(old_of[q]);
    }
    std::sort(x.begin(), x.end());
    std::sort(y.begin(), y.end());
    return x == y;
  };
  for (int l = tree.num_levels() - 1; l >= 1; l--) {
    for (int b : tree.levels[l]) {
      const Box& bx = tree.boxes[b];
      const int ob = old_of[b];
      if (ob < 0 || ot.boxes[ob].leaf != bx.leaf) continue;
      bool s = bx.leaf ? (bool)leaf_same[b] : true;
      if (!bx.leaf)
        for (int ci = 0; ci < nch; ci++) s = s && out_same[bx.child[ci]];
      act_same[b] = s;
    }
    const bool proxy_level = !(l == 1 || (l == 2 && dim == 2));
    for (int b : tree.levels[l]) {
      if (!act_same[b]) continue;
      const int ob = old_of[b];
      const bool id_box = prev.box_factors[ob].n >= min_dofs;   // went through an ID
      bool near = proxy_level && same_list(tree.coarse_nbrs(b), ot.coarse_nbrs(ob)) &&
                  same_list(tree.same_nbrs(b), ot.same_nbrs(ob));
      if (near) {
        for (int o : tree.coarse_nbrs(b)) near = near && leaf_same[o];
        for (int o : tree.same_nbrs(b))
          near = near && (tree.boxes[o].leaf ? leaf_same[o] : act_same[o]);
      }
      if (id_box && near) out[b] = ob;
      out_same[b] = !id_box || out[b] >= 0;
    }
  }
  return out;
}

}  // namespace

// Threads of a k_sweep launch: the autotuner's choice for the bucket, else
// kThreads.
inline int sweep_threads(int bucket) {
  const int ch = tune_choice(kTuneSweep, bucket);
  return ch < 0 ? kThreads : (ch == 0 ? 128 : (ch == 1 ? 256 : 512));
}

// Shared-memory bytes k_sweep needs to stage a factor matrix of `entries`
// entries (the largest of r^2 and k r over the launch's boxes), and the
// largest dynamic shared memory a staged sweep may use.
template <typename T>
size_t sweep_stage_bytes(int entries) {
  return sizeof(T) * (size_t)entries;
}
constexpr size_t kSweepStageCap = 96 * 1024;

// The diagonal solves x_r <- X^-1 x_r of every level's boxes: one launch per
// bin of the all-levels descriptor array.
template <typename T>
void launch_diag_all(Factorization<T>& F, T* x, int ncols, cudaStream_t s) {
  if (!F.d_all_tasks || ncols == 0) return;
  const SweepTask<T>* all = reinterpret_cast<const SweepTask<T>*>(F.d_all_tasks);
  // the bins are independent: on the aux streams when the caller's stream is
  // the factorization's (their fork / join order against it)
  const bool par = s == F.stream && F.diag_bins.size() > 1;
  if (par) F.fork();
  int next = 0;
  for (const auto& b : F.diag_bins) {
    cudaStream_t st = par ? F.aux[(next++) % Factorization<T>::kAux] : s;
    const int ldmax = std::max(1, b[2]) | 1;
    int cw = std::max(1, std::min(ncols, (int)(96 * 1024 / (2 * sizeof(T) * ldmax))));
    cw = std::min(cw, 32);
    dim3 grid(b[1], (ncols + cw - 1) / cw);
    size_t sm = 2 * sizeof(T) * (size_t)ldmax * cw;
    if (sm > 200 * 1024) throw std::runtime_error("box too large for the sweep kernel");
    // kDiag stages X^-1 alone (b[3]: the largest r^2), all at once
    const size_t mats = sweep_stage_bytes<T>(b[3]);
    const int staged = sm + mats <= kSweepStageCap ? 2 : 0;
    if (staged) sm += mats;
    if (sm > 48 * 1024)
      KI_CUDA(cudaFuncSetAttribute(k_sweep<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    const int bucket = sweep_bucket(sizeof(T) == 8, b[2]);
    const bool rec = tune_recording();
    if (rec) F.stage_begin(tune_stage(kTuneSweep, bucket).c_str(), 0, 0, st);
    ki::launch(k_sweep<T>, grid, sweep_threads(bucket), sm, st, all + b[0], x, ncols, ncols, cw, kDiag,
               staged);
    if (rec) F.stage_end(st);
    KI_CUDA(cudaGetLastError());
  }
  if (par) F.join(std::min(next, Factorization<T>::kAux));
}

template <typename T>
void launch_sweep(Factorization<T>& F, int l, int mode, T* x, int ncols, cudaStream_t s) {
  LevelFactor& LF = F.levels[l];
  if (LF.n_comp == 0 || ncols == 0) return;
  // shared memory: the box's rows (n x cw) and the inverse product's
  // temporary (r x cw <= n x cw)
  const int ldmax = std::max(1, LF.max_n) | 1;   // k_sweep's odd leading dimension
  int cw = std::max(1, std::min(ncols, (int)(96 * 1024 / (2 * sizeof(T) * ldmax))));
  cw = std::min(cw, 32);
  dim3 grid(LF.n_comp, (ncols + cw - 1) / cw);
  size_t sm = 2 * sizeof(T) * (size_t)ldmax * cw;
  if (sm > 200 * 1024) throw std::runtime_error("box too large for the sweep kernel");
  const size_t all = sweep_stage_bytes<T>(LF.max_all);
  const size_t mats = sweep_stage_bytes<T>(LF.max_mat);
  const int staged = sm + all <= kSweepStageCap ? 2 : (sm + mats <= kSweepStageCap ? 1 : 0);
  if (staged) sm += staged == 2 ? all : mats;
  if (sm > 48 * 1024)
    KI_CUDA(cudaFuncSetAttribute(k_sweep<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  const int bucket = sweep_bucket(sizeof(T) == 8, LF.max_n);
  const bool rec = tune_recording();
  if (rec) F.stage_begin(tune_stage(kTuneSweep, bucket).c_str(), 0, 0, s);
  ki::launch(k_sweep<T>, grid, sweep_threads(bucket), sm, s, reinterpret_cast<SweepTask<T>*>(LF.d_tasks),
             x, ncols, ncols, cw, mode, staged);
  if (rec) F.stage_end(s);
  KI_CUDA(cudaGetLastError());
}

// Temporaries of one solve (or of the border set-up): taken from the
// library's stream-ordered pool and released, in stream order, when the
// Scratch goes out of scope; or carved from a caller's arena (the
// no-allocation solve), which releases nothing.
template <typename T>
class Scratch {
 public:
  explicit Scratch(cudaStream_t s, ScratchArena* arena = nullptr) : s_(s), arena_(arena) {}
  Scratch(const Scratch&) = delete;
  Scratch& operator=(const Scratch&) = delete;
  ~Scratch() {
    for (void* p : owned_) cudaFreeAsync(p, s_);
  }
  // Bytes one take(elems) consumes at most, alignment included.
  static size_t footprint(size_t elems) { return ((bytes(elems) + 255) & ~size_t(255)) + 256; }
  T* take(size_t elems) {
    if (arena_) {
      void* p = arena_->take(bytes(elems));
      if (!p) throw std::invalid_argument("scratch arena too small for this solve");
      return static_cast<T*>(p);
    }
    void* p = nullptr;
    KI_CUDA(pool_malloc(&p, bytes(elems), s_));
    owned_.push_back(p);
    return static_cast<T*>(p);
  }

 private:
  static size_t bytes(size_t elems) { return sizeof(T) * elems + 16; }
  cudaStream_t s_;
  ScratchArena* arena_;
  std::vector<void*> owned_;
};

// Rows of a DOF-major N x nc array whose flag is set are zeroed.
template <typename T>
__global__ void k_zero_rows(T* X, int nc, const unsigned char* mask, int N) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)N * nc;
       e += (size_t)gridDim.x * blockDim.x)
    if (mask[e / nc]) X[e] = T(0);
}

// k_reduce_partial stages 32 rows of both operands in shared memory and
// keeps na x nc accumulators per block: borders up to 4,096 products use
// it, wider ones the split-K GEMM.
constexpr int kRedWideChunk = 16384;
// (the staged rows, 32 x (na + nc) values, stay within 100 KB of shared memory)
inline bool reduce_is_narrow(int na, int nc) {
  return (long)na * nc <= 16 * 256 && na + nc <= 384;
}

// Elements of the partial-sum buffer reduce_rows takes for (na, nc).
inline size_t reduce_rows_elems(int N, int na, int nc) {
  const int chunk = reduce_is_narrow(na, nc) ? kRedRows : kRedWideChunk;
  return (size_t)((N + chunk - 1) / chunk) * na * nc;
}

// out (na x nc, column-major) = sum over non-skeleton rows i of
// A(i,:)^T B(i,:), A and B DOF-major (N x na, N x nc).  Narrow borders: one
// block per 1,024 rows, then a fixed-order sum of the blocks' partials.
// Wide borders: B's skeleton rows are zeroed in place (B must be a
// temporary), then a split-K GEMM over 16,384-row chunks and a fixed-order
// sum of the slices.
template <typename T>
void reduce_rows(Factorization<T>& F, const T* A, int na, T* B, int nc, T* out, Scratch<T>& sc,
                 cudaStream_t s) {
  const int N = F.N;
  T* partial = sc.take(reduce_rows_elems(N, na, nc));
  if (reduce_is_narrow(na, nc)) {
    const int parts = (N + kRedRows - 1) / kRedRows;
    const int lda = (na + 3) & ~3, ldb = (nc + 1) & ~1;
    if ((lda / 4) * (ldb / 2) <= 2 * 256) {
      const size_t sm = sizeof(T) * 32 * (size_t)(lda + ldb);   // <= 32 x 4,100 values
      if (sm > 48 * 1024)
        KI_CUDA(cudaFuncSetAttribute(k_reduce_tiled<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      ki::launch(k_reduce_tiled<T>, parts, 256, sm, s, A, na, (const T*)B, nc, N, F.d_is_skel, partial);
    } else {
      size_t sm = sizeof(T) * 32 * (size_t)(na + nc);
      if (sm > 48 * 1024)
        KI_CUDA(cudaFuncSetAttribute(k_reduce_partial<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      ki::launch(k_reduce_partial<T>, parts, 256, sm, s, A, na, (const T*)B, nc, N, F.d_is_skel, partial);
    }
    ki::launch(k_reduce_final<T>, std::max(1, (na * nc + 255) / 256), 256, 0, s, (const T*)partial, parts,
               na * nc, out);
    KI_CUDA(cudaGetLastError());
    return;
  }
  ki::launch(k_zero_rows<T>, std::min(8192, (int)(((size_t)N * nc + 255) / 256)), 256, 0, s, B, nc,
             (const unsigned char*)F.d_is_skel, N);
  const int parts = (N + kRedWideChunk - 1) / kRedWideChunk;
  // DOF-major A is the column-major na x N matrix Ac; out = Ac * Bc^T
  dim3 g((na + 63) / 64, (nc + 63) / 64, parts);
  ki::launch(k_gemm<T>, g, 256, 0, s, na, nc, N, T(1), A, na, 0, (const T*)B, nc, 1, T(0), partial, na,
             kRedWideChunk, (int64_t)kRedWideChunk * na, (int64_t)kRedWideChunk * nc, (int64_t)na * nc);
  ki::launch(k_reduce_final<T>, std::max(1, (na * nc + 255) / 256), 256, 0, s, (const T*)partial, parts,
             na * nc, out);
  KI_CUDA(cudaGetLastError());
}

template <typename T>
std::unique_ptr<Factorization<T>> factorize(const Params& prm, int n_points, const double* points,
                                            const double* normals, const double* weights,
                                            const double* curvatures, const HoleDesc& holes,
                                            cudaStream_t stream, const double* d_inputs,
                                            const std::function<void()>& after_tree,
                                            const Factorization<T>* prev) {
  auto t_start = std::chrono::steady_clock::now();
  auto F = std::make_unique<Factorization<T>>();
  F->prm = prm;
  F->stream = stream;
  F->serial = tune_recording();
  F->n_points = n_points;
  Tree& tree = F->tree;
  const int dim = prm.dim;
  cudaStream_t s = stream;

  // point data: interleaved FP64 input (points, normals: dim per point;
  // weights; curvatures) -> SoA in precision T
  double* d_pts_in = nullptr;
  double* d_nrm_in = nullptr;
  double* d_w_in = nullptr;
  {
    const size_t np_ = (size_t)n_points;
    double* d_in = d_inputs ? const_cast<double*>(d_inputs)
                            : (double*)F->alloc(sizeof(double) * np_ * (2 * dim + 2));
    d_pts_in = d_in;
    d_nrm_in = d_in + dim * np_;
    d_w_in = d_in + 2 * dim * np_;
    double* d_k_in = d_w_in + np_;
    if (!d_inputs) {
      KI_CUDA(cudaMemcpyAsync(d_pts_in, points, sizeof(double) * dim * np_, cudaMemcpyHostToDevice, s));
      KI_CUDA(cudaMemcpyAsync(d_nrm_in, normals, sizeof(double) * dim * np_, cudaMemcpyHostToDevice, s));
      KI_CUDA(cudaMemcpyAsync(d_w_in, weights, sizeof(double) * np_, cudaMemcpyHostToDevice, s));
      if (curvatures)
        KI_CUDA(cudaMemcpyAsync(d_k_in, curvatures, sizeof(double) * np_, cudaMemcpyHostToDevice, s));
    }
    T* d = (T*)F->alloc(sizeof(T) * np_ * 11);
    F->d_x = d; F->d_y = d + np_; F->d_nx = d + 2 * np_;
    F->d_ny = d + 3 * np_; F->d_w = d + 4 * np_;
    F->d_kappa = d + 5 * np_;
    if (dim == 3) {
      F->d_z = d + 6 * np_;
      F->d_nz = d + 7 * np_;
    }
    // FP32: low parts of the coordinates
    T* lo = sizeof(T) < sizeof(double) ? d + 8 * np_ : nullptr;
    ki::launch(k_fill_points<T>, std::min(1024, (n_points + 255) / 256), 256, 0, s,
        d_pts_in, d_nrm_in, d_w_in, curvatures ? d_k_in : nullptr, n_points, dim, F->d_x,
        F->d_y, F->d_z, F->d_nx, F->d_ny, F->d_nz, F->d_w, F->d_kappa, lo);
    if (lo) {
      F->d_xl = lo;
      F->d_yl = lo + np_;
      if (dim == 3) F->d_zl = lo + 2 * np_;
    }
    KI_CUDA(cudaGetLastError());
  }
  // the tree on the GPU: descent codes, their sort, boxes, neighbour lists
  // and leaf DOF lists (KI_TREE_BUILD=host: the host partition build, also
  // the fallback when the codes' depth does not reach the leaves)
  {
    const char* tb = std::getenv("KI_TREE_BUILD");
    bool built = false;
    if (!(tb && std::string(tb) == "host")) {
      double c0 = 0, side0 = 0;
      tree_root(points, n_points, dim, &c0, &side0);
      const int depth = tree_code_depth(dim);
      built = tree_build_gpu(d_pts_in, n_points, dim, prm.sol_dim, prm.max_leaf_dofs, c0, side0,
                             depth, &tree, s);
      F->tree_codes_seconds =
          std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    }
    if (!built) tree.build(points, n_points, dim, prm.sol_dim, prm.max_leaf_dofs);
    F->tree_gpu = built;
  }
  if (after_tree) after_tree();
  F->tree_seconds =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  const int sd = prm.sol_dim;
  const int nch = tree.n_children();
  const int N = tree.n_dofs;
  F->N = N;
  const int L = tree.num_levels();

  Points<T> P{F->d_x, F->d_y, F->d_nx, F->d_ny, F->d_w, F->d_kappa};
  P.dim = dim;
  P.z = F->d_z;
  P.nz = F->d_nz;
  P.xl = F->d_xl;
  P.yl = F->d_yl;
  P.zl = F->d_zl;
  P.pde = dim == 2 && prm.sol_dim == 1 ? prm.pde : 0;
  F->d_err = (int*)F->alloc(sizeof(int));
  KI_CUDA(cudaMemsetAsync(F->d_err, 0, sizeof(int), s));

  // 3D diagonal entries (Kernel::compute_diag_entries_3dlaplace/_3dstokes)
  if (dim == 3) {
    const int dpp = sd == 1 ? 1 : 9;
    F->diag_per_point = dpp;
    std::vector<int> glo(n_points), ghi(n_points);
    const int n_outer = holes.n_holes > 0 ? holes.start[0] : n_points;
    for (int p = 0; p < n_outer; p++) { glo[p] = 0; ghi[p] = n_outer; }
    for (int h = 0; h < holes.n_holes; h++)
      for (int p = holes.start[h]; p < holes.start[h] + holes.count[h]; p++) {
        glo[p] = holes.start[h];
        ghi[p] = holes.start[h] + holes.count[h];
      }
    int* d_g = (int*)F->alloc(sizeof(int) * 2 * (size_t)n_points);
    KI_CUDA(cudaMemcpyAsync(d_g, glo.data(), sizeof(int) * n_points, cudaMemcpyHostToDevice, s));
    KI_CUDA(cudaMemcpyAsync(d_g + n_points, ghi.data(), sizeof(int) * n_points, cudaMemcpyHostToDevice, s));
    F->d_diag64 = (double*)F->alloc(sizeof(double) * (size_t)dpp * n_points);
    F->stage_begin("diag3", (sd == 1 ? 20.0 : 80.0) * (double)n_points * n_points, 0);
    const int gx = (n_points + kDiagThreads - 1) / kDiagThreads;
    const char* dmode = std::getenv("KI_DIAG3");
    if (sd == 1 && !(dmode && std::string(dmode) == "fp64")) {
      // Laplace: FP32-pair row sums, the sources split into chunks so that
      // the grid covers the GPU (KI_DIAG3=fp64: the FP64 kernel)
      int sms = 152, dev = 0;
      if (cudaGetDevice(&dev) == cudaSuccess)
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      int chunks = std::max(1, std::min((8 * sms + gx - 1) / gx, n_points / kDiagTile));
      const int chunk_pts = (n_points + chunks - 1) / chunks;
      chunks = (n_points + chunk_pts - 1) / chunk_pts;
      double* part = (double*)F->alloc(sizeof(double) * (size_t)chunks * n_points);
      ki::launch(k_diag3_pair, dim3(gx, chunks), kDiagThreads, 0, s, d_pts_in, d_nrm_in, d_w_in,
                 n_points, d_g, d_g + n_points, chunk_pts, part);
      ki::launch(k_diag3_finish, std::min(2048, (n_points + 255) / 256), 256, 0, s, part, chunks,
                 n_points, n_outer, F->d_diag64);
    } else {
      ki::launch(k_diag3, gx, kDiagThreads, 0, s, d_pts_in, d_nrm_in, d_w_in, n_points, d_g,
                 d_g + n_points, n_outer, sd, F->d_diag64);
    }
    F->stage_end();
    KI_CUDA(cudaGetLastError());
    // synchronize on the (host) group arrays before they go out of scope
    KI_CUDA(cudaStreamSynchronize(s));
    F->d_diag = (T*)F->alloc(sizeof(T) * (size_t)dpp * n_points);
    ki::launch(k_convert<T>, std::min(2048, (dpp * n_points + 255) / 256), 256, 0, s,
        F->d_diag64, (size_t)dpp * n_points, F->d_diag);
    KI_CUDA(cudaGetLastError());
    P.diag = F->d_diag;
  }

  // proxy surface of unit radius (Kernel::get_proxy_mat: 2D angle 2 pi i / P;
  // Kernel::get_proxy_mat3d and the Kernel constructor, kernel/kernel.h:44-62:
  // 3D theta_a = 2 pi a / n_theta, phi_b the Gauss-Legendre nodes on [0, pi],
  // theta outer)
  const int np = prm.num_proxy_points;
  T* d_ptab = (T*)F->alloc(sizeof(T) * 4 * std::max(np, 1));
  ProxyTab<T> ptab{d_ptab, d_ptab + np, d_ptab + 2 * np, d_ptab + 3 * np, np};
  if (dim == 2 && prm.pde == kPdeGauss) ptab.rings = 3;
  {
    std::vector<double> pt(4 * std::max(np, 1), 0.0);
    if (dim == 2) {
      for (int i = 0; i < np; i++) {
        double ang = 2 * M_PI * i * (1.0 / np);
        pt[i] = std::cos(ang);
        pt[np + i] = std::sin(ang);
      }
    } else {
      const int nphi = proxy_phi_count(np), ntheta = 2 * nphi;
      std::vector<double> phi, phw;
      gauss_legendre(nphi, 0.0, M_PI, &phi, &phw);
      for (int a = 0; a < ntheta; a++) {
        const double theta = 2 * M_PI * a * (1.0 / ntheta);
        for (int b = 0; b < nphi; b++) {
          const int i = a * nphi + b;
          pt[i] = std::sin(phi[b]) * std::cos(theta);
          pt[np + i] = std::sin(phi[b]) * std::sin(theta);
          pt[2 * np + i] = std::cos(phi[b]);
          pt[3 * np + i] = (phw[b] * std::sin(phi[b])) * (2 * M_PI / ntheta);
        }
      }
    }
    std::vector<T> ptT(pt.begin(), pt.end());
    upload(d_ptab, ptT, s);
  }

  // integer pool: dof_sorted | per-level active lists | permuted lists
  const int64_t ipool_size = (int64_t)N * (2 * (int64_t)L + 1) + 16;
  int* ipool = (int*)F->alloc(sizeof(int) * ipool_size);
  upload(ipool, tree.dof_sorted, s);
  int64_t ipool_top = N;   // bump pointer for active lists
  int64_t pact_top = (int64_t)N * (L + 1);

  std::vector<HostBox> hb(tree.boxes.size());
  std::vector<SweepTask<T>> all_sw;   // every level's sweep descriptors
  for (size_t b = 0; b < tree.boxes.size(); b++)
    if (tree.boxes[b].leaf) hb[b].n = tree.boxes[b].orig_count;
  F->d_ipool = ipool;
  F->box_factors.assign(tree.boxes.size(), BoxFactor<T>{});

  // re-factorization: per box, the box of prev whose factors are copied
  // (-1: computed here)
  std::vector<int> reuse_of(tree.boxes.size(), -1);
  if (prev && prev->n_points == n_points && same_params(prev->prm, prm)) {
    PointArrays<T> pa{};
    auto add = [&](const T* a, const T* b, int per) {
      if (!a || !b) return;
      pa.a[pa.count] = a;
      pa.b[pa.count] = b;
      pa.per[pa.count++] = per;
    };
    add(F->d_x, prev->d_x, 1);
    add(F->d_y, prev->d_y, 1);
    add(F->d_nx, prev->d_nx, 1);
    add(F->d_ny, prev->d_ny, 1);
    add(F->d_w, prev->d_w, 1);
    add(F->d_kappa, prev->d_kappa, 1);
    add(F->d_xl, prev->d_xl, 1);
    add(F->d_yl, prev->d_yl, 1);
    if (dim == 3) {
      add(F->d_z, prev->d_z, 1);
      add(F->d_nz, prev->d_nz, 1);
      add(F->d_zl, prev->d_zl, 1);
      if (F->diag_per_point == prev->diag_per_point) add(F->d_diag, prev->d_diag, F->diag_per_point);
    }
    // 3D: the diagonal (a sum over the point's curve or surface) is part of
    // every point's data; without a comparable one nothing is reused
    if (dim == 2 || F->diag_per_point == prev->diag_per_point) {
      unsigned char* d_ch = (unsigned char*)F->alloc(std::max(1, n_points));
      ki::launch(k_points_changed<T>, std::min(1024, (n_points + 255) / 256), 256, 0, s, pa, n_points, d_ch);
      KI_CUDA(cudaGetLastError());
      std::vector<unsigned char> ch(n_points);
      KI_CUDA(cudaMemcpyAsync(ch.data(), d_ch, n_points, cudaMemcpyDeviceToHost, s));
      KI_CUDA(cudaStreamSynchronize(s));
      reuse_of = plan_reuse(*prev, tree, ch, prm.min_dofs_to_compress);
    }
  }
  // boxes whose factors are copied: no self block, ID or elimination here
  auto copied = [&](int b) { return reuse_of[b] >= 0 && prev->box_factors[reuse_of[b]].compressed; };

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
        at.nseg = nch;
        for (int ci = 0; ci < nch; ci++) {
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
      double nb = 0;
      for (auto& a : atasks)
        for (int q = 0; q < a.nseg; q++) nb += 8.0 * a.len[q];
      F->stage_begin("active_lists", 0, nb);
      ki::launch(k_build_active, (unsigned)atasks.size(), 128, 0, s, d_at, ipool);
      F->stage_end();
      KI_CUDA(cudaGetLastError());
    }
    if (l == 0) break;

    // ---- self blocks of every box with active DOFs
    std::vector<AsmTask<T>> asm_tasks;
    int64_t kbn_total = 0;
    for (int b : lv)
      if (!copied(b)) kbn_total += (int64_t)hb[b].n * hb[b].n;
    T* d_kbn = (T*)F->alloc(Tsz * (kbn_total + 1));
    std::vector<T*> kbn_of(lv.size(), nullptr);
    {
      int64_t off = 0;
      for (size_t i = 0; i < lv.size(); i++) {
        int b = lv[i];
        const Box& bx = tree.boxes[b];
        HostBox& h = hb[b];
        if (h.n == 0 || copied(b)) continue;
        AsmTask<T> at{};
        at.act = h.act;
        at.n = h.n;
        at.out = d_kbn + off;
        kbn_of[i] = at.out;
        off += (int64_t)h.n * h.n;
        if (!bx.leaf) {
          int o = 0;
          for (int ci = 0; ci < nch; ci++) {
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
      double ne = 0;
      for (auto& a : asm_tasks) ne += (double)a.n * a.n;
      F->stage_begin("assemble", 12.0 * ne, (double)sizeof(T) * ne);
      ki::launch(k_assemble<T>, (unsigned)asm_tasks.size(), kThreads, 0, s, d_as, ipool, P, sd);
      F->stage_end();
      KI_CUDA(cudaGetLastError());
    }

    // ---- ID tasks
    std::vector<int> comp;  // boxes to compress
    std::vector<int> kept;  // boxes whose factors are copied from prev
    for (int b : lv) {
      if (hb[b].n < prm.min_dofs_to_compress || hb[b].n == 0) continue;
      if (reuse_of[b] < 0) {
        comp.push_back(b);
        continue;
      }
      if (hb[b].n != prev->box_factors[reuse_of[b]].n)
        throw std::logic_error("re-factorization: a reused box's active set changed size");
      F->n_reused++;
      if (copied(b)) kept.push_back(b);
    }
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
      it.cx = bx.c[0];
      it.cy = bx.c[1];
      it.cz = bx.c[2];
      it.seg_begin = (int)seg_off.size();
      it.side = bx.side;
      if (l == 1 || (l == 2 && dim == 2)) {
        // Kernel::get_id_mat levels 1/2 (kernel.cpp:441-563): every other box of
        // the level, plus (level 2) the leaves of the levels above; no proxy.
        // Level 2 takes this path in 2D only (`domain_dimension < 3`, :491).
        it.mode = 1;
        for (int o : lv)
          if (o != b) add_seg(hb[o].act, hb[o].n);
        if (l == 2)
          for (int ll = l - 1; ll >= 0; ll--)
            for (int o : tree.levels[ll])
              if (tree.boxes[o].leaf) add_seg(tree.boxes[o].orig_start, tree.boxes[o].orig_count);
      } else {
        it.mode = 0;
        it.rad_filter = std::sqrt((double)dim) * prm.radius_ratio * (bx.side / 2);
        it.rad_proxy = (bx.side / 2) * std::sqrt((double)dim) * prm.radius_ratio;
        for (int o : tree.coarse_nbrs(b)) add_seg(tree.boxes[o].orig_start, tree.boxes[o].orig_count);
        for (int o : tree.same_nbrs(b)) {
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
      ws_cap += n * n + n * n / 4 + 1;
      it.perm = perm_cap;
      perm_cap += n;
      itasks.push_back(it);
    }
    LevelFactor& LF = F->levels[l];
    if (itasks.empty() && kept.empty()) continue;
    int* d_irows = nullptr;   // ID row lists and permutations
    T* d_tws = nullptr;       // ID workspaces (their Tout feeds the elimination)
    std::vector<int> kh;      // ranks of the ID boxes
    if (!itasks.empty()) {
      // scratch
      d_irows = (int*)F->alloc(sizeof(int) * (rows_cap + perm_cap + 16));
      d_tws = (T*)F->alloc(Tsz * (ws_cap + 16));
      for (auto& it : itasks) {
        it.perm += rows_cap;
        it.pact = pact_top;
        pact_top += it.n;
      }
      for (size_t i = 0; i < comp.size(); i++) hb[comp[i]].pact = itasks[i].pact;
      const size_t smem_cap = 225 * 1024;
      IdTask* d_it = (IdTask*)F->alloc(sizeof(IdTask) * itasks.size());
      int64_t* d_soff = (int64_t*)F->alloc(sizeof(int64_t) * (seg_off.size() + 1));
      int* d_slen = (int*)F->alloc(sizeof(int) * (seg_len.size() + 1));
      int* d_k = (int*)F->alloc(sizeof(int) * itasks.size());
      int* d_m = (int*)F->alloc(sizeof(int) * itasks.size());
      upload(d_it, itasks, s);
      upload(d_soff, seg_off, s);
      upload(d_slen, seg_len, s);
      std::string id_name = "id@L" + std::to_string(l);
      F->stage_begin(id_name.c_str(), 0, 0);
      size_t id_rec = F->prof_open.size() - 1;
      // (a) row lists of every box (m is needed to pick the path)
      KI_CUDA(cudaFuncSetAttribute(k_id<T, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_cap));
      KI_CUDA(cudaFuncSetAttribute(k_id<T, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_cap));
      if constexpr (sizeof(T) == 4) {
        KI_CUDA(cudaFuncSetAttribute(k_id<T, 32, kIdBigThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem_cap));
        KI_CUDA(cudaFuncSetAttribute(k_id<T, 64, kIdBigThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem_cap));
      }
      ki::launch(k_id<T, 32>, (unsigned)itasks.size(), kThreads, 0, s, d_it, 0, d_soff, d_slen, ipool, d_irows, d_tws,
                                                           P, sd, ptab, prm.id_tol,
                                                           d_k, d_m, 0, 1, nullptr);
      KI_CUDA(cudaGetLastError());
      // per-box features of the rank predictor and, with a model, the sketch sizes
      const int ntask = (int)itasks.size();
      float* d_feat = (float*)F->alloc(sizeof(float) * kMlpIn * (size_t)ntask);
      int* d_lsk = (int*)F->alloc(sizeof(int) * (size_t)ntask);
      float* d_khat = (float*)F->alloc(sizeof(float) * (size_t)ntask);
      // the network runs in BF16 on the tensor cores (KI_MLP_FP32=1: in FP32
      // inside k_box_features)
      const char* mlp_env = std::getenv("KI_MLP_FP32");
      const bool tc_mlp = prm.rank_model && !(mlp_env && std::string(mlp_env) == "1");
      ki::launch(k_box_features<T>, (ntask + 3) / 4, 128, 0, s,
          d_it, ntask, ipool, P, sd, d_m, proxy_rows(ptab, sd), L > 1 ? (float)l / (float)(L - 1) : 0.f,
          (float)(-std::log10(prm.id_tol) / 10.0), tc_mlp ? nullptr : prm.rank_model,
          prm.sketch_margin, prm.sketch_oversample, d_feat, d_lsk, d_khat);
      KI_CUDA(cudaGetLastError());
      if (tc_mlp) {
        float* d_ratio = (float*)F->alloc(sizeof(float) * (size_t)ntask);
        mlp_predict_bf16(prm.rank_model, d_feat, ntask, d_ratio, F->d_err, s);
        ki::launch(k_sketch_sizes, (ntask + 127) / 128, 128, 0, s, (const IdTask*)d_it, ntask,
                   (const float*)d_ratio, prm.sketch_margin, prm.sketch_oversample, d_lsk, d_khat);
        KI_CUDA(cudaGetLastError());
      }
      kh.assign(itasks.size(), 0);
      std::vector<int> mh(itasks.size()), lh(itasks.size());
      std::vector<float> fh(kMlpIn * (size_t)ntask), khat(itasks.size());
      KI_CUDA(cudaMemcpyAsync(khat.data(), d_khat, sizeof(float) * khat.size(), cudaMemcpyDeviceToHost, s));
      KI_CUDA(cudaMemcpyAsync(lh.data(), d_lsk, sizeof(int) * lh.size(), cudaMemcpyDeviceToHost, s));
      KI_CUDA(cudaMemcpyAsync(fh.data(), d_feat, sizeof(float) * fh.size(), cudaMemcpyDeviceToHost, s));
      KI_CUDA(cudaMemcpyAsync(mh.data(), d_m, sizeof(int) * mh.size(), cudaMemcpyDeviceToHost, s));
      KI_CUDA(cudaStreamSynchronize(s));
      // (b) groups: [narrow, R in smem][narrow, R global][wide, R in smem][wide, R global];
      //     wide = tall ID matrix (folded by the multi-CTA blocked QR) or a
      //     triangle too large for shared memory
      // row threshold of the wide path (environment override KI_WIDE_ROWS, used
      // by the tests to drive every box through it)
      int kWideRows = 1536;
      if (const char* e = std::getenv("KI_WIDE_ROWS")) kWideRows = std::atoi(e);
      // largest shared footprint with the full triangle in shared memory
      // (environment override KI_ID_FULL_CAP, used by the tests)
      size_t full_cap = smem_cap;
      if (const char* e = std::getenv("KI_ID_FULL_CAP")) full_cap = (size_t)std::atol(e);
      // a level of fewer boxes than SMs leaves most SMs idle while one CTA per
      // box folds its rows: with a learned rank its tall boxes take the wide
      // path instead (the sketch formed by many CTAs per box)
      static const int n_sm = device_sm_count();
      const int few_rows = ((int)itasks.size() < n_sm && prm.rank_model) ? 384 : INT_MAX;
      std::vector<int> grp(itasks.size());
      std::vector<char> few(itasks.size(), 0);   // wide only for the level's few boxes
      // KI_TC_SKETCH=1: FP32 sketched boxes of up to 256 columns form their
      // sketch on the tensor cores (k_sketch_tc) instead of k_id's fold
      const char* tc_env = std::getenv("KI_TC_SKETCH");
      const bool tc_sketch = tc_env && std::string(tc_env) == "1";
      for (size_t i = 0; i < itasks.size(); i++) {
        int n = itasks[i].n;
        int md = id_smem_bytes<T>(n, 0) <= full_cap ? 0 : 1;
        const bool tall = mh[i] > kWideRows || (md == 1 && id_smem_bytes<T>(n, 2) > smem_cap);
        few[i] = !tall && mh[i] > few_rows;
        const bool wide = tall || few[i];
        const bool tc = sizeof(T) == 4 && tc_sketch && prm.rank_model && !wide && md == 0 &&
                        lh[i] > 0 && lh[i] < n && lh[i] <= 64 && n <= 256 &&
                        (n > 128 ? 2 : 1) * ((lh[i] + 15) & ~15) <= 128;
        // narrow groups: 0 triangle in shared memory, 1 packed triangle in
        // shared memory (mode 2 of k_id), 4 tensor-core sketch then the
        // pivoted QR of the sketch; wide groups: 2 / 3 by triangle size
        grp[i] = wide ? 2 + md : (tc ? 4 : md);
      }
      auto is_wide = [](int g) { return g == 2 || g == 3; };
      std::vector<int> mode_of(itasks.size());
      {
        std::vector<size_t> order(itasks.size());
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](size_t a2, size_t b2) {
          return grp[a2] != grp[b2] ? grp[a2] < grp[b2] : itasks[a2].n < itasks[b2].n;
        });
        std::vector<IdTask> it2;
        std::vector<int> comp2, grp2, m2, l2;
        std::vector<float> f2;
        for (size_t o : order) {
          it2.push_back(itasks[o]);
          comp2.push_back(comp[o]);
          grp2.push_back(grp[o]);
          m2.push_back(mh[o]);
          // sketches for the shared-memory triangles (group 0) and the wide
          // boxes (groups 2, 3; k_wide_sketch, up to 384 rows; their sketches are
          // cheap next to a fallback, so they get twice the margin and
          // oversampling), not for packed triangles
          // (boxes routed wide only because the level is small keep the narrow
          // path's sketch size)
          int lo = lh[o];
          if (is_wide(grp[o]) && prm.rank_model && !few[o])
            lo = std::min(itasks[o].n, (int)std::ceil((1.f + 2 * prm.sketch_margin) * khat[o]) +
                                           2 * prm.sketch_oversample);
          l2.push_back(grp[o] == 1 || (is_wide(grp[o]) && lo > 384) ? 0 : lo);
          f2.insert(f2.end(), fh.begin() + kMlpIn * o, fh.begin() + kMlpIn * (o + 1));
        }
        itasks.swap(it2);
        comp.swap(comp2);
        grp.swap(grp2);
        mh.swap(m2);
        lh.swap(l2);
        fh.swap(f2);
        for (size_t i = 0; i < comp.size(); i++) {
          hb[comp[i]].pact = itasks[i].pact;
          mode_of[i] = grp[i];
        }
        upload(d_it, itasks, s);
        upload(d_m, mh, s);
        upload(d_lsk, lh, s);
      }
      const bool sketching = prm.rank_model != nullptr;
      int next_aux = 0, n_streams = Factorization<T>::kAux - 1;
      auto launch_range = [&](int g, int flags, cudaStream_t fixed) {
        // tasks of group g are contiguous and sorted by n within the group (see
        // the ordering above); launch them in bins of similar shared-memory
        // size so that small boxes are not limited by the largest one's footprint
        int first = -1, cnt = 0;
        for (size_t i = 0; i < itasks.size(); i++)
          if (grp[i] == g) {
            if (first < 0) first = (int)i;
            cnt++;
          }
        if (cnt == 0) return;
        const int kmode = g == 1 ? 2 : (g & 1);   // group -> k_id storage mode
        // 64-row fold blocks (half the serial steps) where they fit
        auto fold_rows = [&](int n) {
          return (kmode != 1 && (flags & 2) && id_smem_bytes<T>(n, kmode, 64) <= smem_cap) ? 64 : 32;
        };
        int b0 = first;
        while (b0 < first + cnt) {
          const int fr = fold_rows(itasks[b0].n);
          size_t sm0 = id_smem_bytes<T>(itasks[b0].n, kmode, fr, flags);
          // CTAs per SM at this footprint; extend the bin while it stays the same
          int per_sm = std::max(1, (int)(228 * 1024 / (sm0 + 1024)));
          int b1 = b0 + 1;
          size_t sm = sm0;
          while (b1 < first + cnt) {
            if (fold_rows(itasks[b1].n) != fr) break;
            size_t s1 = id_smem_bytes<T>(itasks[b1].n, kmode, fr, flags);
            if (std::max(1, (int)(228 * 1024 / (s1 + 1024))) != per_sm) break;
            sm = std::max(sm, s1);
            b1++;
          }
          if (sm > smem_cap) throw std::runtime_error("box too large for the ID kernel");
          cudaStream_t st = fixed ? fixed : F->aux[(next_aux++) % n_streams];
          // the autotuner's shape for this bin (fold rows, threads), where the
          // fold fits every box of the bin (sorted by n: the last is the largest)
          const int bucket = id_bucket(sizeof(T) == 8, g, itasks[b1 - 1].n);
          const int ch = tune_choice(kTuneId, bucket);
          int fr_use = fr, thr_use = 0;
          size_t sm_use = sm;
          if (ch >= 0) {
            const int want = (ch & 1) ? 64 : 32;
            const size_t s_want = id_smem_bytes<T>(itasks[b1 - 1].n, kmode, want, flags);
            if (want == 32 || (kmode != 1 && (flags & 2) && s_want <= smem_cap)) {
              fr_use = want;
              sm_use = 0;
              for (int q = b0; q < b1; q++)
                sm_use = std::max(sm_use, id_smem_bytes<T>(itasks[q].n, kmode, want, flags));
            }
            thr_use = (sizeof(T) == 4 && (ch & 2)) ? kIdBigThreads : kThreads;
          }
          const bool rec = tune_recording();
          if (rec) F->stage_begin(tune_stage(kTuneId, bucket).c_str(), 0, 0, st);
          launch_k_id<T>(fr_use, thr_use, (unsigned)(b1 - b0), sm_use, st, (const IdTask*)d_it, b0,
                         (const int64_t*)d_soff, (const int*)d_slen, ipool, d_irows, d_tws, P, sd, ptab,
                         prm.id_tol, d_k, d_m, kmode, flags,
                         (const int*)(sketching && g != 1 ? d_lsk : nullptr));
          if (rec) F->stage_end(st);
          KI_CUDA(cudaGetLastError());
          b0 = b1;
        }
      };
      // (c) narrow boxes: fused on-the-fly assembly + TSQR + CPQR, one CTA each;
      //     size bins on aux streams 0..2, the wide path on aux stream 3, all
      //     concurrent
      F->fork();
      launch_range(0, 2, nullptr);
      launch_range(1, 2, nullptr);
      if constexpr (sizeof(T) == 4) {
        // tensor-core sketches (one CTA per box, by accumulator tiles), then
        // the pivoted QR of each sketch, in order on one aux stream
        std::vector<int> list[2];
        for (size_t i = 0; i < itasks.size(); i++)
          if (grp[i] == 4) list[itasks[i].n > 128].push_back((int)i);
        if (!list[0].empty() || !list[1].empty()) {
          cudaStream_t ts = F->aux[0];
          std::string tn = "id_tc_sketch@L" + std::to_string(l);
          double tc_flops = 0;   // Y = Omega M: 2 l m n per box
          for (const auto& lst : list)
            for (int i : lst) tc_flops += 2.0 * lh[i] * (double)mh[i] * itasks[i].n;
          F->stage_begin(tn.c_str(), tc_flops, 0, ts);
          for (int tl = 0; tl < 2; tl++) {
            if (list[tl].empty()) continue;
            int* d_list = (int*)F->alloc(sizeof(int) * list[tl].size());
            upload(d_list, list[tl], ts);
            int nq_max = 16;
            for (int i : list[tl]) nq_max = std::max(nq_max, (lh[i] + 15) & ~15);
            const size_t sm = 2 * tc_sketch_smem(tl + 1, nq_max);   // two stages
            const int ch = ((tl + 1) * nq_max + 31) / 32;   // accumulator chunks per thread
            auto kern = tl ? (ch <= 2 ? k_sketch_tc<2, 2> : k_sketch_tc<2, 4>)
                           : (ch <= 1 ? k_sketch_tc<1, 1> : ch <= 2 ? k_sketch_tc<1, 2> : k_sketch_tc<1, 4>);
            KI_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
            ki::launch(kern, (unsigned)list[tl].size(), kTcThreads, sm, ts, (const IdTask*)d_it,
                       (const int*)d_list, (const int*)d_m, (const int*)d_lsk, (const int*)ipool,
                       (const int*)d_irows, (float*)d_tws, P, sd, ptab, F->d_err);
            KI_CUDA(cudaGetLastError());
          }
          F->stage_end(ts);
          // the pivoted QRs of the sketches (k_cpqr), by sketch rows (32 / 64)
          // and 32-column slabs
          std::vector<int> cls[2][8];
          for (const auto& lst : list)
            for (int i : lst) cls[lh[i] > 32][(itasks[i].n + 31) / 32 - 1].push_back(i);
          std::string qn = "id_cpqr@L" + std::to_string(l);
          F->stage_begin(qn.c_str(), 0, 0, ts);
          for (int lb = 0; lb < 2; lb++)
            for (int wq = 0; wq < 8; wq++) {
              const auto& v = cls[lb][wq];
              if (v.empty()) continue;
              int* d_l2 = (int*)F->alloc(sizeof(int) * v.size());
              upload(d_l2, v, ts);
              int lm = 0, nm = 0;
              for (int i : v) {
                lm = std::max(lm, lh[i]);
                nm = std::max(nm, itasks[i].n);
              }
              const size_t sm = sizeof(float) * (size_t)lm * nm;
              auto kern = lb ? k_cpqr<64> : k_cpqr<32>;
              // the kernel's static shared memory counts against the 48 KB
              // a launch gets without the opt-in attribute
              cudaFuncAttributes fa{};
              KI_CUDA(cudaFuncGetAttributes(&fa, kern));
              if (sm + fa.sharedSizeBytes > 48 * 1024)
                KI_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
              ki::launch(kern, (unsigned)v.size(), 32 * (wq + 1), sm, ts, (const IdTask*)d_it,
                         (const int*)d_l2, (const int*)d_lsk, ipool, d_irows, (float*)d_tws, prm.id_tol, d_k);
              KI_CUDA(cudaGetLastError());
            }
          F->stage_end(ts);
        }
      }
      // (d) wide boxes: explicit ID matrix, blocked Householder QR, then CPQR
      {
        std::vector<WideTask> wt, wsk;   // blocked-QR boxes, sketched boxes
        int64_t mtot = 0, ptot = 0;
        int maxn = 0, max_chunks = 0, max_cb = 0, max_l = 0;
        for (size_t i = 0; i < itasks.size(); i++) {
          if (!is_wide(grp[i])) continue;
          WideTask w{};
          w.task = (int)i;
          w.n = itasks[i].n;
          w.m = mh[i];
          w.nI = (mh[i] - (itasks[i].mode == 0 ? proxy_rows(ptab, sd) : 0)) / 2;
          w.act = itasks[i].act;
          w.rows = itasks[i].rows;
          w.cx = itasks[i].cx;
          w.cy = itasks[i].cy;
          w.cz = itasks[i].cz;
          w.rad = itasks[i].rad_proxy;
          w.R = itasks[i].ws;
          if (sketching && lh[i] > 0 && lh[i] <= w.n && lh[i] <= 384) {
            w.l = lh[i];
            w.chunks = (w.m + kSketchRows - 1) / kSketchRows;
            w.part = ptot;
            ptot += (int64_t)w.chunks * w.l * w.n;
            max_chunks = std::max(max_chunks, w.chunks);
            max_cb = std::max(max_cb, (w.n + kSketchCols - 1) / kSketchCols);
            max_l = std::max(max_l, w.l);
            wsk.push_back(w);
            continue;
          }
          w.M = mtot;
          mtot += (int64_t)w.m * w.n;
          maxn = std::max(maxn, w.n);
          wt.push_back(w);
        }
        cudaStream_t ws3 = F->aux[Factorization<T>::kAux - 1];
        if (!wt.empty() || !wsk.empty()) {
          std::string wq = "wide_qr@L" + std::to_string(l);
          F->stage_begin(wq.c_str(), 0, 0, ws3);
          T* d_wpool = nullptr;
          WideTask* d_wt = nullptr;
          if (!wt.empty()) {
            // the trailing updates' row-chunk partials of V^T A (part 0 then
            // holds W), per box chunks x kQrNb x n
            int64_t ptot_qr = 0;
            int max_m = 0;
            for (auto& w : wt) {
              w.Tf = mtot;
              mtot += kQrNb * kQrNb;
              w.part = ptot_qr;
              ptot_qr += (int64_t)((w.m + kQrChunk - 1) / kQrChunk) * kQrNb * w.n;
              max_m = std::max(max_m, w.m);
            }
            T* d_qparts = nullptr;
            KI_CUDA(pool_malloc((void**)&d_wpool, sizeof(T) * (mtot + 16), ws3));
            KI_CUDA(pool_malloc((void**)&d_qparts, sizeof(T) * (ptot_qr + 16), ws3));
            KI_CUDA(pool_malloc((void**)&d_wt, sizeof(WideTask) * wt.size(), ws3));
            upload(d_wt, wt, ws3);
            ki::launch(k_wide_assemble<T>, dim3((unsigned)wt.size(), (maxn + 7) / 8), 256, 0, ws3,
                d_wt, d_wpool, ipool, d_irows, P, sd, ptab);
            const unsigned nb_w = (unsigned)wt.size();
            // the panels: cooperative launches, `prow` rows per CTA (one box's
            // rows always fit the resident CTAs), over batches of consecutive
            // boxes whose CTAs at the first panel fit them
            int per_sm_coop = 0;
            KI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_coop, k_qr_panel_coop<T>, 256, 0));
            static const int n_sm_coop = device_sm_count();
            const int resident = std::max(1, per_sm_coop) * n_sm_coop;
            const int prow = std::max(512, ((max_m + resident - 1) / resident + 31) & ~31);
            auto box_ctas = [&](const WideTask& w, int p0) {
              return p0 < std::min(w.n, w.m) ? (w.m - p0 + prow - 1) / prow : 0;
            };
            std::vector<std::pair<int, int>> batches;   // [first box, end)
            int batch_max = 0;
            for (int b0 = 0; b0 < (int)wt.size();) {
              int b1 = b0, c = 0;
              while (b1 < (int)wt.size() && (b1 == b0 || c + box_ctas(wt[b1], 0) <= resident)) {
                c += box_ctas(wt[b1], 0);
                b1++;
              }
              batches.push_back({b0, b1});
              batch_max = std::max(batch_max, c);
              b0 = b1;
            }
            T* d_pred = nullptr;
            GridBar* d_bar = nullptr;
            KI_CUDA(pool_malloc((void**)&d_pred, sizeof(T) * (size_t)kPanelRed * (batch_max + 1), ws3));
            KI_CUDA(pool_malloc((void**)&d_bar, sizeof(GridBar), ws3));
            KI_CUDA(cudaMemsetAsync(d_bar, 0, sizeof(GridBar), ws3));
            for (int p0 = 0; p0 < maxn; p0 += kQrNb) {
              for (const auto& bt : batches) {
                int g = 0;
                for (int q = bt.first; q < bt.second; q++) g += box_ctas(wt[q], p0);
                // no box of the batch with rows left below p0: nothing to reflect
                if (g == 0) continue;
                const WideTask* a_t = d_wt + bt.first;
                T* a_pool = d_wpool;
                int a_p = p0, a_rows = prow, a_n = bt.second - bt.first;
                int* a_err = F->d_err;
                void* args[] = {(void*)&a_t, (void*)&a_n, (void*)&a_pool, (void*)&a_p, (void*)&a_rows,
                                (void*)&d_pred, (void*)&d_bar, (void*)&a_err};
                ki::launch_counter().fetch_add(1, std::memory_order_relaxed);
                KI_CUDA(cudaLaunchCooperativeKernel((const void*)k_qr_panel_coop<T>, dim3((unsigned)g),
                                                    dim3(256), args, 0, ws3));
              }
              // trailing columns of the widest box (a box with fewer rows than
              // columns has fewer reflectors in its last panel: one more block)
              const int trail = maxn - p0 - 1;
              if (trail <= 0) continue;
              const unsigned cblk = (unsigned)((trail + kQrWCols - 1) / kQrWCols);
              const unsigned chunks = (unsigned)((max_m - p0 + kQrChunk - 1) / kQrChunk);
              ki::launch(k_qr_wpart<T>, dim3(nb_w, cblk, chunks), 128, 0, ws3, (const WideTask*)d_wt,
                         (const T*)d_wpool, d_qparts, p0);
              ki::launch(k_qr_wsum<T>, dim3(nb_w, cblk), kQrWCols, 0, ws3, (const WideTask*)d_wt,
                         (const T*)d_wpool, d_qparts, p0);
              ki::launch(k_qr_apply<T>, dim3(nb_w, (unsigned)((max_m - p0 + kQrTileRows - 1) / kQrTileRows),
                                             (unsigned)((trail + kQrTileCols - 1) / kQrTileCols)),
                         128, 0, ws3, (const WideTask*)d_wt, d_wpool, (const T*)d_qparts, p0);
            }
            KI_CUDA(cudaFreeAsync(d_qparts, ws3));
            KI_CUDA(cudaFreeAsync(d_pred, ws3));
            KI_CUDA(cudaFreeAsync(d_bar, ws3));
            ki::launch(k_wide_triangle<T>, (unsigned)wt.size(), 256, 0, ws3, d_wt, d_wpool, d_tws);
            KI_CUDA(cudaGetLastError());
          }
          T* d_spool = nullptr;
          WideTask* d_wsk = nullptr;
          if (!wsk.empty()) {
            KI_CUDA(pool_malloc((void**)&d_spool, sizeof(T) * (ptot + 16), ws3));
            KI_CUDA(pool_malloc((void**)&d_wsk, sizeof(WideTask) * wsk.size(), ws3));
            upload(d_wsk, wsk, ws3);
            const size_t skm = sizeof(T) * ((size_t)max_l * kSketchCols + kSketchSub * kSketchCols) +
                               sizeof(uint32_t) * kSketchSub * ((max_l + 31) / 32);
            KI_CUDA(cudaFuncSetAttribute(k_wide_sketch<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem_cap));
            ki::launch(k_wide_sketch<T>, dim3((unsigned)wsk.size(), max_chunks, max_cb), 256, skm, ws3,
                d_wsk, d_spool, ipool, d_irows, P, sd, ptab);
            ki::launch(k_wide_sketch_reduce<T>, (unsigned)wsk.size(), 256, 0, ws3, d_wsk, d_spool, d_tws);
            KI_CUDA(cudaGetLastError());
          }
          F->stage_end(ws3);
          std::string wc = "wide_cpqr@L" + std::to_string(l);
          F->stage_begin(wc.c_str(), 0, 0, ws3);
          // the largest boxes' pivoted QRs over many CTAs each (k_cpqr_coop),
          // in cooperative launches of at most the resident CTAs, on ws3;
          // they leave the per-box k_id bins while those launch (group 5,
          // never launched; they are the last of their groups, which are
          // sorted by n), and get their group back afterwards
          std::vector<std::pair<int, int>> big_grp;
          {
            // (environment override KI_COOP_CPQR_MIN_N, used by the tests to
            // drive every wide box through it)
            int coop_min = kCoopCpqrMinN;
            if (const char* e = std::getenv("KI_COOP_CPQR_MIN_N")) coop_min = std::atoi(e);
            std::vector<int> big;
            for (size_t i = 0; i < itasks.size(); i++)
              if (is_wide(grp[i]) && itasks[i].n >= coop_min) big.push_back((int)i);
            if (!big.empty()) {
              const bool any_sk = sketching;
              size_t sm_max = 0;
              std::vector<CpqrTask> ct;
              int64_t vtot = 0;
              for (int i : big) {
                CpqrTask c{};
                c.task = i;
                c.n = itasks[i].n;
                const bool sk = any_sk && lh[i] > 0 && lh[i] <= itasks[i].n && lh[i] <= 384;
                c.rows = sk ? lh[i] : itasks[i].n;
                c.sketch = sk && lh[i] < itasks[i].n;
                c.jmax = std::min(std::min(c.n, mh[i]), c.rows);
                c.R = itasks[i].ws;
                c.perm = itasks[i].perm;
                c.pact = itasks[i].pact;
                c.act = itasks[i].act;
                c.ctas = (c.n + kCpqrCols - 1) / kCpqrCols;
                c.v = vtot;
                vtot += c.rows + 2;
                sm_max = std::max(sm_max, std::max(sizeof(T) * (size_t)c.rows, sizeof(int) * (size_t)c.n));
                ct.push_back(c);
                big_grp.push_back({i, grp[i]});
                grp[i] = 5;
              }
              if (sm_max > 48 * 1024)
                KI_CUDA(cudaFuncSetAttribute(k_cpqr_coop<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)sm_max));
              int per_sm = 0;
              KI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cpqr_coop<T>, kCpqrCols, sm_max));
              static const int n_sm_cp = device_sm_count();
              const int resident = std::max(1, per_sm) * n_sm_cp;
              T* d_cv = nullptr;
              long long* d_ckey = nullptr;
              int* d_ccol = nullptr;
              int* d_cdone = nullptr;
              GridBar* d_cbar = nullptr;
              int total_ctas = 0;
              for (const auto& c : ct) total_ctas += c.ctas;
              KI_CUDA(pool_malloc((void**)&d_cv, sizeof(T) * (size_t)(vtot + 1), ws3));
              KI_CUDA(pool_malloc((void**)&d_ckey, sizeof(long long) * (size_t)total_ctas, ws3));
              KI_CUDA(pool_malloc((void**)&d_ccol, sizeof(int) * (size_t)total_ctas, ws3));
              KI_CUDA(pool_malloc((void**)&d_cdone, sizeof(int) + sizeof(GridBar) + 16, ws3));
              d_cbar = reinterpret_cast<GridBar*>(d_cdone + 4);
              // launches of consecutive boxes up to the resident CTAs each
              for (size_t g0 = 0; g0 < ct.size();) {
                size_t g1 = g0;
                int ctas = 0;
                while (g1 < ct.size() && (g1 == g0 || ctas + ct[g1].ctas <= resident)) {
                  ct[g1].first = ctas;
                  ctas += ct[g1].ctas;
                  g1++;
                }
                if (ctas > resident)
                  throw std::runtime_error("a box too large for the cooperative pivoted QR");
                std::vector<CpqrTask> part(ct.begin() + g0, ct.begin() + g1);
                CpqrTask* d_ct = nullptr;
                KI_CUDA(pool_malloc((void**)&d_ct, sizeof(CpqrTask) * part.size(), ws3));
                upload(d_ct, part, ws3);
                KI_CUDA(cudaMemsetAsync(d_cdone, 0, sizeof(int) + sizeof(GridBar) + 16, ws3));
                const CpqrTask* a_ct = d_ct;
                int a_nt = (int)part.size();
                T* a_tws = d_tws;
                int* a_irows = d_irows;
                int* a_ipool = ipool;
                double a_tol = prm.id_tol;
                int* a_k = d_k;
                int* a_err = F->d_err;
                void* args[] = {(void*)&a_ct, (void*)&a_nt, (void*)&a_tws, (void*)&a_irows, (void*)&a_ipool,
                                (void*)&d_cv, (void*)&d_ckey, (void*)&d_ccol, (void*)&d_cdone,
                                (void*)&a_tol, (void*)&a_k, (void*)&d_cbar, (void*)&a_err};
                ki::launch_counter().fetch_add(1, std::memory_order_relaxed);
                KI_CUDA(cudaLaunchCooperativeKernel((const void*)k_cpqr_coop<T>, dim3(ctas), dim3(kCpqrCols),
                                                    args, sm_max, ws3));
                KI_CUDA(cudaFreeAsync(d_ct, ws3));
                g0 = g1;
              }
              KI_CUDA(cudaFreeAsync(d_cv, ws3));
              KI_CUDA(cudaFreeAsync(d_ckey, ws3));
              KI_CUDA(cudaFreeAsync(d_ccol, ws3));
              KI_CUDA(cudaFreeAsync(d_cdone, ws3));
            }
          }
          // the pivoted QRs of the wide boxes' sketches / triangles, bins spread
          // over every aux stream (after the sketches on ws3; the upper levels
          // have no narrow boxes to share them with), joined back into ws3
          cudaEvent_t wev[Factorization<T>::kAux];
          for (auto& e : wev) KI_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
          KI_CUDA(cudaEventRecord(wev[0], ws3));
          for (int i = 0; i + 1 < Factorization<T>::kAux; i++) KI_CUDA(cudaStreamWaitEvent(F->aux[i], wev[0], 0));
          n_streams = Factorization<T>::kAux;
          launch_range(2, 4, nullptr);
          launch_range(3, 4, nullptr);
          for (const auto& bg : big_grp) grp[bg.first] = bg.second;
          n_streams = Factorization<T>::kAux - 1;
          for (int i = 0; i + 1 < Factorization<T>::kAux; i++) {
            KI_CUDA(cudaEventRecord(wev[i + 1], F->aux[i]));
            KI_CUDA(cudaStreamWaitEvent(ws3, wev[i + 1], 0));
          }
          for (auto& e : wev) KI_CUDA(cudaEventDestroy(e));
          F->stage_end(ws3);
          if (d_wpool) KI_CUDA(cudaFreeAsync(d_wpool, ws3));
          if (d_wt) KI_CUDA(cudaFreeAsync(d_wt, ws3));
          if (d_spool) KI_CUDA(cudaFreeAsync(d_spool, ws3));
          if (d_wsk) KI_CUDA(cudaFreeAsync(d_wsk, ws3));
        }
      }
      F->join(Factorization<T>::kAux);
      F->stage_end();
      KI_CUDA(cudaGetLastError());
      KI_CUDA(cudaMemcpyAsync(kh.data(), d_k, sizeof(int) * kh.size(), cudaMemcpyDeviceToHost, s));
      KI_CUDA(cudaStreamSynchronize(s));
      if (sketching) {
        // boxes whose sketch did not reveal the rank (k = -1): the plain ID
        std::vector<int> fb;
        for (size_t i = 0; i < kh.size(); i++) {
          if (lh[i] > 0 && (lh[i] < itasks[i].n || is_wide(grp[i]))) F->n_sketched++;
          if (kh[i] < 0) fb.push_back((int)i);
        }
        if (!fb.empty()) {
          // mode 0 (triangle in shared memory) where it fits, else mode 1
          // (triangle in the task's global scratch)
          std::vector<IdTask> t2;
          std::vector<int> m2;
          size_t sm[2] = {0, 0};
          int cnt0 = 0;
          for (int pass = 0; pass < 2; pass++)
            for (int i : fb) {
              const int md = id_smem_bytes<T>(itasks[i].n, 0, 32, 2) <= smem_cap ? 0 : 1;
              if (md != pass) continue;
              t2.push_back(itasks[i]);
              m2.push_back(mh[i]);
              sm[md] = std::max(sm[md], id_smem_bytes<T>(itasks[i].n, md, 32, 2));
              if (md == 0) cnt0++;
            }
          if (sm[1] > smem_cap) throw std::runtime_error("box too large for the ID kernel");
          std::vector<int> fb2;
          for (int pass = 0; pass < 2; pass++)
            for (int i : fb)
              if ((id_smem_bytes<T>(itasks[i].n, 0, 32, 2) <= smem_cap ? 0 : 1) == pass) fb2.push_back(i);
          fb.swap(fb2);
          IdTask* d_t2 = (IdTask*)F->alloc(sizeof(IdTask) * t2.size());
          int* d_m2 = (int*)F->alloc(sizeof(int) * t2.size());
          int* d_k2 = (int*)F->alloc(sizeof(int) * t2.size());
          upload(d_t2, t2, s);
          upload(d_m2, m2, s);
          std::string fname = "id_fallback@L" + std::to_string(l);
          F->stage_begin(fname.c_str(), 0, 0);
          if (cnt0 > 0)
            launch_k_id<T>(32, 0, (unsigned)cnt0, sm[0], s, (const IdTask*)d_t2, 0, (const int64_t*)d_soff,
                           (const int*)d_slen, ipool, d_irows, d_tws, P, sd, ptab, prm.id_tol, d_k2, d_m2,
                           0, 2, (const int*)nullptr);
          if ((int)t2.size() > cnt0)
            launch_k_id<T>(32, 0, (unsigned)(t2.size() - cnt0), sm[1], s, (const IdTask*)d_t2, cnt0,
                           (const int64_t*)d_soff, (const int*)d_slen, ipool, d_irows, d_tws, P, sd, ptab,
                           prm.id_tol, d_k2, d_m2, 1, 2, (const int*)nullptr);
          F->stage_end();
          KI_CUDA(cudaGetLastError());
          std::vector<int> k2(t2.size());
          KI_CUDA(cudaMemcpyAsync(k2.data(), d_k2, sizeof(int) * k2.size(), cudaMemcpyDeviceToHost, s));
          KI_CUDA(cudaStreamSynchronize(s));
          for (size_t j = 0; j < fb.size(); j++) kh[fb[j]] = k2[j];
          F->n_fallback += (int)fb.size();
        }
      }
      // box log: the predictor's features, n, the rank and the level of every ID box
      for (size_t i = 0; i < kh.size(); i++) {
        F->box_log.insert(F->box_log.end(), fh.begin() + kMlpIn * i, fh.begin() + kMlpIn * (i + 1));
        F->box_log.push_back((float)itasks[i].n);
        F->box_log.push_back((float)kh[i]);
        F->box_log.push_back((float)l);
      }
      {
        LevelStat ls;
        ls.level = l;
        ls.boxes = (int)lv.size();
        ls.id_boxes = (int)itasks.size();
        for (size_t i = 0; i < itasks.size(); i++) {
          ls.max_n = std::max(ls.max_n, itasks[i].n);
          ls.max_m = std::max(ls.max_m, mh[i]);
          ls.max_k = std::max(ls.max_k, kh[i]);
          ls.sum_n += itasks[i].n;
          ls.sum_m += mh[i];
          ls.sum_k += kh[i];
          ls.compressed += kh[i] > 0;
          ls.mode_count[grp[i]]++;
        }
        F->level_stats.push_back(ls);
      }
      {
        double fl = 0, by = 0;
        for (size_t i = 0; i < itasks.size(); i++) {
          double m = mh[i], n = itasks[i].n, k = kh[i] > 0 ? kh[i] : std::min(m, n), r = n - k;
          fl += std::max(0.0, 4 * m * n * k - 2 * k * k * (m + n) + 4.0 / 3.0 * k * k * k + k * k * r);
          by += sizeof(T) * (double)k * r;
        }
        F->prof_open[id_rec].flops = fl;
        F->prof_open[id_rec].bytes = by;
      }
    }

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
    for (int b : kept) {
      const BoxFactor<T>& pf = prev->box_factors[reuse_of[b]];
      const int64_t k = pf.k, r = pf.n - pf.k;
      tr_tot += k * r;
      x_tot += r * r;
      r_tot += r;
      kk_tot += k * k;
    }
    LF.n_comp = (int)(ci_list.size() + kept.size());
    if (LF.n_comp == 0) continue;
    T* d_Tp = (T*)F->alloc(Tsz * (tr_tot + 1));
    T* d_LUp = (T*)F->alloc(Tsz * (2 * tr_tot + 1));
    T* d_Xp = (T*)F->alloc(Tsz * (x_tot + 1));
    int* d_pivp = (int*)F->alloc(sizeof(int) * (r_tot + 1));
    T* d_At = (T*)F->alloc(Tsz * (kk_tot + 1));
    T* d_sws = (T*)F->alloc(Tsz * (ws_tot + 1));
    std::vector<SchurTask<T>> st;
    std::vector<SweepTask<T>> sw;
    std::vector<int> sw_box;   // box of each sweep descriptor
    int64_t o_tr = 0, o_x = 0, o_r = 0, o_kk = 0, o_ws = 0;
    for (int i : ci_list) {
      int b = comp[i];
      sw_box.push_back(b);
      int n = itasks[i].n, k = kh[i], r = n - k;
      size_t pos = tree.boxes[b].level_pos;
      SchurTask<T> t{};
      t.K = kbn_of[pos];
      t.n = n;
      t.k = k;
      t.perm = d_irows + itasks[i].perm;
      t.Tin = d_tws + itasks[i].ws + (int64_t)n * n;   // Tout of k_id
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
      LF.max_mat = std::max(LF.max_mat, std::max(r * r, k * r));
      LF.max_all = std::max(LF.max_all, 2 * k * r + r * r);
      LF.sum_kr += (double)k * r;
      LF.sum_r2 += (double)r * r;
      LF.sum_n += n;
      LF.sum_r += r;
    }
    // boxes kept from prev: their lists and factors copied into this level's
    // pools (after the recomputed boxes, whose Schur tasks match sw[0..st))
    std::vector<CopySeg> segs;
    auto copy_seg = [&](const void* src, void* dst, int64_t bytes) {
      if (bytes > 0) segs.push_back(CopySeg{src, dst, bytes / 4});
    };
    for (int b : kept) {
      const BoxFactor<T>& pf = prev->box_factors[reuse_of[b]];
      const int n = pf.n, k = pf.k, r = n - k;
      sw_box.push_back(b);
      SweepTask<T> w{};
      w.n = n;
      w.k = k;
      const int64_t pact = pact_top;
      pact_top += n;
      w.pact = ipool + pact;
      w.Tm = d_Tp + o_tr;
      w.L = d_LUp + 2 * o_tr;
      w.U = d_LUp + 2 * o_tr + (int64_t)k * r;
      w.X = d_Xp + o_x;
      w.piv = d_pivp + o_r;
      w.Xi_formed = 1;
      T* At = d_At + o_kk;
      o_tr += (int64_t)k * r;
      o_x += (int64_t)r * r;
      o_r += r;
      o_kk += (int64_t)k * k;
      copy_seg(prev->d_ipool + pf.pact, ipool + pact, sizeof(int) * (int64_t)n);
      copy_seg(pf.Tm, const_cast<T*>(w.Tm), Tsz * (int64_t)k * r);
      copy_seg(pf.L, const_cast<T*>(w.L), Tsz * (int64_t)k * r);
      copy_seg(pf.U, const_cast<T*>(w.U), Tsz * (int64_t)k * r);
      copy_seg(pf.X, const_cast<T*>(w.X), Tsz * (int64_t)r * r);
      copy_seg(pf.piv, const_cast<int*>(w.piv), sizeof(int) * (int64_t)r);
      copy_seg(pf.tile, At, Tsz * (int64_t)k * k);
      sw.push_back(w);
      HostBox& h = hb[b];
      h.compressed = true;
      h.k = k;
      h.pact = pact;
      h.tile = At;
      F->n_compressed++;
      F->n_redundant += r;
      LF.max_n = std::max(LF.max_n, n);
      LF.max_mat = std::max(LF.max_mat, std::max(r * r, k * r));
      LF.max_all = std::max(LF.max_all, 2 * k * r + r * r);
      LF.sum_kr += (double)k * r;
      LF.sum_r2 += (double)r * r;
      LF.sum_n += n;
      LF.sum_r += r;
    }
    if (sizeof(T) < sizeof(double)) {
      // FP32: explicit inverses of the redundant blocks for the sweeps (the
      // FP64 form keeps the reference's LU substitution)
      int64_t xi_tot = 0;
      for (auto& w : sw) {
        const int64_t r = w.n - w.k;
        if (r <= kInvMax) xi_tot += r * r;
      }
      T* d_xi = (T*)F->alloc(Tsz * (xi_tot + 1));
      int64_t o = 0;
      for (size_t q = 0; q < sw.size(); q++) {
        const int64_t r = sw[q].n - sw[q].k;
        if (r <= kInvMax) {
          sw[q].Xi = d_xi + o;
          if (q < st.size()) st[q].Xi = d_xi + o;
          o += r * r;
        }
      }
      for (size_t q = st.size(); q < sw.size(); q++) {
        const BoxFactor<T>& pf = prev->box_factors[reuse_of[sw_box[q]]];
        if (!sw[q].Xi || !pf.Xi) throw std::logic_error("re-factorization: inverse missing");
        const int64_t r = sw[q].n - sw[q].k;
        copy_seg(pf.Xi, const_cast<T*>(sw[q].Xi), Tsz * r * r);
      }
    }
    if (!segs.empty()) {
      CopySeg* d_seg = (CopySeg*)F->alloc(sizeof(CopySeg) * segs.size());
      upload(d_seg, segs, s);
      double by = 0;
      for (const auto& q : segs) by += 8.0 * q.words;
      F->stage_begin(("reuse@L" + std::to_string(l)).c_str(), 0, by);
      ki::launch(k_copy_segments, (unsigned)segs.size(), 256, 0, s, (const CopySeg*)d_seg);
      F->stage_end();
      KI_CUDA(cudaGetLastError());
    }
    SchurTask<T>* d_st = (SchurTask<T>*)F->alloc(sizeof(SchurTask<T>) * st.size());
    double sf = 0, sb = 0;
    for (auto& q : st) {
      double k = q.k, r = q.n - q.k, n = q.n;
      sf += 2 * r * k * k + 4 * r * r * k + 2 * k * k * r + 2.0 / 3.0 * r * r * r + 4 * r * r * k + 2 * k * k * r;
      sb += sizeof(T) * (n * n + 3 * k * r + r * r + k * k);
    }
    // shared-memory working sets up to this size (environment override
    // KI_SCHUR_SMEM_CAP, used by the tests)
    size_t schur_cap = 225 * 1024;
    if (const char* e = std::getenv("KI_SCHUR_SMEM_CAP")) schur_cap = (size_t)std::atol(e);
    std::string sc_name = "schur@L" + std::to_string(l);
    F->stage_begin(sc_name.c_str(), sf, sb);
    {
      // shared-memory boxes first, then the ones whose working set is global
      // (environment override KI_SCHUR_SMEM_CAP, used by the tests)
      const size_t cap = schur_cap;
      std::vector<SchurTask<T>> st2;
      size_t sm = 0;
      int n_sm = 0;
      // three classes: shared-memory CTA per box; global-memory CTA per box
      // (all in one launch); device-wide launches per box for the few very
      // large ones (n above KI_SCHUR_WIDE_N, default 288)
      int wide_n = 288;
      if (const char* e = std::getenv("KI_SCHUR_WIDE_N")) wide_n = std::atoi(e);
      // FP32: the Gauss-Jordan path where its working set fits, else the LU
      // path (its inverse formed afterwards, xinv)
      for (auto& q : st) q.gj = (q.Xi && schur_bytes<T>(q.n, q.k, true) <= cap) ? 1 : 0;
      for (auto& q : st)
        if (schur_task_bytes<T>(q) <= cap) { st2.push_back(q); sm = std::max(sm, schur_task_bytes<T>(q)); n_sm++; }
      int n_glob = 0;
      for (auto& q : st)
        if (schur_task_bytes<T>(q) > cap && q.n <= wide_n) { st2.push_back(q); n_glob++; }
      for (auto& q : st)
        if (schur_task_bytes<T>(q) > cap && q.n > wide_n) st2.push_back(q);
      for (size_t q = 0; q < st.size(); q++) sw[q].Xi_formed = st[q].gj;
      // shared-memory boxes ascending by footprint, launched in bins of equal
      // CTAs per SM (each bin sized by its largest box) on the aux streams
      std::stable_sort(st2.begin(), st2.begin() + n_sm, [](const SchurTask<T>& a, const SchurTask<T>& b) {
        return schur_task_bytes<T>(a) < schur_task_bytes<T>(b);
      });
      (void)sm;
      upload(d_st, st2, s);
      F->fork();
      int next = 0;
      if (n_sm > 0)
        KI_CUDA(cudaFuncSetAttribute(k_schur<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap));
      auto per_sm = [](size_t bytes) { return std::max(1, (int)(228 * 1024 / (bytes + 1024))); };
      // FP32 Gauss-Jordan bins with redundant blocks of up to 128 rows: the
      // products before and after the inverse in k_schur (phases 1 and 2),
      // the inverse itself by k_gj (KI_SCHUR_SPLIT=0: all in k_schur)
      const char* split_env = std::getenv("KI_SCHUR_SPLIT");
      const bool split_ok = sizeof(T) == 4 && !(split_env && std::string(split_env) == "0");
      for (int b0 = 0; b0 < n_sm;) {
        const int ps = per_sm(schur_task_bytes<T>(st2[b0]));
        int b1 = b0 + 1;
        while (b1 < n_sm && per_sm(schur_task_bytes<T>(st2[b1])) == ps) b1++;
        const size_t bsm = schur_task_bytes<T>(st2[b1 - 1]);
        // a bin of fewer boxes than SMs runs one CTA per SM whatever its footprint
        static const int n_sm = device_sm_count();
        const int thr = schur_threads<T>(b1 - b0 < n_sm ? 1 : ps);
        cudaStream_t bst = F->aux[(next++) % Factorization<T>::kAux];
        int r_max = 0;
        bool all_gj = split_ok;
        for (int q = b0; q < b1; q++) {
          r_max = std::max(r_max, st2[q].n - st2[q].k);
          all_gj = all_gj && st2[q].gj;
        }
        // the autotuner's threads (and, FP32, whether the bin may split)
        const int bucket = schur_bucket(sizeof(T) == 8, r_max, ps);
        const int ch = tune_choice(kTuneSchur, bucket);
        int thr_use = thr;
        if (ch >= 0) {
          if (sizeof(T) == 4) {
            thr_use = ch % 3 == 0 ? 256 : (ch % 3 == 1 ? 512 : 1024);
            all_gj = all_gj && ch < 3;
          } else {
            thr_use = ch == 0 ? 128 : 256;
          }
        }
        const bool rec = tune_recording();
        if (rec) F->stage_begin(tune_stage(kTuneSchur, bucket).c_str(), 0, 0, bst);
        if (all_gj && r_max <= 128) {
          ki::launch(k_schur<T>, (unsigned)(b1 - b0), thr_use, bsm, bst, d_st, b0, 1, F->d_err, 1);
          if constexpr (sizeof(T) == 4) {
            const SchurTask<float>* d_st32 = reinterpret_cast<const SchurTask<float>*>(d_st);
            const int ma = (r_max + 31) / 32;
            auto gj = ma <= 1 ? k_gj<1, kGjLeanCols> : ma == 2 ? k_gj<2, kGjLeanCols>
                    : ma == 3 ? k_gj<3, kGjLeanCols> : k_gj<4, kGjLeanCols>;
            ki::launch(gj, (unsigned)(b1 - b0), 32 * (32 * ma / kGjLeanCols), 0, bst, d_st32, b0, F->d_err);
          }
          ki::launch(k_schur<T>, (unsigned)(b1 - b0), thr_use, bsm, bst, d_st, b0, 1, F->d_err, 2);
        } else {
          ki::launch(k_schur<T>, (unsigned)(b1 - b0), thr_use, bsm, bst, d_st, b0, 1, F->d_err, 0);
        }
        if (rec) F->stage_end(bst);
        b0 = b1;
      }
      if (n_glob > 0)
        ki::launch(k_schur<T>, (unsigned)n_glob, schur_threads<T>(1), 0,
            F->aux[(next++) % Factorization<T>::kAux],
            d_st, n_sm, 0, F->d_err, 0);
      for (size_t q = n_sm + n_glob; q < st2.size(); q++)
        schur_wide<T>(st2[q], F->d_err, F->aux[(next++) % Factorization<T>::kAux]);
      F->join(Factorization<T>::kAux);
    }
    F->stage_end();
    KI_CUDA(cudaGetLastError());
    SweepTask<T>* d_sw = (SweepTask<T>*)F->alloc(sizeof(SweepTask<T>) * sw.size());
    upload(d_sw, sw, s);
    LF.d_tasks = d_sw;
    all_sw.insert(all_sw.end(), sw.begin(), sw.end());
    if (sizeof(T) < sizeof(double)) {
      // inverses of the boxes k_schur factored by LU (global working set)
      std::vector<SweepTask<T>> inv;
      double xf = 0;
      for (auto& w : sw)
        if (w.Xi && !w.Xi_formed) {
          inv.push_back(w);
          xf += 2.0 * std::pow((double)(w.n - w.k), 3);
        }
      if (!inv.empty()) {
        // Xi = I, then the device-wide blocked LU substitution, one box per
        // aux stream
        std::string xi_name = "xinv@L" + std::to_string(l);
        F->stage_begin(xi_name.c_str(), xf, 0);
        F->fork();
        for (size_t q = 0; q < inv.size(); q++) {
          const int r = inv[q].n - inv[q].k;
          cudaStream_t as = F->aux[q % Factorization<T>::kAux];
          T* Xi = const_cast<T*>(inv[q].Xi);
          ki::launch(k_set_identity<T>, std::max(1, std::min(1024, (r * r + 255) / 256)), 256, 0, as, Xi, r);
          dense_lu_solve<T>(inv[q].X, r, inv[q].piv, Xi, r, r, false, as);
        }
        F->join(Factorization<T>::kAux);
        F->stage_end();
        KI_CUDA(cudaGetLastError());
      }
    }
    for (int i : ci_list) F->rank_hist.push_back(kh[i]);
    for (int b : kept) F->rank_hist.push_back(hb[b].k);
    for (size_t q = 0; q < sw.size(); q++) {
      const HostBox& h = hb[sw_box[q]];
      BoxFactor<T>& bf = F->box_factors[sw_box[q]];
      bf.compressed = true;
      bf.k = h.k;
      bf.pact = h.pact;
      bf.tile = (const T*)h.tile;
      bf.Tm = sw[q].Tm;
      bf.L = sw[q].L;
      bf.U = sw[q].U;
      bf.X = sw[q].X;
      bf.piv = sw[q].piv;
      bf.Xi = sw[q].Xi;
    }
  }
  for (size_t b = 0; b < tree.boxes.size(); b++) F->box_factors[b].n = hb[b].n;

  // all levels' sweep descriptors, ascending n, in bins of equal CTAs per SM
  // at 32 columns (the diagonal solves of different levels touch disjoint
  // redundant rows, so they run in one pass)
  if (!all_sw.empty()) {
    std::stable_sort(all_sw.begin(), all_sw.end(),
                     [](const SweepTask<T>& a, const SweepTask<T>& b) { return a.n < b.n; });
    auto per_sm = [](int n) {
      const size_t sm = 2 * sizeof(T) * (size_t)(n | 1) * 32;
      return std::max(1, (int)(228 * 1024 / (sm + 1024)));
    };
    for (int b0 = 0; b0 < (int)all_sw.size();) {
      const int ps = per_sm(all_sw[b0].n);
      int b1 = b0 + 1;
      while (b1 < (int)all_sw.size() && per_sm(all_sw[b1].n) == ps) b1++;
      int mm = 0;
      for (int q = b0; q < b1; q++) {
        const int r = all_sw[q].n - all_sw[q].k;
        mm = std::max(mm, std::max(r * r, all_sw[q].k * r));
      }
      F->diag_bins.push_back({b0, b1 - b0, all_sw[b1 - 1].n, mm});
      b0 = b1;
    }
    SweepTask<T>* d_all = (SweepTask<T>*)F->alloc(sizeof(SweepTask<T>) * all_sw.size());
    upload(d_all, all_sw, s);
    F->d_all_tasks = d_all;
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
        for (int ci = 0; ci < nch; ci++) {
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
      ki::launch(k_assemble<T>, 1, kThreads, 0, s, d_as, ipool, P, sd);
      KI_CUDA(cudaGetLastError());
      F->d_is_skel = (unsigned char*)F->alloc(N);
      KI_CUDA(cudaMemsetAsync(F->d_is_skel, 0, N, s));
      ki::launch(k_mark, std::max(1, (h.n + 255) / 256), 256, 0, s, F->d_root_idx, h.n, F->d_is_skel);
      if (holes.n_holes == 0) {
        F->d_root_lu = A;
        F->d_root_piv = (int*)F->alloc(sizeof(int) * h.n);
        F->stage_begin("root_lu", 2.0 / 3.0 * (double)h.n * h.n * h.n, (double)sizeof(T) * h.n * h.n);
        dense_lu<T>(A, h.n, F->d_root_piv, F->d_err, s);
        F->stage_end();
        KI_CUDA(cudaGetLastError());
        F->n_root_sys = h.n;
      } else {
        // Bordered system (skel_factorization.cpp:311-547): sweep U and Psi^T
        // through every level, apply X_rr^-1 to U's redundant rows, form and
        // factor S.
        const int nh = holes.n_holes;
        const int nb = border_cols_per_hole(dim, sd) * nh;
        F->n_border = nb;
        std::vector<int> hole_of(n_points, -1);
        for (int q = 0; q < nh; q++)
          for (int p = holes.start[q]; p < holes.start[q] + holes.count[q]; p++) hole_of[p] = q;
        int* d_hole_of = (int*)F->alloc(sizeof(int) * n_points);
        upload(d_hole_of, hole_of, s);
        double* d_hc = (double*)F->alloc(sizeof(double) * dim * nh);
        upload(d_hc, holes.centers, s);
        F->d_Umod = (T*)F->alloc(Tsz * (size_t)N * nb);
        F->d_PsiTmod = (T*)F->alloc(Tsz * (size_t)N * nb);
        const size_t bism = sd == 1 && sizeof(T) < sizeof(double) ? sizeof(float) * 2 * dim * nh : 0;
        if (bism > 48 * 1024)
          KI_CUDA(cudaFuncSetAttribute(k_border_init<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)bism));
        ki::launch(k_border_init<T>, std::min(2048, (n_points + 255) / 256), 256, bism, s,
            d_pts_in, d_w_in, n_points, dim, sd, d_hc, nh, d_hole_of, F->d_Umod, F->d_PsiTmod);
        KI_CUDA(cudaGetLastError());
        F->stage_begin("border_sweeps", 0, 0);
        F->stage_begin("border_U_Psi", 0, 0);
        // U~ and Psi~^T are swept independently: one aux stream each
        F->fork();
        for (int l = L - 1; l >= 1; l--) {
          launch_sweep<T>(*F, l, kUp, F->d_Umod, nb, F->aux[0]);
          launch_sweep<T>(*F, l, kPsi, F->d_PsiTmod, nb, F->aux[1]);
        }
        F->join(2);
        F->stage_end();
        T* corr = (T*)F->alloc(Tsz * (size_t)nb * nb);
        {
          Scratch<T> sc(s);
          // D^-1 U~ is kept: the solve forms its redundant rows' result from it
          T* dD = (T*)F->alloc(Tsz * (size_t)N * nb);
          F->d_DinvU = dD;
          KI_CUDA(cudaMemcpyAsync(dD, F->d_Umod, Tsz * (size_t)N * nb, cudaMemcpyDeviceToDevice, s));
          F->stage_begin("border_Dinv", 0, 0);
          launch_diag_all<T>(*F, dD, nb, s);
          F->stage_end();
          F->stage_begin("border_corr", 0, 0);
          reduce_rows<T>(*F, F->d_PsiTmod, nb, dD, nb, corr, sc, s);
          F->stage_end();
          F->stage_end();
        }
        const int ns = h.n + nb;
        T* S = (T*)F->alloc(Tsz * (size_t)ns * ns);
        ki::launch(k_assemble_S<T>, std::min(4096, (int)(((size_t)ns * ns + 255) / 256)), 256, 0, s,
            A, h.n, F->d_root_idx, F->d_Umod, F->d_PsiTmod, corr, nb, S);
        KI_CUDA(cudaGetLastError());
        F->d_root_lu = S;
        F->d_root_piv = (int*)F->alloc(sizeof(int) * ns);
        F->stage_begin("root_lu", 2.0 / 3.0 * (double)ns * ns * ns, (double)sizeof(T) * ns * ns);
        dense_lu<T>(S, ns, F->d_root_piv, F->d_err, s);
        F->stage_end();
        KI_CUDA(cudaGetLastError());
        F->n_root_sys = ns;
      }
    }
  }
  int herr = 0;
  KI_CUDA(cudaMemcpyAsync(&herr, F->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  KI_CUDA(cudaStreamSynchronize(s));
  F->factor_prof = F->collect();
  if (herr == kDevTimeout)
    throw std::runtime_error("a bounded device wait timed out (a tensor-core kernel: the rank "
                             "predictor's inference or an ID sketch)");
  if (herr == kDevSingular) throw std::runtime_error("singular pivot in a Schur or root LU factorization");
  if (herr == kDevNonFinite) throw std::runtime_error("non-finite values in the factorization");
  F->factor_seconds =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  return F;
}

// The factorization's solve (SkelFactorization::solve,
// skel_factorization.cpp:595-778, and multiply_connected_solve, :781-1141),
// every right-hand-side column at once, on F.stream.  Temporaries come from
// `sc`; `prof` brackets the launch groups with profiling events.
template <typename T>
static void solve_core(Factorization<T>& F, T* d_x, int ncols, T* d_alpha, const T* d_g,
                       Scratch<T>& sc, bool prof) {
  cudaStream_t s = F.stream;
  const int L = (int)F.levels.size();
  const int nr = F.n_root;
  auto sb = [&](const char* name, double flops = 0, double bytes = 0) {
    if (prof) F.stage_begin(name, flops, bytes);
  };
  auto se = [&]() { if (prof) F.stage_end(); };
  // Algorithmic work of the sweeps over levels [l0, l1): per box the two
  // k x r factor matrices (T and L up, U and T down) and, with the diagonal
  // solve, the r x r inverse or LU, each read once; the box's n rows of the
  // ncols right-hand sides read and written (plus their indices); flops
  // 4kr (+ 2r^2) per column.
  const double sv = sizeof(T);
  auto sweep_work = [&](int l0, int l1, bool diag, double* flops, double* bytes) {
    double kr = 0, r2 = 0, n = 0;
    for (int l = std::max(1, l0); l < l1; l++) {
      kr += F.levels[l].sum_kr;
      r2 += F.levels[l].sum_r2;
      n += F.levels[l].sum_n;
    }
    *flops = (4 * kr + (diag ? 2 * r2 : 0)) * ncols;
    *bytes = sv * (2 * kr + (diag ? r2 : 0)) + sv * 2 * n * ncols + 4 * n;
  };
  auto sb_sweep = [&](const char* name, int l0, int l1, bool diag) {
    if (!prof) return;
    double fl, by;
    sweep_work(l0, l1, diag, &fl, &by);
    F.stage_begin(name, fl, by);
  };
  // the diagonal solves alone: the r x r matrices and the redundant rows
  auto sb_diag = [&](const char* name) {
    if (!prof) return;
    double r2 = 0, red = 0;
    for (int l = 1; l < L; l++) {
      r2 += F.levels[l].sum_r2;
      red += F.levels[l].sum_r;
    }
    F.stage_begin(name, 2 * r2 * ncols, sv * r2 + sv * 2 * red * ncols + 4 * red);
  };
  if (F.n_border == 0) {
    // the diagonal solves are fused into the upward pass (each box's
    // redundant rows are final once its level has been swept)
    for (int l = L - 1; l >= 1; l--) {
      sb_sweep("sweep_up", l, l + 1, true);
      launch_sweep<T>(F, l, kUpDiag, d_x, ncols, s);
      se();
    }
    if (nr > 0) {
      sb("root_solve");
      T* ws = sc.take((size_t)nr * ncols);
      int gb = std::max(1, std::min(4096, (nr * ncols + 255) / 256));
      ki::launch(k_gather_rows<T>, gb, 256, 0, s, d_x, ncols, F.d_root_idx, nr, ncols, ws);
      dense_lu_solve<T>(F.d_root_lu, nr, F.d_root_piv, ws, nr, ncols, false, s);
      ki::launch(k_scatter_rows<T>, gb, 256, 0, s, d_x, ncols, F.d_root_idx, nr, ncols, ws);
      se();
      KI_CUDA(cudaGetLastError());
    }
    for (int l = 1; l < L; l++) {
      sb_sweep("sweep_down", l, l + 1, false);
      launch_sweep<T>(F, l, kDown, d_x, ncols, s);
      se();
    }
    return;
  }
  const int nb = F.n_border, ns = nr + nb, N = F.N;
  sb_sweep("sweep_up", 1, L, false);
  for (int l = L - 1; l >= 1; l--) launch_sweep<T>(F, l, kUp, d_x, ncols, s);
  se();
  sb_diag("border_diag");
  T* Dw = sc.take((size_t)N * ncols);
  T* t = sc.take((size_t)nb * ncols);
  T* M = sc.take((size_t)ns * ncols);
  KI_CUDA(cudaMemcpyAsync(Dw, d_x, sizeof(T) * (size_t)N * ncols, cudaMemcpyDeviceToDevice, s));
  launch_diag_all<T>(F, Dw, ncols, s);
  se();
  sb("border_reduce");
  reduce_rows<T>(F, F.d_PsiTmod, nb, Dw, ncols, t, sc, s);   // Psi~_r D^-1 w
  se();
  sb("border_root");
  ki::launch(k_mc_rhs<T>, std::max(1, std::min(4096, (ns * ncols + 255) / 256)), 256, 0, s,
      d_x, ncols, F.d_root_idx, nr, t, nb, ncols, M, d_g);
  dense_lu_solve<T>(F.d_root_lu, ns, F.d_root_piv, M, ns, ncols, false, s);
  se();
  // redundant rows: D^-1 (w - U~_r alpha) = D^-1 w - (D^-1 U~)_r alpha
  sb("border_update");
  if (nb <= 64) {
    mc_final<T>(d_x, ncols, Dw, F.d_DinvU, nb, M, nr, N, F.d_is_skel, s);
  } else {
    // x (DOF-major = column-major ncols x N) = Dw - alpha^T (D^-1 U~)^T;
    // skeleton rows are overwritten afterwards, so they need no mask
    KI_CUDA(cudaMemcpyAsync(d_x, Dw, sizeof(T) * (size_t)N * ncols, cudaMemcpyDeviceToDevice, s));
    gemm<T>(s, ncols, N, nb, T(-1), M + nr, ns, true, F.d_DinvU, nb, false, T(1), d_x, ncols);
  }
  KI_CUDA(cudaGetLastError());
  se();
  ki::launch(k_mc_finish<T>, std::max(1, std::min(4096, (ns * ncols + 255) / 256)), 256, 0, s,
      d_x, ncols, F.d_root_idx, M, nr, nb, d_alpha);
  KI_CUDA(cudaGetLastError());
  sb_sweep("sweep_down", 1, L, false);
  for (int l = 1; l < L; l++) launch_sweep<T>(F, l, kDown, d_x, ncols, s);
  se();
}

template <typename T>
void solve_device(Factorization<T>& F, T* d_x, int ncols, T* d_alpha, const T* d_g) {
  Scratch<T> sc(F.stream);
  solve_core<T>(F, d_x, ncols, d_alpha, d_g, sc, F.profile_solve);
}

// ---------------------------------------------------- arena-backed solve --
// solve_device with every temporary carved from a caller-owned buffer: the
// same launch sequence (and so the same results), no allocation, no
// profiling events.
template <typename T>
size_t solve_arena_bytes(const Factorization<T>& F, int ncols) {
  const size_t nr = F.n_root, nb = F.n_border, N = F.N, nc = ncols;
  if (nb == 0) return nr ? Scratch<T>::footprint(nr * nc) : 0;
  return Scratch<T>::footprint(N * nc) + Scratch<T>::footprint(nb * nc) +
         Scratch<T>::footprint((nr + nb) * nc) +
         Scratch<T>::footprint(reduce_rows_elems(F.N, F.n_border, ncols));
}

template <typename T>
void solve_device_arena(Factorization<T>& F, T* d_x, int ncols, T* d_alpha, ScratchArena& arena,
                        cudaStream_t s) {
  cudaStream_t saved = F.stream;
  F.stream = s;
  try {
    Scratch<T> sc(s, &arena);
    solve_core<T>(F, d_x, ncols, d_alpha, nullptr, sc, false);
  } catch (...) {
    F.stream = saved;
    throw;
  }
  F.stream = saved;
}

double tensor_core_selfcheck() {
  const size_t nd = (size_t)kTcCheckRows * kTcCheckQ;
  float* d = nullptr;
  double* ref = nullptr;
  int* err = nullptr;
  KI_CUDA(cudaMalloc(&d, sizeof(float) * nd));
  KI_CUDA(cudaMalloc(&ref, sizeof(double) * nd));
  KI_CUDA(cudaMalloc(&err, sizeof(int)));
  std::vector<float> hd(nd);
  std::vector<double> hr(nd);
  int herr = 0;
  cudaError_t e = cudaMemset(err, 0, sizeof(int));
  const size_t sm = 2 * tc_sketch_smem(2, kTcCheckQ);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_tc_selfcheck, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e == cudaSuccess) {
    ki::launch(k_tc_selfcheck, 1, kTcThreads, sm, (cudaStream_t)0, d, ref, err);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(hd.data(), d, sizeof(float) * nd, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(hr.data(), ref, sizeof(double) * nd, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  cudaFree(ref);
  cudaFree(err);
  if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error: ") + cudaGetErrorString(e));
  if (herr == kDevTimeout) throw std::runtime_error("the tensor-core self-check timed out");
  double dmax = 0, rmax = 0;
  for (size_t i = 0; i < nd; i++) {
    dmax = std::max(dmax, std::fabs((double)hd[i] - hr[i]));
    rmax = std::max(rmax, std::fabs(hr[i]));
  }
  return rmax > 0 ? dmax / rmax : dmax;
}

template size_t solve_arena_bytes<double>(const Factorization<double>&, int);
template size_t solve_arena_bytes<float>(const Factorization<float>&, int);
template void solve_device_arena<double>(Factorization<double>&, double*, int, double*,
                                         ScratchArena&, cudaStream_t);
template void solve_device_arena<float>(Factorization<float>&, float*, int, float*, ScratchArena&,
                                        cudaStream_t);

template std::unique_ptr<Factorization<double>> factorize<double>(
    const Params&, int, const double*, const double*, const double*, const double*,
    const HoleDesc&, cudaStream_t, const double*, const std::function<void()>&,
    const Factorization<double>*);
template std::unique_ptr<Factorization<float>> factorize<float>(
    const Params&, int, const double*, const double*, const double*, const double*,
    const HoleDesc&, cudaStream_t, const double*, const std::function<void()>&,
    const Factorization<float>*);
template void solve_device<double>(Factorization<double>&, double*, int, double*, const double*);
template void solve_device<float>(Factorization<float>&, float*, int, float*, const float*);
template struct Factorization<double>;
template struct Factorization<float>;

}  // namespace ki
