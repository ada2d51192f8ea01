// C ABI (include/ki_gpu.h) over the GPU factorization.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <functional>
#include <future>
#include <memory>
#include <map>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "ki_launch.cuh"
#include "ki_pool.h"
#include "../../include/ki_gpu.h"
#include "ki_common.cuh"
#include "ki_factor.h"
#include "ki_fmm.h"
#include "ki_mlp.h"
#include "ki_tune.h"

namespace {

thread_local std::string g_last_error;

struct ArgError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct StateError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

#define KI_CHECK_CUDA(call)                                                              \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      throw std::runtime_error(std::string("CUDA error: ") + cudaGetErrorString(e_));   \
  } while (0)

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

template <typename F>
int guarded(F&& f) {
  try {
    g_last_error.clear();
    f();
    return KI_OK;
  } catch (const ArgError& e) {
    return fail(KI_ERR_ARG, e.what());
  } catch (const StateError& e) {
    return fail(KI_ERR_STATE, e.what());
  } catch (const std::bad_alloc&) {
    return fail(KI_ERR_OOM, "host allocation failed");
  } catch (const std::invalid_argument& e) {
    return fail(KI_ERR_ARG, e.what());
  } catch (const std::runtime_error& e) {
    std::string m = e.what();
    if (m.find("allocation failed") != std::string::npos || m.find("out of memory") != std::string::npos)
      return fail(KI_ERR_OOM, m);
    if (m.find("singular") != std::string::npos || m.find("non-finite") != std::string::npos)
      return fail(KI_ERR_NUMERIC, m);
    if (m.find("timed out") != std::string::npos) return fail(KI_ERR_TIMEOUT, m);
    return fail(KI_ERR_CUDA, m);
  } catch (...) {
    return fail(KI_ERR_CUDA, "unknown error");
  }
}

// b (column-major, ld) -> x (DOF-major, ld = ncols), with precision change.
template <typename Tin, typename Tout>
__global__ void k_to_dofmajor(const Tin* b, int ldb, int n, int ncols, Tout* x) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * ncols;
       e += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(e % n), c = (int)(e / n);
    x[(size_t)i * ncols + c] = Tout(b[i + (size_t)ldb * c]);
  }
}

template <typename Tin, typename Tout>
__global__ void k_from_dofmajor(const Tin* x, int n, int ncols, Tout* b, int ldb) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * ncols;
       e += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(e % n), c = (int)(e / n);
    b[i + (size_t)ldb * c] = Tout(x[(size_t)i * ncols + c]);
  }
}

// alpha (row-major nb x ncols) -> column-major (ld)
template <typename Tin>
__global__ void k_alpha_out(const Tin* a, int nb, int ncols, double* out, int ld) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nb * ncols; e += gridDim.x * blockDim.x) {
    int i = e / ncols, c = e % ncols;
    out[i + (size_t)ld * c] = double(a[e]);
  }
}

// Dense FP64 operator apply y = K x (+ U alpha), one thread per target DOF,
// sources staged through shared memory.
constexpr int kApplyThreads = 128;
constexpr int kApplyTile = 128;
constexpr int kApplyCols = 8;

// Kernel entry between a target (point data t*, DOF parity tpar) and a source
// point (s*, parity spar), 2D or 3D (Kernel::operator() / get_3d,
// kern_interp/kernel/kernel.cpp:304-429).  diag: the source point's 3D
// diagonal data (used only when the two points coincide).  pde: the 2D
// scalar kernel (Points::pde); fwd: a domain target (the Neumann problem's
// single layer there).
__device__ __forceinline__ double pair_entry(int dim, int sol_dim, int pde, bool fwd, int tpar,
                                             int spar, double tx, double ty, double tz, double tnx,
                                             double tny, double tnz, double sx, double sy,
                                             double sz, double snx, double sny, double snz,
                                             double sw, double sk, const double* diag) {
  if (dim == 3) {
    if (sol_dim == 1)
      return ki::laplace3_entry<double>(tx - sx, ty - sy, tz - sz, snx, sny, snz, sw,
                                        diag ? diag[0] : 0.0);
    return ki::stokes3_entry<double>(tpar, spar, tx - sx, ty - sy, tz - sz, tnx, tny, tnz, snx,
                                     sny, snz, sw, diag);
  }
  if (sol_dim == 1) {
    if (pde == ki::kPdeNeumann && fwd) return ki::neumann_forward_r<double>(tx - sx, ty - sy, sw);
    if (pde) return ki::scalar2_entry_r<double>(pde, tx - sx, ty - sy, tnx, tny, snx, sny, sw, sk);
    return ki::laplace_entry<double>(tx, ty, sx, sy, snx, sny, sw, sk);
  }
  return ki::stokes_entry<double>(tpar, spar, tx, ty, tnx, tny, sx, sy, snx, sny, sw, sk);
}

// Dense FP64 product over one chunk of source points (blockIdx.z):
// out[z][row + ldo c] = sum over the chunk's sources of K(target(row), s) x_s.
// Targets are boundary DOFs (rows[row], or row itself when rows is null; the
// target normal is the DOF's own) or, when tg is given, domain points
// (dim coordinates per point, target normal 0: the reference's forward mode,
// kernel.cpp:335-339 / :390-400).  One thread per target row, sources staged
// through shared memory, kApplyCols columns per blockIdx.y.  With one chunk
// the block writes y directly; otherwise partial sums are reduced in a fixed
// order by k_chunk_reduce.
__global__ void k_dense_apply(ki::Points<double> P, int n_points, int sol_dim, const double* x,
                              int ldx, int ncols, double* out, int ldo, size_t chunk_stride,
                              int chunk_pts, const int* rows, int nrows, const double* tg) {
  __shared__ double sx[kApplyTile], sy[kApplyTile], sz[kApplyTile], snx[kApplyTile],
      sny[kApplyTile], snz[kApplyTile], sw[kApplyTile], sk[kApplyTile];
  const int dim = P.dim;
  const int dpp = dim == 3 ? (sol_dim == 1 ? 1 : 9) : 0;
  const int N = (rows || tg) ? nrows : n_points * sol_dim;
  const int trow = blockIdx.x * blockDim.x + threadIdx.x;
  const int tdof = rows ? (trow < nrows ? rows[trow] : 0) : (trow < N ? trow : 0);
  const int c0 = blockIdx.y * kApplyCols;
  const int nc = min(kApplyCols, ncols - c0);
  const int s_lo = blockIdx.z * chunk_pts, s_hi = min(n_points, s_lo + chunk_pts);
  double* o = out + chunk_stride * blockIdx.z;
  double acc[kApplyCols];
  for (int c = 0; c < kApplyCols; c++) acc[c] = 0.0;
  const int tp = tdof / sol_dim, tpar = tdof - sol_dim * tp;
  double tx, ty, tz, tnx, tny, tnz;
  if (tg) {
    tx = tg[(size_t)dim * tp];
    ty = tg[(size_t)dim * tp + 1];
    tz = dim == 3 ? tg[3 * (size_t)tp + 2] : 0.0;
    tnx = tny = tnz = 0.0;
  } else {
    tx = P.x[tp]; ty = P.y[tp]; tnx = P.nx[tp]; tny = P.ny[tp];
    tz = dim == 3 ? P.z[tp] : 0.0;
    tnz = dim == 3 ? P.nz[tp] : 0.0;
  }
  for (int base = s_lo; base < s_hi; base += kApplyTile) {
    __syncthreads();
    for (int i = threadIdx.x; i < kApplyTile; i += blockDim.x) {
      int p = base + i;
      if (p < s_hi) {
        sx[i] = P.x[p]; sy[i] = P.y[p]; snx[i] = P.nx[p]; sny[i] = P.ny[p]; sw[i] = P.w[p];
        sk[i] = P.kappa[p];
        sz[i] = dim == 3 ? P.z[p] : 0.0;
        snz[i] = dim == 3 ? P.nz[p] : 0.0;
      }
    }
    __syncthreads();
    if (trow >= N) continue;
    int lim = min(kApplyTile, s_hi - base);
    for (int i = 0; i < lim; i++) {
      const double* dg = dpp ? P.diag + (size_t)dpp * (base + i) : nullptr;
      for (int sp = 0; sp < sol_dim; sp++) {
        int sdof = (base + i) * sol_dim + sp;
        double kv = pair_entry(dim, sol_dim, P.pde, tg != nullptr, tpar, sp, tx, ty, tz, tnx,
                               tny, tnz, sx[i], sy[i],
                               sz[i], snx[i], sny[i], snz[i], sw[i], sk[i], dg);
        for (int c = 0; c < nc; c++) acc[c] += kv * x[sdof + (size_t)ldx * (c0 + c)];
      }
    }
  }
  if (trow < N)
    for (int c = 0; c < nc; c++) o[trow + (size_t)ldo * (c0 + c)] = acc[c];
}

// y[row + ldy c] = sum over chunks z (in order) of part[z][row + nrows c].
__global__ void k_chunk_reduce(const double* part, int nchunks, int nrows, int ncols, double* y,
                               int ldy) {
  const size_t tot = (size_t)nrows * ncols;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot;
       e += (size_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int z = 0; z < nchunks; z++) s += part[tot * z + e];
    y[(e % nrows) + (size_t)ldy * (e / nrows)] = s;
  }
}

// Entry (component comp, border column k of one hole) of the border matrix U
// (initialize_U_mat, kern_interp/linear_solve.cpp:19-107); r = x - hole centre.
template <typename R>
__device__ R border_u(int dim, int sol_dim, int comp, int k, const R* r) {
  R r2 = 0;
  for (int d = 0; d < dim; d++) r2 += r[d] * r[d];
  if (sol_dim == 1) return dim == 2 ? R(0.5) * log(r2) : R(1) / sqrt(r2);   // log |r|, 1/|r|
  const R rn = sqrt(r2);
  if (dim == 2) {
    const R sc = R(1.0 / (4 * ki::kPi)), q = rn * rn;
    const R rx = r[0], ry = r[1];
    if (k == 0) return comp == 0 ? sc * (log(1 / rn) + rx * rx / q) : sc * (ry * rx / q);
    if (k == 1) return comp == 0 ? sc * (rx * ry / q) : sc * (log(1 / rn) + ry * ry / q);
    return comp == 0 ? ry * (sc / q) : -rx * (sc / q);
  }
  const R rn3 = rn * rn * rn;
  if (k < 3) return R(1.0 / (8.0 * ki::kPi)) * ((comp == k ? R(1) : R(0)) / rn + r[comp] * r[k] / rn3);
  const R rot = R(-1.0 / (8.0 * ki::kPi)) / rn3;
  const int b = k - 3;
  if (comp == b) return 0;
  // [r]_x entries: (0,1) -r2, (0,2) r1, (1,0) r2, (1,2) -r0, (2,0) -r1, (2,1) r0
  const int o = 3 - comp - b;   // the remaining axis
  const R sgn = ((comp + 1) % 3 == b) ? R(-1) : R(1);
  return rot * sgn * r[o];
}

// FP64 SoA geometry (x, y, nx, ny, w, kappa, z, nz; n each) from the
// interleaved inputs points (dim n) | normals (dim n) | weights | curvatures.
__global__ void k_geo_soa(const double* in, int n, int dim, bool has_kappa, double* geo) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double* p = in + (size_t)dim * i;
    const double* q = in + (size_t)dim * n + (size_t)dim * i;
    geo[i] = p[0];
    geo[n + i] = p[1];
    geo[2 * (size_t)n + i] = q[0];
    geo[3 * (size_t)n + i] = q[1];
    geo[4 * (size_t)n + i] = in[2 * (size_t)dim * n + i];
    geo[5 * (size_t)n + i] = has_kappa ? in[(2 * (size_t)dim + 1) * n + i] : 0.0;
    geo[6 * (size_t)n + i] = dim == 3 ? p[2] : 0.0;
    geo[7 * (size_t)n + i] = dim == 3 ? q[2] : 0.0;
  }
}

// y += U alpha, one thread per listed DOF (rows != nullptr: DOF rows[q] of
// the points; else DOF q).  Points: dim per point with the given stride
// between points (SoA x with stride 1 and separate y/z, or interleaved).
// Each U entry (a log or a reciprocal distance) is evaluated once and
// applied to up to 32 columns held in registers.  R: the arithmetic of the
// entries and sums (float for the residual updates' low-accuracy apply; the
// offsets from the hole centres are formed in FP64).
constexpr int kBorderCols = 32;

// y (column-major, ldy) += U alpha for every DOF (points SoA, stride 1), the
// tiled form: a CTA takes 32 DOFs, forms their U entries once into shared
// memory (32 x nb), stages alpha 32 columns at a time, and lanes are columns
// with warps on DOFs (the U entry broadcast, alpha conflict-free); the tile
// goes out through shared memory so that a warp writes 32 DOFs of one
// column.  Shared memory: sizeof(R) * (32 (nb + 1) + 32 nb + 32 * 33).  In
// FP64 the entries and alpha are held as FP32 pairs and summed with pair_fma
// (the FP32 pipes; the entries themselves are formed in FP64).
constexpr int kBorderTile = 32;
template <typename R>
size_t border_tile_smem(int nb) {
  const size_t b = sizeof(R) * ((size_t)kBorderTile * (nb + 1) + (size_t)nb * 32 + kBorderTile * 33);
  // FP64: the 2D Laplace entries' FP32-pair inputs (points, hole centres, log table)
  return sizeof(R) == 8 ? ((b + 15) & ~size_t(15)) + 16 * (size_t)(kBorderTile + nb) + 8 * 256 : b;
}

// log(1 + (j + 1/2)/256), j < 256, as FP32 pairs: the table of ki::pair_log,
// copied in before each FP64 tile launch.
__device__ float2 g_border_logc[256];
const float2* border_log_table() {
  static const std::vector<float2> tab = [] {
    std::vector<float2> t(256);
    for (int j = 0; j < 256; j++) {
      const double v = std::log(1.0 + (j + 0.5) / 256.0);
      const float h = (float)v;
      t[j] = make_float2(h, (float)(v - (double)h));
    }
    return t;
  }();
  return tab.data();
}
template <typename R>
__global__ void __launch_bounds__(256) k_border_apply_tile(const double* px, const double* py,
                                                           const double* pz, int n_points, int dim,
                                                           int sol_dim, const double* hc, int nh,
                                                           const double* alpha, int lda, int ncols,
                                                           double* y, int ldy) {
  extern __shared__ __align__(16) unsigned char bt_smem[];
  const int cph = sol_dim == 1 ? 1 : (dim == 2 ? 3 : 6);
  const int nb = nh * cph;
  R* Us = reinterpret_cast<R*>(bt_smem);                 // [DOF][nb + 1]
  R* As = Us + (size_t)kBorderTile * (nb + 1);           // [b][32]
  R* out = As + (size_t)nb * 32;                         // [DOF][33]
  const int N = n_points * sol_dim;
  const int d0 = blockIdx.x * kBorderTile;
  const int nd = min(kBorderTile, N - d0);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // FP64, 2D Laplace: the entries 0.5 log |p - c_h|^2 in FP32-pair arithmetic
  // (pair_dist2, pair_log) from the points and centres as pairs
  const bool pair_entries = sizeof(R) == 8 && dim == 2 && sol_dim == 1;
  if constexpr (sizeof(R) == 8) {
    if (pair_entries) {
      const size_t b0 = ((reinterpret_cast<unsigned char*>(out + kBorderTile * 33) - bt_smem) + 15) &
                        ~size_t(15);
      float4* spt = reinterpret_cast<float4*>(bt_smem + b0);
      float4* shc = spt + kBorderTile;
      float2* slog = reinterpret_cast<float2*>(shc + nh);
      auto split4 = [](double x, double y) {
        const float hx = (float)x, hy = (float)y;
        return make_float4(hx, hy, (float)(x - (double)hx), (float)(y - (double)hy));
      };
      for (int i = threadIdx.x; i < 256; i += blockDim.x) slog[i] = g_border_logc[i];
      for (int q = threadIdx.x; q < nd; q += blockDim.x) spt[q] = split4(px[d0 + q], py[d0 + q]);
      for (int h = threadIdx.x; h < nh; h += blockDim.x) shc[h] = split4(hc[2 * h], hc[2 * h + 1]);
      __syncthreads();
      for (int e = threadIdx.x; e < nd * nb; e += blockDim.x) {
        const int q = e / nb, b = e % nb;
        const float2 r2 = ki::pair_dist2(spt[q], shc[b]);
        const float2 lg = ki::pair_log(r2.x, r2.y, slog);
        reinterpret_cast<float2*>(Us)[(size_t)q * (nb + 1) + b] = make_float2(0.5f * lg.x, 0.5f * lg.y);
      }
    }
  }
  for (int e = threadIdx.x; !pair_entries && e < nd * nb; e += blockDim.x) {
    const int q = e / nb, b = e % nb;
    const int dof = d0 + q, p = dof / sol_dim, comp = dof - sol_dim * p;
    const int h = b / cph, kk = b - cph * h;
    const double xp[3] = {px[p], py[p], dim == 3 ? pz[p] : 0.0};
    R rr[3];
    for (int d = 0; d < dim; d++) rr[d] = R(xp[d] - hc[dim * h + d]);
    const R u = border_u<R>(dim, sol_dim, comp, kk, rr);
    if constexpr (sizeof(R) == 8)   // FP64: the entries as FP32 pairs (same bytes)
      reinterpret_cast<float2*>(Us)[(size_t)q * (nb + 1) + b] = ki::split_pair(u);
    else
      Us[(size_t)q * (nb + 1) + b] = u;
  }
  for (int c0 = 0; c0 < ncols; c0 += 32) {
    const int nc = min(32, ncols - c0);
    __syncthreads();
    for (int e = threadIdx.x; e < nb * 32; e += blockDim.x) {
      const int b = e / 32, c = e % 32;
      const double a = c < nc ? alpha[b + (size_t)lda * (c0 + c)] : 0.0;
      if constexpr (sizeof(R) == 8)
        reinterpret_cast<float2*>(As)[e] = ki::split_pair(a);
      else
        As[e] = R(a);
    }
    __syncthreads();
    for (int q = warp; q < nd; q += nw) {
      if constexpr (sizeof(R) == 8) {
        // FP64 sums as FP32-pair products and sums (pair_fma) on the FP32 pipes
        const float2* u = reinterpret_cast<const float2*>(Us) + (size_t)q * (nb + 1);
        const float2* a = reinterpret_cast<const float2*>(As);
        float ah = 0.f, al = 0.f;
        for (int b = 0; b < nb; b++) ki::pair_fma(ah, al, u[b], a[b * 32 + lane]);
        out[q * 33 + lane] = (double)ah + (double)al;
      } else {
        const R* u = Us + (size_t)q * (nb + 1);
        R acc = R(0);
        for (int b = 0; b < nb; b++) acc += u[b] * As[b * 32 + lane];
        out[q * 33 + lane] = acc;
      }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nd * nc; e += blockDim.x) {
      const int c = e / nd, q = e % nd;
      y[(d0 + q) + (size_t)ldy * (c0 + c)] += double(out[q * 33 + c]);
    }
  }
}

template <typename R = double>
__global__ void k_border_apply(const double* px, const double* py, const double* pz, int stride,
                               int n_points, int dim, int sol_dim, const double* hc, int nh,
                               const double* alpha, int lda, int ncols, double* y, int ldy,
                               const int* rows = nullptr, int nrows = 0) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int nq = rows ? nrows : n_points * sol_dim;
  if (q >= nq) return;
  const int dof = rows ? rows[q] : q, p = dof / sol_dim, comp = dof - sol_dim * p;
  const int cph = sol_dim == 1 ? 1 : (dim == 2 ? 3 : 6);
  const double xp[3] = {px[(size_t)stride * p], py[(size_t)stride * p],
                        dim == 3 ? pz[(size_t)stride * p] : 0.0};
  for (int c0 = 0; c0 < ncols; c0 += kBorderCols) {
    const int nc = min(kBorderCols, ncols - c0);
    R acc[kBorderCols];
#pragma unroll
    for (int c = 0; c < kBorderCols; c++) acc[c] = 0;
    for (int h = 0; h < nh; h++) {
      R r[3];
      for (int d = 0; d < dim; d++) r[d] = R(xp[d] - hc[dim * h + d]);
      for (int k = 0; k < cph; k++) {
        const R u = border_u<R>(dim, sol_dim, comp, k, r);
        const double* al = alpha + cph * h + k + (size_t)lda * c0;
#pragma unroll
        for (int c = 0; c < kBorderCols; c++)
          if (c < nc) acc[c] += u * R(al[(size_t)lda * c]);
      }
    }
#pragma unroll
    for (int c = 0; c < kBorderCols; c++)
      if (c < nc) y[q + (size_t)ldy * (c0 + c)] += double(acc[c]);
  }
}

template <typename T>
struct DevBuf {
  T* p = nullptr;
  cudaStream_t s = nullptr;
  DevBuf(size_t n, cudaStream_t st) : s(st) {
    cudaError_t e = ki::pool_malloc((void**)&p, sizeof(T) * (n ? n : 1), st);
    if (e != cudaSuccess) {
      cudaGetLastError();
      throw std::runtime_error("device allocation failed");
    }
  }
  ~DevBuf() {
    if (p) cudaFreeAsync(p, s);
  }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
};

int grid_for(size_t n) { return (int)std::min<size_t>(4096, (n + 255) / 256 + 1); }

// 3D Laplace dense apply y = K x over all boundary DOFs in FP32-pair
// arithmetic (the FP32 pipes run at 64 x the FP64 rate on this part): the
// entry -w_s/(4 pi) (r.n_s)/|r|^3, r = t - s (Kernel::three_d_laplace,
// kern_interp/kernel/kernel.cpp:104-121), from coordinates split hi + lo;
// 1/|r| by one Newton step, y (1 + e/2) with e = 1 - |r|^2 y^2 formed
// exactly enough from the FP32 estimate y (relative error ~2^-23 -> ~2^-46);
// products, dot products and sums carry their rounding errors in the low
// parts.  Each entry keeps ~1e-13 relative accuracy (less where r.n_s
// cancels: ~2^-48 of |r| |n_s| absolute), far below what a refinement
// residual needs.  A coincident pair takes the source's diagonal entry.
// One thread per target DOF, kP3Cols columns per blockIdx.y, sources staged
// per tile in shared memory, blockIdx.z a chunk of the sources (partials
// reduced by k_chunk_reduce in a fixed order).
constexpr int kP3Threads = 128;
constexpr int kP3Tile = 128;
constexpr int kP3Cols = 4;

__global__ void __launch_bounds__(kP3Threads) k_dense_apply3_pair(
    ki::Points<double> P, int n_points, const double* x, int ldx, int ncols, double* out, int ldo,
    size_t chunk_stride, int chunk_pts) {
  __shared__ float4 s_ph[kP3Tile], s_pl[kP3Tile];   // source coordinates hi, lo
  __shared__ float4 s_nh[kP3Tile], s_nl[kP3Tile];   // -w/(4 pi) n_s hi, lo
  __shared__ float2 s_dg[kP3Tile];                  // diagonal entry
  __shared__ float2 s_x[kP3Cols][kP3Tile];          // densities
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int c0 = blockIdx.y * kP3Cols;
  const int nc = min(kP3Cols, ncols - c0);
  const int s_lo = blockIdx.z * chunk_pts, s_hi = min(n_points, s_lo + chunk_pts);
  const int tt = t < n_points ? t : 0;
  const float2 tx = ki::split_pair(P.x[tt]), ty = ki::split_pair(P.y[tt]),
               tz = ki::split_pair(P.z[tt]);
  float ah[kP3Cols], al[kP3Cols];
  for (int c = 0; c < kP3Cols; c++) ah[c] = al[c] = 0.f;
  constexpr double kC = -1.0 / (4.0 * ki::kPi);
  for (int base = s_lo; base < s_hi; base += kP3Tile) {
    __syncthreads();
    for (int i = threadIdx.x; i < kP3Tile; i += blockDim.x) {
      const int sp = base + i;
      if (sp < s_hi) {
        const float2 a = ki::split_pair(P.x[sp]), b = ki::split_pair(P.y[sp]),
                     d = ki::split_pair(P.z[sp]);
        s_ph[i] = make_float4(a.x, b.x, d.x, 0.f);
        s_pl[i] = make_float4(a.y, b.y, d.y, 0.f);
        const double cw = kC * P.w[sp];
        const float2 u = ki::split_pair(cw * P.nx[sp]), v = ki::split_pair(cw * P.ny[sp]),
                     q = ki::split_pair(cw * P.nz[sp]);
        s_nh[i] = make_float4(u.x, v.x, q.x, 0.f);
        s_nl[i] = make_float4(u.y, v.y, q.y, 0.f);
        s_dg[i] = ki::split_pair(P.diag ? P.diag[sp] : 0.0);
        for (int c = 0; c < kP3Cols; c++)
          s_x[c][i] = ki::split_pair(c < nc ? x[sp + (size_t)ldx * (c0 + c)] : 0.0);
      }
    }
    __syncthreads();
    if (t >= n_points) continue;
    const int lim = min(kP3Tile, s_hi - base);
    for (int i = 0; i < lim; i++) {
      float kh, kl;
      if (!ki::pair_dipole3(tx, ty, tz, s_ph[i], s_pl[i], s_nh[i], s_nl[i], kh, kl)) {
        kh = s_dg[i].x;   // coincident pair: the source's diagonal entry
        kl = s_dg[i].y;
      }
      const float2 kv = make_float2(kh, kl);
      for (int c = 0; c < kP3Cols; c++) ki::pair_fma(ah[c], al[c], kv, s_x[c][i]);
    }
  }
  if (t < n_points) {
    double* o = out + chunk_stride * blockIdx.z;
    for (int c = 0; c < nc; c++) o[t + (size_t)ldo * (c0 + c)] = (double)ah[c] + (double)al[c];
  }
}

// y (nrows x ncols, ldy) = dense FP64 product for the given targets (see
// k_dense_apply): all boundary DOFs (rows == tg == null, nrows = N), listed
// DOFs, or domain points.  Few target rows get the source range split into
// chunks so that the launch still fills the GPU; their partial sums are
// added in a fixed order.
void dense_product(const ki::Points<double>& P, int n_points, int sol_dim, const double* x,
                   int ldx, int ncols, double* y, int ldy, const int* rows, int nrows,
                   const double* tg, cudaStream_t s) {
  const int N = (rows || tg) ? nrows : n_points * sol_dim;
  if (N == 0 || ncols == 0) return;
  // 3D Laplace over all boundary DOFs: the FP32-pair kernel (KI_DENSE3=fp64
  // keeps the FP64 one)
  static const bool fp64_only = [] {
    const char* e = std::getenv("KI_DENSE3");
    return e && std::string(e) == "fp64";
  }();
  if (P.dim == 3 && sol_dim == 1 && !rows && !tg && !fp64_only) {
    const int gx = (N + kP3Threads - 1) / kP3Threads;
    const int gy = (ncols + kP3Cols - 1) / kP3Cols;
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess)
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int chunks = std::max(1, std::min((8 * sms + gx * gy - 1) / (gx * gy), n_points / kP3Tile));
    chunks = std::min(chunks, 1024);
    const int chunk_pts = (n_points + chunks - 1) / chunks;
    chunks = (n_points + chunk_pts - 1) / chunk_pts;
    if (chunks == 1) {
      ki::launch(k_dense_apply3_pair, dim3(gx, gy, 1), kP3Threads, 0, s, P, n_points, x, ldx,
                 ncols, y, ldy, (size_t)0, chunk_pts);
      KI_CHECK_CUDA(cudaGetLastError());
      return;
    }
    const size_t stride = (size_t)N * ncols;
    DevBuf<double> part(stride * chunks, s);
    ki::launch(k_dense_apply3_pair, dim3(gx, gy, chunks), kP3Threads, 0, s, P, n_points, x, ldx,
               ncols, part.p, N, stride, chunk_pts);
    ki::launch(k_chunk_reduce, grid_for(stride), 256, 0, s, part.p, chunks, N, ncols, y, ldy);
    KI_CHECK_CUDA(cudaGetLastError());
    return;
  }
  const int gx = (N + kApplyThreads - 1) / kApplyThreads;
  const int gy = (ncols + kApplyCols - 1) / kApplyCols;
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int chunks = std::max(1, std::min((4 * sms + gx * gy - 1) / (gx * gy), n_points / kApplyTile));
  chunks = std::min(chunks, 1024);
  const int chunk_pts = (n_points + chunks - 1) / chunks;
  chunks = (n_points + chunk_pts - 1) / chunk_pts;
  if (chunks == 1) {
    ki::launch(k_dense_apply, dim3(gx, gy, 1), kApplyThreads, 0, s, P, n_points, sol_dim, x, ldx, ncols,
                                                           y, ldy, 0, chunk_pts, rows, nrows, tg);
    KI_CHECK_CUDA(cudaGetLastError());
    return;
  }
  const size_t stride = (size_t)N * ncols;
  DevBuf<double> part(stride * chunks, s);
  ki::launch(k_dense_apply, dim3(gx, gy, chunks), kApplyThreads, 0, s, P, n_points, sol_dim, x, ldx, ncols,
                                                              part.p, N, stride, chunk_pts, rows,
                                                              nrows, tg);
  ki::launch(k_chunk_reduce, grid_for(stride), 256, 0, s, part.p, chunks, N, ncols, y, ldy);
  KI_CHECK_CUDA(cudaGetLastError());
}

}  // namespace

struct ki_factor {
  int precision = KI_PRECISION_FP64;
  int dim = 2;
  int sol_dim = 1;
  int pde = KI_PDE_LAPLACE;
  int n_points = 0;
  int n_dofs = 0;
  int n_holes = 0;
  int n_border = 0;
  cudaStream_t stream = nullptr;
  std::unique_ptr<ki::Factorization<double>> f64;
  std::unique_ptr<ki::Factorization<float>> f32;
  // FP64 geometry on the device (apply / evaluation)
  double* d_geo = nullptr;
  double* d_holes = nullptr;
  double* d_pts = nullptr;     // interleaved coordinates (dim per point)
  float* d_rank_model = nullptr;   // learned rank predictor (FP32 factorizations)
  std::vector<float> rank_model_host;   // its host copy (empty without one)
  int* d_hstart = nullptr;     // hole node ranges
  int* d_hcount = nullptr;
  ki::Points<double> P{};
  // refinement profile (CUDA events; see ki_factor_set_profiling)
  bool profile_refine = false;
  std::vector<ki::StageRec> refine_open;
  std::vector<ki::StageSum> refine_prof;
  // fast FP64 operator apply (2D Laplace): planned and uploaded (on its own
  // stream) by a worker thread while the factorization runs
  std::future<std::unique_ptr<ki::Fmm2d, ki::Fmm2dDeleter>> fmm_ready;
  cudaStream_t fmm_stream = nullptr;
  std::unique_ptr<ki::Fmm2d, ki::Fmm2dDeleter> fmm;
  // host wall-clock milliseconds: create before the factorization (argument
  // copies, geometry upload), the factorization call, waiting for the FMM
  // worker
  double host_prep_ms = 0, host_factor_ms = 0, fmm_wait_ms = 0;
  // exchange every member with o (ki_factor_update installs a new state in
  // the caller's handle; the old one leaves with o)
  void swap_state(ki_factor& o) {
    using std::swap;
    swap(precision, o.precision);
    swap(dim, o.dim);
    swap(sol_dim, o.sol_dim);
    swap(pde, o.pde);
    swap(n_points, o.n_points);
    swap(n_dofs, o.n_dofs);
    swap(n_holes, o.n_holes);
    swap(n_border, o.n_border);
    swap(stream, o.stream);
    swap(f64, o.f64);
    swap(f32, o.f32);
    swap(d_geo, o.d_geo);
    swap(d_holes, o.d_holes);
    swap(d_pts, o.d_pts);
    swap(d_rank_model, o.d_rank_model);
    swap(rank_model_host, o.rank_model_host);
    swap(d_hstart, o.d_hstart);
    swap(d_hcount, o.d_hcount);
    swap(P, o.P);
    swap(profile_refine, o.profile_refine);
    swap(refine_open, o.refine_open);
    swap(refine_prof, o.refine_prof);
    swap(fmm_ready, o.fmm_ready);
    swap(fmm_stream, o.fmm_stream);
    swap(fmm, o.fmm);
    swap(host_prep_ms, o.host_prep_ms);
    swap(host_factor_ms, o.host_factor_ms);
    swap(fmm_wait_ms, o.fmm_wait_ms);
  }
  ~ki_factor() {
    for (auto& r : refine_open) {
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
    if (fmm_ready.valid()) {
      try {
        fmm_ready.get();
      } catch (...) {
      }
    }
    if (stream) cudaStreamSynchronize(stream);   // no apply still reads the FMM buffers
    fmm.reset();
    if (fmm_stream) cudaStreamDestroy(fmm_stream);
    f64.reset();
    f32.reset();
    if (d_geo) cudaFree(d_geo);
    if (d_holes) cudaFree(d_holes);
    if (d_pts) cudaFree(d_pts);
    if (d_rank_model) cudaFree(d_rank_model);
    if (d_hstart) cudaFree(d_hstart);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

template <typename T>
void solve_impl(ki_factor* f, ki::Factorization<T>& F, const double* d_b, int ldb, int nrhs,
                double* d_x, int ldx, double* d_alpha, int ldalpha, cudaStream_t s) {
  const int N = f->n_dofs;
  DevBuf<T> work((size_t)N * nrhs, s);
  DevBuf<T> al((size_t)std::max(1, f->n_border) * nrhs, s);
  ki::launch(k_to_dofmajor<double, T>, grid_for((size_t)N * nrhs), 256, 0, s, d_b, ldb, N, nrhs, work.p);
  KI_CHECK_CUDA(cudaGetLastError());
  cudaStream_t saved = F.stream;
  F.stream = s;
  try {
    ki::solve_device<T>(F, work.p, nrhs, al.p);
  } catch (...) {
    F.stream = saved;
    throw;
  }
  F.stream = saved;
  ki::launch(k_from_dofmajor<T, double>, grid_for((size_t)N * nrhs), 256, 0, s, work.p, N, nrhs, d_x, ldx);
  KI_CHECK_CUDA(cudaGetLastError());
  if (f->n_border > 0 && d_alpha) {
    ki::launch(k_alpha_out<T>, grid_for((size_t)f->n_border * nrhs), 256, 0, s, al.p, f->n_border, nrhs,
                                                                       d_alpha, ldalpha);
    KI_CHECK_CUDA(cudaGetLastError());
  }
}

static_assert(KI_PDE_LAPLACE_NEUMANN == ki::kPdeNeumann && KI_PDE_GAUSS == ki::kPdeGauss,
              "Points::pde takes the ki_pde values");

void check_desc(const ki_problem_desc* d) {
  if (!d) throw ArgError("desc is NULL");
  if (d->domain_dimension != 2 && d->domain_dimension != 3)
    throw ArgError("domain_dimension must be 2 or 3");
  const int dim = d->domain_dimension;
  if (d->n_points <= 0) throw ArgError("n_points must be positive");
  if (d->pde == KI_PDE_LAPLACE) {
    if (d->solution_dimension != 1) throw ArgError("Laplace needs solution_dimension 1");
  } else if (d->pde == KI_PDE_STOKES) {
    if (d->solution_dimension != dim)
      throw ArgError("Stokes needs solution_dimension equal to domain_dimension");
  } else if (d->pde == KI_PDE_LAPLACE_NEUMANN || d->pde == KI_PDE_GAUSS) {
    if (dim != 2 || d->solution_dimension != 1)
      throw ArgError("the Neumann and Gaussian kernels need domain_dimension 2 and "
                     "solution_dimension 1");
  } else {
    throw ArgError("unknown pde");
  }
  // the Gaussian kernel reads neither normals nor weights: NULL reads as zeros,
  // as the reference's empty arrays do (Kernel::boundary_normals, kernel.cpp:12-22)
  if (!d->points || (d->pde != KI_PDE_GAUSS && (!d->normals || !d->weights)))
    throw ArgError("points/normals/weights must be non-NULL");
  if (!(d->id_tol > 0) || !std::isfinite(d->id_tol)) throw ArgError("id_tol must be positive");
  if (d->precision != KI_PRECISION_FP64 && d->precision != KI_PRECISION_FP32)
    throw ArgError("unknown precision");
  if (d->precision == KI_PRECISION_FP32 && d->id_tol < 5e-8)
    throw ArgError("an FP32 factorization needs id_tol >= 5e-8 (FP32 rounding); use "
                   "ki_solve_refined to reach tighter residuals");
  if (d->n_holes < 0) throw ArgError("n_holes must be >= 0");
  if (d->n_holes > 0 && (!d->hole_centers || !d->hole_node_start || !d->hole_node_count))
    throw ArgError("hole arrays must be non-NULL when n_holes > 0");
  for (int h = 0; h < d->n_holes; h++) {
    int s = d->hole_node_start[h], c = d->hole_node_count[h];
    if (s < 0 || c <= 0 || s + c > d->n_points) throw ArgError("hole node range out of bounds");
  }
  if (dim == 3 && d->num_proxy_points > 0) {
    int q = (int)std::lround(std::sqrt(d->num_proxy_points / 2.0));
    if (q < 1 || 2 * q * q != d->num_proxy_points)
      throw ArgError("3D num_proxy_points must be 2 q^2 (a theta x phi grid of 2q x q points)");
  }
  for (long i = 0; i < (long)dim * d->n_points; i++)
    if (!std::isfinite(d->points[i]) || (d->normals && !std::isfinite(d->normals[i])))
      throw ArgError("non-finite point or normal");
  for (int i = 0; i < d->n_points; i++) {
    if (d->weights && !std::isfinite(d->weights[i])) throw ArgError("non-finite weight");
    if (d->curvatures && !std::isfinite(d->curvatures[i])) throw ArgError("non-finite curvature");
  }
  if (d->max_leaf_dofs < 0 || d->num_proxy_points < 0 || d->min_dofs_to_compress < 0 ||
      d->radius_ratio < 0)
    throw ArgError("tree/proxy parameters must be >= 0 (0 = reference default)");
}

// ---------------------------------------------------------------------------
// Allocation-free solve.  Callers that cannot allocate device memory while
// solving -- applications that reserve all device memory up front for their
// own allocator and account for every byte, or latency-critical loops that
// cannot absorb the implicit synchronization of cudaMalloc/cudaFree -- call
// ki_solve_device_noalloc.  Its temporaries live in this fixed, file-scope
// device array instead of coming from the stream-ordered allocator.
// Every GPU that loads the library holds the array until the process exits.
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;   // 32 MiB
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch per device, looked up once (with that
// device current) on the first no-allocation call made on it.  The host-side
// name g_noalloc_scratch is only a stand-in: never hand it to a kernel.
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[256] = {};

void* noalloc_scratch_for_current_device() {
  int dev = 0;
  KI_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) throw std::runtime_error("device index out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      throw std::runtime_error(std::string("cudaGetSymbolAddress of the no-allocation scratch failed: ") +
                               cudaGetErrorString(e));
    g_noalloc_ptr[dev] = p;
  }
  return g_noalloc_ptr[dev];
}

template <typename T>
void solve_impl_noalloc(ki_factor* f, ki::Factorization<T>& F, const double* d_b, int ldb,
                        int nrhs, double* d_x, int ldx, double* d_alpha, int ldalpha,
                        cudaStream_t s) {
  const int N = f->n_dofs;
  auto piece = [](size_t b) { return ((b + 255) & ~size_t(255)) + 256; };
  const size_t need = piece(sizeof(T) * (size_t)N * nrhs) +
                      piece(sizeof(T) * (size_t)std::max(1, f->n_border) * nrhs) +
                      ki::solve_arena_bytes<T>(F, nrhs);
  if (need > kNoAllocScratchBytes)
    throw ArgError("ki_solve_device_noalloc: this solve needs " + std::to_string(need) +
                   " bytes of scratch but the fixed scratch holds " +
                   std::to_string(kNoAllocScratchBytes) +
                   " bytes (32 MiB); use fewer right-hand sides per call or ki_solve_device");
  ki::ScratchArena arena;
  arena.base = static_cast<char*>(noalloc_scratch_for_current_device());
  arena.size = kNoAllocScratchBytes;
  T* work = static_cast<T*>(arena.take(sizeof(T) * (size_t)N * nrhs));
  T* al = static_cast<T*>(arena.take(sizeof(T) * (size_t)std::max(1, f->n_border) * nrhs));
  if (!work || !al) throw ArgError("ki_solve_device_noalloc: scratch exhausted");
  // every temporary is written before it is read: nothing needs clearing
  ki::launch(k_to_dofmajor<double, T>, grid_for((size_t)N * nrhs), 256, 0, s, d_b, ldb, N, nrhs, work);
  KI_CHECK_CUDA(cudaGetLastError());
  ki::solve_device_arena<T>(F, work, nrhs, al, arena, s);
  ki::launch(k_from_dofmajor<T, double>, grid_for((size_t)N * nrhs), 256, 0, s, work, N, nrhs, d_x, ldx);
  KI_CHECK_CUDA(cudaGetLastError());
  if (f->n_border > 0 && d_alpha) {
    ki::launch(k_alpha_out<T>, grid_for((size_t)f->n_border * nrhs), 256, 0, s, al, f->n_border, nrhs,
                                                                       d_alpha, ldalpha);
    KI_CHECK_CUDA(cudaGetLastError());
  }
}

// FMA-throughput microbenchmark: register-resident independent FMA chains,
// 8 CTAs of 256 threads per SM.  Gives the compute denominators of the
// roofline for CUDA-core work (the pipe the factorization kernels use).
template <typename T>
__global__ void k_fma_peak(T* out, int iters) {
  T a0 = T(threadIdx.x) * T(1e-3), a1 = a0 + T(1), a2 = a0 + T(2), a3 = a0 + T(3);
  T a4 = a0 + T(4), a5 = a0 + T(5), a6 = a0 + T(6), a7 = a0 + T(7);
  const T b = T(0.999999), c = T(1e-7);
  for (int i = 0; i < iters; i++) {
    a0 = a0 * b + c; a1 = a1 * b + c; a2 = a2 * b + c; a3 = a3 * b + c;
    a4 = a4 * b + c; a5 = a5 * b + c; a6 = a6 * b + c; a7 = a7 * b + c;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

template <typename T>
double fma_peak_gflops(int sms, int iters) {
  const int blocks = sms * 8, threads = 256;
  T* out = nullptr;
  KI_CHECK_CUDA(cudaMalloc(&out, sizeof(T) * blocks * threads));
  ki::launch(k_fma_peak<T>, blocks, threads, 0, 0, out, 16);
  cudaEvent_t e0, e1;
  KI_CHECK_CUDA(cudaEventCreate(&e0));
  KI_CHECK_CUDA(cudaEventCreate(&e1));
  KI_CHECK_CUDA(cudaEventRecord(e0));
  ki::launch(k_fma_peak<T>, blocks, threads, 0, 0, out, iters);
  KI_CHECK_CUDA(cudaEventRecord(e1));
  KI_CHECK_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  KI_CHECK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  return 2.0 * 8 * (double)iters * blocks * threads / (ms * 1e-3) / 1e9;
}

// ---------------------------------------------------------------------------
// Iterative refinement with an FP64 residual.  The bordered operator
// [K U; Psi -I] (the reference's multiply connected system,
// kern_interp/skel_factorization/skel_factorization.cpp:781-1141; plain K
// without holes) is applied in FP64; the factorization (FP32 or FP64) solves
// for the correction.

// Entry (border row k of one hole, DOF component comp) of Psi
// (initialize_Psi_mat, kern_interp/linear_solve.cpp:110-199): x absolute
// coordinates, r = x - hole centre.
__device__ double psi_entry(int dim, int sol_dim, int k, int comp, double w, const double* x,
                            const double* r) {
  if (sol_dim == 1) return w;
  if (dim == 2) {
    if (k < 2) return comp == k ? w : 0.0;
    return comp == 0 ? w * x[1] : -w * x[0];
  }
  if (k < 3) return comp == k ? w : 0.0;
  const int b = k - 3;
  if (comp == b) return 0.0;
  const int o = 3 - comp - b;
  const double sgn = ((comp + 1) % 3 == b) ? -1.0 : 1.0;
  return -w * sgn * r[o];
}

// y2 (n_border x ncols, column-major) = Psi mu - alpha: one block per
// (border row, column), the hole's nodes summed in a fixed order.
__global__ void k_psi_apply(const double* pts, const double* w, int dim, int sol_dim,
                            const double* hc, const int* hstart, const int* hcount, int cph,
                            const double* mu, int ldmu, const double* alpha, int lda, double* y2,
                            int ldy) {
  __shared__ double red[256];
  const int row = blockIdx.x, c = blockIdx.y;
  const int h = row / cph, k = row - cph * h;
  double acc = 0.0;
  for (int p = hstart[h] + threadIdx.x; p < hstart[h] + hcount[h]; p += blockDim.x) {
    double x[3] = {pts[(size_t)dim * p], pts[(size_t)dim * p + 1],
                   dim == 3 ? pts[3 * (size_t)p + 2] : 0.0};
    double r[3];
    for (int d = 0; d < dim; d++) r[d] = x[d] - hc[dim * h + d];
    for (int comp = 0; comp < sol_dim; comp++)
      acc += psi_entry(dim, sol_dim, k, comp, w[p], x, r) * mu[(size_t)p * sol_dim + comp + (size_t)ldmu * c];
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) y2[row + (size_t)ldy * c] = red[0] - alpha[row + (size_t)lda * c];
}

// Per-column sums of squares of an (n x ncols, ld) column-major array:
// partial sums per block (fixed order), then a fixed-order final sum.
constexpr int kNormBlocks = 64;
__global__ void k_colsq_partial(const double* a, int n, int ld, double* part) {
  __shared__ double red[256];
  const int c = blockIdx.y;
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double v = a[i + (size_t)ld * c];
    acc += v * v;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x + (size_t)gridDim.x * c] = red[0];
}

__global__ void k_colsq_final(const double* part, int nparts, int ncols, double* out, int accumulate) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncols) return;
  double s = 0.0;
  for (int q = 0; q < nparts; q++) s += part[q + (size_t)nparts * c];
  out[c] = accumulate ? out[c] + s : s;
}

// r = b - y (b may be null: r = -y), column-major with leading dimensions.
__global__ void k_residual(const double* b, int ldb, const double* y, int ldy, int n, int ncols,
                           double* r, int ldr) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * ncols;
       e += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(e % n), c = (int)(e / n);
    r[i + (size_t)ldr * c] = (b ? b[i + (size_t)ldb * c] : 0.0) - y[i + (size_t)ldy * c];
  }
}

// x (column-major, ldx) += d (DOF-major in precision T, ld = ncols); with
// dcol, d is also stored there in FP64 (column-major, ld = n).
template <typename T>
__global__ void k_add_dofmajor(const T* d, int n, int ncols, double* x, int ldx,
                               double* dcol = nullptr) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * ncols;
       e += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(e % n), c = (int)(e / n);
    const double v = double(d[(size_t)i * ncols + c]);
    x[i + (size_t)ldx * c] += v;
    if (dcol) dcol[e] = v;
  }
}

// column-major (ld) FP64 -> row-major (n x ncols) precision T, and back with +=.
template <typename T>
__global__ void k_to_rowmajor(const double* a, int lda, int n, int ncols, T* out) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * ncols; e += gridDim.x * blockDim.x) {
    int i = e % n, c = e / n;
    out[(size_t)i * ncols + c] = T(a[i + (size_t)lda * c]);
  }
}

template <typename T>
__global__ void k_add_rowmajor(const T* d, int n, int ncols, double* a, int lda,
                               double* dcol = nullptr) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * ncols; e += gridDim.x * blockDim.x) {
    int i = e % n, c = e / n;
    const double v = double(d[(size_t)i * ncols + c]);
    a[i + (size_t)lda * c] += v;
    if (dcol) dcol[e] = v;
  }
}

// y1 = K mu + U alpha, y2 = Psi mu - alpha (FP64, column-major, ld = N / nb).
// low: K by the FP32 FMM at kLowOrder terms (requires use_fmm).
void apply_bordered(ki_factor* f, const double* mu, const double* alpha, int ncols, double* y1,
                    double* y2, cudaStream_t s, double target, ki::StageRecorder* rec,
                    bool low = false);
bool use_fmm(const ki_factor* f);

// The low-accuracy apply of residual updates: FMM terms, and the relative
// error (2-norm, per column) it is credited with.  12 terms leave a
// truncation error near 4e-7 (1.4e-8 * 0.43^(12 - 16)); FP32 arithmetic adds
// rounding of the same order; 1e-5 keeps a margin over both.
constexpr int kLowOrder = 12;
constexpr double kLowRelErr = 1e-5;

// CUDA-event recorder of the refinement's launch groups (into the handle).
struct RefineRecorder : ki::StageRecorder {
  ki_factor* f;
  cudaStream_t s;
  RefineRecorder(ki_factor* f_, cudaStream_t s_) : f(f_), s(s_) {}
  void begin(const char* name, double flops) override {
    ki::StageRec r;
    r.stage = name;
    r.flops = flops;
    KI_CHECK_CUDA(cudaEventCreate(&r.a));
    KI_CHECK_CUDA(cudaEventCreate(&r.b));
    KI_CHECK_CUDA(cudaEventRecord(r.a, s));
    f->refine_open.push_back(r);
  }
  void end() override { KI_CHECK_CUDA(cudaEventRecord(f->refine_open.back().b, s)); }
};

// Per-column relative residual of [mu; alpha] for right-hand side b:
// returns max over columns of ||[b;0] - A[mu;alpha]|| / ||b||, leaves r1/r2.
double column_norms(ki_factor* f, const double* b, const double* r1, const double* r2, int ncols,
                    double* work, std::vector<double>* rel, cudaStream_t s);

double residual_norms(ki_factor* f, const double* b, const double* mu, const double* alpha,
                      int ncols, double* r1, double* r2, double* work, std::vector<double>* rel,
                      cudaStream_t s, double target, ki::StageRecorder* rec) {
  const int N = f->n_dofs, nb = f->n_border;
  apply_bordered(f, mu, alpha, ncols, r1, r2, s, target, rec);
  if (rec) rec->begin("residual_other", 0);
  ki::launch(k_residual, grid_for((size_t)N * ncols), 256, 0, s, b, N, r1, N, N, ncols, r1, N);
  if (nb > 0) ki::launch(k_residual, grid_for((size_t)nb * ncols), 256, 0, s, nullptr, 0, r2, nb, nb, ncols, r2, nb);
  KI_CHECK_CUDA(cudaGetLastError());
  const double worst = column_norms(f, b, r1, r2, ncols, work, rel, s);
  if (rec) rec->end();
  return worst;
}

// The residual update after a correction [d; d_alpha]: [r1; r2] -= A_low
// [d; d_alpha] (y1, y2: scratch of the residual's shape), then the column
// norms.
double update_residual(ki_factor* f, const double* b, const double* d, const double* dal,
                       int ncols, double* r1, double* r2, double* y1, double* y2, double* work,
                       std::vector<double>* rel, cudaStream_t s, ki::StageRecorder* rec) {
  const int N = f->n_dofs, nb = f->n_border;
  apply_bordered(f, d, dal, ncols, y1, y2, s, 0.0, rec, true);
  if (rec) rec->begin("residual_other", 0);
  ki::launch(k_residual, grid_for((size_t)N * ncols), 256, 0, s, r1, N, y1, N, N, ncols, r1, N);
  if (nb > 0) ki::launch(k_residual, grid_for((size_t)nb * ncols), 256, 0, s, r2, nb, y2, nb, nb, ncols, r2, nb);
  KI_CHECK_CUDA(cudaGetLastError());
  const double worst = column_norms(f, b, r1, r2, ncols, work, rel, s);
  if (rec) rec->end();
  return worst;
}

// Per-column ||[r1; r2]|| / ||b|| (host vector rel), returns the largest.
double column_norms(ki_factor* f, const double* b, const double* r1, const double* r2, int ncols,
                    double* work, std::vector<double>* rel, cudaStream_t s) {
  const int N = f->n_dofs, nb = f->n_border;
  // work: part (kNormBlocks x ncols) | sq_r (ncols) | sq_b (ncols)
  double* part = work;
  double* sq = work + (size_t)kNormBlocks * ncols;
  double* sqb = sq + ncols;
  ki::launch(k_colsq_partial, dim3(kNormBlocks, ncols), 256, 0, s, r1, N, N, part);
  ki::launch(k_colsq_final, (ncols + 127) / 128, 128, 0, s, part, kNormBlocks, ncols, sq, 0);
  if (nb > 0) {
    ki::launch(k_colsq_partial, dim3(1, ncols), 256, 0, s, r2, nb, nb, part);
    ki::launch(k_colsq_final, (ncols + 127) / 128, 128, 0, s, part, 1, ncols, sq, 1);
  }
  ki::launch(k_colsq_partial, dim3(kNormBlocks, ncols), 256, 0, s, b, N, N, part);
  ki::launch(k_colsq_final, (ncols + 127) / 128, 128, 0, s, part, kNormBlocks, ncols, sqb, 0);
  KI_CHECK_CUDA(cudaGetLastError());
  std::vector<double> h(2 * (size_t)ncols);
  KI_CHECK_CUDA(cudaMemcpyAsync(h.data(), sq, sizeof(double) * 2 * ncols, cudaMemcpyDeviceToHost, s));
  KI_CHECK_CUDA(cudaStreamSynchronize(s));
  double worst = 0.0;
  rel->assign(ncols, 0.0);
  for (int c = 0; c < ncols; c++) {
    double v = h[ncols + c] > 0 ? std::sqrt(h[c] / h[ncols + c]) : std::sqrt(h[c]);
    (*rel)[c] = v;
    worst = std::max(worst, v);
  }
  return worst;
}

// One correction: [mu; alpha] += M^-1 [r1; r2], M the factorization (precision T).
// With dcol / dal, the correction is also stored there in FP64 (column-
// major, ld = N / nb).
template <typename T>
void correct(ki_factor* f, ki::Factorization<T>& F, const double* r1, const double* r2, int ncols,
             double* mu, double* alpha, cudaStream_t s, double* dcol = nullptr,
             double* dal = nullptr) {
  const int N = f->n_dofs, nb = f->n_border;
  DevBuf<T> work((size_t)N * ncols, s), al((size_t)std::max(1, nb) * ncols, s),
      g((size_t)std::max(1, nb) * ncols, s);
  ki::launch(k_to_dofmajor<double, T>, grid_for((size_t)N * ncols), 256, 0, s, r1, N, N, ncols, work.p);
  if (nb > 0) ki::launch(k_to_rowmajor<T>, grid_for((size_t)nb * ncols), 256, 0, s, r2, nb, nb, ncols, g.p);
  KI_CHECK_CUDA(cudaGetLastError());
  cudaStream_t saved = F.stream;
  F.stream = s;
  try {
    ki::solve_device<T>(F, work.p, ncols, al.p, nb > 0 ? g.p : nullptr);
  } catch (...) {
    F.stream = saved;
    throw;
  }
  F.stream = saved;
  ki::launch(k_add_dofmajor<T>, grid_for((size_t)N * ncols), 256, 0, s, work.p, N, ncols, mu, N, dcol);
  if (nb > 0)
    ki::launch(k_add_rowmajor<T>, grid_for((size_t)nb * ncols), 256, 0, s, al.p, nb, ncols, alpha, nb, dal);
  KI_CHECK_CUDA(cudaGetLastError());
}

// Refined solve on device buffers (b, mu: N x ncols, alpha: nb x ncols,
// column-major with ld = N / nb).
void refined_solve(ki_factor* f, const double* b, int ncols, double* mu, double* alpha,
                   double tol, int max_steps, ki_refine_info* info, cudaStream_t s) {
  const int N = f->n_dofs, nb = f->n_border;
  DevBuf<double> r1((size_t)N * ncols, s), r2((size_t)std::max(1, nb) * ncols, s),
      work((size_t)(kNormBlocks + 2) * ncols, s);
  KI_CHECK_CUDA(cudaMemsetAsync(mu, 0, sizeof(double) * (size_t)N * ncols, s));
  if (nb > 0) KI_CHECK_CUDA(cudaMemsetAsync(alpha, 0, sizeof(double) * (size_t)nb * ncols, s));
  KI_CHECK_CUDA(cudaMemcpyAsync(r1.p, b, sizeof(double) * (size_t)N * ncols, cudaMemcpyDeviceToDevice, s));
  if (nb > 0) KI_CHECK_CUDA(cudaMemsetAsync(r2.p, 0, sizeof(double) * (size_t)nb * ncols, s));
  RefineRecorder recorder(f, s);
  ki::StageRecorder* rec = f->profile_refine ? &recorder : nullptr;
  // residual updates (see ki_solve_refined): the low-accuracy FMM apply of
  // the correction instead of a new FP64 product, while the accumulated
  // drift bound stays below tol / 20
  const char* ue = std::getenv("KI_REFINE_UPDATE");
  const bool may_update = use_fmm(f) && !(ue && std::string(ue) == "0");
  DevBuf<double> dcol(may_update ? (size_t)N * ncols : 1, s),
      dal(may_update ? (size_t)std::max(1, nb) * ncols : 1, s),
      y1(may_update ? (size_t)N * ncols : 1, s),
      y2(may_update ? (size_t)std::max(1, nb) * ncols : 1, s);
  auto corr = [&](bool keep) {
    if (rec) rec->begin("precond_solve", 0);
    double* dc = keep ? dcol.p : nullptr;
    double* da = keep && nb > 0 ? dal.p : nullptr;
    if (f->f64) correct<double>(f, *f->f64, r1.p, r2.p, ncols, mu, alpha, s, dc, da);
    else correct<float>(f, *f->f32, r1.p, r2.p, ncols, mu, alpha, s, dc, da);
    if (rec) rec->end();
  };
  corr(false);   // x0 = M^-1 b
  std::vector<double> rel, rel_old;
  double res = residual_norms(f, b, mu, alpha, ncols, r1.p, r2.p, work.p, &rel, s, tol, rec);
  info->residual0 = res;
  std::vector<double> drift(ncols, 0.0);
  auto bound = [&] {
    double w = 0.0;
    for (int c = 0; c < ncols; c++) w = std::max(w, rel[c] + drift[c]);
    return w;
  };
  int steps = 0, updates = 0;
  while (bound() > tol && steps < max_steps) {
    // an update is tried when the bound stays below tol / 20 in every
    // column for a correction that removes most of the residual
    // (||r_after|| << ||r_before||); if the actual ||r_after|| pushes it
    // over, the FP64 residual is recomputed (and the bound reset) after all
    bool update = may_update;
    for (int c = 0; c < ncols && update; c++)
      update = drift[c] + kLowRelErr * rel[c] <= tol / 20;
    corr(update);
    steps++;
    bool recompute = !update;
    if (update) {
      rel_old = rel;
      res = update_residual(f, b, dcol.p, nb > 0 ? dal.p : nullptr, ncols, r1.p, r2.p, y1.p,
                            y2.p, work.p, &rel, s, rec);
      for (int c = 0; c < ncols; c++) {
        drift[c] += kLowRelErr * (rel_old[c] + rel[c]);
        recompute = recompute || drift[c] > tol / 20;
      }
      updates++;
    }
    if (recompute) {
      res = residual_norms(f, b, mu, alpha, ncols, r1.p, r2.p, work.p, &rel, s, tol, rec);
      std::fill(drift.begin(), drift.end(), 0.0);
    }
  }
  info->steps = steps;
  info->residual = bound();
  info->updates = updates;
  info->drift_bound = *std::max_element(drift.begin(), drift.end());
  if (rec) {
    // aggregate this solve's records by stage
    KI_CHECK_CUDA(cudaStreamSynchronize(s));
    f->refine_prof.clear();
    for (auto& r : f->refine_open) {
      float ms = 0;
      KI_CHECK_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
      auto it = std::find_if(f->refine_prof.begin(), f->refine_prof.end(),
                             [&](const ki::StageSum& q) { return q.stage == r.stage; });
      if (it == f->refine_prof.end()) {
        f->refine_prof.push_back(ki::StageSum{r.stage, 0, 0, 0, 0});
        it = f->refine_prof.end() - 1;
      }
      it->launches++;
      it->ms += ms;
      it->flops += r.flops;
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
    f->refine_open.clear();
  }
}

}  // namespace

// The bordered FP64 operator: K by the FMM (2D Laplace, n_dofs >= 4096 or
// KI_RESIDUAL_APPLY=fmm) or the dense Nystrom apply (one thread per target
// DOF, sources through shared memory; KI_RESIDUAL_APPLY=dense forces it),
// border columns, Psi rows.
namespace {
bool fmm_capable(const ki_factor* f) {
  return f->dim == 2 && f->sol_dim == 1 && f->pde == KI_PDE_LAPLACE;
}

// Expansion terms of the FMM plan (translation matrices for every lower
// order are leading blocks, so one plan serves any accuracy).
int fmm_order() {
  int p = 32;
  if (const char* e = std::getenv("KI_FMM_P")) p = std::atoi(e);
  return p;
}

// Terms for a refinement target: the smallest order whose expected relative
// error, 1.4e-8 * 0.43^(p - 16) (measured max-norm error of K x for random x
// on the 2D Laplace disc-with-ellipses family at 1,048,576 unknowns: 1.4e-8
// at 16 terms, 4.8e-10 at 20, 1.6e-11 at 24), is 20x below the target.
int fmm_order_for(double target, int plan_order) {
  if (const char* e = std::getenv("KI_FMM_P")) return std::atoi(e);
  int p = 12;
  while (p < plan_order && 1.4e-8 * std::pow(0.43, p - 16) > target / 20) p++;
  return p;
}

ki::Fmm2d& fmm_for(ki_factor* f, cudaStream_t s) {
  if (!f->fmm && f->fmm_ready.valid()) {
    const auto t0 = std::chrono::steady_clock::now();
    f->fmm = f->fmm_ready.get();   // uploaded: the worker synchronized its stream
    f->fmm_wait_ms = std::chrono::duration<double, std::milli>(
                         std::chrono::steady_clock::now() - t0).count();
  }
  if (!f->fmm) {
    // geometry back from the device copy (the handle keeps no host arrays)
    const int n = f->n_points;
    std::vector<double> geo((size_t)6 * n), pts(2 * (size_t)n), nrm(2 * (size_t)n);
    KI_CHECK_CUDA(cudaMemcpyAsync(geo.data(), f->d_geo, sizeof(double) * geo.size(),
                                  cudaMemcpyDeviceToHost, s));
    KI_CHECK_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < n; i++) {
      pts[2 * i] = geo[i];
      pts[2 * i + 1] = geo[n + i];
      nrm[2 * i] = geo[2 * (size_t)n + i];
      nrm[2 * i + 1] = geo[3 * (size_t)n + i];
    }
    f->fmm = ki::fmm2d_build(pts.data(), nrm.data(), geo.data() + 4 * (size_t)n,
                             geo.data() + 5 * (size_t)n, n, fmm_order(), s);
  }
  return *f->fmm;
}

bool use_fmm(const ki_factor* f) {
  if (!fmm_capable(f)) return false;
  const char* e = std::getenv("KI_RESIDUAL_APPLY");
  if (e && std::string(e) == "dense") return false;
  if (e && std::string(e) == "fmm") return true;
  return f->n_dofs >= 4096;
}

// fast: FMM with `order` terms (0: 24, relative error ~2e-11)
void apply_K(ki_factor* f, const double* mu, int ncols, double* y1, cudaStream_t s, bool fast,
             int order = 0, ki::StageRecorder* rec = nullptr,
             ki::FmmArith arith = ki::FmmArith::kF64) {
  const int N = f->n_dofs;
  if (fast) {
    ki::Fmm2d& F = fmm_for(f, s);
    ki::fmm2d_apply(F, mu, N, ncols, y1, N, s, order > 0 ? order : std::min(24, ki::fmm2d_order(F)),
                    rec, arith);
    return;
  }
  if (rec) rec->begin("dense_apply", 0);
  dense_product(f->P, f->n_points, f->sol_dim, mu, N, ncols, y1, N, nullptr, 0, nullptr, s);
  if (rec) rec->end();
}

void apply_bordered(ki_factor* f, const double* mu, const double* alpha, int ncols, double* y1,
                    double* y2, cudaStream_t s, double target, ki::StageRecorder* rec, bool low) {
  const int N = f->n_dofs, nb = f->n_border;
  const bool fast = use_fmm(f);
  if (low && !fast) throw std::logic_error("low-accuracy apply without the FMM");
  if (low)
    apply_K(f, mu, ncols, y1, s, true, kLowOrder, rec, ki::FmmArith::kF32);
  else
    apply_K(f, mu, ncols, y1, s, fast,
            fast ? fmm_order_for(target, ki::fmm2d_order(fmm_for(f, s))) : 0, rec);
  if (nb > 0) {
    if (rec) rec->begin("border_apply", 0);
    const size_t tsm = low ? border_tile_smem<float>(nb) : border_tile_smem<double>(nb);
    if (tsm <= 100 * 1024) {
      auto tile = low ? k_border_apply_tile<float> : k_border_apply_tile<double>;
      if (!low)
        KI_CHECK_CUDA(cudaMemcpyToSymbolAsync(g_border_logc, border_log_table(), sizeof(float2) * 256, 0,
                                              cudaMemcpyHostToDevice, s));
      KI_CHECK_CUDA(cudaFuncSetAttribute(tile, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         100 * 1024));
      ki::launch(tile, (N + kBorderTile - 1) / kBorderTile, 256, tsm, s,
          f->P.x, f->P.y, f->P.z, f->n_points, f->dim, f->sol_dim, f->d_holes, f->n_holes, alpha,
          nb, ncols, y1, N);
    } else {
      auto border = low ? k_border_apply<float> : k_border_apply<double>;
      ki::launch(border, (N + 127) / 128, 128, 0, s, f->P.x, f->P.y, f->P.z, 1, f->n_points, f->dim,
                                             f->sol_dim, f->d_holes, f->n_holes, alpha, nb, ncols,
                                             y1, N, nullptr, 0);
    }
    const int cph = nb / f->n_holes;
    ki::launch(k_psi_apply, dim3(nb, ncols), 256, 0, s, f->d_pts, f->P.w, f->dim, f->sol_dim, f->d_holes,
                                                f->d_hstart, f->d_hcount, cph, mu, N, alpha, nb,
                                                y2, nb);
    KI_CHECK_CUDA(cudaGetLastError());
    if (rec) rec->end();
  }
}
}  // namespace

namespace {

// Timing of one factorization (and, for the sweep knob, one solve of nrhs
// columns) with the tuner's recording on: device ms per (knob, bucket).
template <typename T>
void tune_times(ki_factor* f, ki::Factorization<T>& F, int knob, const double* d_b, double* d_x,
                double* d_al, int nrhs, std::map<int, double>* out) {
  // the factorization's records (its border sweeps included), and for the
  // sweep knob a solve's
  std::vector<ki::StageSum> recs = F.factor_prof;
  if (knob == ki::kTuneSweep) {
    solve_impl<T>(f, F, d_b, f->n_dofs, nrhs, d_x, f->n_dofs, d_al, std::max(1, f->n_border), f->stream);
    KI_CHECK_CUDA(cudaStreamSynchronize(f->stream));
    const std::vector<ki::StageSum> sv = F.collect();
    recs.insert(recs.end(), sv.begin(), sv.end());
  }
  for (const auto& r : recs) {
    int k = -1, b = -1;
    if (ki::tune_parse_stage(r.stage, &k, &b) && k == knob) (*out)[b] += r.ms;
  }
}

}  // namespace

extern "C" {

namespace {

// A new handle's state for desc (ki_factor_create).  With prev (a handle of
// the same problem before a boundary perturbation, same precision, sizes,
// parameters and rank model), the boxes of prev's factorization that the
// perturbation left unchanged are copied rather than recomputed.
void build_factor(ki_factor* f, const ki_problem_desc* desc_in, const ki_factor* prev,
                  bool plan_fmm = true) {
  const auto t_create = std::chrono::steady_clock::now();
  // the Neumann and Gaussian problems have no border: the reference's
  // initialize_U_mat / initialize_Psi_mat give them empty matrices
  // (kern_interp/linear_solve.cpp:101-104, :193-196), so holes are ignored;
  // absent normals and weights (Gaussian kernel) read as zeros
  ki_problem_desc dd = *desc_in;
  const ki_problem_desc* desc = &dd;
  const bool scalar_other = dd.pde == KI_PDE_LAPLACE_NEUMANN || dd.pde == KI_PDE_GAUSS;
  if (scalar_other) dd.n_holes = 0;
  std::vector<double> zeros;
  if (!dd.normals || !dd.weights) {
    zeros.assign((size_t)dd.domain_dimension * dd.n_points, 0.0);
    if (!dd.normals) dd.normals = zeros.data();
    if (!dd.weights) dd.weights = zeros.data();
  }
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) {
    cudaGetLastError();
    throw std::runtime_error("no CUDA device available");
  }
  f->precision = desc->precision;
  const int dim = desc->domain_dimension;
  f->dim = dim;
  f->sol_dim = desc->solution_dimension;
  f->pde = desc->pde;
  f->n_points = desc->n_points;
  f->n_dofs = desc->n_points * desc->solution_dimension;
  f->n_holes = desc->n_holes;
  f->n_border = desc->n_holes * ki::border_cols_per_hole(dim, desc->solution_dimension);
  KI_CHECK_CUDA(cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking));
  ki::Params prm;
  prm.dim = dim;
  prm.sol_dim = desc->solution_dimension;
  prm.pde = scalar_other ? desc->pde : 0;   // ki::kPdeNeumann / ki::kPdeGauss
  prm.max_leaf_dofs = desc->max_leaf_dofs ? desc->max_leaf_dofs : 64;
  // reference defaults: NUM_PROXY_POINTS = 128 (2D); the 3D proxy sphere is
  // the Kernel constructor's 8 x 4 grid (kern_interp/kernel/kernel.h:44-62)
  prm.num_proxy_points = desc->num_proxy_points ? desc->num_proxy_points : (dim == 2 ? 128 : 32);
  prm.radius_ratio = desc->radius_ratio > 0 ? desc->radius_ratio : 2.0;
  prm.min_dofs_to_compress = desc->min_dofs_to_compress ? desc->min_dofs_to_compress : 64;
  prm.id_tol = desc->id_tol;
  if (desc->rank_model && desc->precision == KI_PRECISION_FP32) {
    for (int i = 0; i < ki::kMlpModelFloats; i++)
      if (!std::isfinite(desc->rank_model[i])) throw ArgError("non-finite rank model");
    KI_CHECK_CUDA(cudaMalloc(&f->d_rank_model, sizeof(float) * ki::kMlpModelFloats));
    KI_CHECK_CUDA(cudaMemcpy(f->d_rank_model, desc->rank_model, sizeof(float) * ki::kMlpModelFloats,
                             cudaMemcpyHostToDevice));
    prm.rank_model = f->d_rank_model;
    f->rank_model_host.assign(desc->rank_model, desc->rank_model + ki::kMlpModelFloats);
  }
  ki::HoleDesc holes;
  holes.n_holes = desc->n_holes;
  for (int h = 0; h < desc->n_holes; h++) {
    for (int d = 0; d < dim; d++) holes.centers.push_back(desc->hole_centers[dim * h + d]);
    holes.start.push_back(desc->hole_node_start[h]);
    holes.count.push_back(desc->hole_node_count[h]);
  }
  // the caller's arrays uploaded once, interleaved as given: points (dim n) |
  // normals (dim n) | weights (n) | curvatures (n); the factorization reads
  // them in place, and the FP64 SoA geometry of the apply / evaluation
  // kernels is formed from them on the device
  const int n = desc->n_points;
  {
    const size_t nn = (size_t)n;
    KI_CHECK_CUDA(cudaMalloc(&f->d_pts, sizeof(double) * (2 * dim + 2) * nn));
    double* d_in = f->d_pts;
    KI_CHECK_CUDA(cudaMemcpyAsync(d_in, desc->points, sizeof(double) * dim * nn,
                                  cudaMemcpyHostToDevice, f->stream));
    KI_CHECK_CUDA(cudaMemcpyAsync(d_in + dim * nn, desc->normals, sizeof(double) * dim * nn,
                                  cudaMemcpyHostToDevice, f->stream));
    KI_CHECK_CUDA(cudaMemcpyAsync(d_in + 2 * dim * nn, desc->weights, sizeof(double) * nn,
                                  cudaMemcpyHostToDevice, f->stream));
    if (desc->curvatures)
      KI_CHECK_CUDA(cudaMemcpyAsync(d_in + (2 * dim + 1) * nn, desc->curvatures,
                                    sizeof(double) * nn, cudaMemcpyHostToDevice, f->stream));
    KI_CHECK_CUDA(cudaMalloc(&f->d_geo, sizeof(double) * 8 * nn));
    ki::launch(k_geo_soa, std::min(2048, (n + 255) / 256), 256, 0, f->stream,
        d_in, n, dim, desc->curvatures != nullptr, f->d_geo);
    KI_CHECK_CUDA(cudaGetLastError());
  }
  f->P = ki::Points<double>{f->d_geo, f->d_geo + n, f->d_geo + 2 * (size_t)n,
                            f->d_geo + 3 * (size_t)n, f->d_geo + 4 * (size_t)n,
                            f->d_geo + 5 * (size_t)n};
  f->P.dim = dim;
  f->P.pde = prm.pde;
  if (dim == 3) {
    f->P.z = f->d_geo + 6 * (size_t)n;
    f->P.nz = f->d_geo + 7 * (size_t)n;
  }
  if (desc->n_holes > 0) {
    KI_CHECK_CUDA(cudaMalloc(&f->d_holes, sizeof(double) * dim * desc->n_holes));
    KI_CHECK_CUDA(cudaMemcpy(f->d_holes, desc->hole_centers, sizeof(double) * dim * desc->n_holes,
                             cudaMemcpyHostToDevice));
    KI_CHECK_CUDA(cudaMalloc(&f->d_hstart, sizeof(int) * 2 * desc->n_holes));
    f->d_hcount = f->d_hstart + desc->n_holes;
    KI_CHECK_CUDA(cudaMemcpy(f->d_hstart, desc->hole_node_start, sizeof(int) * desc->n_holes,
                             cudaMemcpyHostToDevice));
    KI_CHECK_CUDA(cudaMemcpy(f->d_hcount, desc->hole_node_count, sizeof(int) * desc->n_holes,
                             cudaMemcpyHostToDevice));
  }

  // 2D Laplace: the FMM for refinement residuals, planned and uploaded by a
  // worker thread on its own stream, concurrent with the factorization (it
  // copies the caller's arrays first, and this call returns only after the
  // copy; it plans once the factorization's tree is built, so that the two
  // do not compete for the host cores)
  std::promise<void> copied;
  std::future<void> copied_f = copied.get_future();
  std::promise<void> tree_done;
  std::shared_future<void> tree_done_f = tree_done.get_future().share();
  bool tree_signalled = false;
  auto signal_tree = [&] {
    if (!tree_signalled) {
      tree_signalled = true;
      tree_done.set_value();
    }
  };
  bool planning = false;
  if (plan_fmm && fmm_capable(f) && f->n_dofs >= 4096 && !std::getenv("KI_NO_FMM_PREPLAN")) {
    planning = true;
    const double *pp = desc->points, *nn = desc->normals, *ww = desc->weights,
                 *kk = desc->curvatures;
    const int order = fmm_order();
    KI_CHECK_CUDA(cudaStreamCreateWithFlags(&f->fmm_stream, cudaStreamNonBlocking));
    cudaStream_t us = f->fmm_stream;
    int dev = 0;
    KI_CHECK_CUDA(cudaGetDevice(&dev));
    f->fmm_ready = std::async(std::launch::async, [pp, nn, ww, kk, n, order, us, dev, &copied,
                                                    tree_done_f] {
      std::vector<double> P, Nn, W, K;
      try {
        P.assign(pp, pp + 2 * (size_t)n);
        Nn.assign(nn, nn + 2 * (size_t)n);
        W.assign(ww, ww + n);
        if (kk) K.assign(kk, kk + n);
        else K.assign(n, 0.0);
      } catch (...) {
        copied.set_value();
        throw;
      }
      copied.set_value();
      tree_done_f.wait();
      auto plan = ki::fmm2d_plan(P.data(), Nn.data(), W.data(), K.data(), n, order);
      KI_CHECK_CUDA(cudaSetDevice(dev));   // the caller's device, not the thread default
      return ki::fmm2d_upload(*plan, us);
    });
  }
  struct WaitCopy {   // the caller's arrays stay valid until the worker has copied them;
                      // the worker is released from its wait on every path out
    bool on;
    std::future<void>& fut;
    std::function<void()> release;
    ~WaitCopy() {
      release();
      if (on) fut.wait();
    }
  } wait_copy{planning, copied_f, signal_tree};
  const auto t_factor = std::chrono::steady_clock::now();
  f->host_prep_ms = std::chrono::duration<double, std::milli>(t_factor - t_create).count();
  // prev's factorization serves only a problem of the same kind and size
  // with the same rank model (factorize checks the parameters)
  const bool reuse = prev && prev->precision == f->precision && prev->dim == f->dim &&
                     prev->sol_dim == f->sol_dim && prev->pde == f->pde &&
                     prev->n_points == f->n_points &&
                     prev->rank_model_host == f->rank_model_host;
  if (f->precision == KI_PRECISION_FP64)
    f->f64 = ki::factorize<double>(prm, n, desc->points, desc->normals, desc->weights,
                                   desc->curvatures, holes, f->stream, f->d_pts, signal_tree,
                                   reuse ? prev->f64.get() : nullptr);
  else
    f->f32 = ki::factorize<float>(prm, n, desc->points, desc->normals, desc->weights,
                                  desc->curvatures, holes, f->stream, f->d_pts, signal_tree,
                                  reuse ? prev->f32.get() : nullptr);
  f->host_factor_ms = std::chrono::duration<double, std::milli>(
                          std::chrono::steady_clock::now() - t_factor).count();
  // the FP64 3D diagonal of the factorization serves the FP64 apply
  f->P.diag = f->f64 ? f->f64->d_diag64 : f->f32->d_diag64;
}

}  // namespace

int ki_factor_create(const ki_problem_desc* desc, ki_factor** out) {
  return guarded([&] {
    if (!out) throw ArgError("out is NULL");
    *out = nullptr;
    check_desc(desc);
    std::unique_ptr<ki_factor> f(new ki_factor());
    build_factor(f.get(), desc, nullptr);
    *out = f.release();
  });
}

int ki_tune_set(const char* json) {
  return guarded([&] {
    if (!json) throw ArgError("json is NULL");
    try {
      ki::tune_from_json(json);
    } catch (const std::invalid_argument& e) {
      throw ArgError(e.what());
    }
  });
}

int ki_tune_get(char* buf, int len) {
  return guarded([&] {
    const std::string js = ki::tune_to_json();
    if (!buf || len < (int)js.size() + 1) throw ArgError("buffer too small: need " + std::to_string(js.size() + 1));
    std::memcpy(buf, js.c_str(), js.size() + 1);
  });
}

int ki_autotune(const ki_problem_desc* desc, int nrhs, int repeats, char* out, int len) {
  return guarded([&] {
    check_desc(desc);
    if (nrhs <= 0 || repeats <= 0) throw ArgError("nrhs and repeats must be positive");
    if (!out || len <= 0) throw ArgError("output buffer is NULL");
    struct Restore {
      ~Restore() {
        ki::tune_set_recording(false);
        for (int k = 0; k < ki::kTuneKnobs; k++) ki::tune_force(k, -1);
      }
    } restore;
    ki::tune_set_recording(true);
    const bool fp64 = desc->precision == KI_PRECISION_FP64;
    const size_t N = (size_t)desc->n_points * desc->solution_dimension;
    const int nb_max = std::max(1, desc->n_holes * 6);
    // right-hand sides: a fixed pseudo-random set (the sweeps' cost does not
    // depend on the values)
    std::vector<double> hb(N * nrhs);
    uint64_t st = 0x9e3779b97f4a7c15ull;
    for (auto& v : hb) {
      st = st * 6364136223846793005ull + 1442695040888963407ull;
      v = (double)(st >> 11) * (1.0 / 9007199254740992.0) - 0.5;
    }
    DevBuf<double> d_b(N * nrhs, nullptr), d_x(N * nrhs, nullptr), d_al((size_t)nb_max * nrhs, nullptr);
    KI_CHECK_CUDA(cudaMemcpy(d_b.p, hb.data(), sizeof(double) * hb.size(), cudaMemcpyHostToDevice));
    std::string report = "{";
    for (int knob = 0; knob < ki::kTuneKnobs; knob++) {
      int ncand = ki::kTuneCandidates[knob];
      if (fp64 && knob != ki::kTuneSweep) ncand = 2;   // FP64: fold rows / 128-256 threads only
      std::map<int, std::vector<double>> ms;            // bucket -> best ms per candidate
      for (int c = 0; c < ncand; c++) {
        ki::tune_force(knob, c);
        for (int rep = 0; rep < repeats; rep++) {
          std::unique_ptr<ki_factor> f(new ki_factor());
          build_factor(f.get(), desc, nullptr, false);
          std::map<int, double> t;
          if (f->f64) tune_times<double>(f.get(), *f->f64, knob, d_b.p, d_x.p, d_al.p, nrhs, &t);
          else tune_times<float>(f.get(), *f->f32, knob, d_b.p, d_x.p, d_al.p, nrhs, &t);
          for (const auto& kv : t) {
            auto& v = ms[kv.first];
            if (v.empty()) v.assign(ncand, -1.0);
            if (v[c] < 0 || kv.second < v[c]) v[c] = kv.second;
          }
        }
      }
      ki::tune_force(knob, -1);
      for (const auto& kv : ms) {
        int best = -1;
        for (int c = 0; c < ncand; c++)
          if (kv.second[c] >= 0 && (best < 0 || kv.second[c] < kv.second[best])) best = c;
        if (best >= 0) ki::tune_set(knob, kv.first, best);
        report += (report.size() > 1 ? ", " : "") + std::string("\"") +
                  ki::tune_stage(knob, kv.first).substr(5) + "\": [";
        for (int c = 0; c < ncand; c++) {
          char num[32];
          std::snprintf(num, sizeof(num), "%s%.6f", c ? ", " : "", kv.second[c]);
          report += num;
        }
        report += "]";
      }
    }
    report += "}";
    const std::string js = "{\"table\": " + ki::tune_to_json() + ", \"ms\": " + report + "}";
    if (len < (int)js.size() + 1) throw ArgError("buffer too small: need " + std::to_string(js.size() + 1));
    std::memcpy(out, js.c_str(), js.size() + 1);
  });
}

int ki_factor_update(ki_factor* f, const ki_problem_desc* desc) {
  return guarded([&] {
    if (!f) throw ArgError("f is NULL");
    check_desc(desc);
    // the old state stays in f until the new one is complete: a failure
    // leaves the handle as it was
    std::unique_ptr<ki_factor> nf(new ki_factor());
    nf->profile_refine = f->profile_refine;
    build_factor(nf.get(), desc, f);
    f->swap_state(*nf);
  });
}

int ki_factor_destroy(ki_factor* f) {
  return guarded([&] { delete f; });
}

int ki_factor_get_info(const ki_factor* f, ki_factor_info* info) {
  return guarded([&] {
    if (!f || !info) throw ArgError("NULL argument");
    std::memset(info, 0, sizeof(*info));
    info->n_dofs = f->n_dofs;
    info->n_border = f->n_border;
    auto fill = [&](const auto& F) {
      info->n_levels = F.tree.num_levels();
      info->n_compressed = F.n_compressed;
      info->n_redundant = F.n_redundant;
      info->n_root = F.n_root;
      info->factor_seconds = F.factor_seconds;
      info->device_bytes = (long)F.device_bytes;
      info->n_sketched = F.n_sketched;
      info->n_fallback = F.n_fallback;
      info->n_reused = F.n_reused;
    };
    if (f->f64) fill(*f->f64);
    if (f->f32) fill(*f->f32);
  });
}

int ki_solve_device(ki_factor* f, const double* d_b, int ldb, int nrhs, double* d_x, int ldx,
                    double* d_alpha, int ldalpha, void* stream) {
  return guarded([&] {
    if (!f) throw ArgError("factor is NULL");
    if (nrhs < 0 || ldb < f->n_dofs || ldx < f->n_dofs) throw ArgError("bad leading dimension / nrhs");
    if (f->n_border > 0 && d_alpha && ldalpha < f->n_border) throw ArgError("bad ldalpha");
    if (nrhs == 0) return;
    if (!d_b || !d_x) throw ArgError("NULL b or x");
    cudaStream_t s = stream ? (cudaStream_t)stream : f->stream;
    if (f->f64) solve_impl<double>(f, *f->f64, d_b, ldb, nrhs, d_x, ldx, d_alpha, ldalpha, s);
    else solve_impl<float>(f, *f->f32, d_b, ldb, nrhs, d_x, ldx, d_alpha, ldalpha, s);
  });
}

int ki_solve_device_noalloc(ki_factor* f, const double* d_b, int ldb, int nrhs, double* d_x,
                            int ldx, double* d_alpha, int ldalpha, void* stream) {
  return guarded([&] {
    if (!f) throw ArgError("factor is NULL");
    if (nrhs < 0 || ldb < f->n_dofs || ldx < f->n_dofs) throw ArgError("bad leading dimension / nrhs");
    if (f->n_border > 0 && d_alpha && ldalpha < f->n_border) throw ArgError("bad ldalpha");
    if (nrhs == 0) return;
    if (!d_b || !d_x) throw ArgError("NULL b or x");
    cudaStream_t s = stream ? (cudaStream_t)stream : f->stream;
    if (f->f64) solve_impl_noalloc<double>(f, *f->f64, d_b, ldb, nrhs, d_x, ldx, d_alpha, ldalpha, s);
    else solve_impl_noalloc<float>(f, *f->f32, d_b, ldb, nrhs, d_x, ldx, d_alpha, ldalpha, s);
  });
}

int ki_solve(ki_factor* f, const double* b, int ldb, int nrhs, double* x, int ldx, double* alpha,
             int ldalpha) {
  return guarded([&] {
    if (!f) throw ArgError("factor is NULL");
    if (nrhs < 0 || ldb < f->n_dofs || ldx < f->n_dofs) throw ArgError("bad leading dimension / nrhs");
    if (f->n_border > 0 && alpha && ldalpha < f->n_border) throw ArgError("bad ldalpha");
    if (nrhs == 0) return;
    if (!b || !x) throw ArgError("NULL b or x");
    cudaStream_t s = f->stream;
    const int N = f->n_dofs;
    DevBuf<double> db((size_t)N * nrhs, s), dx((size_t)N * nrhs, s);
    DevBuf<double> da((size_t)std::max(1, f->n_border) * nrhs, s);
    KI_CHECK_CUDA(cudaMemcpy2DAsync(db.p, sizeof(double) * N, b, sizeof(double) * ldb,
                                    sizeof(double) * N, nrhs, cudaMemcpyHostToDevice, s));
    if (f->f64) solve_impl<double>(f, *f->f64, db.p, N, nrhs, dx.p, N, da.p, f->n_border, s);
    else solve_impl<float>(f, *f->f32, db.p, N, nrhs, dx.p, N, da.p, f->n_border, s);
    KI_CHECK_CUDA(cudaMemcpy2DAsync(x, sizeof(double) * ldx, dx.p, sizeof(double) * N,
                                    sizeof(double) * N, nrhs, cudaMemcpyDeviceToHost, s));
    if (f->n_border > 0 && alpha)
      KI_CHECK_CUDA(cudaMemcpy2DAsync(alpha, sizeof(double) * ldalpha, da.p,
                                      sizeof(double) * f->n_border, sizeof(double) * f->n_border,
                                      nrhs, cudaMemcpyDeviceToHost, s));
    KI_CHECK_CUDA(cudaStreamSynchronize(s));
  });
}

int ki_apply(ki_factor* f, const double* x, int ldx, int ncols, const double* alpha, int ldalpha,
             double* y, int ldy) {
  return guarded([&] {
    if (!f || !x || !y) throw ArgError("NULL argument");
    const int N = f->n_dofs;
    if (ncols < 0 || ldx < N || ldy < N) throw ArgError("bad leading dimension / ncols");
    if (ncols == 0) return;
    cudaStream_t s = f->stream;
    DevBuf<double> dx((size_t)N * ncols, s), dy((size_t)N * ncols, s);
    KI_CHECK_CUDA(cudaMemcpy2DAsync(dx.p, sizeof(double) * N, x, sizeof(double) * ldx,
                                    sizeof(double) * N, ncols, cudaMemcpyHostToDevice, s));
    dense_product(f->P, f->n_points, f->sol_dim, dx.p, N, ncols, dy.p, N, nullptr, 0, nullptr, s);
    if (f->n_border > 0 && alpha) {
      if (ldalpha < f->n_border) throw ArgError("bad ldalpha");
      DevBuf<double> da((size_t)f->n_border * ncols, s);
      KI_CHECK_CUDA(cudaMemcpy2DAsync(da.p, sizeof(double) * f->n_border, alpha,
                                      sizeof(double) * ldalpha, sizeof(double) * f->n_border,
                                      ncols, cudaMemcpyHostToDevice, s));
      ki::launch(k_border_apply<double>, (N + 127) / 128, 128, 0, s,
          f->P.x, f->P.y, f->P.z, 1, f->n_points, f->dim, f->sol_dim, f->d_holes, f->n_holes, da.p,
          f->n_border, ncols, dy.p, N, (const int*)nullptr, 0);
      KI_CHECK_CUDA(cudaGetLastError());
      KI_CHECK_CUDA(cudaMemcpy2DAsync(y, sizeof(double) * ldy, dy.p, sizeof(double) * N,
                                      sizeof(double) * N, ncols, cudaMemcpyDeviceToHost, s));
      KI_CHECK_CUDA(cudaStreamSynchronize(s));
      return;
    }
    KI_CHECK_CUDA(cudaMemcpy2DAsync(y, sizeof(double) * ldy, dy.p, sizeof(double) * N,
                                    sizeof(double) * N, ncols, cudaMemcpyDeviceToHost, s));
    KI_CHECK_CUDA(cudaStreamSynchronize(s));
  });
}

int ki_apply_fmm(ki_factor* f, const double* x, int ldx, int ncols, const double* alpha,
                 int ldalpha, double* y, int ldy) {
  return ki_apply_fmm_ex(f, x, ldx, ncols, alpha, ldalpha, y, ldy, 0, 0);
}

int ki_apply_fmm_ex(ki_factor* f, const double* x, int ldx, int ncols, const double* alpha,
                    int ldalpha, double* y, int ldy, int order, int fp32) {
  return guarded([&] {
    if (!f || !x || !y) throw ArgError("NULL argument");
    if (!fmm_capable(f)) throw StateError("ki_apply_fmm: 2D Laplace problems only");
    if (order < 0 || order > 32) throw ArgError("order out of range");
    const int N = f->n_dofs, nb = f->n_border;
    if (ncols < 0 || ldx < N || ldy < N) throw ArgError("bad leading dimension / ncols");
    if (ncols == 0) return;
    cudaStream_t s = f->stream;
    DevBuf<double> dx((size_t)N * ncols, s), dy((size_t)N * ncols, s);
    KI_CHECK_CUDA(cudaMemcpy2DAsync(dx.p, sizeof(double) * N, x, sizeof(double) * ldx,
                                    sizeof(double) * N, ncols, cudaMemcpyHostToDevice, s));
    apply_K(f, dx.p, ncols, dy.p, s, true, order, nullptr,
            fp32 ? ki::FmmArith::kF32 : ki::FmmArith::kF64);
    if (nb > 0 && alpha) {
      if (ldalpha < nb) throw ArgError("bad ldalpha");
      DevBuf<double> da((size_t)nb * ncols, s);
      KI_CHECK_CUDA(cudaMemcpy2DAsync(da.p, sizeof(double) * nb, alpha, sizeof(double) * ldalpha,
                                      sizeof(double) * nb, ncols, cudaMemcpyHostToDevice, s));
      ki::launch(k_border_apply<double>, (N + 127) / 128, 128, 0, s, f->P.x, f->P.y, f->P.z, 1,
                 f->n_points, f->dim, f->sol_dim, f->d_holes, f->n_holes, da.p, nb, ncols, dy.p, N,
                 (const int*)nullptr, 0);
      KI_CHECK_CUDA(cudaGetLastError());
      KI_CHECK_CUDA(cudaStreamSynchronize(s));
    }
    KI_CHECK_CUDA(cudaMemcpy2DAsync(y, sizeof(double) * ldy, dy.p, sizeof(double) * N,
                                    sizeof(double) * N, ncols, cudaMemcpyDeviceToHost, s));
    KI_CHECK_CUDA(cudaStreamSynchronize(s));
  });
}

int ki_apply_rows(ki_factor* f, const int* rows, int nrows, const double* x, int ldx, int ncols,
                  const double* alpha, int ldalpha, double* y, int ldy) {
  return guarded([&] {
    if (!f || !rows || !x || !y) throw ArgError("NULL argument");
    const int N = f->n_dofs;
    if (nrows < 0 || ncols < 0 || ldx < N || ldy < nrows) throw ArgError("bad sizes");
    for (int i = 0; i < nrows; i++)
      if (rows[i] < 0 || rows[i] >= N) throw ArgError("row index out of range");
    if (nrows == 0 || ncols == 0) return;
    cudaStream_t s = f->stream;
    DevBuf<double> dx((size_t)N * ncols, s), dy((size_t)nrows * ncols, s);
    DevBuf<int> dr((size_t)nrows, s);
    KI_CHECK_CUDA(cudaMemcpyAsync(dr.p, rows, sizeof(int) * nrows, cudaMemcpyHostToDevice, s));
    KI_CHECK_CUDA(cudaMemcpy2DAsync(dx.p, sizeof(double) * N, x, sizeof(double) * ldx,
                                    sizeof(double) * N, ncols, cudaMemcpyHostToDevice, s));
    dense_product(f->P, f->n_points, f->sol_dim, dx.p, N, ncols, dy.p, nrows, dr.p, nrows, nullptr,
                  s);
    if (f->n_border > 0 && alpha) {
      if (ldalpha < f->n_border) throw ArgError("bad ldalpha");
      DevBuf<double> da((size_t)f->n_border * ncols, s);
      KI_CHECK_CUDA(cudaMemcpy2DAsync(da.p, sizeof(double) * f->n_border, alpha,
                                      sizeof(double) * ldalpha, sizeof(double) * f->n_border,
                                      ncols, cudaMemcpyHostToDevice, s));
      ki::launch(k_border_apply<double>, (nrows + 127) / 128, 128, 0, s,
          f->P.x, f->P.y, f->P.z, 1, f->n_points, f->dim, f->sol_dim, f->d_holes, f->n_holes, da.p,
          f->n_border, ncols, dy.p, nrows, (const int*)dr.p, nrows);
      KI_CHECK_CUDA(cudaGetLastError());
      KI_CHECK_CUDA(cudaStreamSynchronize(s));
    }
    KI_CHECK_CUDA(cudaMemcpy2DAsync(y, sizeof(double) * ldy, dy.p, sizeof(double) * nrows,
                                    sizeof(double) * nrows, ncols, cudaMemcpyDeviceToHost, s));
    KI_CHECK_CUDA(cudaStreamSynchronize(s));
  });
}

int ki_eval_targets(ki_factor* f, const double* targets, int n_targets, const double* mu, int ldmu,
                    int ncols, const double* alpha, int ldalpha, double* out, int ldout) {
  return guarded([&] {
    if (!f || !targets || !mu || !out) throw ArgError("NULL argument");
    const int N = f->n_dofs;
    const int NT = n_targets * f->sol_dim;
    if (n_targets < 0 || ncols < 0 || ldmu < N || ldout < NT) throw ArgError("bad sizes");
    if (n_targets == 0 || ncols == 0) return;
    cudaStream_t s = f->stream;
    const int dim = f->dim;
    DevBuf<double> dt((size_t)dim * n_targets, s), dm((size_t)N * ncols, s), dout((size_t)NT * ncols, s);
    KI_CHECK_CUDA(cudaMemcpyAsync(dt.p, targets, sizeof(double) * dim * n_targets, cudaMemcpyHostToDevice, s));
    KI_CHECK_CUDA(cudaMemcpy2DAsync(dm.p, sizeof(double) * N, mu, sizeof(double) * ldmu,
                                    sizeof(double) * N, ncols, cudaMemcpyHostToDevice, s));
    dense_product(f->P, f->n_points, f->sol_dim, dm.p, N, ncols, dout.p, NT, nullptr, NT, dt.p, s);
    KI_CHECK_CUDA(cudaGetLastError());
    if (f->n_border > 0 && alpha) {
      if (ldalpha < f->n_border) throw ArgError("bad ldalpha");
      DevBuf<double> da((size_t)f->n_border * ncols, s);
      KI_CHECK_CUDA(cudaMemcpy2DAsync(da.p, sizeof(double) * f->n_border, alpha,
                                      sizeof(double) * ldalpha, sizeof(double) * f->n_border,
                                      ncols, cudaMemcpyHostToDevice, s));
      ki::launch(k_border_apply<double>, (NT + 127) / 128, 128, 0, s, dt.p, dt.p + 1, dt.p + 2,
                 dim, n_targets, dim, f->sol_dim, f->d_holes, f->n_holes, da.p, f->n_border, ncols,
                 dout.p, NT, (const int*)nullptr, 0);
      KI_CHECK_CUDA(cudaGetLastError());
      KI_CHECK_CUDA(cudaStreamSynchronize(s));
    }
    KI_CHECK_CUDA(cudaMemcpy2DAsync(out, sizeof(double) * ldout, dout.p, sizeof(double) * NT,
                                    sizeof(double) * NT, ncols, cudaMemcpyDeviceToHost, s));
    KI_CHECK_CUDA(cudaStreamSynchronize(s));
  });
}

int ki_solve_refined_device(ki_factor* f, const double* d_b, int nrhs, double* d_x,
                            double* d_alpha, double tol, int max_steps, ki_refine_info* info,
                            void* stream) {
  return guarded([&] {
    if (!f || !info) throw ArgError("NULL argument");
    if (nrhs < 0 || max_steps < 0 || !(tol >= 0)) throw ArgError("bad nrhs / max_steps / tol");
    std::memset(info, 0, sizeof(*info));
    if (nrhs == 0) return;
    if (!d_b || !d_x || (f->n_border > 0 && !d_alpha)) throw ArgError("NULL b, x or alpha");
    cudaStream_t s = stream ? (cudaStream_t)stream : f->stream;
    refined_solve(f, d_b, nrhs, d_x, d_alpha, tol, max_steps, info, s);
    KI_CHECK_CUDA(cudaStreamSynchronize(s));
  });
}

int ki_solve_refined(ki_factor* f, const double* b, int ldb, int nrhs, double* x, int ldx,
                     double* alpha, int ldalpha, double tol, int max_steps, ki_refine_info* info) {
  return guarded([&] {
    if (!f || !info) throw ArgError("NULL argument");
    const int N = f->n_dofs, nb = f->n_border;
    if (nrhs < 0 || ldb < N || ldx < N || max_steps < 0 || !(tol >= 0))
      throw ArgError("bad leading dimension / nrhs / max_steps / tol");
    if (nb > 0 && alpha && ldalpha < nb) throw ArgError("bad ldalpha");
    std::memset(info, 0, sizeof(*info));
    if (nrhs == 0) return;
    if (!b || !x) throw ArgError("NULL b or x");
    cudaStream_t s = f->stream;
    DevBuf<double> db((size_t)N * nrhs, s), dx((size_t)N * nrhs, s),
        da((size_t)std::max(1, nb) * nrhs, s);
    KI_CHECK_CUDA(cudaMemcpy2DAsync(db.p, sizeof(double) * N, b, sizeof(double) * ldb,
                                    sizeof(double) * N, nrhs, cudaMemcpyHostToDevice, s));
    refined_solve(f, db.p, nrhs, dx.p, da.p, tol, max_steps, info, s);
    KI_CHECK_CUDA(cudaMemcpy2DAsync(x, sizeof(double) * ldx, dx.p, sizeof(double) * N,
                                    sizeof(double) * N, nrhs, cudaMemcpyDeviceToHost, s));
    if (nb > 0 && alpha)
      KI_CHECK_CUDA(cudaMemcpy2DAsync(alpha, sizeof(double) * ldalpha, da.p, sizeof(double) * nb,
                                      sizeof(double) * nb, nrhs, cudaMemcpyDeviceToHost, s));
    KI_CHECK_CUDA(cudaStreamSynchronize(s));
  });
}

int ki_factor_set_profiling(ki_factor* f, int on) {
  return guarded([&] {
    if (!f) throw ArgError("factor is NULL");
    if (f->f64) f->f64->profile_solve = on != 0;
    if (f->f32) f->f32->profile_solve = on != 0;
    f->profile_refine = on != 0;
  });
}

int ki_factor_get_profile(ki_factor* f, char* buf, int len) {
  return guarded([&] {
    if (!f || !buf || len <= 0) throw ArgError("NULL argument");
    auto dump = [](const std::vector<ki::StageSum>& v) {
      std::string o = "[";
      for (size_t i = 0; i < v.size(); i++) {
        char tmp[256];
        snprintf(tmp, sizeof(tmp),
                 "%s{\"stage\": \"%s\", \"launches\": %d, \"ms\": %.6f, \"flops\": %.6e, \"bytes\": %.6e}",
                 i ? ", " : "", v[i].stage.c_str(), v[i].launches, v[i].ms, v[i].flops, v[i].bytes);
        o += tmp;
      }
      return o + "]";
    };
    std::string j;
    auto fill = [&](auto& F) {
      auto now = F.collect();
      if (!now.empty()) F.solve_prof = now;
      std::string lv = "[";
      for (size_t i = 0; i < F.level_stats.size(); i++) {
        const auto& q = F.level_stats[i];
        char tmp[512];
        snprintf(tmp, sizeof(tmp),
                 "%s{\"level\": %d, \"boxes\": %d, \"id_boxes\": %d, \"compressed\": %d, "
                 "\"max_n\": %d, \"mean_n\": %.1f, \"max_m\": %d, \"mean_m\": %.1f, "
                 "\"max_k\": %d, \"mean_k\": %.1f, \"paths\": [%d, %d, %d, %d, %d]}",
                 i ? ", " : "", q.level, q.boxes, q.id_boxes, q.compressed, q.max_n,
                 q.sum_n / std::max(1, q.id_boxes), q.max_m, q.sum_m / std::max(1, q.id_boxes),
                 q.max_k, q.sum_k / std::max(1, q.id_boxes), q.mode_count[0], q.mode_count[1],
                 q.mode_count[2], q.mode_count[3], q.mode_count[4]);
        lv += tmp;
      }
      lv += "]";
      char host[384];
      snprintf(host, sizeof(host),
               "{\"create_prep_ms\": %.3f, \"factor_call_ms\": %.3f, \"tree_ms\": %.3f, "
               "\"tree_gpu_ms\": %.3f, \"tree_built_on_gpu\": %d, \"fmm_wait_ms\": %.3f}",
               f->host_prep_ms, f->host_factor_ms, F.tree_seconds * 1e3,
               F.tree_codes_seconds * 1e3, F.tree_gpu ? 1 : 0, f->fmm_wait_ms);
      j = "{\"factor\": " + dump(F.factor_prof) + ", \"solve\": " + dump(F.solve_prof) +
          ", \"refine\": " + dump(f->refine_prof) + ", \"levels\": " + lv +
          ", \"host\": " + host + "}";
    };
    if (f->f64) fill(*f->f64);
    if (f->f32) fill(*f->f32);
    if ((int)j.size() + 1 > len) throw ArgError("profile buffer too small");
    std::memcpy(buf, j.c_str(), j.size() + 1);
  });
}

int ki_measure_fma_peak(double* fp64_gflops, double* fp32_gflops) {
  return guarded([&] {
    if (!fp64_gflops || !fp32_gflops) throw ArgError("NULL argument");
    int dev = 0, sms = 0;
    KI_CHECK_CUDA(cudaGetDevice(&dev));
    KI_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    *fp64_gflops = fma_peak_gflops<double>(sms, 20000);
    *fp32_gflops = fma_peak_gflops<float>(sms, 200000);
  });
}

int ki_tensor_core_check(double* max_rel_err) {
  return guarded([&] {
    if (!max_rel_err) throw ArgError("NULL argument");
    *max_rel_err = ki::tensor_core_selfcheck();
  });
}

int ki_rank_model_floats(void) { return ki::kMlpModelFloats; }

int ki_rank_model_train(const float* features, const float* ratios, int n, int epochs, float lr,
                        unsigned seed, float* model, float* loss) {
  return guarded([&] {
    if (!features || !ratios || !model || !loss) throw ArgError("NULL argument");
    if (n <= 0 || epochs < 0 || !(lr > 0)) throw ArgError("bad n / epochs / lr");
    const int F = ki::kMlpIn, H = ki::kMlpHidden;
    for (long i = 0; i < (long)n * F; i++)
      if (!std::isfinite(features[i])) throw ArgError("non-finite feature");
    for (int i = 0; i < n; i++)
      if (!(ratios[i] >= 0 && ratios[i] <= 1)) throw ArgError("ratios must lie in [0, 1]");
    std::vector<float> m(ki::kMlpModelFloats, 0.f);
    // standardization from the data
    for (int f = 0; f < F; f++) {
      double s1 = 0, s2 = 0;
      for (int i = 0; i < n; i++) { s1 += features[(size_t)i * F + f]; s2 += (double)features[(size_t)i * F + f] * features[(size_t)i * F + f]; }
      double mu = s1 / n, var = std::max(0.0, s2 / n - mu * mu);
      m[ki::kMlpMean + f] = (float)mu;
      m[ki::kMlpScale + f] = (float)(var > 1e-12 ? std::sqrt(var) : 1.0);
    }
    // He-scaled uniform weights from a 64-bit linear congruential generator
    uint64_t st = 0x9E3779B97F4A7C15ull ^ seed;
    auto unif = [&]() {
      st = st * 6364136223846793005ull + 1442695040888963407ull;
      return (float)((st >> 40) * (1.0 / 16777216.0)) * 2.f - 1.f;
    };
    const float a1 = std::sqrt(6.f / F), a2 = std::sqrt(6.f / H);
    for (int e = 0; e < H * F; e++) m[ki::kMlpW1 + e] = a1 * unif();
    for (int e = 0; e < H * H; e++) m[ki::kMlpW2 + e] = a2 * unif();
    for (int e = 0; e < H; e++) m[ki::kMlpW3 + e] = a2 * unif();
    cudaStream_t s = nullptr;
    DevBuf<float> dm(ki::kMlpModelFloats, s), dx((size_t)n * F, s), dy(n, s);
    KI_CHECK_CUDA(cudaMemcpyAsync(dm.p, m.data(), sizeof(float) * m.size(), cudaMemcpyHostToDevice, s));
    KI_CHECK_CUDA(cudaMemcpyAsync(dx.p, features, sizeof(float) * (size_t)n * F, cudaMemcpyHostToDevice, s));
    KI_CHECK_CUDA(cudaMemcpyAsync(dy.p, ratios, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    *loss = ki::mlp_train(dm.p, dx.p, dy.p, n, epochs, lr, s);
    KI_CHECK_CUDA(cudaMemcpyAsync(model, dm.p, sizeof(float) * m.size(), cudaMemcpyDeviceToHost, s));
    KI_CHECK_CUDA(cudaStreamSynchronize(s));
  });
}

int ki_rank_model_predict(const float* model, const float* features, int n, float* ratios) {
  return guarded([&] {
    if (!model || !features || !ratios) throw ArgError("NULL argument");
    if (n < 0) throw ArgError("bad n");
    if (n == 0) return;
    cudaStream_t s = nullptr;
    DevBuf<float> dm(ki::kMlpModelFloats, s), dx((size_t)n * ki::kMlpIn, s), dy(n, s);
    KI_CHECK_CUDA(cudaMemcpyAsync(dm.p, model, sizeof(float) * ki::kMlpModelFloats, cudaMemcpyHostToDevice, s));
    KI_CHECK_CUDA(cudaMemcpyAsync(dx.p, features, sizeof(float) * (size_t)n * ki::kMlpIn, cudaMemcpyHostToDevice, s));
    ki::mlp_predict(dm.p, dx.p, n, dy.p, s);
    KI_CHECK_CUDA(cudaMemcpyAsync(ratios, dy.p, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    KI_CHECK_CUDA(cudaStreamSynchronize(s));
  });
}

int ki_rank_model_predict_bf16(const float* model, const float* features, int n, float* ratios) {
  return guarded([&] {
    if (!model || !features || !ratios) throw ArgError("NULL argument");
    if (n < 0) throw ArgError("bad n");
    if (n == 0) return;
    cudaStream_t s = nullptr;
    DevBuf<float> dm(ki::kMlpModelFloats, s), dx((size_t)n * ki::kMlpIn, s), dy(n, s);
    DevBuf<int> de(1, s);
    KI_CHECK_CUDA(cudaMemsetAsync(de.p, 0, sizeof(int), s));
    KI_CHECK_CUDA(cudaMemcpyAsync(dm.p, model, sizeof(float) * ki::kMlpModelFloats, cudaMemcpyHostToDevice, s));
    KI_CHECK_CUDA(cudaMemcpyAsync(dx.p, features, sizeof(float) * (size_t)n * ki::kMlpIn, cudaMemcpyHostToDevice, s));
    ki::mlp_predict_bf16(dm.p, dx.p, n, dy.p, de.p, s);
    int herr = 0;
    KI_CHECK_CUDA(cudaMemcpyAsync(&herr, de.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    KI_CHECK_CUDA(cudaMemcpyAsync(ratios, dy.p, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    KI_CHECK_CUDA(cudaStreamSynchronize(s));
    if (herr) throw std::runtime_error("a bounded device wait timed out (tensor-core MLP inference)");
  });
}

int ki_rank_model_grad(const float* model, const float* features, const float* ratios, int n,
                       float* grad, float* loss) {
  return guarded([&] {
    if (!model || !features || !ratios || !grad || !loss) throw ArgError("NULL argument");
    if (n <= 0) throw ArgError("bad n");
    cudaStream_t s = nullptr;
    DevBuf<float> dm(ki::kMlpModelFloats, s), dx((size_t)n * ki::kMlpIn, s), dy(n, s),
        dg(ki::kMlpModelFloats, s);
    KI_CHECK_CUDA(cudaMemcpyAsync(dm.p, model, sizeof(float) * ki::kMlpModelFloats, cudaMemcpyHostToDevice, s));
    KI_CHECK_CUDA(cudaMemcpyAsync(dx.p, features, sizeof(float) * (size_t)n * ki::kMlpIn, cudaMemcpyHostToDevice, s));
    KI_CHECK_CUDA(cudaMemcpyAsync(dy.p, ratios, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    ki::mlp_loss_grad(dm.p, dx.p, dy.p, n, dg.p, loss, s);
    KI_CHECK_CUDA(cudaMemcpyAsync(grad, dg.p, sizeof(float) * ki::kMlpModelFloats, cudaMemcpyDeviceToHost, s));
    KI_CHECK_CUDA(cudaStreamSynchronize(s));
  });
}

int ki_factor_get_box_log(const ki_factor* f, float* out, int max_rows, int* rows) {
  return guarded([&] {
    if (!f || !rows || (max_rows > 0 && !out)) throw ArgError("NULL argument");
    const std::vector<float>& log = f->f64 ? f->f64->box_log : f->f32->box_log;
    const int total = (int)(log.size() / 15);
    *rows = total;
    const int w = std::min(total, std::max(0, max_rows));
    if (w > 0) std::memcpy(out, log.data(), sizeof(float) * 15 * (size_t)w);
  });
}

int ki_trim_memory(void) {
  return guarded([&] { KI_CHECK_CUDA(ki::pool_trim()); });
}

long long ki_launch_count(void) { return ki::launch_counter().load(); }

const char* ki_last_error(void) { return g_last_error.c_str(); }

const char* ki_version(void) { return "kern-interp-gb300 0.1 (sm_103a)"; }

}  // extern "C"
