// Uniform-depth 2D FMM for the Laplace double-layer Nystrom operator (see
// ki_fmm.h).  Host: Morton-sorted points, one tree level per refinement
// step down to a leaf level with about 40 points per non-empty leaf, near
// lists (the 3 x 3 leaf neighbourhood) and interaction lists (children of
// the parent's neighbours that are not adjacent), translation matrices.
// Device, FP64: P2M per leaf, M2M up, M2L per box over its interaction list
// (the matrix depends only on the integer offset between the two boxes, so
// 49 matrices serve every level), L2L down, and per leaf the local
// expansion plus the direct near-field sum with the exact kernel entries.
// All 32 columns of a pass share every kernel-entry and translation-matrix
// load.
#include "ki_common.cuh"
#include "ki_launch.cuh"
#include "ki_pool.h"
#include "ki_fmm.h"
#include "ki_parallel.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

namespace ki {

namespace {

#define KI_FMM_CUDA(call)                                                                  \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      throw std::runtime_error(std::string("CUDA error (fmm): ") + cudaGetErrorString(e_)); \
  } while (0)

constexpr int kCols = 32;        // columns per pass
constexpr int kMaxP = 32;        // expansion terms (upper bound)
constexpr int kChunk = 32;       // source points staged per shared-memory chunk
constexpr double kPi2 = 6.283185307179586476925286766559;

// The FP64-accurate apply's arithmetic: an FP32 pair (value h + l, about 48
// significant bits), operated on the FP32 pipes, which run at 64x the FP64
// rate on this part.  Products split the high parts exactly (fma) and carry
// the cross terms; sums use Knuth's two-sum.  Results are not renormalised
// (l stays within a few ulps of h), which the first-order cross terms of the
// next operation absorb; every step adds an error near 2^-47 of its operands,
// far under the expansions' truncation error.  The _rn intrinsics keep the
// compiler from fusing the separately rounded steps.
struct pr {
  float h, l;
  pr() = default;
  __host__ __device__ __forceinline__ pr(float hi, float lo) : h(hi), l(lo) {}
  __device__ __forceinline__ pr(double v) {
    h = (float)v;
    l = (float)(v - (double)h);
  }
  __device__ __forceinline__ pr(int v) : h((float)v), l(0.f) {}
  __device__ __forceinline__ explicit operator double() const { return (double)h + (double)l; }
};
__device__ __forceinline__ pr operator-(pr a) { return pr(-a.h, -a.l); }
__device__ __forceinline__ pr operator*(pr a, pr b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return pr(p, e);
}
__device__ __forceinline__ pr operator+(pr a, pr b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  return pr(s, __fadd_rn(e, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ pr operator-(pr a, pr b) { return a + (-b); }
struct cpr {
  pr x, y;
};

// Complex values of the expansions: pairs (the FP64-accurate apply) or float2
// (FP32 arithmetic, the low-accuracy apply of residual updates).
template <typename R> struct Cplx;
template <> struct Cplx<pr> { using type = cpr; };
template <> struct Cplx<float> { using type = float2; };
template <typename R> using cplx_t = typename Cplx<R>::type;

__device__ __forceinline__ pr fmx(pr a, pr b, pr c) { return c + a * b; }
__device__ __forceinline__ float fmx(float a, float b, float c) { return __fmaf_rn(a, b, c); }

template <typename V> __device__ __forceinline__ V czero() {
  V r;
  r.x = 0;
  r.y = 0;
  return r;
}
template <typename V> __device__ __forceinline__ V cmul(V a, V b) {
  V r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
template <typename V> __device__ __forceinline__ V cfma(V a, V b, V c) {   // a*b + c
  V r;
  r.x = fmx(a.x, b.x, fmx(-a.y, b.y, c.x));
  r.y = fmx(a.x, b.y, fmx(a.y, b.x, c.y));
  return r;
}
// an FP64 complex value rounded to the expansion type
template <typename V> __device__ __forceinline__ V cround(double x, double y) {
  V r;
  r.x = (decltype(r.x))x;
  r.y = (decltype(r.y))y;
  return r;
}

// u[i kCols + c] = mu[perm[i] + ldmu (c0 + c)]: the densities in sorted
// order, point-major (a point's columns contiguous), in the expansion type.
// Block (32, 8) per 32 points: columns read along the points (coalesced in
// mu), written along the columns through shared memory.
template <typename R>
__global__ void k_densities(const int* perm, int n, const double* mu, int ldmu, int c0, int nc,
                            R* u) {
  __shared__ R tile[32][kCols + 1];
  const int i0 = blockIdx.x * 32;
  const int i = i0 + threadIdx.x;
  if (i < n) {
    const int o = perm[i];
    for (int c = threadIdx.y; c < nc; c += blockDim.y)
      tile[threadIdx.x][c] = (R)mu[o + (size_t)ldmu * (c0 + c)];
  }
  __syncthreads();
  const int cnt = min(32, n - i0);
  for (int e = threadIdx.y * 32 + threadIdx.x; e < cnt * nc; e += 32 * blockDim.y) {
    const int r = e / nc, c = e % nc;
    u[(size_t)(i0 + r) * kCols + c] = tile[r][c];
  }
}

// Multipole expansion of every leaf: me[(g nc + c) p + k] = sum_s q_s w_s^k,
// w_s = (z_s - centre) / side (formed in FP64), q_s = nw_s mu_s with mu_s
// real: the column-independent factors nw_s w_s^k are formed once per point
// and each column adds mu_s times them (real-by-complex products).
template <typename R>
__global__ void k_p2m(const int* leaf_start, const int* leaf_box, const double2* centre,
                      double side, const double2* z, const double2* nw, const R* u, int nc, int p,
                      cplx_t<R>* me) {
  using V = cplx_t<R>;
  __shared__ V pw[kChunk][kMaxP];
  __shared__ R us[kChunk][kCols];
  const int lf = blockIdx.x, g = leaf_box[lf];
  const int s0 = leaf_start[lf], s1 = leaf_start[lf + 1];
  const double2 c = centre[g];
  const int nout = p * nc;
  V acc[4];
  for (int r = 0; r < 4; r++) acc[r] = czero<V>();
  for (int base = s0; base < s1; base += kChunk) {
    const int cnt = min(kChunk, s1 - base);
    __syncthreads();
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
      const V w = cround<V>((z[base + i].x - c.x) / side, (z[base + i].y - c.y) / side);
      V t = cround<V>(nw[base + i].x, nw[base + i].y);
      for (int k = 0; k < p; k++) {
        pw[i][k] = t;
        t = cmul(t, w);
      }
    }
    for (int e = threadIdx.x; e < cnt * nc; e += blockDim.x) {
      int i = e / nc, cc = e % nc;
      us[i][cc] = u[(size_t)(base + i) * kCols + cc];
    }
    __syncthreads();
    for (int r = 0; r < 4; r++) {
      int o = threadIdx.x + r * blockDim.x;
      if (o >= nout) break;
      int k = o % p, cc = o / p;
      V a = acc[r];
      for (int i = 0; i < cnt; i++) {
        const R m = us[i][cc];
        a.x = fmx(m, pw[i][k].x, a.x);
        a.y = fmx(m, pw[i][k].y, a.y);
      }
      acc[r] = a;
    }
  }
  for (int r = 0; r < 4; r++) {
    int o = threadIdx.x + r * blockDim.x;
    if (o >= nout) break;
    me[(size_t)g * nout + o] = acc[r];
  }
}

// Multipole of each box of one level from its children (M2M), in rotated
// form: with the child offset d = |d| e^(i theta) (parent-side units),
// T(k, j) = C(k, j) 0.5^j d^(k-j) = e^(i theta k) Tr(k, j) e^(-i theta j), Tr
// real lower triangular (leading dimension ldm >= p), so
// me[P]_k += e^(i theta k) sum_(j<=k) Tr(k, j) (e^(-i theta j) me[C]_j).
// Each child's rotated expansions and its Tr are staged in shared memory;
// output (k, c) is thread c + nc k.
template <typename R>
__global__ void k_m2m(int b0, const int* child, const int* child_pos, const R* Tr,
                      const cplx_t<R>* Tph, int ldm, int nc, int p, cplx_t<R>* me) {
  using V = cplx_t<R>;
  __shared__ V sm_x[kCols * (kMaxP + 1)];
  __shared__ R sm_T[kMaxP * kMaxP];
  const int g = b0 + blockIdx.x;
  const int nout = p * nc, ld = p + 1;
  V acc[4];
  for (int r = 0; r < 4; r++) acc[r] = czero<V>();
  for (int q = 0; q < 4; q++) {
    const int ch = child[4 * g + q];
    if (ch < 0) continue;
    __syncthreads();
    const int pos = child_pos[ch];
    const V* ph = Tph + (size_t)pos * ldm;   // e^(i theta k)
    const V* src = me + (size_t)ch * nout;
    for (int e = threadIdx.x; e < nout; e += blockDim.x) {
      const int j = e % p, cc = e / p;
      V cph = ph[j];
      cph.y = -cph.y;
      sm_x[cc * ld + j] = cmul(cph, src[e]);
    }
    const R* Tm = Tr + (size_t)pos * ldm * ldm;
    for (int e = threadIdx.x; e < p * p; e += blockDim.x) sm_T[e] = Tm[(size_t)(e / p) * ldm + e % p];
    __syncthreads();
    for (int r = 0; r < 4; r++) {
      int o = threadIdx.x + r * blockDim.x;
      if (o >= nout) break;
      const int cc = o % nc, k = o / nc;
      V ck = czero<V>();
      const R* row = sm_T + k * p;
      const V* x = sm_x + cc * ld;
      for (int jj = 0; jj <= k; jj++) {
        ck.x = fmx(row[jj], x[jj].x, ck.x);
        ck.y = fmx(row[jj], x[jj].y, ck.y);
      }
      acc[r] = cfma(ph[k], ck, acc[r]);
    }
  }
  for (int r = 0; r < 4; r++) {
    int o = threadIdx.x + r * blockDim.x;
    if (o >= nout) break;
    const int cc = o % nc, k = o / nc;
    me[(size_t)g * nout + (size_t)cc * p + k] = acc[r];
  }
}

// Local expansion contributions over the interaction list (M2L): for every
// box g of one level, le[g] = (1/side) sum_v M_code(v) me[src(v)].  The
// translation for offset d, M(m, k) = (-1)^m C(k+m, m) rho^(k+m+1) with
// rho = 1/d, is applied in rotated form: with rho = |rho| e^(i phi),
// M(m, k) = e^(i phi (m+1)) Rr(m, k) e^(i phi k), Rr real, so each pair
// costs p^2 real-by-complex products (half the complex ones) plus 2p phase
// rotations.  Output (m, c) is thread c + nc m: a warp shares one row of Rr
// (broadcast) and reads 32 columns of the staged, rotated multipoles (row
// stride p + 1: conflict-free).
template <typename R>
__global__ void k_m2l(int b0, const int* v_off, const int* v_src, const int* v_code,
                      const R* Mr, const cplx_t<R>* Mph, int ldm, double inv_side, int nc, int p,
                      const cplx_t<R>* me, cplx_t<R>* le) {
  using V = cplx_t<R>;
  __shared__ V sm_me[kCols * (kMaxP + 1)];
  __shared__ R sm_R[kMaxP * kMaxP];
  const int g = b0 + blockIdx.x;
  const int nout = p * nc;
  const int ld = p + 1;
  V acc[4];
  for (int r = 0; r < 4; r++) acc[r] = czero<V>();
  for (int v = v_off[g]; v < v_off[g + 1]; v++) {
    __syncthreads();
    const V* src = me + (size_t)v_src[v] * nout;
    const int code = v_code[v];
    const V* ph = Mph + (size_t)code * (ldm + 1);   // e^(i phi k), k = 0..ldm
    for (int e = threadIdx.x; e < nout; e += blockDim.x) {
      const int k = e % p, cc = e / p;
      sm_me[cc * ld + k] = cmul(ph[k], src[e]);
    }
    const R* Rm = Mr + (size_t)code * ldm * ldm;
    for (int e = threadIdx.x; e < p * p; e += blockDim.x) sm_R[e] = Rm[(size_t)(e / p) * ldm + e % p];
    __syncthreads();
    for (int r = 0; r < 4; r++) {
      int o = threadIdx.x + r * blockDim.x;
      if (o >= nout) break;
      const int cc = o % nc, m = o / nc;
      V cm = czero<V>();
      const R* row = sm_R + m * p;
      const V* x = sm_me + cc * ld;
      for (int k = 0; k < p; k++) {
        cm.x = fmx(row[k], x[k].x, cm.x);
        cm.y = fmx(row[k], x[k].y, cm.y);
      }
      acc[r] = cfma(ph[m + 1], cm, acc[r]);
    }
  }
  const R is = (R)inv_side;
  for (int r = 0; r < 4; r++) {
    int o = threadIdx.x + r * blockDim.x;
    if (o >= nout) break;
    const int cc = o % nc, m = o / nc;
    V out;
    out.x = acc[r].x * is;
    out.y = acc[r].y * is;
    le[(size_t)g * nout + (size_t)cc * p + m] = out;
  }
}

// Local expansion of each box of one level += its parent's, translated (L2L),
// in rotated form: S(j, m) = C(m, j) 0.5^j d^(m-j) = e^(-i theta j) Sr(j, m)
// e^(i theta m), Sr real upper triangular (leading dimension ldm), so
// le[C]_j += e^(-i theta j) sum_(m>=j) Sr(j, m) (e^(i theta m) le[P]_m); the
// parent's rotated expansions and Sr staged in shared memory, output (j, c)
// is thread c + nc j.
template <typename R>
__global__ void k_l2l(int b0, const int* parent, const int* child_pos, const R* Sr,
                      const cplx_t<R>* Tph, int ldm, int nc, int p, cplx_t<R>* le) {
  using V = cplx_t<R>;
  __shared__ V sm_x[kCols * (kMaxP + 1)];
  __shared__ R sm_S[kMaxP * kMaxP];
  const int g = b0 + blockIdx.x;
  const int par = parent[g];
  const int pos = child_pos[g];
  const V* ph = Tph + (size_t)pos * ldm;   // e^(i theta m)
  const int nout = p * nc, ld = p + 1;
  const V* src = le + (size_t)par * nout;
  for (int e = threadIdx.x; e < nout; e += blockDim.x) {
    const int m = e % p, cc = e / p;
    sm_x[cc * ld + m] = cmul(ph[m], src[e]);
  }
  const R* Sm = Sr + (size_t)pos * ldm * ldm;
  for (int e = threadIdx.x; e < p * p; e += blockDim.x) sm_S[e] = Sm[(size_t)(e / p) * ldm + e % p];
  __syncthreads();
  for (int o = threadIdx.x; o < nout; o += blockDim.x) {
    const int cc = o % nc, j = o / nc;
    const size_t dst = (size_t)g * nout + (size_t)cc * p + j;
    V cj = czero<V>();
    const R* row = sm_S + j * p;
    const V* x = sm_x + cc * ld;
    for (int m = j; m < p; m++) {
      cj.x = fmx(row[m], x[m].x, cj.x);
      cj.y = fmx(row[m], x[m].y, cj.y);
    }
    V cph = ph[j];
    cph.y = -cph.y;
    le[dst] = cfma(cph, cj, le[dst]);
  }
}

// The Nystrom entry (nw_s . (t - s)) / |t - s|^2 in FP32-pair arithmetic from
// pairs t, s, nw = (hi x, hi y, lo x, lo y): the difference by two_diff, the
// dot products and squared distance with exact products (p = a b,
// fma(a, b, -p)) and the low-order terms, the quotient by long division with
// one remainder step (Dekker's double-length division, 1971): q1 = num_h / r2_h
// through the rounded reciprocal, then (num - q1 r2) / r2_h.  Relative error
// ~1e-13, far under the FMM truncation error; returned as a normalised pair.
__device__ __forceinline__ float2 pair_entry(const float4& t, const float4& s, const float4& nw) {
  float dxh, dxl, dyh, dyl;
  two_diff(t.x, s.x, dxh, dxl);
  two_diff(t.y, s.y, dyh, dyl);
  fast_two_sum(dxh, __fadd_rn(dxl, __fsub_rn(t.z, s.z)), dxh, dxl);
  fast_two_sum(dyh, __fadd_rn(dyl, __fsub_rn(t.w, s.w)), dyh, dyl);
  // r2 = dx^2 + dy^2
  const float a = __fmul_rn(dxh, dxh), b = __fmul_rn(dyh, dyh);
  float r2h, r2l;
  two_sum(a, b, r2h, r2l);
  r2l = __fadd_rn(r2l, __fadd_rn(fmaf(dxh, dxh, -a), fmaf(dyh, dyh, -b)));
  r2l = fmaf(2.f * dxh, dxl, fmaf(2.f * dyh, dyl, r2l));
  fast_two_sum(r2h, r2l, r2h, r2l);
  // num = nw . d
  const float c = __fmul_rn(nw.x, dxh), d = __fmul_rn(nw.y, dyh);
  float nh, nl;
  two_sum(c, d, nh, nl);
  nl = __fadd_rn(nl, __fadd_rn(fmaf(nw.x, dxh, -c), fmaf(nw.y, dyh, -d)));
  nl = fmaf(nw.x, dxl, fmaf(nw.z, dxh, fmaf(nw.y, dyl, fmaf(nw.w, dyh, nl))));
  fast_two_sum(nh, nl, nh, nl);
  // q = num / r2
  const float inv = __frcp_rn(r2h);
  const float q1 = __fmul_rn(nh, inv);
  const float p = __fmul_rn(q1, r2h);
  float rem = __fsub_rn(nh, p);   // exact: p is within a factor two of nh
  rem = __fsub_rn(rem, fmaf(q1, r2h, -p));
  rem = fmaf(-q1, r2l, __fadd_rn(rem, nl));
  float qh, ql;
  fast_two_sum(q1, __fmul_rn(rem, inv), qh, ql);
  return make_float2(qh, ql);
}

// Near-field points are staged as FP32 pairs (hi x, hi y, lo x, lo y), hi =
// fl(x), lo = fl(x - hi), in both applies, so that differences of nearby nodes
// keep their full relative accuracy; nw_s = -(w_s / 2 pi) n_s likewise as
// pairs in the FP64 apply, rounded in the FP32 one.
template <typename R> struct NearNw;
template <> struct NearNw<pr> { using type = float4; };
template <> struct NearNw<float> { using type = float2; };

// The Nystrom entry Re(nw_s / (t - s)) = (nw_s . (t - s)) / |t - s|^2 in FP32
// (the FP32 apply): t - s = (t_hi - s_hi) + (t_lo - s_lo).
__device__ __forceinline__ float near_entry(const float4& t, const float4& s, float2 nws) {
  const float dx = (t.x - s.x) + (t.z - s.z), dy = (t.y - s.y) + (t.w - s.w);
  return (nws.x * dx + nws.y * dy) * __frcp_rn(dx * dx + dy * dy);
}

// Per leaf: far field from the local expansion, near field by direct
// summation over the 3 x 3 leaf neighbourhood (exact entries, the
// coincident point excluded), diagonal term (FP64); written unsorted into y.
//
// Lanes are columns: a warp evaluates one target at a time for all 32
// columns, so every FMA instruction has 32 useful lanes whatever the leaf's
// size (a leaf holds 8 to 40 points).  The targets of a pass (up to 32)
// are split over the four warps (target k of warp w: w + 4k, a warp-uniform
// branch), each lane accumulating its column for its warp's targets.  Per
// pass: the powers w_t^m of the targets and the kernel entries 1/(t - s) of
// each 32-source chunk are formed once in shared memory (one entry per
// thread) and broadcast to the lanes; charges and local expansions are read
// [point or term][column] (conflict-free).  The output goes through shared
// memory so that a warp writes 32 targets of one column.  The near field is
// the real Nystrom matrix times the real densities: one entry per pair, one
// FMA per pair and column.
constexpr int kLeafThreads = 128;
constexpr int kLeafWarps = kLeafThreads / 32;
constexpr int kPassTargets = 32;
constexpr int kWarpTargets = kPassTargets / kLeafWarps;
constexpr int kSrcChunk = 32;
static_assert(kSrcChunk == kMaxP, "bufA holds powers [t][m] and entries [t][s] in turn");
static_assert(kPassTargets <= kCols, "bufB holds the output tile");

template <typename R>
__global__ void __launch_bounds__(kLeafThreads)
    k_leaf_eval(const int* leaf_start, const int* leaf_box, const int* near_off,
                const int* near_leaf, const double2* centre, double side, const double2* z,
                const float4* zf, const float2* nw32, const float4* nwf,
                const double* diag,
                const int* perm, const R* u, const cplx_t<R>* le, int nc, int p,
                const double* mu, int ldmu, int c0, double* y, int ldy) {
  using V = cplx_t<R>;
  using W = typename NearNw<R>::type;
  __shared__ V bufA[kPassTargets * kMaxP];   // powers [t][m] (complex), then entries [t][s] (real)
  __shared__ V bufB[kSrcChunk * kCols];      // local expansion [m][c], densities [s][c] (real), output
  __shared__ float4 st[kPassTargets];
  __shared__ float4 ss[kSrcChunk];
  __shared__ W snw[kSrcChunk];
  R* ent = reinterpret_cast<R*>(bufA);
  R* dens = reinterpret_cast<R*>(bufB);
  const int lf = blockIdx.x, g = leaf_box[lf];
  const int t0 = leaf_start[lf], t1 = leaf_start[lf + 1];
  const double2 c = centre[g];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool col_on = lane < nc;
  const int nout = p * nc;
  for (int tb = t0; tb < t1; tb += kPassTargets) {
    const int nt = min(kPassTargets, t1 - tb);
    __syncthreads();   // the previous pass's output is written
    if (threadIdx.x < nt) {
      const int t = tb + threadIdx.x;
      st[threadIdx.x] = zf[t];
      const double2 zt = z[t];
      const V w = cround<V>((zt.x - c.x) / side, (zt.y - c.y) / side);
      V pw = cround<V>(1, 0);
      for (int m = 0; m < p; m++) {
        bufA[threadIdx.x * kMaxP + m] = pw;
        pw = cmul(pw, w);
      }
    }
    for (int e = threadIdx.x; e < nout; e += blockDim.x) {
      const int m = e % p, cc = e / p;
      bufB[m * kCols + cc] = le[(size_t)g * nout + e];
    }
    __syncthreads();
    R acc[kWarpTargets];
#pragma unroll
    for (int k = 0; k < kWarpTargets; k++) acc[k] = 0;
    // far field: Re sum_m le_m w^m
    if (col_on) {
      for (int m = 0; m < p; m++) {
        const V b = bufB[m * kCols + lane];
#pragma unroll
        for (int k = 0; k < kWarpTargets; k++) {
          const int tt = warp + kLeafWarps * k;
          if (tt < nt) {
            const V a = bufA[tt * kMaxP + m];
            acc[k] = fmx(b.x, a.x, fmx(-b.y, a.y, acc[k]));
          }
        }
      }
    }
    // near field: sum_s Re(nw_s / (t - s)) mu_s, one real entry per pair.
    // FP64 apply: entries (pair_entry) and densities as FP32 pairs, summed with
    // pair_fma: the FP32 pipes instead of the FP64 pipe, which runs at 1/64 of
    // their rate on this part.
    if constexpr (std::is_same<R, pr>::value) {
      const float2* u2 = reinterpret_cast<const float2*>(u);   // the pairs' layout
      float2* ent2 = reinterpret_cast<float2*>(bufA);    // [t][s]
      float2* dens2 = reinterpret_cast<float2*>(bufB);   // [s][c]
      float nh[kWarpTargets], nl[kWarpTargets];
#pragma unroll
      for (int k = 0; k < kWarpTargets; k++) nh[k] = nl[k] = 0.f;
      for (int v = near_off[lf]; v < near_off[lf + 1]; v++) {
        const int sl = near_leaf[v];
        const int s0 = leaf_start[sl], s1 = leaf_start[sl + 1];
        for (int base = s0; base < s1; base += kSrcChunk) {
          const int cnt = min(kSrcChunk, s1 - base);
          __syncthreads();   // readers of bufA / bufB done
          for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
            ss[i] = zf[base + i];
            snw[i] = nwf[base + i];
          }
          for (int e = threadIdx.x; e < cnt * nc; e += blockDim.x) {
            const int i = e / nc, cc = e % nc;
            dens2[i * kCols + cc] = u2[(size_t)(base + i) * kCols + cc];
          }
          __syncthreads();
          for (int e = threadIdx.x; e < nt * cnt; e += blockDim.x) {
            const int tt = e / cnt, i = e % cnt;
            ent2[tt * kSrcChunk + i] = (tb + tt != base + i) ? pair_entry(st[tt], ss[i], snw[i])
                                                             : make_float2(0.f, 0.f);
          }
          __syncthreads();
          if (col_on) {
            for (int i = 0; i < cnt; i++) {
              const float2 dv = dens2[i * kCols + lane];
#pragma unroll
              for (int k = 0; k < kWarpTargets; k++) {
                const int tt = warp + kLeafWarps * k;
                if (tt < nt) pair_fma(nh[k], nl[k], ent2[tt * kSrcChunk + i], dv);
              }
            }
          }
        }
      }
#pragma unroll
      for (int k = 0; k < kWarpTargets; k++) acc[k] = acc[k] + pr(nh[k], nl[k]);
    } else
    for (int v = near_off[lf]; v < near_off[lf + 1]; v++) {
      const int sl = near_leaf[v];
      const int s0 = leaf_start[sl], s1 = leaf_start[sl + 1];
      for (int base = s0; base < s1; base += kSrcChunk) {
        const int cnt = min(kSrcChunk, s1 - base);
        __syncthreads();   // readers of bufA / bufB done
        for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
          ss[i] = zf[base + i];
          snw[i] = nw32[base + i];
        }
        for (int e = threadIdx.x; e < cnt * nc; e += blockDim.x) {
          const int i = e / nc, cc = e % nc;
          dens[i * kCols + cc] = u[(size_t)(base + i) * kCols + cc];
        }
        __syncthreads();
        for (int e = threadIdx.x; e < nt * cnt; e += blockDim.x) {
          const int tt = e / cnt, i = e % cnt;
          ent[tt * kSrcChunk + i] = (tb + tt != base + i) ? near_entry(st[tt], ss[i], snw[i]) : R(0);
        }
        __syncthreads();
        if (col_on) {
          for (int i = 0; i < cnt; i++) {
            const R dv = dens[i * kCols + lane];
#pragma unroll
            for (int k = 0; k < kWarpTargets; k++) {
              const int tt = warp + kLeafWarps * k;
              if (tt < nt) acc[k] = fmx(dv, ent[tt * kSrcChunk + i], acc[k]);
            }
          }
        }
      }
    }
    __syncthreads();   // bufB becomes the output tile [t][c] (stride kCols + 1)
    R* so = reinterpret_cast<R*>(bufB);
    if (col_on) {
#pragma unroll
      for (int k = 0; k < kWarpTargets; k++) {
        const int tt = warp + kLeafWarps * k;
        if (tt < nt) so[tt * (kCols + 1) + lane] = acc[k];
      }
    }
    __syncthreads();
    const int tt = threadIdx.x % kPassTargets;
    if (tt < nt) {
      const int t = tb + tt, orig = perm[t];
      const double dg = diag[t];
      for (int cc = threadIdx.x / kPassTargets; cc < nc; cc += kLeafThreads / kPassTargets)
        y[orig + (size_t)ldy * (c0 + cc)] =
            (double)so[tt * (kCols + 1) + cc] + dg * mu[orig + (size_t)ldmu * (c0 + cc)];
    }
  }
}

// FP64 -> FP32 copies for the FP32 apply: complex arrays, and the sorted
// points (and nw) as hi/lo pairs.
__global__ void k_round_cplx(const double2* a, size_t count, float2* out) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count;
       e += (size_t)gridDim.x * blockDim.x)
    out[e] = make_float2((float)a[e].x, (float)a[e].y);
}
// FP64 -> FP32 pairs for the FP64-accurate apply's tables.
__global__ void k_pair_cplx(const double2* a, size_t count, cpr* out) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count;
       e += (size_t)gridDim.x * blockDim.x) {
    out[e].x = pr(a[e].x);
    out[e].y = pr(a[e].y);
  }
}
__global__ void k_pair_real(const double* a, size_t count, pr* out) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count;
       e += (size_t)gridDim.x * blockDim.x)
    out[e] = pr(a[e]);
}
__global__ void k_round_real(const double* a, size_t count, float* out) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count;
       e += (size_t)gridDim.x * blockDim.x)
    out[e] = (float)a[e];
}
__global__ void k_split_points(const double2* z, int n, float4* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float hx = (float)z[i].x, hy = (float)z[i].y;
    out[i] = make_float4(hx, hy, (float)(z[i].x - (double)hx), (float)(z[i].y - (double)hy));
  }
}

// Morton key of a cell: bit b of ix at position 2b + 1, of iy at 2b.
inline uint64_t spread2(uint32_t v) {
  uint64_t x = v;
  x = (x | (x << 16)) & 0x0000FFFF0000FFFFull;
  x = (x | (x << 8)) & 0x00FF00FF00FF00FFull;
  x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0Full;
  x = (x | (x << 2)) & 0x3333333333333333ull;
  x = (x | (x << 1)) & 0x5555555555555555ull;
  return x;
}
inline uint32_t compact2(uint64_t x) {
  x &= 0x5555555555555555ull;
  x = (x | (x >> 1)) & 0x3333333333333333ull;
  x = (x | (x >> 2)) & 0x0F0F0F0F0F0F0F0Full;
  x = (x | (x >> 4)) & 0x00FF00FF00FF00FFull;
  x = (x | (x >> 8)) & 0x0000FFFF0000FFFFull;
  x = (x | (x >> 16)) & 0x00000000FFFFFFFFull;
  return (uint32_t)x;
}
inline uint64_t morton(uint32_t ix, uint32_t iy) { return (spread2(ix) << 1) | spread2(iy); }
inline void demorton(uint64_t k, uint32_t* ix, uint32_t* iy) {
  *ix = compact2(k >> 1);
  *iy = compact2(k);
}

// Stable least-significant-digit radix sort of (key, index) pairs by the
// low `bits` bits of the keys (11-bit digits).  Each pass: per-part digit
// histograms, offsets digit-major then part-major, and each part scattering
// its keys in order -- stable whatever the number of parts.
void radix_sort_pairs(std::vector<uint64_t>* key, std::vector<int>* idx, int bits) {
  constexpr int D = 11, B = 1 << D;
  const int n = (int)key->size();
  std::vector<uint64_t> k2(n);
  std::vector<int> i2(n);
  const int parts = parallel_part_count(n, 1 << 16);
  std::vector<std::vector<size_t>> cnt(parts, std::vector<size_t>(B));
  for (int sh = 0; sh < bits; sh += D) {
    const uint64_t* k = key->data();
    const int* v = idx->data();
    parallel_parts(n, [&](int t, int lo, int hi) {
      std::fill(cnt[t].begin(), cnt[t].end(), 0);
      for (int i = lo; i < hi; i++) cnt[t][(k[i] >> sh) & (B - 1)]++;
    }, 1 << 16);
    size_t run = 0;
    for (int d = 0; d < B; d++)
      for (int t = 0; t < parts; t++) {
        const size_t c = cnt[t][d];
        cnt[t][d] = run;
        run += c;
      }
    parallel_parts(n, [&](int t, int lo, int hi) {
      size_t* off = cnt[t].data();
      for (int i = lo; i < hi; i++) {
        const size_t o = off[(k[i] >> sh) & (B - 1)]++;
        k2[o] = k[i];
        i2[o] = v[i];
      }
    }, 1 << 16);
    key->swap(k2);
    idx->swap(i2);
  }
}

// Box key -> global box index for one level: open addressing, linear
// probing, power-of-two table (keys are below 2^40, so ~0 marks a free slot).
struct KeyIndex {
  std::vector<uint64_t> keys;
  std::vector<int> vals;
  uint64_t mask = 0;
  int shift = 64;
  void build(const std::vector<uint64_t>& ks, int base) {
    size_t cap = 16;
    int lg = 4;
    while (cap < 2 * ks.size()) {
      cap <<= 1;
      lg++;
    }
    keys.assign(cap, ~0ull);
    vals.assign(cap, -1);
    mask = cap - 1;
    shift = 64 - lg;
    for (size_t i = 0; i < ks.size(); i++) {
      size_t h = slot(ks[i]);
      while (keys[h] != ~0ull) h = (h + 1) & mask;
      keys[h] = ks[i];
      vals[h] = base + (int)i;
    }
  }
  size_t slot(uint64_t k) const { return (size_t)((k * 0x9E3779B97F4A7C15ull) >> shift); }
  int find(uint64_t k) const {
    size_t h = slot(k);
    for (;;) {
      if (keys[h] == k) return vals[h];
      if (keys[h] == ~0ull) return -1;
      h = (h + 1) & mask;
    }
  }
};

double binom(int n, int k) {
  double r = 1;
  for (int i = 1; i <= k; i++) r = r * (n - k + i) / i;
  return std::round(r);
}

template <typename V>
V* upload_vec(const std::vector<V>& v, std::vector<void*>* owned, cudaStream_t s) {
  V* d = nullptr;
  KI_FMM_CUDA(pool_malloc((void**)&d, sizeof(V) * std::max<size_t>(1, v.size()), s));
  owned->push_back(d);
  if (!v.empty())
    KI_FMM_CUDA(cudaMemcpyAsync(d, v.data(), sizeof(V) * v.size(), cudaMemcpyHostToDevice, s));
  return d;
}

}  // namespace

struct Fmm2d {
  int n = 0, p = 0, L = 0, nleaf = 0, nbox = 0;
  long m2l_pairs = 0, near_pairs = 0, near_point_pairs = 0;
  double lo = 0, side0 = 0;
  std::vector<int> lvl_off;   // global box index range of each level
  int *d_perm = nullptr, *d_leaf_start = nullptr, *d_leaf_box = nullptr;
  int *d_near_off = nullptr, *d_near_leaf = nullptr;
  int *d_child = nullptr, *d_parent = nullptr, *d_child_pos = nullptr;
  int *d_v_off = nullptr, *d_v_src = nullptr, *d_v_code = nullptr;
  double2 *d_z = nullptr, *d_nw = nullptr, *d_centre = nullptr;
  double2 *d_Tph = nullptr, *d_Mph = nullptr;
  double *d_Tr = nullptr, *d_Sr = nullptr, *d_Mr = nullptr;
  double* d_diag = nullptr;
  // FP32 copies for the low-accuracy apply, made on its first use
  float2 *d_Tph32 = nullptr, *d_Mph32 = nullptr, *d_nw32 = nullptr;
  float *d_Tr32 = nullptr, *d_Sr32 = nullptr, *d_Mr32 = nullptr;
  float4* d_zf = nullptr;
  // FP32-pair copies for the FP64-accurate apply: nw (hi x, hi y, lo x, lo y)
  // for the near field, and the translation tables
  float4* d_nwf = nullptr;
  cpr *d_Tph2 = nullptr, *d_Mph2 = nullptr;
  pr *d_Tr2 = nullptr, *d_Sr2 = nullptr, *d_Mr2 = nullptr;
  std::vector<void*> owned;
  cudaStream_t stream = nullptr;   // the upload stream; frees are ordered on it
  ~Fmm2d() {
    for (void* q : owned) cudaFreeAsync(q, stream);
  }
};

void Fmm2dDeleter::operator()(Fmm2d* f) const { delete f; }

// Host-side plan: everything fmm2d_upload copies to the device.
struct Fmm2dPlan {
  int n = 0, p = 0, L = 0, nleaf = 0, nbox = 0;
  long near_point_pairs = 0;   // (target, source) pairs of the near field, self excluded
  double lo = 0, side0 = 0;
  std::vector<int> lvl_off, order, leaf_start, leaf_box, near_off, near_leaf, child, parent,
      child_pos, v_off, v_src, v_code;
  std::vector<double2> z, nw, centre, Tph, Mph;
  std::vector<double> Tr, Sr, Mr;
  std::vector<double> diag;
};

void Fmm2dPlanDeleter::operator()(Fmm2dPlan* f) const { delete f; }

std::unique_ptr<Fmm2dPlan, Fmm2dPlanDeleter> fmm2d_plan(const double* pts, const double* nrm,
                                                        const double* wts, const double* kap,
                                                        int n, int p) {
  if (n <= 0) throw std::invalid_argument("fmm: no points");
  if (p < 4 || p > kMaxP) throw std::invalid_argument("fmm: expansion order out of range");
  std::unique_ptr<Fmm2dPlan, Fmm2dPlanDeleter> F(new Fmm2dPlan());
  F->n = n;
  F->p = p;
  double mn = pts[0], mx = pts[0];
  for (int i = 0; i < 2 * n; i++) {
    mn = std::min(mn, pts[i]);
    mx = std::max(mx, pts[i]);
  }
  F->lo = mn - 0.01;
  F->side0 = (mx + 0.01) - F->lo;
  auto cell = [&](double x, int L) {
    long m = 1L << L;
    long i = (long)std::floor((x - F->lo) / F->side0 * m);
    return (uint32_t)std::min(m - 1, std::max(0L, i));
  };
  // Morton keys at the finest admissible level, one stable sort (ties by
  // point index); a coarser level's key is a right shift.  The leaf level is
  // the first from 2 at which the non-empty leaves hold 40 points or fewer
  // on average: consecutive sorted keys first differ at level
  // kLmax - floor(msb(a ^ b) / 2), so one pass counts the boxes of every level.
  constexpr int kLmax = 20;
  std::vector<uint64_t> skey(n);
  std::vector<int> order(n);
  parallel_ranges(n, [&](int lo, int hi) {
    for (int i = lo; i < hi; i++) {
      skey[i] = morton(cell(pts[2 * i], kLmax), cell(pts[2 * i + 1], kLmax));
      order[i] = i;
    }
  });
  radix_sort_pairs(&skey, &order, 2 * kLmax);
  std::vector<long> first_diff(kLmax + 1, 0);
  for (int i = 1; i < n; i++) {
    const uint64_t d = skey[i] ^ skey[i - 1];
    if (d) first_diff[kLmax - (63 - __builtin_clzll(d)) / 2]++;
  }
  int L = 2;
  for (;; L++) {
    long nl = 1;
    for (int l = 0; l <= L; l++) nl += first_diff[l];
    if ((double)n / nl <= 40.0 || L >= kLmax) break;
  }
  F->L = L;
  // leaves and levels (global box index: level 0 first)
  std::vector<std::vector<uint64_t>> lk(L + 1);
  std::vector<int> leaf_start;
  const int shL = 2 * (kLmax - L);
  for (int i = 0; i < n; i++) {
    const uint64_t k = skey[i] >> shL;
    if (lk[L].empty() || lk[L].back() != k) {
      lk[L].push_back(k);
      leaf_start.push_back(i);
    }
  }
  leaf_start.push_back(n);
  for (int l = L - 1; l >= 0; l--)
    for (uint64_t k : lk[l + 1])
      if (lk[l].empty() || lk[l].back() != (k >> 2)) lk[l].push_back(k >> 2);
  F->lvl_off.assign(L + 2, 0);
  for (int l = 0; l <= L; l++) F->lvl_off[l + 1] = F->lvl_off[l] + (int)lk[l].size();
  const int nbox = F->lvl_off[L + 1];
  F->nbox = nbox;
  F->nleaf = (int)lk[L].size();
  std::vector<KeyIndex> idx(L + 1);
  for (int l = 0; l <= L; l++) idx[l].build(lk[l], F->lvl_off[l]);
  std::vector<double2> centre(nbox);
  std::vector<int> parent(nbox, -1), child(4 * (size_t)nbox, -1), child_pos(nbox, 0);
  for (int l = 0; l <= L; l++) {
    const double side = F->side0 / (double)(1L << l);
    for (size_t i = 0; i < lk[l].size(); i++) {
      uint32_t ix, iy;
      demorton(lk[l][i], &ix, &iy);
      int g = F->lvl_off[l] + (int)i;
      centre[g] = make_double2(F->lo + (ix + 0.5) * side, F->lo + (iy + 0.5) * side);
      child_pos[g] = (int)(lk[l][i] & 3u);
      if (l > 0) {
        int pg = idx[l - 1].find(lk[l][i] >> 2);
        parent[g] = pg;
        child[4 * (size_t)pg + child_pos[g]] = g;
      }
    }
  }
  // near lists (leaf indices) and interaction lists, built in parallel parts
  // and joined in box order
  auto level_of = [&](int g) {
    int l = 0;
    while (F->lvl_off[l + 1] <= g) l++;
    return l;
  };
  std::vector<int> near_off(1, 0), near_leaf;
  {
    const int nl = (int)lk[L].size();
    const int parts = parallel_part_count(nl, 2048);
    std::vector<std::vector<int>> pl(parts), pc(parts);
    parallel_parts(nl, [&](int t, int lo, int hi) {
      for (int i = lo; i < hi; i++) {
        uint32_t ix, iy;
        demorton(lk[L][i], &ix, &iy);
        int c = 0;
        for (int di = -1; di <= 1; di++)
          for (int dj = -1; dj <= 1; dj++) {
            long a = (long)ix + di, b = (long)iy + dj;
            if (a < 0 || b < 0) continue;
            const int f = idx[L].find(morton((uint32_t)a, (uint32_t)b));
            if (f >= 0) {
              pl[t].push_back(f - F->lvl_off[L]);
              c++;
            }
          }
        pc[t].push_back(c);
      }
    }, 2048);
    for (int t = 0; t < parts; t++) {
      near_leaf.insert(near_leaf.end(), pl[t].begin(), pl[t].end());
      for (int c : pc[t]) near_off.push_back(near_off.back() + c);
    }
  }
  std::vector<int> v_off(1, 0), v_src, v_code;
  {
    const int parts = parallel_part_count(nbox, 2048);
    std::vector<std::vector<int>> ps(parts), pcd(parts), pc(parts);
    parallel_parts(nbox, [&](int t, int lo, int hi) {
      if (lo >= hi) return;
      int l = level_of(lo);
      for (int g = lo; g < hi; g++) {
        while (F->lvl_off[l + 1] <= g) l++;
        int c = 0;
        if (l >= 2) {
          uint32_t ix, iy;
          demorton(lk[l][g - F->lvl_off[l]], &ix, &iy);
          long px = ix >> 1, py = iy >> 1;
          for (int a = -1; a <= 1; a++)
            for (int b = -1; b <= 1; b++)
              for (int u = 0; u < 2; u++)
                for (int w = 0; w < 2; w++) {
                  long sx = 2 * (px + a) + u, sy = 2 * (py + b) + w;
                  if (sx < 0 || sy < 0) continue;
                  long di = (long)ix - sx, dj = (long)iy - sy;
                  if (std::labs(di) <= 1 && std::labs(dj) <= 1) continue;
                  const int f = idx[l].find(morton((uint32_t)sx, (uint32_t)sy));
                  if (f < 0) continue;
                  ps[t].push_back(f);
                  pcd[t].push_back((int)((di + 3) * 7 + (dj + 3)));
                  c++;
                }
        }
        pc[t].push_back(c);
      }
    }, 2048);
    for (int t = 0; t < parts; t++) {
      v_src.insert(v_src.end(), ps[t].begin(), ps[t].end());
      v_code.insert(v_code.end(), pcd[t].begin(), pcd[t].end());
      for (int c : pc[t]) v_off.push_back(v_off.back() + c);
    }
  }
  // translation matrices
  std::vector<double2> Tph(4 * (size_t)p), Mph(49 * (size_t)(p + 1));
  std::vector<double> Tr(4 * (size_t)p * p, 0.0), Sr(4 * (size_t)p * p, 0.0),
      Mr(49 * (size_t)p * p);
  for (int pos = 0; pos < 4; pos++) {
    // child offset from the parent centre in units of the parent side,
    // d = |d| e^(i theta): real cores C(k, j) 0.5^j |d|^(k-j) (M2M rows k,
    // L2L rows j) and the phases e^(i theta k)
    const std::complex<double> d((pos & 2) ? 0.25 : -0.25, (pos & 1) ? 0.25 : -0.25);
    const double ad = std::abs(d), th = std::arg(d);
    for (int k = 0; k < p; k++) {
      const std::complex<double> e = std::polar(1.0, th * k);
      Tph[(size_t)pos * p + k] = make_double2(e.real(), e.imag());
      for (int j = 0; j <= k; j++) {
        const double v = binom(k, j) * std::pow(0.5, j) * std::pow(ad, k - j);
        Tr[(size_t)pos * p * p + (size_t)k * p + j] = v;   // M2M: row k, column j
        Sr[(size_t)pos * p * p + (size_t)j * p + k] = v;   // L2L: row j, column m = k
      }
    }
  }
  for (int di = -3; di <= 3; di++)
    for (int dj = -3; dj <= 3; dj++) {
      int code = (di + 3) * 7 + (dj + 3);
      if (std::abs(di) <= 1 && std::abs(dj) <= 1) continue;
      // rho = 1/d = |rho| e^(i phi): real part Rr(m, k) = (-1)^m C(k+m, m)
      // |rho|^(k+m+1), phases e^(i phi k) for k = 0..p
      const std::complex<double> rho = 1.0 / std::complex<double>(di, dj);
      const double ar = std::abs(rho), phi = std::arg(rho);
      for (int m = 0; m < p; m++)
        for (int k = 0; k < p; k++)
          Mr[(size_t)code * p * p + (size_t)m * p + k] =
              binom(k + m, m) * ((m & 1) ? -1.0 : 1.0) * std::pow(ar, k + m + 1);
      for (int k = 0; k <= p; k++) {
        const std::complex<double> e = std::polar(1.0, phi * k);
        Mph[(size_t)code * (p + 1) + k] = make_double2(e.real(), e.imag());
      }
    }
  // sorted point data
  std::vector<double2> z(n), nw(n);
  std::vector<double> dg(n);
  parallel_ranges(n, [&](int lo, int hi) {
    for (int i = lo; i < hi; i++) {
      int o = order[i];
      z[i] = make_double2(pts[2 * o], pts[2 * o + 1]);
      double w = wts[o] / kPi2;
      nw[i] = make_double2(-w * nrm[2 * o], -w * nrm[2 * o + 1]);
      // Kernel::one_d_kern's coincident-point limit (kernel.cpp:37-38)
      dg[i] = 0.5 + 0.5 * (kap ? kap[o] : 0.0) * wts[o] * (1.0 / kPi2);
    }
  });
  std::vector<int> leaf_box(F->nleaf);
  for (int i = 0; i < F->nleaf; i++) leaf_box[i] = F->lvl_off[L] + i;
  for (int i = 0; i < F->nleaf; i++) {
    long src = 0;
    for (int v = near_off[i]; v < near_off[i + 1]; v++)
      src += leaf_start[near_leaf[v] + 1] - leaf_start[near_leaf[v]];
    F->near_point_pairs += (long)(leaf_start[i + 1] - leaf_start[i]) * src;
  }
  F->near_point_pairs -= n;
  F->order = std::move(order);
  F->leaf_start = std::move(leaf_start);
  F->leaf_box = std::move(leaf_box);
  F->near_off = std::move(near_off);
  F->near_leaf = std::move(near_leaf);
  F->child = std::move(child);
  F->parent = std::move(parent);
  F->child_pos = std::move(child_pos);
  F->v_off = std::move(v_off);
  F->v_src = std::move(v_src);
  F->v_code = std::move(v_code);
  F->z = std::move(z);
  F->nw = std::move(nw);
  F->centre = std::move(centre);
  F->Tr = std::move(Tr);
  F->Sr = std::move(Sr);
  F->Tph = std::move(Tph);
  F->Mr = std::move(Mr);
  F->Mph = std::move(Mph);
  F->diag = std::move(dg);
  return F;
}

std::unique_ptr<Fmm2d, Fmm2dDeleter> fmm2d_upload(const Fmm2dPlan& P, cudaStream_t s) {
  std::unique_ptr<Fmm2d, Fmm2dDeleter> F(new Fmm2d());
  F->stream = s;
  F->n = P.n;
  F->p = P.p;
  F->L = P.L;
  F->nleaf = P.nleaf;
  F->nbox = P.nbox;
  F->lo = P.lo;
  F->side0 = P.side0;
  F->lvl_off = P.lvl_off;
  F->m2l_pairs = (long)P.v_src.size();
  F->near_pairs = (long)P.near_leaf.size();
  F->near_point_pairs = P.near_point_pairs;
  F->d_perm = upload_vec(P.order, &F->owned, s);
  F->d_leaf_start = upload_vec(P.leaf_start, &F->owned, s);
  F->d_leaf_box = upload_vec(P.leaf_box, &F->owned, s);
  F->d_near_off = upload_vec(P.near_off, &F->owned, s);
  F->d_near_leaf = upload_vec(P.near_leaf, &F->owned, s);
  F->d_child = upload_vec(P.child, &F->owned, s);
  F->d_parent = upload_vec(P.parent, &F->owned, s);
  F->d_child_pos = upload_vec(P.child_pos, &F->owned, s);
  F->d_v_off = upload_vec(P.v_off, &F->owned, s);
  F->d_v_src = upload_vec(P.v_src, &F->owned, s);
  F->d_v_code = upload_vec(P.v_code, &F->owned, s);
  F->d_z = upload_vec(P.z, &F->owned, s);
  F->d_nw = upload_vec(P.nw, &F->owned, s);
  F->d_centre = upload_vec(P.centre, &F->owned, s);
  F->d_Tr = upload_vec(P.Tr, &F->owned, s);
  F->d_Sr = upload_vec(P.Sr, &F->owned, s);
  F->d_Tph = upload_vec(P.Tph, &F->owned, s);
  F->d_Mr = upload_vec(P.Mr, &F->owned, s);
  F->d_Mph = upload_vec(P.Mph, &F->owned, s);
  F->d_diag = upload_vec(P.diag, &F->owned, s);
  KI_FMM_CUDA(cudaStreamSynchronize(s));
  return F;
}

std::unique_ptr<Fmm2d, Fmm2dDeleter> fmm2d_build(const double* pts, const double* nrm,
                                                 const double* wts, const double* kap, int n,
                                                 int p, cudaStream_t s) {
  return fmm2d_upload(*fmm2d_plan(pts, nrm, wts, kap, n, p), s);
}

namespace {

// The FP32 copies of the translation matrices and the hi/lo split points.
void ensure_fp32(Fmm2d& F, cudaStream_t s) {
  if (F.d_zf) return;
  auto round = [&](const double2* a, size_t count) {
    float2* d = nullptr;
    KI_FMM_CUDA(pool_malloc((void**)&d, sizeof(float2) * count, s));
    F.owned.push_back(d);
    ki::launch(k_round_cplx, (int)std::min<size_t>(1024, (count + 255) / 256), 256, 0, s, a, count, d);
    return d;
  };
  const size_t pp = (size_t)F.p * F.p;
  F.d_Tph32 = round(F.d_Tph, 4 * (size_t)F.p);
  F.d_Mph32 = round(F.d_Mph, 49 * (size_t)(F.p + 1));
  F.d_nw32 = round(F.d_nw, (size_t)F.n);
  auto round_real = [&](const double* a, size_t count) {
    float* d = nullptr;
    KI_FMM_CUDA(pool_malloc((void**)&d, sizeof(float) * count, s));
    F.owned.push_back(d);
    ki::launch(k_round_real, (int)std::min<size_t>(1024, (count + 255) / 256), 256, 0, s, a, count, d);
    return d;
  };
  F.d_Mr32 = round_real(F.d_Mr, 49 * pp);
  F.d_Tr32 = round_real(F.d_Tr, 4 * pp);
  F.d_Sr32 = round_real(F.d_Sr, 4 * pp);
  auto pair_cplx = [&](const double2* a, size_t count) {
    cpr* d = nullptr;
    KI_FMM_CUDA(pool_malloc((void**)&d, sizeof(cpr) * count, s));
    F.owned.push_back(d);
    ki::launch(k_pair_cplx, (int)std::min<size_t>(1024, (count + 255) / 256), 256, 0, s, a, count, d);
    return d;
  };
  auto pair_real = [&](const double* a, size_t count) {
    pr* d = nullptr;
    KI_FMM_CUDA(pool_malloc((void**)&d, sizeof(pr) * count, s));
    F.owned.push_back(d);
    ki::launch(k_pair_real, (int)std::min<size_t>(1024, (count + 255) / 256), 256, 0, s, a, count, d);
    return d;
  };
  F.d_Tph2 = pair_cplx(F.d_Tph, 4 * (size_t)F.p);
  F.d_Mph2 = pair_cplx(F.d_Mph, 49 * (size_t)(F.p + 1));
  F.d_Mr2 = pair_real(F.d_Mr, 49 * pp);
  F.d_Tr2 = pair_real(F.d_Tr, 4 * pp);
  F.d_Sr2 = pair_real(F.d_Sr, 4 * pp);
  float4* zf = nullptr;
  KI_FMM_CUDA(pool_malloc((void**)&zf, sizeof(float4) * (size_t)F.n, s));
  F.owned.push_back(zf);
  ki::launch(k_split_points, (F.n + 255) / 256, 256, 0, s, F.d_z, F.n, zf);
  float4* nwf = nullptr;
  KI_FMM_CUDA(pool_malloc((void**)&nwf, sizeof(float4) * (size_t)F.n, s));
  F.owned.push_back(nwf);
  ki::launch(k_split_points, (F.n + 255) / 256, 256, 0, s, F.d_nw, F.n, nwf);
  KI_FMM_CUDA(cudaGetLastError());
  F.d_zf = zf;
  F.d_nwf = nwf;
}

template <typename R>
void apply_impl(Fmm2d& F, const R* Tr, const R* Sr, const cplx_t<R>* Tph, const R* Mr,
                const cplx_t<R>* Mph,
                const double* mu, int ldmu, int ncols, double* y, int ldy, cudaStream_t s, int p,
                StageRecorder* rec, const char* const* names) {
  using V = cplx_t<R>;
  const int n = F.n, L = F.L, nbox = F.nbox, ldm = F.p;
  const int nc_max = std::min(ncols, kCols);
  R* q = nullptr;
  V *me = nullptr, *le = nullptr;
  KI_FMM_CUDA(pool_malloc((void**)&q, sizeof(R) * (size_t)n * kCols, s));
  KI_FMM_CUDA(pool_malloc((void**)&me, sizeof(V) * (size_t)nbox * p * nc_max, s));
  KI_FMM_CUDA(pool_malloc((void**)&le, sizeof(V) * (size_t)nbox * p * nc_max, s));
  for (int c0 = 0; c0 < ncols; c0 += kCols) {
    const int nc = std::min(kCols, ncols - c0);
    // algorithmic flops per column (complex FMA = 8, real-by-complex = 4,
    // rotation = 6): P2M 4 n p (+ 6 n p column-independent), M2M and L2L
    // (rotated) 2 p(p+1) + 14 p per child link / per box below level 2, M2L
    // (rotated) 4 p^2 + 14 p per interaction pair, near field 2 per point
    // pair (+ 12 per pair for the entry), local expansion 4 n p (+ 6 n p)
    const double pp = p, cx = nc;
    const int nl2 = F.lvl_off[L + 1] - F.lvl_off[3 > L ? L + 1 : 3];
    if (rec) rec->begin(names[0], (double)n * pp * (4.0 * cx + 6.0) +
                                  cx * (double)(nbox - 1) * (2.0 * pp * (pp + 1) + 14.0 * pp));
    ki::launch(k_densities<R>, (n + 31) / 32, dim3(32, 8), 0, s, F.d_perm, n, mu, ldmu, c0, nc, q);
    ki::launch(k_p2m<R>, F.nleaf, 256, 0, s, F.d_leaf_start, F.d_leaf_box, F.d_centre,
                                     F.side0 / (double)(1L << L), F.d_z, F.d_nw, q, nc, p, me);
    for (int l = L; l >= 1; l--) {
      const int b0 = F.lvl_off[l - 1], cnt = F.lvl_off[l] - b0;
      ki::launch(k_m2m<R>, cnt, 256, 0, s, b0, F.d_child, F.d_child_pos, Tr, Tph, ldm, nc, p, me);
    }
    if (rec) rec->end();
    KI_FMM_CUDA(cudaMemsetAsync(le, 0, sizeof(V) * (size_t)F.lvl_off[2] * p * nc, s));
    // M2L in rotated form: p^2 real-by-complex products (4 flops) and 2p
    // complex rotations per pair and column
    if (rec) rec->begin(names[1], cx * (double)F.m2l_pairs * (4.0 * pp * pp + 14.0 * pp));
    for (int l = 2; l <= L; l++) {
      const int b0 = F.lvl_off[l], cnt = F.lvl_off[l + 1] - b0;
      ki::launch(k_m2l<R>, cnt, 256, 0, s, b0, F.d_v_off, F.d_v_src, F.d_v_code, Mr, Mph, ldm,
                                   (double)(1L << l) / F.side0, nc, p, me, le);
    }
    if (rec) rec->end();
    if (rec) rec->begin(names[2], cx * (double)nl2 * (2.0 * pp * (pp + 1) + 14.0 * pp));
    for (int l = 3; l <= L; l++) {
      const int b0 = F.lvl_off[l], cnt = F.lvl_off[l + 1] - b0;
      ki::launch(k_l2l<R>, cnt, 256, 0, s, b0, F.d_parent, F.d_child_pos, Sr, Tph, ldm, nc, p, le);
    }
    if (rec) rec->end();
    if (rec) rec->begin(names[3], (double)F.near_point_pairs * (2.0 * cx + 12.0) +
                                  (double)n * pp * (4.0 * cx + 6.0));
    ki::launch(k_leaf_eval<R>, F.nleaf, kLeafThreads, 0, s,
        F.d_leaf_start, F.d_leaf_box, F.d_near_off, F.d_near_leaf, F.d_centre,
        F.side0 / (double)(1L << L), F.d_z, F.d_zf, F.d_nw32, F.d_nwf, F.d_diag, F.d_perm, q, le,
        nc, p, mu, ldmu, c0, y, ldy);
    if (rec) rec->end();
    KI_FMM_CUDA(cudaGetLastError());
  }
  KI_FMM_CUDA(cudaFreeAsync(q, s));
  KI_FMM_CUDA(cudaFreeAsync(me, s));
  KI_FMM_CUDA(cudaFreeAsync(le, s));
}

}  // namespace

void fmm2d_apply(Fmm2d& F, const double* mu, int ldmu, int ncols, double* y, int ldy,
                 cudaStream_t s, int order, StageRecorder* rec, FmmArith arith) {
  const int p = order > 0 ? std::min(order, F.p) : F.p;
  if (arith == FmmArith::kF32) {
    static const char* const names[4] = {"fmm32_upward", "fmm32_m2l", "fmm32_l2l", "fmm32_near"};
    ensure_fp32(F, s);
    apply_impl<float>(F, F.d_Tr32, F.d_Sr32, F.d_Tph32, F.d_Mr32, F.d_Mph32, mu, ldmu, ncols, y,
                      ldy, s, p, rec, names);
  } else {
    static const char* const names[4] = {"fmm_upward", "fmm_m2l", "fmm_l2l", "fmm_near"};
    ensure_fp32(F, s);   // the pair tables and the near field's point and nw pairs
    apply_impl<pr>(F, F.d_Tr2, F.d_Sr2, F.d_Tph2, F.d_Mr2, F.d_Mph2, mu, ldmu, ncols, y, ldy, s,
                       p, rec, names);
  }
}

int fmm2d_order(const Fmm2d& f) { return f.p; }

void fmm2d_stats(const Fmm2d& f, int* level, int* leaves, int* boxes, long* m2l_pairs,
                 long* near_pairs) {
  *level = f.L;
  *leaves = f.nleaf;
  *boxes = f.nbox;
  *m2l_pairs = f.m2l_pairs;
  *near_pairs = f.near_pairs;
}

}  // namespace ki
