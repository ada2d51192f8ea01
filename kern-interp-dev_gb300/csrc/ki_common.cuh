// Shared device-side definitions: point data, the Nystrom kernel entries and
// small CTA-cooperative dense linear-algebra helpers.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace ki {

// Point data, structure-of-arrays, resident in HBM for the whole factorization.
// 2D uses x, y, nx, ny, w, kappa; 3D adds z, nz and the precomputed diagonal
// entries (Kernel::compute_diag_entries_3dlaplace / _3dstokes,
// kern_interp/kernel/kernel.cpp:124-301): one per point for Laplace, a
// row-major 3 x 3 tensor per point for Stokes.
template <typename T>
struct Points {
  const T* x;
  const T* y;
  const T* nx;
  const T* ny;
  const T* w;
  const T* kappa;
  const T* z = nullptr;
  const T* nz = nullptr;
  const T* diag = nullptr;
  int dim = 2;
  // FP32 form: low parts of the coordinates (x = x + xl exactly to ~2^-48
  // relative), so that differences of nearby points are formed without the
  // cancellation of rounded absolute coordinates; nullptr in FP64.
  const T* xl = nullptr;
  const T* yl = nullptr;
  const T* zl = nullptr;
  // 2D scalar kernels other than the Laplace double layer (Kernel::Pde,
  // kern_interp/kernel/kernel.h:19-24): kPdeNeumann, kPdeGauss; 0 otherwise
  int pde = 0;
};

// Kernel::Pde values of the scalar 2D kernels that Points::pde selects.
constexpr int kPdeNeumann = 1;
constexpr int kPdeGauss = 2;

// Coordinate difference a - b from (hi, lo) pairs: hi[a] - hi[b] is exact for
// nearby points (Sterbenz), so the difference keeps full relative accuracy.
template <typename T>
__device__ __forceinline__ T pdiff(const T* hi, const T* lo, int a, int b) {
  return lo ? (hi[a] - hi[b]) + (lo[a] - lo[b]) : hi[a] - hi[b];
}

constexpr double kPi = 3.14159265358979323846;

// Nystrom entry K(target dof, source dof) of the 2D double-layer kernels.
// Laplace: Kernel::one_d_kern (kern_interp/kernel/kernel.cpp:33-43);
// Stokes:  Kernel::two_d_kern (kern_interp/kernel/kernel.cpp:65-87).
// r = t - s; an exactly coincident pair takes the diagonal limit.
template <typename T>
__device__ __forceinline__ T laplace_entry_r(T r1, T r2, T snx, T sny, T sw, T sk) {
  if (r1 == T(0) && r2 == T(0)) return T(0.5) + T(0.5) * sk * sw * T(1.0 / (2 * kPi));
  return -sw * T(1.0 / (2 * kPi)) * (r1 * snx + r2 * sny) / (r1 * r1 + r2 * r2);
}

template <typename T>
__device__ __forceinline__ T laplace_entry(T tx, T ty, T sx, T sy, T snx, T sny, T sw, T sk) {
  return laplace_entry_r<T>(tx - sx, ty - sy, snx, sny, sw, sk);
}

// Interior Neumann problem (Kernel::one_d_kern, LAPLACE_NEUMANN,
// kern_interp/kernel/kernel.cpp:44-54): the adjoint double layer
// w/(2 pi) (r.n_t)/|r|^2 plus the rank-one term w that removes the constant
// null space; a coincident pair takes w - 1/2 + kappa w/(4 pi).  Domain
// targets (forward) take the single layer w/(2 pi) log|r|.
template <typename T>
__device__ __forceinline__ T neumann_entry_r(T r1, T r2, T tnx, T tny, T sw, T sk) {
  if (r1 == T(0) && r2 == T(0)) return sw - T(0.5) + T(0.5) * sk * sw * T(1.0 / (2 * kPi));
  return sw + sw * T(1.0 / (2 * kPi)) * (r1 * tnx + r2 * tny) / (r1 * r1 + r2 * r2);
}
template <typename T>
__device__ __forceinline__ T neumann_forward_r(T r1, T r2, T sw) {
  return sw * T(1.0 / (2 * kPi)) * log(sqrt(r1 * r1 + r2 * r2));
}

// Gaussian covariance kernel (Kernel::one_d_kern, GAUSS, kernel.cpp:55-60):
// exp(-|r|^2), 5 on the diagonal; no quadrature weight, the same for domain
// targets.
template <typename T>
__device__ __forceinline__ T gauss_entry_r(T r1, T r2) {
  if (r1 == T(0) && r2 == T(0)) return T(5);
  return exp(-(r1 * r1 + r2 * r2));
}

// Scalar 2D entry of Points::pde between target (normal tn) and source.
template <typename T>
__device__ __forceinline__ T scalar2_entry_r(int pde, T r1, T r2, T tnx, T tny, T snx, T sny, T sw,
                                             T sk) {
  if (pde == kPdeNeumann) return neumann_entry_r<T>(r1, r2, tnx, tny, sw, sk);
  if (pde == kPdeGauss) return gauss_entry_r<T>(r1, r2);
  return laplace_entry_r<T>(r1, r2, snx, sny, sw, sk);
}

template <typename T>
__device__ __forceinline__ T stokes_entry_r(int tpar, int spar, T r1, T r2, T tnx, T tny,
                                            T snx, T sny, T sw, T sk) {
  T sn[2] = {snx, sny};
  T tn[2] = {tnx, tny};
  int is_diag = (tpar + spar + 1) % 2;
  if (r1 == T(0) && r2 == T(0)) {
    return T(-0.5) * T(is_diag) +
           T(1 - 2 * is_diag) * T(0.5) * sk * sw * T(1.0 / kPi) * sn[(tpar + 1) % 2] *
               sn[(spar + 1) % 2] +
           sw * tn[tpar] * sn[spar];
  }
  T r[2] = {r1, r2};
  T rr = r1 * r1 + r2 * r2;
  return sw * T(1.0 / kPi) * (r1 * snx + r2 * sny) / (rr * rr) * r[tpar] * r[spar] +
         sw * tn[tpar] * sn[spar];
}

template <typename T>
__device__ __forceinline__ T stokes_entry(int tpar, int spar, T tx, T ty, T tnx, T tny, T sx,
                                          T sy, T snx, T sny, T sw, T sk) {
  return stokes_entry_r<T>(tpar, spar, tx - sx, ty - sy, tnx, tny, snx, sny, sw, sk);
}

// 3D Laplace double layer (Kernel::three_d_laplace, kernel.cpp:104-121):
// -w/(4 pi) (r.n_s)/|r|^3, r = t - s; a coincident pair takes `diag`.
template <typename T>
__device__ __forceinline__ T laplace3_entry(T r1, T r2, T r3, T snx, T sny, T snz, T sw, T diag) {
  if (r1 == T(0) && r2 == T(0) && r3 == T(0)) return diag;
  T rr = r1 * r1 + r2 * r2 + r3 * r3;
  return -sw * T(1.0 / (4 * kPi)) * (r1 * snx + r2 * sny + r3 * snz) / (rr * sqrt(rr));
}

// 3D Stokes completed double layer (Kernel::three_d_stokes, kernel.cpp:89-102):
// -3/(4 pi) w (r.n_s) r_i r_j / |r|^5 + w n_t,i n_s,j; a coincident pair
// takes the (i, j) element of the source point's diagonal tensor.
template <typename T>
__device__ __forceinline__ T stokes3_entry(int tpar, int spar, T r1, T r2, T r3, T tnx, T tny,
                                           T tnz, T snx, T sny, T snz, T sw, const T* diag9) {
  if (r1 == T(0) && r2 == T(0) && r3 == T(0)) return diag9 ? diag9[3 * tpar + spar] : T(0);
  const T r[3] = {r1, r2, r3};
  const T tn[3] = {tnx, tny, tnz};
  const T sn[3] = {snx, sny, snz};
  T rr = r1 * r1 + r2 * r2 + r3 * r3;
  return sw * T(-3.0 / (4 * kPi)) * (r1 * snx + r2 * sny + r3 * snz) / (rr * rr * sqrt(rr)) *
             r[tpar] * r[spar] +
         sw * tn[tpar] * sn[spar];
}

// Entry between two boundary DOFs: 2D Laplace (sol_dim 1), 2D Stokes
// (sol_dim 2, DOF 2p+i = node p component i), 3D Laplace (sol_dim 1), 3D
// Stokes (sol_dim 3, DOF 3p+i).
template <typename T>
__device__ __forceinline__ T kernel_entry(const Points<T>& P, int sol_dim, int tdof, int sdof) {
  if (P.dim == 3) {
    if (sol_dim == 1)
      return laplace3_entry<T>(pdiff(P.x, P.xl, tdof, sdof), pdiff(P.y, P.yl, tdof, sdof),
                               pdiff(P.z, P.zl, tdof, sdof), P.nx[sdof], P.ny[sdof], P.nz[sdof],
                               P.w[sdof], P.diag ? P.diag[sdof] : T(0));
    const int tp = tdof / 3, sp = sdof / 3;
    return stokes3_entry<T>(tdof - 3 * tp, sdof - 3 * sp, pdiff(P.x, P.xl, tp, sp),
                            pdiff(P.y, P.yl, tp, sp), pdiff(P.z, P.zl, tp, sp), P.nx[tp], P.ny[tp],
                            P.nz[tp], P.nx[sp], P.ny[sp], P.nz[sp], P.w[sp],
                            P.diag ? P.diag + 9 * (size_t)sp : nullptr);
  }
  if (sol_dim == 1) {
    if (P.pde)
      return scalar2_entry_r<T>(P.pde, pdiff(P.x, P.xl, tdof, sdof), pdiff(P.y, P.yl, tdof, sdof),
                                P.nx[tdof], P.ny[tdof], P.nx[sdof], P.ny[sdof], P.w[sdof],
                                P.kappa[sdof]);
    return laplace_entry_r<T>(pdiff(P.x, P.xl, tdof, sdof), pdiff(P.y, P.yl, tdof, sdof),
                              P.nx[sdof], P.ny[sdof], P.w[sdof], P.kappa[sdof]);
  }
  int tp = tdof >> 1, sp = sdof >> 1;
  return stokes_entry_r<T>(tdof & 1, sdof & 1, pdiff(P.x, P.xl, tp, sp), pdiff(P.y, P.yl, tp, sp),
                           P.nx[tp], P.ny[tp], P.nx[sp], P.ny[sp], P.w[sp], P.kappa[sp]);
}

// Point of a DOF.
__device__ __forceinline__ int dof_point(int dof, int sol_dim) {
  return sol_dim == 1 ? dof : (sol_dim == 2 ? dof >> 1 : dof / 3);
}

// ------------------------------------------------------------------------
// FP32-pair arithmetic (a value as hi + lo, |lo| <= ulp(hi)/2) for FP64-accurate
// sums on the FP32 pipes, which run at 64x the FP64 rate on this part.

// An FP64 value as an FP32 pair: hi = fl(v), lo = fl(v - hi) (48 bits kept).
__device__ __forceinline__ float2 split_pair(double v) {
  const float h = (float)v;
  return make_float2(h, (float)(v - (double)h));
}

// h + l += e * d for FP32 pairs (value = hi + lo): the product of the high
// parts is split exactly (p + fma(e_h, d_h, -p)), the cross terms join its
// error, and p enters the sum through Knuth's two-sum, whose rounding error
// goes to l with the rest.  The _rn intrinsics keep the compiler from fusing
// the separately rounded steps.  Each step adds an error near 2^-48 of the
// partial sum, so a near-field sum of a few hundred pairs keeps ~1e-13
// relative accuracy while the arithmetic runs on the FP32 pipes.
__device__ __forceinline__ void pair_fma(float& h, float& l, float2 e, float2 d) {
  const float p = __fmul_rn(e.x, d.x);
  float q = fmaf(e.x, d.x, -p);
  q = fmaf(e.x, d.y, q);
  q = fmaf(e.y, d.x, q);
  const float sum = __fadd_rn(h, p);
  const float bp = __fsub_rn(sum, h);
  const float err = __fadd_rn(__fsub_rn(h, __fsub_rn(sum, bp)), __fsub_rn(p, bp));
  l = __fadd_rn(l, __fadd_rn(err, q));
  h = sum;
}

// Error-free transforms (Knuth's two-sum and two-difference, Dekker's fast
// two-sum for |a| >= |b|): hi + lo equals the exact result.
__device__ __forceinline__ void two_sum(float a, float b, float& hi, float& lo) {
  hi = __fadd_rn(a, b);
  const float bb = __fsub_rn(hi, a);
  lo = __fadd_rn(__fsub_rn(a, __fsub_rn(hi, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void two_diff(float a, float b, float& hi, float& lo) {
  hi = __fsub_rn(a, b);
  const float bb = __fsub_rn(hi, a);
  lo = __fsub_rn(__fsub_rn(a, __fsub_rn(hi, bb)), __fadd_rn(b, bb));
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& hi, float& lo) {
  hi = __fadd_rn(a, b);
  lo = __fsub_rn(b, __fsub_rn(hi, a));
}

// h + l = (ah + al)(bh + bl) to ~2^-47 relative: the high product split
// exactly by an fma, the cross terms added to its error.
__device__ __forceinline__ void pair_mul(float ah, float al, float bh, float bl, float& h,
                                         float& l) {
  h = __fmul_rn(ah, bh);
  l = __fmaf_rn(ah, bl, __fmaf_rn(al, bh, __fmaf_rn(ah, bh, -h)));
}

// The 3D double-layer pair term (r . c) / |r|^3, r = t - s, in FP32-pair
// arithmetic: t = (tx, ty, tz) and s = (sh + sl) as hi/lo pairs, c = ch + cl
// (the source's normal scaled by its weight and -1/(4 pi)).  r by
// two-differences of the hi parts plus the lo differences; |r|^2 with exact
// squares; 1/|r| by one Newton step y0 (1 + e/2), e = 1 - |r|^2 y0^2, from
// the FP32 estimate y0 (relative error ~2^-23 -> ~2^-46); the dot product
// and the products with their rounding errors carried.  ~1e-13 relative
// (where r . c cancels, ~2^-48 of |r| |c| absolute).  Returns false, with
// nothing written, when r is exactly zero.
__device__ __forceinline__ bool pair_dipole3(float2 tx, float2 ty, float2 tz, float4 sh, float4 sl,
                                             float4 ch, float4 cl, float& kh, float& kl) {
  float dxh, dxl, dyh, dyl, dzh, dzl;
  two_diff(tx.x, sh.x, dxh, dxl);
  two_diff(ty.x, sh.y, dyh, dyl);
  two_diff(tz.x, sh.z, dzh, dzl);
  fast_two_sum(dxh, __fadd_rn(dxl, __fsub_rn(tx.y, sl.x)), dxh, dxl);
  fast_two_sum(dyh, __fadd_rn(dyl, __fsub_rn(ty.y, sl.y)), dyh, dyl);
  fast_two_sum(dzh, __fadd_rn(dzl, __fsub_rn(tz.y, sl.z)), dzh, dzl);
  const float a = __fmul_rn(dxh, dxh), b = __fmul_rn(dyh, dyh), d = __fmul_rn(dzh, dzh);
  float s1h, s1l, r2h, r2l;
  two_sum(a, b, s1h, s1l);
  two_sum(s1h, d, r2h, r2l);
  float lo = __fadd_rn(__fmaf_rn(dxh, dxh, -a),
                       __fadd_rn(__fmaf_rn(dyh, dyh, -b), __fmaf_rn(dzh, dzh, -d)));
  lo = __fmaf_rn(2.f * dxh, dxl, __fmaf_rn(2.f * dyh, dyl, __fmaf_rn(2.f * dzh, dzl, lo)));
  r2l = __fadd_rn(r2l, __fadd_rn(s1l, lo));
  fast_two_sum(r2h, r2l, r2h, r2l);
  if (r2h == 0.f) return false;
  const float y0 = rsqrtf(r2h);
  const float p = __fmul_rn(y0, y0), pe = __fmaf_rn(y0, y0, -p);
  const float q = __fmul_rn(r2h, p);
  const float qe = __fmaf_rn(r2h, pe, __fmaf_rn(r2l, p, __fmaf_rn(r2h, p, -q)));
  const float e = __fsub_rn(__fsub_rn(1.f, q), qe);
  float yh, yl;
  fast_two_sum(y0, __fmul_rn(__fmul_rn(0.5f, y0), e), yh, yl);
  float y2h, y2l, y3h, y3l;
  pair_mul(yh, yl, yh, yl, y2h, y2l);
  pair_mul(y2h, y2l, yh, yl, y3h, y3l);
  float m1h, m1l, m2h, m2l, m3h, m3l;
  pair_mul(dxh, dxl, ch.x, cl.x, m1h, m1l);
  pair_mul(dyh, dyl, ch.y, cl.y, m2h, m2l);
  pair_mul(dzh, dzl, ch.z, cl.z, m3h, m3l);
  float uh, ul, vh, vl;
  two_sum(m1h, m2h, uh, ul);
  two_sum(uh, m3h, vh, vl);
  vl = __fadd_rn(vl, __fadd_rn(ul, __fadd_rn(m1l, __fadd_rn(m2l, m3l))));
  fast_two_sum(vh, vl, vh, vl);
  pair_mul(vh, vl, y3h, y3l, kh, kl);
  return true;
}

// Squared distance |t - s|^2 of two points given as FP32 pairs
// (hi x, hi y, lo x, lo y), as a pair (value r2.x + r2.y).
__device__ __forceinline__ float2 pair_dist2(const float4& t, const float4& s) {
  float dxh, dxl, dyh, dyl;
  two_diff(t.x, s.x, dxh, dxl);
  two_diff(t.y, s.y, dyh, dyl);
  fast_two_sum(dxh, __fadd_rn(dxl, __fsub_rn(t.z, s.z)), dxh, dxl);
  fast_two_sum(dyh, __fadd_rn(dyl, __fsub_rn(t.w, s.w)), dyh, dyl);
  const float a = __fmul_rn(dxh, dxh), b = __fmul_rn(dyh, dyh);
  float r2h, r2l;
  two_sum(a, b, r2h, r2l);
  r2l = __fadd_rn(r2l, __fadd_rn(__fmaf_rn(dxh, dxh, -a), __fmaf_rn(dyh, dyh, -b)));
  r2l = __fmaf_rn(2.f * dxh, dxl, __fmaf_rn(2.f * dyh, dyl, r2l));
  fast_two_sum(r2h, r2l, r2h, r2l);
  return make_float2(r2h, r2l);
}

// log(x) of a positive normal FP32 pair x = xh + xl, as a pair, by Tang's
// table-driven method (ACM TOMS 16, 1990): x = 2^e m, m in [1, 2); with
// c = 1 + (j + 1/2)/256 for the leading 8 bits j of m's fraction,
// log x = e ln2 + log c + log1p(t), t = (m - c)/c, |t| <= 2^-9, where log c
// comes from `logc` (pairs, formed in FP64 on the host) and log1p(t) from its
// series t - t^2/2 + t^3/3 - t^4/4 + t^5/5 (the next term is below 2^-56), the
// first two terms in pair arithmetic.  ln2 is split in three so that e ln2_h
// is exact.  Absolute error about 2^-47 |log x|.
__device__ __forceinline__ float2 pair_log(float xh, float xl, const float2* logc) {
  constexpr double kLn2 = 0.69314718055994530942;
  constexpr float kLn2H = 0.693145751953125f;   // 45426 / 2^16
  constexpr float kLn2M = (float)(kLn2 - 0.693145751953125);
  constexpr float kLn2L = (float)(kLn2 - 0.693145751953125 - (double)kLn2M);
  const int bits = __float_as_int(xh);
  const int e = ((bits >> 23) & 0xff) - 127;
  const float m = __int_as_float((bits & 0x007fffff) | 0x3f800000);
  const int j = (bits >> 15) & 0xff;
  const float c = 1.f + ((float)j + 0.5f) * (1.f / 256.f);   // exact
  const float dl = __fmul_rn(xl, __int_as_float((127 - e) << 23));   // xl 2^-e, exact
  const float dh = __fsub_rn(m, c);                                   // exact (Sterbenz)
  const float rc = __frcp_rn(c);
  const float th = __fmul_rn(dh, rc);
  const float tl = __fmul_rn(__fadd_rn(__fmaf_rn(-th, c, dh), dl), rc);
  const float q = __fmul_rn(th, th);
  const float qe = __fmaf_rn(th, th, -q);
  const float rest = __fmul_rn(__fmul_rn(th, q),
                               __fmaf_rn(-th, __fmaf_rn(-th, 0.2f, 0.25f), 1.f / 3.f));
  float sh, sl;
  two_sum(th, -0.5f * q, sh, sl);
  sl = __fadd_rn(sl, __fadd_rn(__fsub_rn(tl, __fmaf_rn(0.5f, qe, th * tl)), rest));
  const float2 lc = logc[j];
  const float fe = (float)e;
  const float pm = __fmul_rn(fe, kLn2M);
  float s1, e1, s2, e2, s3, e3;
  two_sum(fe * kLn2H, lc.x, s1, e1);
  two_sum(s1, pm, s2, e2);
  two_sum(s2, sh, s3, e3);
  const float lo = __fadd_rn(__fadd_rn(__fadd_rn(e1, e2), __fadd_rn(e3, __fmaf_rn(fe, kLn2M, -pm))),
                             __fadd_rn(__fmaf_rn(fe, kLn2L, lc.y), sl));
  float rh, rl;
  two_sum(s3, lo, rh, rl);
  return make_float2(rh, rl);
}

// ------------------------------------------------------------------------
// CTA-cooperative dense helpers on column-major matrices (shared or global
// memory).  All threads of the block must call them.

// Register-tiled body of cta_gemm_to: each thread owns TI x TJ outputs,
// rows r0 + ii*mt and columns c0 + jj*nt (strided, so that consecutive
// threads touch consecutive rows), and keeps TI + TJ operands in registers
// per step of the inner dimension.  op(A)(i, l) = A[i*sai + l*sal] and
// op(B)(l, j) = B[l*sbl + j*sbj].  Every output is the sum over l in
// increasing order, as in the one-output-per-thread form.
template <typename T, int TI, int TJ>
__device__ __forceinline__ void cta_gemm_rt(int m, int n, int kk, T alpha, const T* A, int sai,
                                            int sal, const T* B, int sbl, int sbj, T beta,
                                            const T* Cin, int ldci, T* C, int ldc) {
  const int mt = (m + TI - 1) / TI, nt = (n + TJ - 1) / TJ;
  for (int t = threadIdx.x; t < mt * nt; t += blockDim.x) {
    const int r0 = t % mt, c0 = t / mt;
    int ia[TI], jb[TJ];
#pragma unroll
    for (int ii = 0; ii < TI; ii++) ia[ii] = min(r0 + ii * mt, m - 1) * sai;
#pragma unroll
    for (int jj = 0; jj < TJ; jj++) jb[jj] = min(c0 + jj * nt, n - 1) * sbj;
    T acc[TI][TJ];
#pragma unroll
    for (int ii = 0; ii < TI; ii++)
#pragma unroll
      for (int jj = 0; jj < TJ; jj++) acc[ii][jj] = T(0);
    int oa = 0, ob = 0;
    for (int l = 0; l < kk; l++) {
      T a[TI], b[TJ];
#pragma unroll
      for (int ii = 0; ii < TI; ii++) a[ii] = A[ia[ii] + oa];
#pragma unroll
      for (int jj = 0; jj < TJ; jj++) b[jj] = B[jb[jj] + ob];
#pragma unroll
      for (int ii = 0; ii < TI; ii++)
#pragma unroll
        for (int jj = 0; jj < TJ; jj++) acc[ii][jj] += a[ii] * b[jj];
      oa += sal;
      ob += sbl;
    }
#pragma unroll
    for (int ii = 0; ii < TI; ii++)
#pragma unroll
      for (int jj = 0; jj < TJ; jj++) {
        const int i = r0 + ii * mt, j = c0 + jj * nt;
        if (i < m && j < n)
          C[i + (size_t)ldc * j] =
              (beta == T(0) ? T(0) : beta * Cin[i + (size_t)ldci * j]) + alpha * acc[ii][jj];
      }
  }
}

// C(m x n) = beta*Cin + alpha * op(A) * op(B); op(A) is m x kk; Cin may be C.
// The thread tile (1x1, 2x2, 4x2 or 4x4 outputs) is the one with the fewest
// instructions on a thread's path: rounds over the block times (FMAs + loads)
// per inner step, ties to the larger tile (fewer loads in total).
template <typename T>
__device__ void cta_gemm_to(int m, int n, int kk, T alpha, const T* A, int lda, bool ta,
                            const T* B, int ldb, bool tb, T beta, const T* Cin, int ldci, T* C,
                            int ldc) {
  if (m <= 0 || n <= 0) return;
  const int sai = ta ? lda : 1, sal = ta ? 1 : lda;
  const int sbl = tb ? ldb : 1, sbj = tb ? 1 : ldb;
  const int nth = blockDim.x;
  auto cost = [&](int ti, int tj) {
    const int tiles = ((m + ti - 1) / ti) * ((n + tj - 1) / tj);
    return ((tiles + nth - 1) / nth) * (ti * tj + ti + tj);
  };
  const int c11 = cost(1, 1), c22 = cost(2, 2), c42 = cost(4, 2), c44 = cost(4, 4);
  if (c44 <= c42 && c44 <= c22 && c44 <= c11)
    cta_gemm_rt<T, 4, 4>(m, n, kk, alpha, A, sai, sal, B, sbl, sbj, beta, Cin, ldci, C, ldc);
  else if (c42 <= c22 && c42 <= c11)
    cta_gemm_rt<T, 4, 2>(m, n, kk, alpha, A, sai, sal, B, sbl, sbj, beta, Cin, ldci, C, ldc);
  else if (c22 <= c11)
    cta_gemm_rt<T, 2, 2>(m, n, kk, alpha, A, sai, sal, B, sbl, sbj, beta, Cin, ldci, C, ldc);
  else
    cta_gemm_rt<T, 1, 1>(m, n, kk, alpha, A, sai, sal, B, sbl, sbj, beta, Cin, ldci, C, ldc);
}

// C(m x n) = beta*C + alpha * op(A) * op(B); op(A) is m x kk.
template <typename T>
__device__ void cta_gemm(int m, int n, int kk, T alpha, const T* A, int lda, bool ta,
                         const T* B, int ldb, bool tb, T beta, T* C, int ldc) {
  cta_gemm_to<T>(m, n, kk, alpha, A, lda, ta, B, ldb, tb, beta, C, ldc, C, ldc);
}

// f(i, c) for the elements e = threadIdx.x, threadIdx.x + blockDim.x, ... of
// a rows x cols rectangle, i = e % rows, c = e / rows, advanced without a
// division per element.
template <typename F>
__device__ __forceinline__ void cta_for_2d(int rows, int cols, F f) {
  if (rows <= 0 || cols <= 0) return;
  const int nth = blockDim.x;
  int i = (int)threadIdx.x % rows, c = (int)threadIdx.x / rows;
  const int di = nth % rows, dc = nth / rows;
  while (c < cols) {
    f(i, c);
    i += di;
    c += dc;
    if (i >= rows) {
      i -= rows;
      c++;
    }
  }
}

// In-place LU with partial pivoting (dgetrf semantics, 0-based pivots:
// row i was swapped with piv[i]).  Returns the first zero pivot + 1, or 0.
template <typename T>
__device__ int cta_lu(int n, T* A, int lda, int* piv, int* s_flag, T* s_red, int* s_idx) {
  int info = 0;
  for (int j = 0; j < n; j++) {
    // pivot search: warp 0 scans rows j..n-1
    if (threadIdx.x < 32) {
      T best = T(-1);
      int bi = j;
      for (int i = j + threadIdx.x; i < n; i += 32) {
        T v = fabs(A[i + (size_t)lda * j]);
        if (v > best) { best = v; bi = i; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        T ov = __shfl_down_sync(0xffffffff, best, o);
        int oi = __shfl_down_sync(0xffffffff, bi, o);
        if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
      }
      if (threadIdx.x == 0) { *s_idx = bi; *s_red = best; }
    }
    __syncthreads();
    int p = *s_idx;
    T pv = *s_red;
    if (threadIdx.x == 0) piv[j] = p;
    if (p != j) {
      for (int c = threadIdx.x; c < n; c += blockDim.x) {
        T t = A[j + (size_t)lda * c];
        A[j + (size_t)lda * c] = A[p + (size_t)lda * c];
        A[p + (size_t)lda * c] = t;
      }
    }
    __syncthreads();
    if (pv == T(0)) {
      if (info == 0) info = j + 1;
      continue;
    }
    T d = A[j + (size_t)lda * j];
    for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) A[i + (size_t)lda * j] /= d;
    __syncthreads();
    const int rows = n - j - 1;
    cta_for_2d(rows, rows, [&](int ii, int cc) {
      const int i = j + 1 + ii, c = j + 1 + cc;
      A[i + (size_t)lda * c] -= A[i + (size_t)lda * j] * A[j + (size_t)lda * c];
    });
    __syncthreads();
  }
  (void)s_flag;
  return info;
}

// In-place inverse by Gauss-Jordan elimination with partial pivoting: at
// step j the row of the largest |A(i, j)|, i >= j, is swapped into row j
// (piv[j], device memory), row j is scaled by 1/pivot with A(j, j) taken as
// 1, and column j is eliminated from every other row, A(i, j) becoming
// -A(i, j)/pivot; the interchanges are finally undone on the columns in
// reverse order.  colj: n entries of scratch (shared memory); s_val: 2.
// Returns the first zero pivot + 1, or 0.
template <typename T>
__device__ int cta_gj_inverse(int n, T* A, int lda, int* piv, T* colj, T* s_val, int* s_idx) {
  int info = 0;
  for (int j = 0; j < n; j++) {
    if (threadIdx.x < 32) {
      T best = T(-1);
      int bi = j;
      for (int i = j + threadIdx.x; i < n; i += 32) {
        T v = fabs(A[i + (size_t)lda * j]);
        if (v > best) { best = v; bi = i; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        T ov = __shfl_down_sync(0xffffffff, best, o);
        int oi = __shfl_down_sync(0xffffffff, bi, o);
        if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
      }
      if (threadIdx.x == 0) {
        *s_idx = bi;
        s_val[0] = A[bi + (size_t)lda * j];
        s_val[1] = A[j + (size_t)lda * j];
        piv[j] = bi;
      }
    }
    __syncthreads();
    const int p = *s_idx;
    const T pv = s_val[0], ajj = s_val[1];
    if (pv == T(0)) {   // the same branch in every thread
      if (info == 0) info = j + 1;
      continue;
    }
    // column j after the interchange (rows other than j and p are not written here)
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      colj[i] = (i == j) ? pv : (i == p ? ajj : A[i + (size_t)lda * j]);
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
      T a = A[j + (size_t)lda * c], b = A[p + (size_t)lda * c];
      if (c == j) { a = ajj; b = pv; }
      A[j + (size_t)lda * c] = (c == j ? T(1) : b) / pv;
      if (p != j) A[p + (size_t)lda * c] = a;
    }
    __syncthreads();
    // elimination over the rows other than j (row j is scaled; A(j, j) = 1/pivot)
    cta_for_2d(n - 1, n, [&](int ii, int c) {
      const int i = ii < j ? ii : ii + 1;
      if (c == j) A[i + (size_t)lda * j] = -colj[i] * A[j + (size_t)lda * j];
      else A[i + (size_t)lda * c] -= colj[i] * A[j + (size_t)lda * c];
    });
    __syncthreads();
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    for (int j = n - 1; j >= 0; j--) {
      const int q = piv[j];
      if (q != j) {
        T t = A[i + (size_t)lda * j];
        A[i + (size_t)lda * j] = A[i + (size_t)lda * q];
        A[i + (size_t)lda * q] = t;
      }
    }
  __syncthreads();
  return info;
}

// The same inverse with the matrix held in registers: lane x of warp w owns
// rows x + 32 a (a < MA) and columns w + W b (b < MAXB), W warps, so that
// each step is one FMA per owned element with the pivot column (per lane) and
// the pivot row (broadcast per warp) read from shared memory.  Rows are not
// swapped: step j takes as pivot the unused row p of largest |A(p, j)| (ties
// to the lowest row; every warp finds it from the staged column, so no
// barrier is spent on the search) and eliminates column j with it in place
// (A(p, j) = 1/pivot, A(p, c) /= pivot, A(i, j) = -A(i, j)/pivot,
// A(i, c) -= A(i, j) A(p, c)); the result is the inverse with rows and
// columns permuted, X^-1(j, m) = A(p_j, c) with p_c = m, which the final store
// undoes.  Two barriers per column.  Requires n <= 32 MA and n <= W MAXB;
// scratch: 3n of T and 2n ints (shared).  piv[j] = p_j (device memory).
// Returns the first zero pivot + 1, or 0.  Not inlined, so that the register
// tile does not compete with the calling kernel's live values (inlined into
// the 64-register Schur kernel it spilled about twice as much).
template <typename T, int MA, int MAXB>
__device__ __noinline__ int cta_gj_inverse_reg(int n, T* A, int lda, int* piv, T* scratch) {
  T* colbuf = scratch;                   // [2][n]: column j (double-buffered)
  T* rowbuf = scratch + 2 * n;           // pivot row after scaling
  int* spiv = reinterpret_cast<int*>(scratch + 3 * n);   // p_j
  int* spinv = spiv + n;                  // j of pivot row p
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, W = blockDim.x >> 5;
  T a[MA][MAXB];
#pragma unroll
  for (int ia = 0; ia < MA; ia++)
#pragma unroll
    for (int ib = 0; ib < MAXB; ib++) {
      const int i = lane + 32 * ia, c = w + W * ib;
      a[ia][ib] = (i < n && c < n) ? A[i + (size_t)lda * c] : T(0);
    }
  // column j of the register tile into colbuf[j & 1] (warp j % W, uniform)
  auto stage_col = [&](int j) {
    if (w != j % W) return;
    const int jb = j / W;
    T* dst = colbuf + (j & 1) * n;
#pragma unroll
    for (int ib = 0; ib < MAXB; ib++)
      if (ib == jb)
#pragma unroll
        for (int ia = 0; ia < MA; ia++) {
          const int i = lane + 32 * ia;
          if (i < n) dst[i] = a[ia][ib];
        }
  };
  stage_col(0);
  unsigned used = 0;   // bit ia: row lane + 32 ia already a pivot row
  int info = 0;
  for (int j = 0; j < n; j++) {
    const T* cj = colbuf + (j & 1) * n;
    __syncthreads();   // column j staged; the previous step's readers of rowbuf done
    T f[MA];
    T best = T(-1);
    int bi = n;
#pragma unroll
    for (int ia = 0; ia < MA; ia++) {
      const int i = lane + 32 * ia;
      f[ia] = i < n ? cj[i] : T(0);
      if (i < n && !((used >> ia) & 1u)) {
        T v = fabs(f[ia]);
        if (!(v == v)) v = T(3e38);   // a NaN orders first, so the choice stays a valid row
        if (v > best) { best = v; bi = i; }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const T ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
    }
    const int p = bi;
    const int pa = p >> 5;
    const bool p_mine = (p & 31) == lane;
    if (p_mine) used |= 1u << pa;
    if (threadIdx.x == 0) {
      piv[j] = p;
      spiv[j] = p;
      spinv[p] = j;
    }
    const T pv = cj[p];
    if (pv == T(0)) {   // the same branch in every thread
      if (info == 0) info = j + 1;
      if (j + 1 < n) stage_col(j + 1);
      continue;
    }
    const T inv = T(1) / pv;
    // the pivot row, scaled, by its owners (lane p % 32 of every warp)
    if (p_mine) {
#pragma unroll
      for (int ia = 0; ia < MA; ia++)
        if (ia == pa)
#pragma unroll
          for (int ib = 0; ib < MAXB; ib++) {
            const int c = w + W * ib;
            if (c < n) {
              const T v = (c == j) ? inv : a[ia][ib] * inv;
              a[ia][ib] = v;
              rowbuf[c] = v;
            }
          }
    }
    __syncthreads();   // rowbuf written
    // every other row: A(i, c) -= f_i A(p, c); column j: -f_i / pivot
#pragma unroll
    for (int ia = 0; ia < MA; ia++)
      if (p_mine && ia == pa) f[ia] = T(0);
#pragma unroll
    for (int ib = 0; ib < MAXB; ib++) {
      const int c = w + W * ib;
      const T rb = c < n ? rowbuf[c] : T(0);
#pragma unroll
      for (int ia = 0; ia < MA; ia++) a[ia][ib] = fma(-f[ia], rb, a[ia][ib]);
    }
    if (w == j % W) {
      const int jb = j / W;
#pragma unroll
      for (int ib = 0; ib < MAXB; ib++)
        if (ib == jb)
#pragma unroll
          for (int ia = 0; ia < MA; ia++)
            if (!(p_mine && ia == pa)) a[ia][ib] = -f[ia] * inv;
    }
    if (j + 1 < n) stage_col(j + 1);
  }
  __syncthreads();   // every step's pivots recorded
  // X^-1(spinv[i], spiv[c]) = a(i, c)
#pragma unroll
  for (int ia = 0; ia < MA; ia++)
#pragma unroll
    for (int ib = 0; ib < MAXB; ib++) {
      const int i = lane + 32 * ia, c = w + W * ib;
      if (i < n && c < n) A[spinv[i] + (size_t)lda * spiv[c]] = a[ia][ib];
    }
  __syncthreads();
  return info;
}

// B(n x nrhs) <- A^-1 B (trans=false) or A^-T B (trans=true) from cta_lu.
template <typename T>
__device__ void cta_lu_solve(int n, const T* LU, int lda, const int* piv, bool trans, T* B,
                             int ldb, int nrhs) {
  if (!trans) {
    // apply row swaps, forward (unit L), backward (U); one thread per column
    for (int c = threadIdx.x; c < nrhs; c += blockDim.x) {
      T* b = B + (size_t)ldb * c;
      for (int i = 0; i < n; i++) {
        int p = piv[i];
        if (p != i) { T t = b[i]; b[i] = b[p]; b[p] = t; }
      }
      for (int i = 0; i < n; i++) {
        T s = b[i];
        for (int l = 0; l < i; l++) s -= LU[i + (size_t)lda * l] * b[l];
        b[i] = s;
      }
      for (int i = n - 1; i >= 0; i--) {
        T s = b[i];
        for (int l = i + 1; l < n; l++) s -= LU[i + (size_t)lda * l] * b[l];
        b[i] = s / LU[i + (size_t)lda * i];
      }
    }
  } else {
    // A^T = U^T L^T P : solve U^T y = b, L^T z = y, then undo swaps reversed
    for (int c = threadIdx.x; c < nrhs; c += blockDim.x) {
      T* b = B + (size_t)ldb * c;
      for (int i = 0; i < n; i++) {
        T s = b[i];
        for (int l = 0; l < i; l++) s -= LU[l + (size_t)lda * i] * b[l];
        b[i] = s / LU[i + (size_t)lda * i];
      }
      for (int i = n - 1; i >= 0; i--) {
        T s = b[i];
        for (int l = i + 1; l < n; l++) s -= LU[l + (size_t)lda * i] * b[l];
        b[i] = s;
      }
      for (int i = n - 1; i >= 0; i--) {
        int p = piv[i];
        if (p != i) { T t = b[i]; b[i] = b[p]; b[p] = t; }
      }
    }
  }
  __syncthreads();
}

// The same solves with every thread of the block: pivots by column, then
// column-oriented substitution (one barrier per row), the update of the
// remaining rows spread over (row, column) pairs.
template <typename T>
__device__ void cta_lu_solve_par(int n, const T* LU, int lda, const int* piv, bool trans, T* B,
                                 int ldb, int nrhs) {
  const int tid = threadIdx.x, nth = blockDim.x;
  if (!trans) {
    for (int c = tid; c < nrhs; c += nth) {
      T* b = B + (size_t)ldb * c;
      for (int i = 0; i < n; i++) {
        int p = piv[i];
        if (p != i) { T t = b[i]; b[i] = b[p]; b[p] = t; }
      }
    }
    __syncthreads();
    for (int l = 0; l < n - 1; l++) {          // unit lower
      cta_for_2d(n - 1 - l, nrhs, [&](int ii, int c) {
        const int i = l + 1 + ii;
        B[i + (size_t)ldb * c] -= LU[i + (size_t)lda * l] * B[l + (size_t)ldb * c];
      });
      __syncthreads();
    }
    for (int l = n - 1; l >= 0; l--) {         // upper
      for (int c = tid; c < nrhs; c += nth) B[l + (size_t)ldb * c] /= LU[l + (size_t)lda * l];
      __syncthreads();
      cta_for_2d(l, nrhs, [&](int i, int c) {
        B[i + (size_t)ldb * c] -= LU[i + (size_t)lda * l] * B[l + (size_t)ldb * c];
      });
      __syncthreads();
    }
  } else {
    for (int l = 0; l < n; l++) {              // U^T (lower, U's diagonal)
      for (int c = tid; c < nrhs; c += nth) B[l + (size_t)ldb * c] /= LU[l + (size_t)lda * l];
      __syncthreads();
      cta_for_2d(n - 1 - l, nrhs, [&](int ii, int c) {
        const int i = l + 1 + ii;
        B[i + (size_t)ldb * c] -= LU[l + (size_t)lda * i] * B[l + (size_t)ldb * c];
      });
      __syncthreads();
    }
    for (int l = n - 1; l >= 1; l--) {         // L^T (unit upper)
      cta_for_2d(l, nrhs, [&](int i, int c) {
        B[i + (size_t)ldb * c] -= LU[l + (size_t)lda * i] * B[l + (size_t)ldb * c];
      });
      __syncthreads();
    }
    for (int c = tid; c < nrhs; c += nth) {
      T* b = B + (size_t)ldb * c;
      for (int i = n - 1; i >= 0; i--) {
        int p = piv[i];
        if (p != i) { T t = b[i]; b[i] = b[p]; b[p] = t; }
      }
    }
  }
  __syncthreads();
}

}  // namespace ki
