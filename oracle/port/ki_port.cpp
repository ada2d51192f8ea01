// CPU restatement of the reference's recursive-skeletonization factor and
// solve (kern_interp), used as the ORACLE: the checker in tests and the
// timed CPU baseline in bench.py.  TEST INFRASTRUCTURE ONLY -- the product
// path never links, loads or calls it.
//
// Each function names the reference function it restates (paths relative to
// the reference project).  The dense linear algebra calls the same LAPACK
// routines as the reference (dgeqp3, dtrtrs, dgetrf, dgetrs, dgemm), resolved
// at run time from whichever OpenBLAS the caller has loaded into the process
// (scipy's bundled build, whose symbols may carry a "scipy_" prefix).
//
// Deliberate differences, none of which changes the arithmetic:
//  * Schur-update gathering (quadtree/quadtree.cpp:1545-1632) uses a hash map
//    from DOF to position instead of the reference's quadratic list scan.
//  * The ID matrix's update blocks for near rows (kernel/kernel.cpp:612-619)
//    are omitted: descendants' updates only touch DOFs inside the box, so
//    those blocks are identically zero.
//  * multiply_connected_solve handles every right-hand-side column at once
//    (the reference handles column 0 only, skel_factorization.cpp:915-916);
//    each column's arithmetic is the same.
#include <dlfcn.h>
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace {

// ---------------------------------------------------------------- LAPACK --
typedef void (*dgeqp3_t)(const int*, const int*, double*, const int*, int*, double*,
                         double*, const int*, int*);
typedef void (*dgetrf_t)(const int*, const int*, double*, const int*, int*, int*);
typedef void (*dgetrs_t)(const char*, const int*, const int*, const double*, const int*,
                         const int*, double*, const int*, int*, size_t);
typedef void (*dtrtrs_t)(const char*, const char*, const char*, const int*, const int*,
                         const double*, const int*, double*, const int*, int*, size_t,
                         size_t, size_t);
typedef void (*dgemm_t)(const char*, const char*, const int*, const int*, const int*,
                        const double*, const double*, const int*, const double*,
                        const int*, const double*, double*, const int*, size_t, size_t);
typedef void (*setthreads_t)(int);

struct Lapack {
  dgeqp3_t dgeqp3 = nullptr;
  dgetrf_t dgetrf = nullptr;
  dgetrs_t dgetrs = nullptr;
  dtrtrs_t dtrtrs = nullptr;
  dgemm_t dgemm = nullptr;
  setthreads_t set_threads = nullptr;
};

void* find_symbol(const char* name) {
  std::string pre = std::string("scipy_") + name;
  void* p = dlsym(RTLD_DEFAULT, pre.c_str());
  if (!p) p = dlsym(RTLD_DEFAULT, name);
  return p;
}

const Lapack& lapack() {
  static Lapack L = [] {
    Lapack l;
    l.dgeqp3 = (dgeqp3_t)find_symbol("dgeqp3_");
    l.dgetrf = (dgetrf_t)find_symbol("dgetrf_");
    l.dgetrs = (dgetrs_t)find_symbol("dgetrs_");
    l.dtrtrs = (dtrtrs_t)find_symbol("dtrtrs_");
    l.dgemm = (dgemm_t)find_symbol("dgemm_");
    l.set_threads = (setthreads_t)find_symbol("openblas_set_num_threads");
    return l;
  }();
  return L;
}

// ---------------------------------------------------------------- Matrix --
// Column-major owning matrix with the reference's ki_Mat semantics
// (ki_mat.h:19-104): lda == height.
struct Mat {
  int h = 0, w = 0;
  std::vector<double> a;
  Mat() {}
  Mat(int h_, int w_) : h(h_), w(w_), a((size_t)h_ * w_, 0.0) {}
  double& operator()(int i, int j) { return a[i + (size_t)h * j]; }
  double operator()(int i, int j) const { return a[i + (size_t)h * j]; }
  double* data() { return a.data(); }
  const double* data() const { return a.data(); }
};

// C = alpha * op(A) op(B) + beta * C  (ki_Mat::operator*, ki_mat.cpp:328-335)
void gemm(bool ta, bool tb, double alpha, const Mat& A, const Mat& B, double beta, Mat* C) {
  int m = ta ? A.w : A.h, k = ta ? A.h : A.w, n = tb ? B.h : B.w;
  if (C->h != m || C->w != n) *C = Mat(m, n);
  if (m == 0 || n == 0) return;
  if (k == 0) {
    for (auto& v : C->a) v *= beta;
    return;
  }
  char ca = ta ? 'T' : 'N', cb = tb ? 'T' : 'N';
  int lda = std::max(1, A.h), ldb = std::max(1, B.h), ldc = std::max(1, C->h);
  lapack().dgemm(&ca, &cb, &m, &n, &k, &alpha, A.data(), &lda, B.data(), &ldb, &beta,
                 C->data(), &ldc, 1, 1);
}

Mat mul(const Mat& A, const Mat& B, bool ta = false, bool tb = false) {
  Mat C;
  gemm(ta, tb, 1.0, A, B, 0.0, &C);
  return C;
}

Mat sub(const Mat& A, const std::vector<int>& I, const std::vector<int>& J) {
  Mat R((int)I.size(), (int)J.size());
  for (size_t j = 0; j < J.size(); j++)
    for (size_t i = 0; i < I.size(); i++) R((int)i, (int)j) = A(I[i], J[j]);
  return R;
}

// LU with partial pivoting (ki_Mat::LU_factorize, ki_mat.cpp:445-453).
void lu(Mat* A, std::vector<int>* piv) {
  int n = A->h, info = 0, lda = std::max(1, n);
  piv->assign(n, 0);
  if (n == 0) return;
  lapack().dgetrf(&n, &n, A->data(), &lda, piv->data(), &info);
  if (info < 0) throw std::runtime_error("dgetrf failed");
}

// B <- op(A)^-1 B using an LU factor (dgetrs; ki_mat.cpp:455-513).
void lu_solve(const Mat& LU, const std::vector<int>& piv, bool trans, Mat* B) {
  int n = LU.h, nrhs = B->w, info = 0, lda = std::max(1, n), ldb = std::max(1, B->h);
  if (n == 0 || nrhs == 0) return;
  char t = trans ? 'T' : 'N';
  lapack().dgetrs(&t, &n, &nrhs, LU.data(), &lda, piv.data(), B->data(), &ldb, &info, 1);
  if (info != 0) throw std::runtime_error("dgetrs failed");
}

Mat transpose(const Mat& A) {
  Mat T(A.w, A.h);
  for (int j = 0; j < A.w; j++)
    for (int i = 0; i < A.h; i++) T(j, i) = A(i, j);
  return T;
}

// Interpolative decomposition by column-pivoted QR (ki_Mat::id,
// ki_mat.cpp:525-568): k = first i >= 1 with |R_ii| < tol |R_00|, 0 when no
// such i exists; T = R11^-1 R12 (k x (n-k)); perm = 0-based pivots.
int interp_decomp(Mat M, double tol, std::vector<int>* perm, Mat* T) {
  int m = M.h, n = M.w, info = 0, lda = std::max(1, m);
  std::vector<int> jpvt(n, 0);
  std::vector<double> tau(std::min(m, n) + 1);
  int lwork = -1;
  double wq = 0;
  lapack().dgeqp3(&m, &n, M.data(), &lda, jpvt.data(), tau.data(), &wq, &lwork, &info);
  lwork = std::max(1, (int)wq);
  std::vector<double> work(lwork);
  lapack().dgeqp3(&m, &n, M.data(), &lda, jpvt.data(), tau.data(), work.data(), &lwork, &info);
  if (info != 0) throw std::runtime_error("dgeqp3 failed");
  int k = 0;
  double thresh = std::fabs(tol * M(0, 0));
  for (int i = 1; i < std::min(m, n); i++) {
    if (std::fabs(M(i, i)) < thresh) {
      k = i;
      break;
    }
  }
  if (k == 0) return 0;
  perm->resize(n);
  for (int i = 0; i < n; i++) (*perm)[i] = jpvt[i] - 1;
  int r = n - k;
  char U = 'U', N = 'N';
  dtrtrs_t trs = lapack().dtrtrs;
  trs(&U, &N, &N, &k, &r, M.data(), &lda, M.data() + (size_t)lda * k, &lda, &info, 1, 1, 1);
  if (info != 0) throw std::runtime_error("dtrtrs failed");
  *T = Mat(k, r);
  for (int j = 0; j < r; j++)
    for (int i = 0; i < k; i++) (*T)(i, j) = M(i, k + j);
  return k;
}

// ---------------------------------------------------------------- Kernel --
struct Geometry {
  int n_points = 0, dim = 2, sol_dim = 1, pde = 0;
  const double* pts = nullptr;   // interleaved (x, y[, z])
  const double* nrm = nullptr;   // interleaved
  const double* wts = nullptr;
  const double* curv = nullptr;
  std::vector<double> diag;      // 3D: 1 (Laplace) or 9 (Stokes) per point
  std::vector<double> pxy_thetas, pxy_theta_w, pxy_phis, pxy_phi_w;   // 3D proxy sphere
};

// Kernel::one_d_kern / two_d_kern (kernel/kernel.cpp:33-87) and
// three_d_laplace / three_d_stokes (:89-121).  diag: the source point's 3D
// diagonal data (nullptr: zeros, as the proxy rows pass).
inline double entry(const Geometry& g, int tgt_dof, int src_dof, const double* tp,
                    const double* tn, const double* sp, const double* sn, double sw,
                    double sc, const double* diag = nullptr) {
  if (g.dim == 3) {
    double r1 = tp[0] - sp[0], r2 = tp[1] - sp[1], r3 = tp[2] - sp[2];
    if (g.sol_dim == 1) {
      if (r1 == 0. && r2 == 0. && r3 == 0.) return diag ? diag[0] : 0.;
      return -sw * (1.0 / (4 * M_PI)) * (r1 * sn[0] + r2 * sn[1] + r3 * sn[2]) /
             std::pow(r1 * r1 + r2 * r2 + r3 * r3, 1.5);
    }
    int tpar = tgt_dof % 3, spar = src_dof % 3;
    if (r1 == 0. && r2 == 0. && r3 == 0.) return diag ? diag[3 * tpar + spar] : 0.;
    double r[3] = {r1, r2, r3};
    double scale = -3.0 / (4.0 * M_PI);
    return sw * scale * (r1 * sn[0] + r2 * sn[1] + r3 * sn[2]) /
               std::pow(r1 * r1 + r2 * r2 + r3 * r3, 2.5) * r[tpar] * r[spar] +
           sw * tn[tpar] * sn[spar];
  }
  double r1 = tp[0] - sp[0], r2 = tp[1] - sp[1];
  if (g.sol_dim == 1 && g.pde == 1) {   // LAPLACE_NEUMANN (kernel.cpp:44-54), not forward
    if (r1 == 0. && r2 == 0.) return sw - 0.5 + 0.5 * sc * sw * (1.0 / (2 * M_PI));
    return sw + sw * (1.0 / (2 * M_PI)) * (r1 * tn[0] + r2 * tn[1]) / (r1 * r1 + r2 * r2);
  }
  if (g.sol_dim == 1 && g.pde == 2) {   // GAUSS (kernel.cpp:55-60)
    if (r1 == 0. && r2 == 0.) return 5.;
    return std::exp(-(r1 * r1 + r2 * r2));
  }
  if (g.sol_dim == 1) {
    if (r1 == 0. && r2 == 0.) return 0.5 + 0.5 * sc * sw * (1.0 / (2 * M_PI));
    return -sw * (1.0 / (2 * M_PI)) * (r1 * sn[0] + r2 * sn[1]) / (r1 * r1 + r2 * r2);
  }
  int tpar = tgt_dof % 2, spar = src_dof % 2;
  double r[2] = {r1, r2};
  double scale = 1 / M_PI;
  int is_diag = (tpar + spar + 1) % 2;
  if (r1 == 0. && r2 == 0.) {
    return -0.5 * is_diag + (1 - 2 * is_diag) * 0.5 * sc * sw * scale * sn[(tpar + 1) % 2] *
               sn[(spar + 1) % 2] +
           sw * tn[tpar] * sn[spar];
  }
  double rr = r1 * r1 + r2 * r2;
  return sw * scale * (r1 * sn[0] + r2 * sn[1]) / (rr * rr) * r[tpar] * r[spar] +
         sw * tn[tpar] * sn[spar];
}

// Kernel::operator() / get_3d (kernel/kernel.cpp:304-429): dense block K(tgt, src).
Mat kernel_block(const Geometry& g, const std::vector<int>& tgt, const std::vector<int>& src) {
  const int d = g.dim;
  const int dpp = d == 3 ? (g.sol_dim == 1 ? 1 : 9) : 0;
  Mat R((int)tgt.size(), (int)src.size());
  for (size_t j = 0; j < src.size(); j++) {
    int sp = src[j] / g.sol_dim;
    const double* s = g.pts + d * sp;
    const double* sn = g.nrm + d * sp;
    double sw = g.wts[sp], sc = g.curv ? g.curv[sp] : 0.;
    const double* dg = dpp ? g.diag.data() + (size_t)dpp * sp : nullptr;
    for (size_t i = 0; i < tgt.size(); i++) {
      int tpi = tgt[i] / g.sol_dim;
      R((int)i, (int)j) = entry(g, tgt[i], src[j], g.pts + d * tpi, g.nrm + d * tpi, s, sn, sw, sc, dg);
    }
  }
  return R;
}

// Kernel::get_proxy_mat (kernel/kernel.cpp:646-717), 2D.  The Gaussian
// kernel takes three rings per angle, radii r - 1, r, r + 1 (ring-minor rows).
Mat proxy_block(const Geometry& g, const double* c, int P, double r, const std::vector<int>& box) {
  double pw = 2.0 * M_PI * r / P;
  int c_dim = g.sol_dim;
  if (c_dim == 1 && g.pde == 2) {
    Mat R(6 * P, (int)box.size());
    for (size_t j = 0; j < box.size(); j++) {
      const double* b = g.pts + 2 * box[j];
      for (int i = 0; i < P; i++) {
        double ang = 2 * M_PI * i * (1.0 / P);
        for (int k = 0; k < 3; k++) {
          double rr = r + (k - 1);
          double pp[2] = {c[0] + rr * std::cos(ang), c[1] + rr * std::sin(ang)};
          double pn[2] = {std::cos(ang), std::sin(ang)};
          R(3 * i + k, (int)j) = entry(g, 0, 0, pp, pn, b, b, 0., 0);
          R(3 * P + 3 * i + k, (int)j) = entry(g, 0, 0, b, b, pp, pn, pw, 0);
        }
      }
    }
    return R;
  }
  int lda = c_dim * 2 * P;
  Mat R(lda, (int)box.size());
  for (size_t j = 0; j < box.size(); j++) {
    int bp = box[j] / g.sol_dim;
    const double* b = g.pts + 2 * bp;
    const double* bn = g.nrm + 2 * bp;
    double bw = g.wts[bp];
    for (int i = 0; i < P; i++) {
      double ang = 2 * M_PI * i * (1.0 / P);
      double pp[2] = {c[0] + r * std::cos(ang), c[1] + r * std::sin(ang)};
      double pn[2] = {std::cos(ang), std::sin(ang)};
      if (c_dim == 1) {
        R(i, (int)j) = entry(g, 0, 0, pp, pn, b, bn, bw, 0);
        R(P + i, (int)j) = entry(g, 0, 0, b, bn, pp, pn, pw, 0);
      } else {
        for (int par = 0; par < 2; par++) {
          R(2 * i + par, (int)j) = entry(g, par, box[j], pp, pn, b, bn, bw, 0);
          R(2 * P + 2 * i + par, (int)j) = entry(g, box[j], par, b, bn, pp, pn, pw, 0);
        }
      }
    }
  }
  return R;
}

// Kernel::get_proxy_mat3d (kernel/kernel.cpp:720-790): theta x phi grid,
// theta outer; rows [0, c P) box -> proxy, [c P, 2 c P) proxy -> box.
Mat proxy_block3(const Geometry& g, const double* c, double r, const std::vector<int>& box) {
  std::vector<double> pp, pn, pw;
  for (size_t i = 0; i < g.pxy_thetas.size(); i++) {
    double theta = g.pxy_thetas[i];
    for (size_t j = 0; j < g.pxy_phis.size(); j++) {
      double phi = g.pxy_phis[j];
      pp.push_back(c[0] + r * std::sin(phi) * std::cos(theta));
      pp.push_back(c[1] + r * std::sin(phi) * std::sin(theta));
      pp.push_back(c[2] + r * std::cos(phi));
      pn.push_back(std::sin(phi) * std::cos(theta));
      pn.push_back(std::sin(phi) * std::sin(theta));
      pn.push_back(std::cos(phi));
      pw.push_back(std::pow(r, 2) * g.pxy_phi_w[j] * g.pxy_theta_w[i]);
    }
  }
  const int P = (int)pw.size(), cd = g.sol_dim;
  const int lda = 2 * cd * P;
  Mat R(lda, (int)box.size());
  for (size_t j = 0; j < box.size(); j++) {
    int bp = box[j] / cd;
    const double* b = g.pts + 3 * bp;
    const double* bn = g.nrm + 3 * bp;
    double bw = g.wts[bp];
    for (int i = 0; i < P; i++) {
      const double* q = pp.data() + 3 * i;
      const double* qn = pn.data() + 3 * i;
      if (cd == 1) {
        R(i, (int)j) = entry(g, 0, 0, q, qn, b, bn, bw, 0);
        R(P + i, (int)j) = entry(g, 0, 0, b, bn, q, qn, pw[i], 0);
      } else {
        for (int par = 0; par < 3; par++) {
          R(3 * i + par, (int)j) = entry(g, par, box[j], q, qn, b, bn, bw, 0);
          R(3 * P + 3 * i + par, (int)j) = entry(g, box[j], par, b, bn, q, qn, pw[i], 0);
        }
      }
    }
  }
  return R;
}

// Gauss-Legendre nodes/weights on [a, b], ascending, by Newton's method on
// the Legendre recurrence (the reference calls cgqf for the proxy
// latitudes, kernel/kernel.h:44-62).
void gauss_legendre(int n, double a, double b, std::vector<double>* x, std::vector<double>* w) {
  x->assign(n, 0.);
  w->assign(n, 0.);
  for (int i = 0; i < n; i++) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), pd = 1.;
    for (int it = 0; it < 100; it++) {
      double p0 = 1., p1 = z;
      for (int k = 2; k <= n; k++) {
        double p2 = ((2. * k - 1.) * z * p1 - (k - 1.) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      pd = n == 1 ? 1. : n * (z * p1 - p0) / (z * z - 1.);
      double dz = p1 / pd;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    double p0 = 1., p1 = z;
    for (int k = 2; k <= n; k++) {
      double p2 = ((2. * k - 1.) * z * p1 - (k - 1.) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    pd = n == 1 ? 1. : n * (z * p1 - p0) / (z * z - 1.);
    (*x)[n - 1 - i] = 0.5 * (b - a) * z + 0.5 * (b + a);
    (*w)[n - 1 - i] = (b - a) / ((1. - z * z) * pd * pd);
  }
}

// The Kernel constructor's proxy sphere (kernel/kernel.h:44-62): n_theta
// equispaced longitudes, n_theta/2 Gauss-Legendre latitudes on [0, pi],
// latitude weight w_j sin(phi_j), longitude weight 2 pi / n_theta.
void proxy_sphere(Geometry* g, int n_theta) {
  int n_phi = n_theta / 2;
  std::vector<double> ph, pw;
  gauss_legendre(n_phi, 0., M_PI, &ph, &pw);
  g->pxy_thetas.clear(); g->pxy_theta_w.clear(); g->pxy_phis.clear(); g->pxy_phi_w.clear();
  for (int i = 0; i < n_theta; i++) {
    g->pxy_thetas.push_back(2 * M_PI * i * (1.0 / n_theta));
    g->pxy_theta_w.push_back(2 * M_PI / n_theta);
  }
  for (int j = 0; j < n_phi; j++) {
    g->pxy_phis.push_back(ph[j]);
    g->pxy_phi_w.push_back(pw[j] * std::sin(ph[j]));
  }
}

// Kernel::compute_diag_entries_3dlaplace / _3dstokes (kernel/kernel.cpp:124-301):
// row sums over the point's own surface (outer nodes [0, n_outer), or its
// hole's range), then 1 - sum / I - sum on the outer surface, -sum on holes.
void compute_diag3(Geometry* g, int n_outer, const std::vector<int>& hs, const std::vector<int>& hn,
                   int threads) {
  const int n = g->n_points;
  const bool lap = g->sol_dim == 1;
  g->diag.assign((size_t)n * (lap ? 1 : 9), 0.);
  std::vector<int> lo(n), hi(n);
  for (int p = 0; p < n_outer; p++) { lo[p] = 0; hi[p] = n_outer; }
  for (size_t h = 0; h < hs.size(); h++)
    for (int p = hs[h]; p < hs[h] + hn[h]; p++) { lo[p] = hs[h]; hi[p] = hs[h] + hn[h]; }
  const double* P = g->pts;
  const double* Nn = g->nrm;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 16)
  for (int t = 0; t < n; t++) {
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int s = lo[t]; s < hi[t]; s++) {
      if (s == t) continue;
      double r1 = P[3 * t] - P[3 * s], r2 = P[3 * t + 1] - P[3 * s + 1], r3 = P[3 * t + 2] - P[3 * s + 2];
      double sn[3] = {Nn[3 * s], Nn[3 * s + 1], Nn[3 * s + 2]};
      double sw = g->wts[s];
      if (lap) {
        acc[0] += (-sw * (1.0 / (4 * M_PI)) * (r1 * sn[0] + r2 * sn[1] + r3 * sn[2]) /
                   std::pow(r1 * r1 + r2 * r2 + r3 * r3, 1.5));
      } else {
        double r[3] = {r1, r2, r3};
        double tn[3] = {Nn[3 * t], Nn[3 * t + 1], Nn[3 * t + 2]};
        double scale = -3.0 / (4.0 * M_PI);
        for (int a = 0; a < 3; a++)
          for (int b = 0; b < 3; b++)
            acc[3 * a + b] += sw * scale * (r1 * sn[0] + r2 * sn[1] + r3 * sn[2]) /
                                  std::pow(r1 * r1 + r2 * r2 + r3 * r3, 2.5) * r[a] * r[b] +
                              sw * tn[a] * sn[b];
      }
    }
    double one = t < n_outer ? 1. : 0.;
    if (lap) {
      g->diag[t] = one - acc[0];
    } else {
      for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) g->diag[9 * (size_t)t + 3 * a + b] = (a == b ? one : 0.) - acc[3 * a + b];
    }
  }
}

// Border matrices of a multiply connected boundary (initialize_U_mat /
// initialize_Psi_mat, kern_interp/linear_solve.cpp:19-199), hole membership
// from node ranges: U restricted to the DOF rows `rows` (|rows| x n_border)
// and the whole Psi (n_border x N).  Columns per hole: 1 (Laplace), 3 (2D
// Stokes: Stokeslets in x and y, rotlet), 6 (3D Stokes: 3 Stokeslets, 3
// rotlets).
void border_matrices(const Geometry& g, int n_holes, const double* hole_centers,
                     const int* hole_start, const int* hole_count, const std::vector<int>& rows,
                     Mat* Um, Mat* Psi) {
  const int d = g.dim, sd = g.sol_dim;
  const int c = sd == 1 ? 1 : (d == 2 ? 3 : 6);
  const int N = g.n_points * sd;
  const double* points = g.pts;
  const double* weights = g.wts;
  *Um = Mat((int)rows.size(), c * n_holes);
  *Psi = Mat(c * n_holes, N);
  for (int h = 0; h < n_holes; h++) {
    const double* hc = hole_centers + d * h;
    for (size_t i = 0; i < rows.size(); i++) {
      const int p = rows[i] / sd, a = rows[i] % sd;
      Mat& U = *Um;
      if (d == 3) {
        // linear_solve.cpp:26-36 (Laplace), :49-76 (Stokes)
        double r[3] = {points[3 * p] - hc[0], points[3 * p + 1] - hc[1], points[3 * p + 2] - hc[2]};
        double rn = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        if (sd == 1) {
          U((int)i, h) = 1.0 / rn;
          continue;
        }
        for (int b = 0; b < 3; b++)
          U((int)i, 6 * h + b) =
              (1.0 / (8.0 * M_PI)) * ((a == b ? 1 : 0) / rn + r[a] * r[b] / std::pow(rn, 3));
        double rot = -1.0 / (8.0 * M_PI * std::pow(rn, 3));
        if (a == 0) {
          U((int)i, 6 * h + 4) = rot * (-r[2]);
          U((int)i, 6 * h + 5) = rot * (r[1]);
        } else if (a == 1) {
          U((int)i, 6 * h + 3) = rot * (r[2]);
          U((int)i, 6 * h + 5) = rot * (-r[0]);
        } else {
          U((int)i, 6 * h + 3) = rot * (-r[1]);
          U((int)i, 6 * h + 4) = rot * (r[0]);
        }
        continue;
      }
      double rx = points[2 * p] - hc[0], ry = points[2 * p + 1] - hc[1];
      double rn = std::sqrt(rx * rx + ry * ry);
      if (sd == 1) {
        U((int)i, h) = std::log(rn);          // linear_solve.cpp:37-45
      } else {                                 // linear_solve.cpp:77-97
        double sc = 1.0 / (4 * M_PI), r2 = rn * rn;
        if (a == 0) {
          U((int)i, 3 * h) = sc * (std::log(1 / rn) + rx * rx / r2);
          U((int)i, 3 * h + 1) = sc * (rx * ry / r2);
          U((int)i, 3 * h + 2) = ry * (sc / r2);
        } else {
          U((int)i, 3 * h) = sc * (ry * rx / r2);
          U((int)i, 3 * h + 1) = sc * (std::log(1 / rn) + ry * ry / r2);
          U((int)i, 3 * h + 2) = -rx * (sc / r2);
        }
      }
    }
    // linear_solve.cpp:114-129, 131-143 (Laplace); :146-163 (3D Stokes),
    // :164-177 (2D Stokes, absolute-coordinate rotation row)
    for (int p = hole_start[h]; p < hole_start[h] + hole_count[h]; p++) {
      double w = weights[p];
      if (sd == 1) {
        (*Psi)(h, p) = w;
      } else if (d == 2) {
        (*Psi)(3 * h, 2 * p) = w;
        (*Psi)(3 * h + 1, 2 * p + 1) = w;
        (*Psi)(3 * h + 2, 2 * p) = w * points[2 * p + 1];
        (*Psi)(3 * h + 2, 2 * p + 1) = -w * points[2 * p];
      } else {
        double r[3] = {points[3 * p] - hc[0], points[3 * p + 1] - hc[1], points[3 * p + 2] - hc[2]};
        (*Psi)(6 * h, 3 * p) = w;
        (*Psi)(6 * h + 1, 3 * p + 1) = w;
        (*Psi)(6 * h + 2, 3 * p + 2) = w;
        (*Psi)(6 * h + 4, 3 * p) = -w * (-r[2]);
        (*Psi)(6 * h + 5, 3 * p) = -w * (r[1]);
        (*Psi)(6 * h + 3, 3 * p + 1) = -w * (r[2]);
        (*Psi)(6 * h + 5, 3 * p + 1) = -w * (-r[0]);
        (*Psi)(6 * h + 3, 3 * p + 2) = -w * (-r[1]);
        (*Psi)(6 * h + 4, 3 * p + 2) = -w * (r[0]);
      }
    }
  }
}

// ------------------------------------------------------------------ Tree --
struct Node {
  int level = 0;
  bool leaf = true, compressed = false;
  double c[3] = {0, 0, 0}, side = 0;
  int parent = -1;
  std::vector<int> children, neighbors;
  std::vector<int> orig, act, skel, red, near, perm;
  Mat T, L, U, Xlu, S;
  std::vector<int> piv;
};

struct Params {
  int leaf = 64, proxy = 128, min_compress = 64;
  double ratio = 2.0, tol = 1e-10;
  int threads = 1;
};

struct Tree {
  Geometry g;
  Params p;
  std::vector<Node> nodes;
  std::vector<std::vector<int>> levels;
  Mat allskel_lu, U, Psi, S_lu;
  std::vector<int> allskel_piv, S_piv;

  int new_node() {
    nodes.emplace_back();
    return (int)nodes.size() - 1;
  }

  // Child index (quadtree/quadtree.cpp:324-330, 398-405): coordinate d at or
  // above the centre adds 2^(dim-1-d).
  int child_index(int pt, const double* c) const {
    int ci = 0;
    for (int d = 0; d < g.dim; d++)
      if (g.pts[g.dim * pt + d] >= c[d]) ci += 1 << (g.dim - 1 - d);
    return ci;
  }

  // QuadTree::node_subdivide (quadtree/quadtree.cpp:372-413).
  void subdivide(int ni) {
    nodes[ni].leaf = false;
    const int nch = 1 << g.dim;
    int kids[8];
    for (int ci = 0; ci < nch; ci++) {
      int k = new_node();
      kids[ci] = k;
      Node& n = nodes[ni];
      Node& ch = nodes[k];
      for (int d = 0; d < g.dim; d++)
        ch.c[d] = n.c[d] + (((ci >> (g.dim - 1 - d)) & 1) ? n.side / 4. : -n.side / 4.);
      ch.level = n.level + 1;
      ch.side = n.side / 2.0;
      ch.parent = ni;
    }
    Node& n = nodes[ni];
    for (int ci = 0; ci < nch; ci++) n.children.push_back(kids[ci]);
    if ((int)levels.size() < n.level + 2) levels.emplace_back();
    for (int ci = 0; ci < nch; ci++) levels[n.level + 1].push_back(kids[ci]);
    std::vector<int> orig = n.orig;
    double c[3] = {n.c[0], n.c[1], n.c[2]};
    for (size_t idx = 0; idx < orig.size(); idx += g.sol_dim) {
      int dof = orig[idx];
      int pt = dof / g.sol_dim;
      int ci = child_index(pt, c);
      for (int s = 0; s < g.sol_dim; s++) nodes[kids[ci]].orig.push_back(dof + s);
    }
    for (int ci = 0; ci < nch; ci++)
      if ((int)nodes[kids[ci]].orig.size() > p.leaf) subdivide(kids[ci]);
  }

  // QuadTree::recursive_add (quadtree/quadtree.cpp:317-344).
  void add(int ni, int pt) {
    for (int s = 0; s < g.sol_dim; s++) nodes[ni].orig.push_back(g.sol_dim * pt + s);
    if (!nodes[ni].leaf) {
      add(nodes[ni].children[child_index(pt, nodes[ni].c)], pt);
    } else if ((int)nodes[ni].orig.size() > p.leaf) {
      subdivide(ni);
    }
  }

  // QuadTree::get_descendent_neighbors (quadtree/quadtree.cpp:292-314).
  void descendent_neighbors(int big, int small) {
    bool nb = true;
    for (int d = 0; d < g.dim; d++) {
      double dist = std::fabs(nodes[big].c[d] - nodes[small].c[d]);
      double pred = (nodes[big].side + nodes[small].side) / 2.;
      if (dist - pred > 1e-9) {
        nb = false;
        break;
      }
    }
    if (nb) {
      nodes[big].neighbors.push_back(small);
      nodes[small].neighbors.push_back(big);
    }
    for (int ch : std::vector<int>(nodes[small].children)) descendent_neighbors(big, ch);
  }

  // QuadTree::compute_neighbor_lists (quadtree/quadtree.cpp:192-237).
  void neighbor_lists() {
    for (size_t l = 0; l < levels.size(); l++) {
      for (int a : levels[l]) {
        int par = nodes[a].parent;
        if (par >= 0) {
          for (int sib : nodes[par].children)
            if (sib != a) nodes[a].neighbors.push_back(sib);
          for (int pn : std::vector<int>(nodes[par].neighbors)) {
            for (int cousin : nodes[pn].children) {
              if (nodes[cousin].level != nodes[a].level) continue;
              double dist = 0.;
              for (int d = 0; d < g.dim; d++)
                dist += std::pow(nodes[a].c[d] - nodes[cousin].c[d], 2);
              dist = std::sqrt(dist);
              if (dist < nodes[a].side * std::sqrt((double)g.dim) + 1e-9)
                nodes[a].neighbors.push_back(cousin);
            }
          }
        }
        if (nodes[a].leaf) {
          for (size_t k = 0; k < nodes[a].neighbors.size(); k++) {
            int nb = nodes[a].neighbors[k];
            if (nodes[nb].level != nodes[a].level) continue;
            for (int ch : std::vector<int>(nodes[nb].children)) descendent_neighbors(a, ch);
          }
        }
      }
    }
  }

  // QuadTree::initialize_tree (quadtree/quadtree.cpp:240-287).
  void build() {
    double mn = g.pts[0], mx = g.pts[0];
    for (int i = 0; i < g.dim * g.n_points; i++) {
      mn = std::min(mn, g.pts[i]);
      mx = std::max(mx, g.pts[i]);
    }
    double tmin = mn - 0.01, tmax = mx + 0.01;
    int root = new_node();
    for (int d = 0; d < g.dim; d++) nodes[root].c[d] = (tmin + tmax) / 2.0;
    nodes[root].side = tmax - tmin;
    levels.push_back({root});
    nodes.reserve(8 * (g.n_points * g.sol_dim / std::max(1, p.leaf) + 4));
    for (int i = 0; i < g.n_points; i++) add(root, i);
    neighbor_lists();
  }

  // QuadTree::remove_inactive_dofs_at_box (quadtree/quadtree.cpp:1172-1204).
  void refresh_box(int ni) {
    Node& n = nodes[ni];
    n.skel.clear();
    n.red.clear();
    n.act.clear();
    if (!n.leaf) {
      for (int ch : n.children) {
        const Node& c = nodes[ch];
        const std::vector<int>& src = c.compressed ? c.skel : c.act;
        n.act.insert(n.act.end(), src.begin(), src.end());
      }
    } else {
      n.act = n.orig;
    }
  }

  // QuadTree::remove_inactive_dofs_at_level (quadtree/quadtree.cpp:1142-1169).
  void refresh_level(int l) {
    for (int ni : levels[l])
      if (!nodes[ni].compressed) refresh_box(ni);
    for (int ni : levels[l]) {
      Node& a = nodes[ni];
      a.near.clear();
      for (int nb : a.neighbors) {
        const Node& b = nodes[nb];
        if (b.level > a.level) continue;
        const std::vector<int>& src = b.leaf ? b.orig : b.act;
        a.near.insert(a.near.end(), src.begin(), src.end());
      }
    }
  }

  // Kernel::get_id_mat (kernel/kernel.cpp:432-641).
  Mat id_matrix(int ni) {
    const Node& n = nodes[ni];
    const std::vector<int>& A = n.act;
    std::vector<int> outside;
    bool proxy = true;
    if (n.level == 1 || (n.level == 2 && g.dim < 3)) {
      proxy = false;
      for (int o : levels[n.level])
        if (o != ni) outside.insert(outside.end(), nodes[o].act.begin(), nodes[o].act.end());
      if (n.level == 2) {
        for (int l = n.level - 1; l >= 0; l--)
          for (int o : levels[l])
            if (nodes[o].leaf) outside.insert(outside.end(), nodes[o].orig.begin(), nodes[o].orig.end());
      }
    } else {
      double rad = std::sqrt((double)g.dim) * p.ratio * (n.side / 2);
      for (int dof : n.near) {
        int pt = dof / g.sol_dim;
        double dist = 0.;
        for (int d = 0; d < g.dim; d++) dist += std::pow(n.c[d] - g.pts[g.dim * pt + d], 2);
        dist = std::sqrt(dist);
        if (dist < rad) outside.push_back(dof);
      }
    }
    Mat Kia = kernel_block(g, outside, A);
    Mat Kai = kernel_block(g, A, outside);
    Mat pxy;
    if (proxy) {
      double rad = (n.side / 2) * std::sqrt((double)g.dim) * p.ratio;
      pxy = g.dim == 3 ? proxy_block3(g, n.c, rad, A) : proxy_block(g, n.c, p.proxy, rad, A);
    }
    int o = (int)outside.size();
    Mat M(2 * o + pxy.h, (int)A.size());
    for (int j = 0; j < (int)A.size(); j++) {
      for (int i = 0; i < o; i++) M(i, j) = Kia(i, j);
      for (int i = 0; i < o; i++) M(o + i, j) = Kai(j, i);
      for (int i = 0; i < pxy.h; i++) M(2 * o + i, j) = pxy(i, j);
    }
    return M;
  }

  // get_descendents_updates / get_update (quadtree/quadtree.cpp:1545-1632):
  // sum of the Schur updates of every compressed strict descendant,
  // restricted to rows x cols.
  void add_descendant_updates(int ni, const std::vector<int>& rows, const std::vector<int>& cols,
                              Mat* upd) {
    std::unordered_map<int, int> rpos, cpos;
    for (size_t i = 0; i < rows.size(); i++) rpos[rows[i]] = (int)i;
    for (size_t j = 0; j < cols.size(); j++) cpos[cols[j]] = (int)j;
    std::vector<int> stack(nodes[ni].children.begin(), nodes[ni].children.end());
    while (!stack.empty()) {
      int d = stack.back();
      stack.pop_back();
      const Node& nd = nodes[d];
      for (int ch : nd.children) stack.push_back(ch);
      if (!nd.compressed) continue;
      std::vector<std::pair<int, int>> sr, sc;
      for (size_t s = 0; s < nd.skel.size(); s++) {
        auto it = rpos.find(nd.skel[s]);
        if (it != rpos.end()) sr.push_back({(int)s, it->second});
        auto jt = cpos.find(nd.skel[s]);
        if (jt != cpos.end()) sc.push_back({(int)s, jt->second});
      }
      for (auto& b : sc)
        for (auto& a : sr) (*upd)(a.second, b.second) += nd.S(a.first, b.first);
    }
  }

  // SkelFactorization::decouple (skel_factorization.cpp:91-127).
  void decouple(int ni) {
    Node& n = nodes[ni];
    int k = n.T.h, r = n.T.w;
    Mat upd((int)n.act.size(), (int)n.act.size());
    add_descendant_updates(ni, n.act, n.act, &upd);
    Mat K = kernel_block(g, n.act, n.act);
    for (size_t i = 0; i < K.a.size(); i++) K.a[i] -= upd.a[i];
    std::vector<int> s(n.perm.begin(), n.perm.begin() + k), rr(n.perm.begin() + k, n.perm.end());
    Mat Kss = sub(K, s, s), Ksr = sub(K, s, rr), Krs = sub(K, rr, s), Krr = sub(K, rr, rr);
    Mat Krs_t = Krs;
    gemm(true, false, -1.0, n.T, Kss, 1.0, &Krs_t);           // K_rs - T^T K_ss
    Mat X = Krr;
    gemm(true, false, -1.0, n.T, Ksr, 1.0, &X);                // - T^T K_sr
    gemm(false, false, -1.0, Krs_t, n.T, 1.0, &X);             // - K~_rs T
    Mat Ksr_t = Ksr;
    gemm(false, false, -1.0, Kss, n.T, 1.0, &Ksr_t);           // K_sr - K_ss T
    n.Xlu = X;
    lu(&n.Xlu, &n.piv);
    // L = K~_sr X^-1  via  X^T L^T = K~_sr^T
    Mat Lt = transpose(Ksr_t);
    lu_solve(n.Xlu, n.piv, true, &Lt);
    n.L = transpose(Lt);
    n.U = Krs_t;
    lu_solve(n.Xlu, n.piv, false, &n.U);
    n.S = mul(n.L, Krs_t);
    (void)r;
    n.compressed = true;
  }

  // SkelFactorization::id_compress (skel_factorization.cpp:36-58).
  int id_compress(int ni) {
    Node& n = nodes[ni];
    Mat M = id_matrix(ni);
    if (M.h == 0) return 0;
    std::vector<int> perm;
    Mat T;
    int k = interp_decomp(std::move(M), p.tol, &perm, &T);
    if (k == 0) return 0;
    n.T = T;
    n.perm = perm;
    n.skel.clear();
    n.red.clear();
    for (int i = 0; i < k; i++) n.skel.push_back(n.act[perm[i]]);
    for (size_t i = k; i < perm.size(); i++) n.red.push_back(n.act[perm[i]]);
    return T.w;
  }

  std::vector<int> allskel, allred;

  // SkelFactorization::skeletonize (skel_factorization.cpp:173-551).
  void skeletonize() {
    if (lapack().set_threads) lapack().set_threads(1);
    int L = (int)levels.size();
    for (int l = L - 1; l >= 1; l--) {
      refresh_level(l);
      const std::vector<int>& lv = levels[l];
      std::vector<char> err(lv.size(), 0);
#pragma omp parallel for num_threads(p.threads) schedule(dynamic, 1)
      for (int i = 0; i < (int)lv.size(); i++) {
        int ni = lv[i];
        if (nodes[ni].compressed || (int)nodes[ni].act.size() < p.min_compress) continue;
        try {
          if (id_compress(ni) == 0) continue;
          decouple(ni);
        } catch (...) {
          err[i] = 1;
        }
      }
      for (char e : err)
        if (e) throw std::runtime_error("LAPACK failure during skeletonization");
    }
    for (int l = L - 1; l >= 0; l--) refresh_level(l);
    allskel = nodes[levels[0][0]].act;
    Mat A;
    if (!allskel.empty()) {
      Mat upd((int)allskel.size(), (int)allskel.size());
      add_descendant_updates(levels[0][0], allskel, allskel, &upd);
      A = kernel_block(g, allskel, allskel);
      for (size_t i = 0; i < A.a.size(); i++) A.a[i] -= upd.a[i];
    }
    int N = g.n_points * g.sol_dim;
    std::vector<char> is_skel(N, 0);
    for (int s : allskel) is_skel[s] = 1;
    allred.clear();
    for (int i = 0; i < N; i++)
      if (!is_skel[i]) allred.push_back(i);
    if (U.w == 0) {
      allskel_lu = A;
      lu(&allskel_lu, &allskel_piv);
      return;
    }
    // Bordered system (skel_factorization.cpp:311-547).
    std::unordered_map<int, int> red_pos;
    for (size_t i = 0; i < allred.size(); i++) red_pos[allred[i]] = (int)i;
    Mat mU = U, mPsiT = transpose(Psi);
    up_sweep(&mU, false);
    psi_sweep(&mPsiT);
    Mat Psi_m = transpose(mPsiT);
    Mat DinvC = sub(mU, allred, range(mU.w));
    diag_solve_small(&DinvC, red_pos);
    int ns = (int)allskel.size(), nh = Psi.h;
    Mat S(ns + nh, ns + nh);
    Mat PsiR = sub(Psi_m, range(nh), allred), PsiS = sub(Psi_m, range(nh), allskel);
    Mat Us = sub(mU, allskel, range(U.w));
    Mat corr = mul(PsiR, DinvC);
    for (int j = 0; j < ns; j++)
      for (int i = 0; i < ns; i++) S(i, j) = A(i, j);
    for (int j = 0; j < ns; j++)
      for (int i = 0; i < nh; i++) S(ns + i, j) = PsiS(i, j);
    for (int j = 0; j < nh; j++)
      for (int i = 0; i < ns; i++) S(i, ns + j) = Us(i, j);
    for (int j = 0; j < nh; j++)
      for (int i = 0; i < nh; i++) S(ns + i, ns + j) = -(i == j ? 1.0 : 0.0) - corr(i, j);
    S_lu = S;
    lu(&S_lu, &S_piv);
  }

  static std::vector<int> range(int n) {
    std::vector<int> r(n);
    for (int i = 0; i < n; i++) r[i] = i;
    return r;
  }

  // apply_sweep_matrix (skel_factorization.cpp:555-572): x(b) += op(M) x(a).
  static void sweep(const Mat& M, bool trans, double sign, Mat* x, const std::vector<int>& a,
                    const std::vector<int>& b) {
    if (a.empty() || b.empty()) return;
    Mat xa = sub(*x, a, range(x->w));
    Mat prod;
    gemm(trans, false, sign, M, xa, 0.0, &prod);
    for (int j = 0; j < x->w; j++)
      for (size_t i = 0; i < b.size(); i++) (*x)(b[i], j) += prod((int)i, j);
  }

  // Upward pass of SkelFactorization::solve (skel_factorization.cpp:626-673).
  void up_sweep(Mat* x, bool with_diag) {
    int L = (int)levels.size();
    for (int l = L - 1; l >= 0; l--) {
      const std::vector<int>& lv = levels[l];
#pragma omp parallel for num_threads(p.threads) schedule(dynamic, 4)
      for (int i = 0; i < (int)lv.size(); i++) {
        const Node& n = nodes[lv[i]];
        if (!n.compressed) continue;
        sweep(n.T, true, -1.0, x, n.skel, n.red);
        sweep(n.L, false, -1.0, x, n.red, n.skel);
      }
    }
    if (with_diag) diag_solve(x);
  }

  // Transposed down-sweep applied to Psi^T (skel_factorization.cpp:416-465).
  void psi_sweep(Mat* x) {
    int L = (int)levels.size();
    for (int l = L - 1; l >= 0; l--) {
      const std::vector<int>& lv = levels[l];
#pragma omp parallel for num_threads(p.threads) schedule(dynamic, 4)
      for (int i = 0; i < (int)lv.size(); i++) {
        const Node& n = nodes[lv[i]];
        if (!n.compressed) continue;
        sweep(n.T, true, -1.0, x, n.skel, n.red);
        sweep(n.U, true, -1.0, x, n.red, n.skel);
      }
    }
  }

  // apply_diag_inv_matrix over all boxes (skel_factorization.cpp:676-687).
  void diag_solve(Mat* x) {
    std::vector<int> all;
    for (int l = (int)levels.size() - 1; l >= 0; l--)
      for (int ni : levels[l]) all.push_back(ni);
#pragma omp parallel for num_threads(p.threads) schedule(dynamic, 4)
    for (int i = 0; i < (int)all.size(); i++) {
      const Node& n = nodes[all[i]];
      if (!n.compressed || n.red.empty()) continue;
      Mat xr = sub(*x, n.red, range(x->w));
      lu_solve(n.Xlu, n.piv, false, &xr);
      for (int j = 0; j < x->w; j++)
        for (size_t q = 0; q < n.red.size(); q++) (*x)(n.red[q], j) = xr((int)q, j);
    }
  }

  // The same on a matrix indexed by position within allred.
  void diag_solve_small(Mat* x, const std::unordered_map<int, int>& red_pos) {
    std::vector<int> all;
    for (int l = (int)levels.size() - 1; l >= 0; l--)
      for (int ni : levels[l]) all.push_back(ni);
#pragma omp parallel for num_threads(p.threads) schedule(dynamic, 4)
    for (int i = 0; i < (int)all.size(); i++) {
      const Node& n = nodes[all[i]];
      if (!n.compressed || n.red.empty()) continue;
      std::vector<int> sm;
      for (int d : n.red) sm.push_back(red_pos.at(d));
      Mat xr = sub(*x, sm, range(x->w));
      lu_solve(n.Xlu, n.piv, false, &xr);
      for (int j = 0; j < x->w; j++)
        for (size_t q = 0; q < sm.size(); q++) (*x)(sm[q], j) = xr((int)q, j);
    }
  }

  // Downward pass (skel_factorization.cpp:725-777).
  void down_sweep(Mat* x) {
    int L = (int)levels.size();
    for (int l = 0; l < L; l++) {
      const std::vector<int>& lv = levels[l];
#pragma omp parallel for num_threads(p.threads) schedule(dynamic, 4)
      for (int i = (int)lv.size() - 1; i >= 0; i--) {
        const Node& n = nodes[lv[i]];
        if (!n.compressed) continue;
        sweep(n.U, false, -1.0, x, n.skel, n.red);
        sweep(n.T, false, -1.0, x, n.red, n.skel);
      }
    }
  }

  // SkelFactorization::solve (skel_factorization.cpp:595-778).
  void solve(Mat* x) {
    up_sweep(x, true);
    if (!allskel.empty()) {
      Mat xs = sub(*x, allskel, range(x->w));
      lu_solve(allskel_lu, allskel_piv, false, &xs);
      for (int j = 0; j < x->w; j++)
        for (size_t q = 0; q < allskel.size(); q++) (*x)(allskel[q], j) = xs((int)q, j);
    }
    down_sweep(x);
  }

  // SkelFactorization::multiply_connected_solve (skel_factorization.cpp:781-1141).
  void mc_solve(Mat* mu, Mat* alpha) {
    std::unordered_map<int, int> red_pos;
    for (size_t i = 0; i < allred.size(); i++) red_pos[allred[i]] = (int)i;
    Mat mU = U, mPsiT = transpose(Psi);
    up_sweep(mu, false);
    up_sweep(&mU, false);
    Mat w = sub(*mu, allred, range(mu->w));
    Mat z = sub(*mu, allskel, range(mu->w));
    psi_sweep(&mPsiT);
    Mat Psi_m = transpose(mPsiT);
    Mat Dw = w;
    diag_solve_small(&Dw, red_pos);
    int ns = (int)allskel.size(), nh = Psi.h, nc = mu->w;
    Mat PsiR = sub(Psi_m, range(nh), allred);
    Mat t = mul(PsiR, Dw);
    Mat M(ns + nh, nc);
    for (int j = 0; j < nc; j++) {
      for (int i = 0; i < ns; i++) M(i, j) = z(i, j);
      for (int i = 0; i < nh; i++) M(ns + i, j) = -t(i, j);
    }
    lu_solve(S_lu, S_piv, false, &M);
    *alpha = Mat(nh, nc);
    for (int j = 0; j < nc; j++)
      for (int i = 0; i < nh; i++) (*alpha)(i, j) = M(ns + i, j);
    Mat Ur = sub(mU, allred, range(mU.w));
    Mat Nm = w;
    gemm(false, false, -1.0, Ur, *alpha, 1.0, &Nm);
    diag_solve_small(&Nm, red_pos);
    for (int j = 0; j < nc; j++) {
      for (size_t q = 0; q < allred.size(); q++) (*mu)(allred[q], j) = Nm((int)q, j);
      for (int q = 0; q < ns; q++) (*mu)(allskel[q], j) = M(q, j);
    }
    down_sweep(mu);
  }
};

thread_local std::string g_err;

}  // namespace

extern "C" {

int kiport_dense_dim(int n_points, int domain_dim, int solution_dim, const double* points,
                     const double* normals, const double* weights, const double* curvatures,
                     double* out);

const char* kiport_last_error() { return g_err.c_str(); }

// Factor + solve, the same contract as the reference driver's kiref_solve:
// column-major rhs (N x nrhs), outputs mu (N x nrhs) and alpha
// (n_border x nrhs).  stats: [0] factor s, [1] solve s, [2] levels,
// [3] root skeleton size, [4] compressed boxes, [5] redundant DOFs.
int kiport_solve(int n_points, int domain_dim, int solution_dim, int pde,
                 const double* points, const double* normals, const double* weights,
                 const double* curvatures, int n_holes, const double* hole_centers,
                 const int* hole_start, const int* hole_count, const double* rhs, int nrhs,
                 double id_tol, int threads, int leaf, int proxy, double ratio,
                 int min_compress, double* mu_out, double* alpha_out, double* stats) {
  try {
    if (domain_dim != 2 && domain_dim != 3) throw std::runtime_error("domain_dim must be 2 or 3");
    if (!lapack().dgeqp3 || !lapack().dgemm)
      throw std::runtime_error("LAPACK symbols not found: load OpenBLAS first");
    Tree t;
    t.g.n_points = n_points;
    t.g.dim = domain_dim;
    t.g.sol_dim = solution_dim;
    t.g.pde = pde;
    // the Neumann and Gaussian problems have no border (initialize_U_mat gives
    // them an empty U, linear_solve.cpp:101-104)
    if (pde == 1 || pde == 2) n_holes = 0;
    t.g.pts = points;
    t.g.nrm = normals;
    t.g.wts = weights;
    t.g.curv = curvatures;
    t.p.tol = id_tol;
    t.p.threads = std::max(1, threads);
    t.p.leaf = leaf;
    if (proxy <= 0) proxy = domain_dim == 2 ? 128 : 32;
    t.p.proxy = proxy;
    t.p.ratio = ratio;
    t.p.min_compress = min_compress;
    int N = n_points * solution_dim;
    double t0 = omp_get_wtime();
    if (domain_dim == 3) {
      int q = (int)std::lround(std::sqrt(proxy / 2.0));
      if (2 * q * q != proxy) throw std::runtime_error("3D proxy count must be 2 q^2");
      proxy_sphere(&t.g, 2 * q);
      std::vector<int> hs(hole_start, hole_start + n_holes), hn(hole_count, hole_count + n_holes);
      compute_diag3(&t.g, n_holes > 0 ? hole_start[0] : n_points, hs, hn, t.p.threads);
    }
    t.build();
    if (n_holes > 0) {
      std::vector<int> all(N);
      for (int i = 0; i < N; i++) all[i] = i;
      border_matrices(t.g, n_holes, hole_centers, hole_start, hole_count, all, &t.U, &t.Psi);
    }
    t.skeletonize();
    double t1 = omp_get_wtime();
    Mat x(N, nrhs);
    std::memcpy(x.data(), rhs, sizeof(double) * (size_t)N * nrhs);
    if (n_holes > 0) {
      Mat alpha;
      t.mc_solve(&x, &alpha);
      if (alpha_out) std::memcpy(alpha_out, alpha.data(), sizeof(double) * alpha.a.size());
    } else {
      t.solve(&x);
    }
    double t2 = omp_get_wtime();
    std::memcpy(mu_out, x.data(), sizeof(double) * (size_t)N * nrhs);
    if (stats) {
      int comp = 0;
      long red = 0;
      for (auto& n : t.nodes)
        if (n.compressed) {
          comp++;
          red += (long)n.red.size();
        }
      stats[0] = t1 - t0;
      stats[1] = t2 - t1;
      stats[2] = (double)t.levels.size();
      stats[3] = (double)t.allskel.size();
      stats[4] = comp;
      stats[5] = (double)red;
    }
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

// Dense kernel matrix K(all, all), column-major (Kernel::operator()); 3D
// with the diagonal of compute_diag3 (no holes).
int kiport_dense(int n_points, int solution_dim, const double* points, const double* normals,
                 const double* weights, const double* curvatures, double* out) {
  return kiport_dense_dim(n_points, 2, solution_dim, points, normals, weights, curvatures, out);
}

int kiport_dense_dim(int n_points, int domain_dim, int solution_dim, const double* points,
                     const double* normals, const double* weights, const double* curvatures,
                     double* out) {
  Geometry g;
  g.n_points = n_points;
  g.dim = domain_dim;
  g.sol_dim = solution_dim;
  g.pts = points;
  g.nrm = normals;
  g.wts = weights;
  g.curv = curvatures;
  if (domain_dim == 3) compute_diag3(&g, n_points, {}, {}, 8);
  int N = n_points * solution_dim;
  std::vector<int> all(N);
  for (int i = 0; i < N; i++) all[i] = i;
  Mat K = kernel_block(g, all, all);
  std::memcpy(out, K.data(), sizeof(double) * (size_t)N * N);
  return 0;
}

// Residual rows of the (bordered) boundary-integral system, for checking a
// solution at sizes where the dense operator does not fit:
//   res[i, c]   = sum_j K(rows[i], j) mu[j, c] + sum_b U(rows[i], b) alpha[b, c] - f[rows[i], c]
//   res_b[b, c] = sum_j Psi(b, j) mu[j, c] - alpha[b, c]          (n_holes > 0)
// K is Kernel::operator() (kern_interp/kernel/kernel.cpp:304-429; 3D with the
// row-sum diagonal, O(N^2)), U/Psi initialize_U_mat/initialize_Psi_mat.
// Column-major mu (N x nrhs), alpha (n_border x nrhs), f (N x nrhs), res
// (nrows x nrhs), res_b (n_border x nrhs).
int kiport_residual_rows(int n_points, int domain_dim, int solution_dim, const double* points,
                         const double* normals, const double* weights, const double* curvatures,
                         int n_holes, const double* hole_centers, const int* hole_start,
                         const int* hole_count, const double* mu, const double* alpha,
                         const double* f, int nrhs, const int* rows, int nrows, int threads,
                         double* res, double* res_b) {
  try {
    Geometry g;
    g.n_points = n_points;
    g.dim = domain_dim;
    g.sol_dim = solution_dim;
    g.pts = points;
    g.nrm = normals;
    g.wts = weights;
    g.curv = curvatures;
    threads = std::max(1, threads);
    const int N = n_points * solution_dim;
    if (domain_dim == 3) {
      std::vector<int> hs(hole_start, hole_start + n_holes), hn(hole_count, hole_count + n_holes);
      compute_diag3(&g, n_holes > 0 ? hole_start[0] : n_points, hs, hn, threads);
    }
    const int d = domain_dim, dpp = d == 3 ? (solution_dim == 1 ? 1 : 9) : 0;
    // densities point-major so that one source's columns are contiguous
    std::vector<double> mt((size_t)N * nrhs);
    for (int c = 0; c < nrhs; c++)
      for (int j = 0; j < N; j++) mt[(size_t)j * nrhs + c] = mu[j + (size_t)N * c];
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
    for (int i = 0; i < nrows; i++) {
      std::vector<double> acc(nrhs, 0.0);
      const int t = rows[i], tp = t / solution_dim;
      for (int j = 0; j < N; j++) {
        const int sp = j / solution_dim;
        const double* dg = dpp ? g.diag.data() + (size_t)dpp * sp : nullptr;
        const double e = entry(g, t, j, points + d * tp, normals + d * tp, points + d * sp,
                               normals + d * sp, weights[sp], curvatures ? curvatures[sp] : 0., dg);
        const double* m = mt.data() + (size_t)j * nrhs;
        for (int c = 0; c < nrhs; c++) acc[c] += e * m[c];
      }
      for (int c = 0; c < nrhs; c++) res[i + (size_t)nrows * c] = acc[c] - f[t + (size_t)N * c];
    }
    if (n_holes > 0) {
      Mat U, Psi;
      std::vector<int> rv(rows, rows + nrows);
      border_matrices(g, n_holes, hole_centers, hole_start, hole_count, rv, &U, &Psi);
      const int nb = U.w;
      for (int c = 0; c < nrhs; c++) {
        for (int i = 0; i < nrows; i++) {
          double a = 0.;
          for (int b = 0; b < nb; b++) a += U(i, b) * alpha[b + (size_t)nb * c];
          res[i + (size_t)nrows * c] += a;
        }
        for (int b = 0; b < nb; b++) {
          // Psi's row b is nonzero only on its hole's DOFs
          const int h = b / (nb / n_holes);
          const int j0 = hole_start[h] * solution_dim, j1 = j0 + hole_count[h] * solution_dim;
          double a = 0.;
          for (int j = j0; j < j1; j++) a += Psi(b, j) * mu[j + (size_t)N * c];
          res_b[b + (size_t)nb * c] = a - alpha[b + (size_t)nb * c];
        }
      }
    }
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

}  // extern "C"
