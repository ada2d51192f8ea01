// Reference-shaped C++ surface over the C ABI (ki_gpu.h): the classes and
// free functions a kern_interp driver calls -- ki_Mat, PointVec, Boundary,
// Kernel, QuadTree, SkelFactorization, linear_solve, boundary_integral_solve
// -- with the reference's names and argument meanings, so that a driver
// written against the reference's headers compiles against this one and
// runs the GPU factorization.  Header-only; link with -lki_gpu.
//
// Interfaces restated (paths relative to the reference project):
//   ki_Mat                 kern_interp/ki_mat.h:19-104 (column-major, lda == height,
//                          deep-copy semantics)
//   PointVec               kern_interp/pointvec.h:8-20
//   Hole, Boundary         kern_interp/boundaries/boundary.h:11-70
//   Kernel                 kern_interp/kernel/kernel.h:17-66
//   QuadTree               kern_interp/quadtree/quadtree.h:110-125 (initialize_tree)
//   SkelFactorization      kern_interp/skel_factorization/skel_factorization.h:20-57
//   linear_solve, boundary_integral_solve   kern_interp/linear_solve.h:17-31,
//                          kern_interp/linear_solve.cpp:202-303
//
// Differences, by design:
//   * The factorization lives on the GPU, owned by the QuadTree (in the
//     reference it is stored in the tree's nodes too): skeletonize creates it
//     from the boundary the tree was initialized with, the tree destroys it.
//   * fact_threads is accepted and ignored; the 3D diagonal entries
//     (Kernel::compute_diag_entries_3d*) are computed inside skeletonize.
//   * Hole membership comes from node ranges: the outer boundary's nodes come
//     first (num_outer_nodes of them, or all nodes not in holes), then each
//     hole's num_nodes nodes in order -- the layout the reference's boundaries
//     build (boundary.h:61-62).
//   * Errors throw std::runtime_error with the library's message instead of
//     asserting.
//   * multiply_connected_solve handles every column of b (the reference
//     solves column 0 only, skel_factorization.cpp:915-916).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "ki_gpu.h"

namespace kern_interp {

namespace detail {
inline void check(int rc) {
  if (rc != KI_OK) throw std::runtime_error(std::string("kern_interp_gb300: ") + ki_last_error());
}
}  // namespace detail

// --------------------------------------------------------------------- ki_Mat
struct ki_Mat {
  double* mat = nullptr;
  int lda_ = 0, height_ = 0, width_ = 0;

  ki_Mat() {}
  ki_Mat(int h, int w) : lda_(h), height_(h), width_(w) {
    if (h < 0 || w < 0) throw std::invalid_argument("ki_Mat: negative size");
    if (h > 0 && w > 0) {
      mat = new double[(size_t)h * w];
      std::fill(mat, mat + (size_t)h * w, 0.0);
    }
  }
  ki_Mat(const ki_Mat& o) : ki_Mat(o.height_, o.width_) {
    if (mat) std::memcpy(mat, o.mat, sizeof(double) * (size_t)height_ * width_);
  }
  ki_Mat(ki_Mat&& o) noexcept : mat(o.mat), lda_(o.lda_), height_(o.height_), width_(o.width_) {
    o.mat = nullptr;
    o.lda_ = o.height_ = o.width_ = 0;
  }
  ki_Mat& operator=(const ki_Mat& o) {
    if (this != &o) {
      ki_Mat c(o);
      *this = std::move(c);
    }
    return *this;
  }
  ki_Mat& operator=(ki_Mat&& o) noexcept {
    if (this != &o) {
      delete[] mat;
      mat = o.mat;
      lda_ = o.lda_;
      height_ = o.height_;
      width_ = o.width_;
      o.mat = nullptr;
      o.lda_ = o.height_ = o.width_ = 0;
    }
    return *this;
  }
  ~ki_Mat() { delete[] mat; }

  double get(int i, int j) const { return mat[i + (size_t)lda_ * j]; }
  void set(int i, int j, double a) { mat[i + (size_t)lda_ * j] = a; }
  int height() const { return height_; }
  int width() const { return width_; }
  double frob_norm() const {
    double s = 0;
    for (size_t e = 0; e < (size_t)height_ * width_; e++) s += mat[e] * mat[e];
    return std::sqrt(s);
  }
  ki_Mat operator-(const ki_Mat& o) const {
    if (o.height_ != height_ || o.width_ != width_) throw std::invalid_argument("ki_Mat: size mismatch");
    ki_Mat r(*this);
    for (size_t e = 0; e < (size_t)height_ * width_; e++) r.mat[e] -= o.mat[e];
    return r;
  }
};

// ------------------------------------------------------------------- PointVec
struct PointVec {
  std::vector<double> a;
  PointVec() {}
  PointVec(double m, double n) : a{m, n} {}
  PointVec(double x, double y, double z) : a{x, y, z} {}
  explicit PointVec(const std::vector<double>& b) : a(b) {}
  double norm() const { return std::sqrt(dot(*this)); }
  double dot(const PointVec& o) const {
    double s = 0;
    for (size_t i = 0; i < a.size(); i++) s += a[i] * o.a[i];
    return s;
  }
  PointVec operator-(const PointVec& o) const {
    PointVec r(*this);
    for (size_t i = 0; i < a.size(); i++) r.a[i] -= o.a[i];
    return r;
  }
  PointVec operator+(const PointVec& o) const {
    PointVec r(*this);
    for (size_t i = 0; i < a.size(); i++) r.a[i] += o.a[i];
    return r;
  }
  PointVec operator*(const double d) const {
    PointVec r(*this);
    for (double& v : r.a) v *= d;
    return r;
  }
};

// ------------------------------------------------------------------- Boundary
struct Hole {
  PointVec center;
  double radius = 0;
  int num_nodes = 0;
};

// The reference's boundary-condition selector; concrete boundaries (not part
// of this library) interpret it.
enum BoundaryCondition {
  ELECTRON_3D, LAPLACE_PIPE_HOLES, LAPLACE_COW_MESH, SINGLE_ELECTRON, ALL_ONES, ALL_NEG_ONES,
  ALL_ZEROS, TANGENT_VEC, REVERSE_TANGENT_VEC, NORMAL_VEC, REVERSE_NORMAL_VEC, EX1,
  LEFT_TO_RIGHT_FLOW, NO_SLIP, HORIZONTAL_VEC, EX3A, EX3B, LAPLACE_CHECK_2D, LAPLACE_CHECK_3D,
  STOKES_SPHERES, STOKES_PIPE_HOLES, STOKES_COW_MESH, STOKES_2D_MIX, DEFAULT
};

class Boundary {
 public:
  int num_outer_nodes = -1;
  std::vector<double> perturbation_parameters;
  std::vector<double> points, normals, curvatures, weights;
  std::vector<Hole> holes;
  ki_Mat boundary_values;
  virtual std::unique_ptr<Boundary> clone() const = 0;
  virtual ~Boundary() {}
  virtual void initialize(int n, BoundaryCondition bc) = 0;
  virtual bool is_in_domain(const PointVec& a) const = 0;
};

// --------------------------------------------------------------------- Kernel
struct Kernel {
  // the order of ki_pde
  enum Pde { LAPLACE, LAPLACE_NEUMANN, GAUSS, STOKES };
  int solution_dimension = 1, domain_dimension = 2;
  Kernel::Pde pde = LAPLACE;
  std::vector<double> boundary_points_, boundary_normals_, boundary_weights_, boundary_curvatures_,
      domain_points;
  Kernel() {}
  Kernel(int solution_dimension_, int domain_dimension_, Kernel::Pde pde_, Boundary* boundary,
         std::vector<double> domain_points_)
      : solution_dimension(solution_dimension_), domain_dimension(domain_dimension_), pde(pde_),
        boundary_points_(boundary->points), boundary_normals_(boundary->normals),
        boundary_weights_(boundary->weights), boundary_curvatures_(boundary->curvatures),
        domain_points(std::move(domain_points_)) {}
  // computed on the GPU inside SkelFactorization::skeletonize
  void compute_diag_entries_3dlaplace(Boundary*) {}
  void compute_diag_entries_3dstokes(Boundary*) {}
  void update_data(Boundary* boundary) {
    boundary_points_ = boundary->points;
    boundary_normals_ = boundary->normals;
    boundary_weights_ = boundary->weights;
    boundary_curvatures_ = boundary->curvatures;
  }
};

// ------------------------------------------------------------------- QuadTree
// Holds the boundary the tree is built over and, after skeletonize, the GPU
// factorization (the tree and its boxes are built on the GPU).
class QuadTree {
 public:
  int solution_dimension = 1, domain_dimension = 2;
  int no_proxy_level = 0;
  ki_Mat U, Psi;   // kept for drivers that set them; the GPU forms its own
  QuadTree() {}
  QuadTree(const QuadTree&) = delete;
  QuadTree& operator=(const QuadTree&) = delete;
  ~QuadTree() { reset(); }

  void initialize_tree(Boundary* boundary, int solution_dimension_, int domain_dimension_) {
    if (!boundary) throw std::invalid_argument("initialize_tree: NULL boundary");
    reset();
    boundary_ = boundary;
    solution_dimension = solution_dimension_;
    domain_dimension = domain_dimension_;
  }

  // QuadTree::perturb (quadtree.cpp:581-890): the tree now describes
  // new_boundary (points identified by index; the boundary must outlive the
  // tree's use of it), and the next skeletonize keeps the factors of the
  // boxes the change left alone (ki_factor_update).
  void perturb(const Boundary& new_boundary) {
    if (!boundary_) throw std::invalid_argument("perturb: tree not initialized");
    boundary_ = &new_boundary;
  }

  // The GPU factorization (NULL before skeletonize).
  ki_factor* factor() const { return factor_; }
  const Boundary* boundary() const { return boundary_; }
  int n_border() const {
    // the factorization's own count once it exists (the Neumann and Gaussian
    // kernels have no border whatever holes the boundary has)
    ki_factor_info info;
    if (factor_ && ki_factor_get_info(factor_, &info) == KI_OK) return info.n_border;
    if (!boundary_ || boundary_->holes.empty()) return 0;
    const int c = solution_dimension == 1 ? 1 : (domain_dimension == 2 ? 3 : 6);
    return c * (int)boundary_->holes.size();
  }
  void reset() {
    if (factor_) ki_factor_destroy(factor_);
    factor_ = nullptr;
  }

 private:
  friend class SkelFactorization;
  const Boundary* boundary_ = nullptr;
  ki_factor* factor_ = nullptr;
};

// ---------------------------------------------------------- SkelFactorization
class SkelFactorization {
 public:
  double id_tol = 1e-6;
  int fact_threads = 1;   // no meaning on the GPU
  bool using_hif = false;
  // Beyond the reference: the factorization's precision (KI_PRECISION_FP64,
  // the reference's arithmetic, or KI_PRECISION_FP32) and its tree / proxy
  // parameters (0: the reference's defaults).
  int precision = KI_PRECISION_FP64;
  int max_leaf_dofs = 0, num_proxy_points = 0, min_dofs_to_compress = 0;
  double radius_ratio = 0;

  SkelFactorization() {}
  SkelFactorization(double id_tol_, int fact_threads_, bool using_hif_ = false)
      : id_tol(id_tol_), fact_threads(fact_threads_), using_hif(using_hif_) {
    if (using_hif) throw std::invalid_argument("SkelFactorization: HIF levels are not supported");
  }

  // Factor the boundary the tree was initialized with, or perturbed to (the
  // kernel gives the PDE and dimensions); the factorization is stored in the
  // tree.  A tree factorized before is re-factorized keeping the factors of
  // unchanged boxes, as the reference's skeletonize skips boxes still
  // compressed (skel_factorization.cpp:199-208).
  void skeletonize(const Kernel& K, QuadTree* tree) const {
    if (!tree || !tree->boundary_) throw std::invalid_argument("skeletonize: tree not initialized");
    const Boundary& b = *tree->boundary_;
    const int dim = K.domain_dimension;
    const int n = (int)b.weights.size();
    std::vector<double> hc;
    std::vector<int> hs, hn;
    int hole_nodes = 0;
    for (const Hole& h : b.holes) hole_nodes += h.num_nodes;
    int start = b.num_outer_nodes >= 0 ? b.num_outer_nodes : n - hole_nodes;
    for (const Hole& h : b.holes) {
      if ((int)h.center.a.size() < dim) throw std::invalid_argument("skeletonize: hole centre dimension");
      for (int q = 0; q < dim; q++) hc.push_back(h.center.a[q]);
      hs.push_back(start);
      hn.push_back(h.num_nodes);
      start += h.num_nodes;
    }
    ki_problem_desc d;
    std::memset(&d, 0, sizeof(d));
    d.n_points = n;
    d.domain_dimension = dim;
    d.solution_dimension = K.solution_dimension;
    d.pde = (int)K.pde;
    d.points = b.points.data();
    d.normals = b.normals.data();
    d.weights = b.weights.data();
    d.curvatures = b.curvatures.empty() ? nullptr : b.curvatures.data();
    d.n_holes = (int)b.holes.size();
    d.hole_centers = hc.empty() ? nullptr : hc.data();
    d.hole_node_start = hs.empty() ? nullptr : hs.data();
    d.hole_node_count = hn.empty() ? nullptr : hn.data();
    d.max_leaf_dofs = max_leaf_dofs;
    d.num_proxy_points = num_proxy_points;
    d.radius_ratio = radius_ratio;
    d.min_dofs_to_compress = min_dofs_to_compress;
    d.id_tol = id_tol;
    d.precision = precision;
    tree->solution_dimension = K.solution_dimension;
    tree->domain_dimension = dim;
    if (tree->factor_)
      detail::check(ki_factor_update(tree->factor_, &d));
    else
      detail::check(ki_factor_create(&d, &tree->factor_));
  }

  // x = A^-1 b for every column of b (simply connected problems).
  void solve(const QuadTree& tree, ki_Mat* x, const ki_Mat& b) const {
    if (tree.n_border()) throw std::invalid_argument("solve: the problem has holes (multiply_connected_solve)");
    run(tree, x, nullptr, b);
  }

  // [mu; alpha] of the bordered system [K U; Psi -I] [mu; alpha] = [b; 0].
  void multiply_connected_solve(const QuadTree& tree, ki_Mat* mu, ki_Mat* alpha, const ki_Mat& b) const {
    run(tree, mu, alpha, b);
  }

 private:
  void run(const QuadTree& tree, ki_Mat* x, ki_Mat* alpha, const ki_Mat& b) const {
    if (!tree.factor_) throw std::invalid_argument("solve: not skeletonized");
    if (!x) throw std::invalid_argument("solve: NULL x");
    const int N = b.height(), nrhs = b.width(), nb = tree.n_border();
    ki_Mat out(N, nrhs), al(std::max(nb, 1), nrhs);
    detail::check(ki_solve(tree.factor_, b.mat, std::max(1, b.lda_), nrhs, out.mat, std::max(1, N),
                           al.mat, std::max(nb, 1)));
    *x = std::move(out);
    if (alpha) {
      ki_Mat a(nb, nrhs);
      for (int c = 0; c < nrhs; c++)
        for (int i = 0; i < nb; i++) a.set(i, c, al.get(i, c));
      *alpha = std::move(a);
    }
  }
};

// ------------------------------------------------------------ free functions
// linear_solve (linear_solve.cpp:202-227): mu (and alpha for a problem with
// holes) for the right-hand side f.
inline void linear_solve(const SkelFactorization& skel_factorization, const QuadTree& quadtree,
                         const ki_Mat& f, ki_Mat* mu, ki_Mat* alpha = nullptr) {
  if (alpha == nullptr && quadtree.n_border() == 0) {
    skel_factorization.solve(quadtree, mu, f);
  } else {
    ki_Mat a;
    skel_factorization.multiply_connected_solve(quadtree, mu, &a, f);
    if (alpha) *alpha = std::move(a);
  }
}

// boundary_integral_solve (linear_solve.cpp:257-303): factor the boundary
// (skeletonize into quadtree, which initialize_tree prepared), solve for the
// boundary values, and evaluate the solution at the domain points
// (domain_points, or the kernel's when empty); points the boundary reports
// outside its domain get 0, as in the reference.
inline ki_Mat boundary_integral_solve(const Kernel& kernel, const Boundary& boundary,
                                      QuadTree* quadtree, double id_tol, int fact_threads,
                                      const std::vector<double>& domain_points) {
  SkelFactorization skel(id_tol, fact_threads);
  skel.skeletonize(kernel, quadtree);
  ki_Mat mu, alpha;
  const int nb = quadtree->n_border();
  linear_solve(skel, *quadtree, boundary.boundary_values, &mu, nb ? &alpha : nullptr);
  const std::vector<double>& tg = domain_points.empty() ? kernel.domain_points : domain_points;
  const int dim = kernel.domain_dimension, sd = kernel.solution_dimension;
  const int nt = (int)tg.size() / dim;
  ki_Mat out(nt * sd, 1);
  if (nt > 0)
    detail::check(ki_eval_targets(quadtree->factor(), tg.data(), nt, mu.mat, mu.height(), 1,
                                  nb ? alpha.mat : nullptr, std::max(nb, 1), out.mat, out.height()));
  for (int p = 0; p < nt; p++) {
    PointVec pt(std::vector<double>(tg.begin() + (size_t)p * dim, tg.begin() + (size_t)(p + 1) * dim));
    if (!boundary.is_in_domain(pt))
      for (int j = 0; j < sd; j++) out.set(sd * p + j, 0, 0.0);
  }
  return out;
}

}  // namespace kern_interp
