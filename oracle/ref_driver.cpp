// Driver around the UNMODIFIED reference CPU solver (kern_interp), compiled
// from the reference's own sources by oracle/build_ref.py into oracle/_ref/.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product links, loads or calls
// this file; tests and the fixture generator use it as the checker.
//
// It exposes one extern "C" entry point that mirrors the reference's
// boundary_integral_solve flow (kern_interp/linear_solve.cpp:257-303):
//   Boundary data -> QuadTree::initialize_tree -> SkelFactorization::skeletonize
//   -> SkelFactorization::solve / multiply_connected_solve (one column at a
//   time, because multiply_connected_solve handles column 0 only,
//   kern_interp/skel_factorization/skel_factorization.cpp:915-916).
// Hole border matrices are built from node ranges: U with the reference's own
// initialize_U_mat (centres only, kern_interp/linear_solve.cpp:19-107) and Psi
// from the ranges, because the reference's circle-membership test in
// initialize_Psi_mat (kern_interp/linear_solve.cpp:137) misclassifies
// non-circular holes.
#include <omp.h>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "kern_interp/boundaries/boundary.h"
#include "kern_interp/kernel/kernel.h"
#include "kern_interp/linear_solve.h"
#include "kern_interp/quadtree/quadtree.h"
#include "kern_interp/skel_factorization/skel_factorization.h"

namespace {

using kern_interp::Boundary;
using kern_interp::BoundaryCondition;
using kern_interp::PointVec;

// A Boundary whose data vectors are filled directly from caller arrays.
class ArrayBoundary : public Boundary {
 public:
  std::unique_ptr<Boundary> clone() const override {
    return std::unique_ptr<Boundary>(new ArrayBoundary(*this));
  }
  void initialize(int, BoundaryCondition) override {}
  bool is_in_domain(const PointVec&) const override { return true; }
};

}  // namespace

extern "C" {

// Stats written by kiref_solve (doubles): [0] factor seconds, [1] solve
// seconds (all columns), [2] number of tree levels, [3] root skeleton size,
// [4] number of compressed boxes, [5] sum of redundant DOFs.
int kiref_solve(int n_points, int domain_dim, int solution_dim, int pde,
                const double* points, const double* normals,
                const double* weights, const double* curvatures,
                int n_holes, const double* hole_centers,
                const int* hole_start, const int* hole_count,
                const double* rhs, int nrhs, double id_tol, int threads,
                double* mu_out, double* alpha_out, double* stats) {
  const int d = domain_dim;
  const int N = n_points * solution_dim;
  // As the reference's experiment drivers do before factorizing
  // (kern_interp/experiments/pde_acc.cpp:97): one BLAS thread per box.
  openblas_set_num_threads(1);
  ArrayBoundary boundary;
  boundary.points.assign(points, points + (size_t)n_points * d);
  boundary.normals.assign(normals, normals + (size_t)n_points * d);
  boundary.weights.assign(weights, weights + n_points);
  if (curvatures) boundary.curvatures.assign(curvatures, curvatures + n_points);
  for (int h = 0; h < n_holes; h++) {
    kern_interp::Hole hole;
    std::vector<double> c(hole_centers + (size_t)h * d, hole_centers + (size_t)(h + 1) * d);
    hole.center = PointVec(c);
    hole.radius = 0.;
    hole.num_nodes = hole_count[h];
    boundary.holes.push_back(hole);
  }
  boundary.num_outer_nodes = n_points;
  if (n_holes > 0) boundary.num_outer_nodes = hole_start[0];
  boundary.boundary_values = kern_interp::ki_Mat(N, 1);

  kern_interp::Kernel kernel(solution_dim, d, (kern_interp::Kernel::Pde)pde,
                             &boundary, std::vector<double>());
  // 3D diagonals, as the reference's 3D drivers do before factorizing
  // (kern_interp/experiments/ex1_concentric_spheres.cpp:88)
  if (d == 3) {
    if (solution_dim == 1) kernel.compute_diag_entries_3dlaplace(&boundary);
    else kernel.compute_diag_entries_3dstokes(&boundary);
  }
  kern_interp::QuadTree quadtree;
  quadtree.initialize_tree(&boundary, solution_dim, d);

  // the Neumann and Gaussian kernels get an empty U (initialize_U_mat,
  // kern_interp/linear_solve.cpp:101-104): no border, holes ignored
  if (n_holes > 0 && pde != kern_interp::Kernel::Pde::LAPLACE_NEUMANN &&
      pde != kern_interp::Kernel::Pde::GAUSS) {
    quadtree.U = kern_interp::initialize_U_mat(kernel.pde, boundary.holes,
                                               boundary.points, d);
    // Psi from node ranges (Laplace: weights; Stokes: reference layout,
    // kern_interp/linear_solve.cpp:146-177).
    int c = quadtree.U.width() / n_holes;
    kern_interp::ki_Mat Psi(c * n_holes, N);
    for (int h = 0; h < n_holes; h++) {
      for (int p = hole_start[h]; p < hole_start[h] + hole_count[h]; p++) {
        double w = weights[p];
        if (solution_dim == 1) {
          Psi.set(h, p, w);
        } else if (d == 3) {
          double r[3];
          for (int q = 0; q < 3; q++) r[q] = points[3 * p + q] - hole_centers[3 * h + q];
          Psi.set(6 * h, 3 * p, w);
          Psi.set(6 * h + 1, 3 * p + 1, w);
          Psi.set(6 * h + 2, 3 * p + 2, w);
          Psi.set(6 * h + 4, 3 * p, -w * (-r[2]));
          Psi.set(6 * h + 5, 3 * p, -w * (r[1]));
          Psi.set(6 * h + 3, 3 * p + 1, -w * (r[2]));
          Psi.set(6 * h + 5, 3 * p + 1, -w * (-r[0]));
          Psi.set(6 * h + 3, 3 * p + 2, -w * (-r[1]));
          Psi.set(6 * h + 4, 3 * p + 2, -w * (r[0]));
        } else {
          double x = points[2 * p], y = points[2 * p + 1];
          Psi.set(3 * h, 2 * p, w);
          Psi.set(3 * h + 1, 2 * p + 1, w);
          Psi.set(3 * h + 2, 2 * p, w * y);
          Psi.set(3 * h + 2, 2 * p + 1, -w * x);
        }
      }
    }
    quadtree.Psi = Psi;
  }

  kern_interp::SkelFactorization skel(id_tol, threads);
  double t0 = omp_get_wtime();
  skel.skeletonize(kernel, &quadtree);
  double t1 = omp_get_wtime();
  for (int col = 0; col < nrhs; col++) {
    kern_interp::ki_Mat f(N, 1);
    std::memcpy(f.mat, rhs + (size_t)col * N, sizeof(double) * N);
    kern_interp::ki_Mat mu(N, 1);
    // as linear_solve decides (kern_interp/linear_solve.cpp:236): the bordered
    // solve only when U has columns
    if (quadtree.U.width() > 0) {
      kern_interp::ki_Mat alpha(quadtree.U.width(), 1);
      skel.multiply_connected_solve(quadtree, &mu, &alpha, f);
      if (alpha_out)
        std::memcpy(alpha_out + (size_t)col * quadtree.U.width(), alpha.mat,
                    sizeof(double) * quadtree.U.width());
    } else {
      skel.solve(quadtree, &mu, f);
    }
    std::memcpy(mu_out + (size_t)col * N, mu.mat, sizeof(double) * N);
  }
  double t2 = omp_get_wtime();
  if (stats) {
    int compressed = 0;
    long redundant = 0;
    for (auto* level : quadtree.levels)
      for (auto* node : level->nodes)
        if (node->compressed) {
          compressed++;
          redundant += node->dof_lists.redundant.size();
        }
    stats[0] = t1 - t0;
    stats[1] = t2 - t1;
    stats[2] = quadtree.levels.size();
    stats[3] = quadtree.root->dof_lists.active_box.size();
    stats[4] = compressed;
    stats[5] = (double)redundant;
  }
  return 0;
}

// Incremental re-factorization as the reference's updating experiments run
// it (kern_interp/experiments/experiment_two.cpp:49-70, the updating test
// kern_interp/kern_interp_test.cpp:424-465): frame 0 is initialized and
// skeletonized; each later frame's boundary data replace the previous ones,
// then Kernel::update_data, QuadTree::perturb and a skeletonize that skips
// the boxes perturb left compressed, then the bordered or plain solve of the
// frame's one right-hand side.  Arrays hold `frames` frames back to back
// (points/normals dim n, weights/curvatures n, hole centres dim n_holes,
// rhs N; the hole node ranges are the same in every frame).  Outputs per
// frame: mu (N), alpha (border columns), stats[2 f] skeletonize seconds and
// stats[2 f + 1] boxes compressed after it.
int kiref_update_solve(int n_points, int domain_dim, int solution_dim, int pde, int frames,
                       const double* points, const double* normals, const double* weights,
                       const double* curvatures, int n_holes, const double* hole_centers,
                       const int* hole_start, const int* hole_count, const double* rhs,
                       double id_tol, int threads, double* mu_out, double* alpha_out,
                       double* stats) {
  const int d = domain_dim;
  const int N = n_points * solution_dim;
  openblas_set_num_threads(1);
  ArrayBoundary boundary;
  auto load = [&](int f) {
    boundary.points.assign(points + (size_t)f * n_points * d, points + (size_t)(f + 1) * n_points * d);
    boundary.normals.assign(normals + (size_t)f * n_points * d,
                            normals + (size_t)(f + 1) * n_points * d);
    boundary.weights.assign(weights + (size_t)f * n_points, weights + (size_t)(f + 1) * n_points);
    if (curvatures)
      boundary.curvatures.assign(curvatures + (size_t)f * n_points,
                                 curvatures + (size_t)(f + 1) * n_points);
    boundary.holes.clear();
    for (int h = 0; h < n_holes; h++) {
      kern_interp::Hole hole;
      const double* c0 = hole_centers + ((size_t)f * n_holes + h) * d;
      hole.center = PointVec(std::vector<double>(c0, c0 + d));
      hole.radius = 0.;
      hole.num_nodes = hole_count[h];
      boundary.holes.push_back(hole);
    }
    boundary.num_outer_nodes = n_holes > 0 ? hole_start[0] : n_points;
    boundary.boundary_values = kern_interp::ki_Mat(N, 1);
  };
  load(0);
  kern_interp::Kernel kernel(solution_dim, d, (kern_interp::Kernel::Pde)pde, &boundary,
                             std::vector<double>());
  kern_interp::QuadTree quadtree;
  quadtree.initialize_tree(&boundary, solution_dim, d);
  kern_interp::SkelFactorization skel(id_tol, threads);
  for (int f = 0; f < frames; f++) {
    if (f > 0) {
      load(f);
      kernel.update_data(&boundary);
      quadtree.perturb(boundary);
    }
    if (d == 3) {
      if (solution_dim == 1) kernel.compute_diag_entries_3dlaplace(&boundary);
      else kernel.compute_diag_entries_3dstokes(&boundary);
    }
    const double* pts = points + (size_t)f * n_points * d;
    const double* w = weights + (size_t)f * n_points;
    const double* hc = hole_centers + (size_t)f * n_holes * d;
    if (n_holes > 0) {
      quadtree.U = kern_interp::initialize_U_mat(kernel.pde, boundary.holes, boundary.points, d);
      const int c = quadtree.U.width() / n_holes;
      kern_interp::ki_Mat Psi(c * n_holes, N);
      for (int h = 0; h < n_holes; h++)
        for (int p = hole_start[h]; p < hole_start[h] + hole_count[h]; p++) {
          if (solution_dim == 1) {
            Psi.set(h, p, w[p]);
          } else if (d == 2) {
            Psi.set(3 * h, 2 * p, w[p]);
            Psi.set(3 * h + 1, 2 * p + 1, w[p]);
            Psi.set(3 * h + 2, 2 * p, w[p] * pts[2 * p + 1]);
            Psi.set(3 * h + 2, 2 * p + 1, -w[p] * pts[2 * p]);
          } else {
            double r[3];
            for (int q = 0; q < 3; q++) r[q] = pts[3 * p + q] - hc[3 * h + q];
            Psi.set(6 * h, 3 * p, w[p]);
            Psi.set(6 * h + 1, 3 * p + 1, w[p]);
            Psi.set(6 * h + 2, 3 * p + 2, w[p]);
            Psi.set(6 * h + 4, 3 * p, w[p] * r[2]);
            Psi.set(6 * h + 5, 3 * p, -w[p] * r[1]);
            Psi.set(6 * h + 3, 3 * p + 1, -w[p] * r[2]);
            Psi.set(6 * h + 5, 3 * p + 1, w[p] * r[0]);
            Psi.set(6 * h + 3, 3 * p + 2, w[p] * r[1]);
            Psi.set(6 * h + 4, 3 * p + 2, -w[p] * r[0]);
          }
        }
      quadtree.Psi = Psi;
    }
    double t0 = omp_get_wtime();
    skel.skeletonize(kernel, &quadtree);
    double t1 = omp_get_wtime();
    kern_interp::ki_Mat fv(N, 1);
    std::memcpy(fv.mat, rhs + (size_t)f * N, sizeof(double) * N);
    kern_interp::ki_Mat mu(N, 1);
    if (n_holes > 0) {
      kern_interp::ki_Mat alpha(quadtree.U.width(), 1);
      skel.multiply_connected_solve(quadtree, &mu, &alpha, fv);
      if (alpha_out)
        std::memcpy(alpha_out + (size_t)f * quadtree.U.width(), alpha.mat,
                    sizeof(double) * quadtree.U.width());
    } else {
      skel.solve(quadtree, &mu, fv);
    }
    std::memcpy(mu_out + (size_t)f * N, mu.mat, sizeof(double) * N);
    int compressed = 0;
    for (auto* level : quadtree.levels)
      for (auto* node : level->nodes) compressed += node->compressed;
    if (stats) {
      stats[2 * f] = t1 - t0;
      stats[2 * f + 1] = compressed;
    }
  }
  return 0;
}

// Dense Nystrom matrix K(all, all) of the reference kernel
// (Kernel::operator(), kern_interp/kernel/kernel.cpp:304-360), column-major.
int kiref_dense(int n_points, int domain_dim, int solution_dim, int pde,
                const double* points, const double* normals,
                const double* weights, const double* curvatures, double* out) {
  const int d = domain_dim;
  const int N = n_points * solution_dim;
  ArrayBoundary boundary;
  boundary.points.assign(points, points + (size_t)n_points * d);
  boundary.normals.assign(normals, normals + (size_t)n_points * d);
  boundary.weights.assign(weights, weights + n_points);
  if (curvatures) boundary.curvatures.assign(curvatures, curvatures + n_points);
  boundary.num_outer_nodes = n_points;
  kern_interp::Kernel kernel(solution_dim, d, (kern_interp::Kernel::Pde)pde,
                             &boundary, std::vector<double>());
  if (d == 3) {
    if (solution_dim == 1) kernel.compute_diag_entries_3dlaplace(&boundary);
    else kernel.compute_diag_entries_3dstokes(&boundary);
  }
  std::vector<int> all(N);
  for (int i = 0; i < N; i++) all[i] = i;
  kern_interp::ki_Mat K = kernel(all, all);
  std::memcpy(out, K.mat, sizeof(double) * (size_t)N * N);
  return 0;
}

}  // extern "C"
