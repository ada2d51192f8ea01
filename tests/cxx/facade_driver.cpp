// A reference-style driver written against include/kern_interp_gb300.hpp
// only: it subclasses Boundary, fills its data vectors, builds the Kernel and
// QuadTree, and calls SkelFactorization::skeletonize, linear_solve and
// boundary_integral_solve as a kern_interp driver does.
//
// Input (binary, little-endian): int32 n, dim, sd, n_targets, n_holes,
// num_outer_nodes, leaf, proxy, min_compress; double id_tol, ratio; then
// doubles points (dim n), normals (dim n), weights (n), curvatures (n),
// f (sd n), targets (dim n_targets), hole centres (dim n_holes); int32 hole
// node counts (n_holes).
// Optionally followed by int32 n_frames and, per frame, doubles points
// (dim n) and hole centres (dim n_holes): perturbation frames, each applied
// with QuadTree::perturb and skeletonize on the first tree, as the
// reference's updating experiments do.
// Output (binary): doubles mu (sd n), alpha (border columns), u at the
// targets (sd n_targets), then per frame mu and alpha.  Exit status 3 when
// the library reports an error.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <memory>
#include <vector>

#include "kern_interp_gb300.hpp"

using namespace kern_interp;

class ArrayBoundary : public Boundary {
 public:
  std::unique_ptr<Boundary> clone() const override {
    return std::unique_ptr<Boundary>(new ArrayBoundary(*this));
  }
  void initialize(int, BoundaryCondition) override {}
  bool is_in_domain(const PointVec&) const override { return true; }
};

template <typename T>
static std::vector<T> take(std::ifstream& in, size_t n) {
  std::vector<T> v(n);
  in.read(reinterpret_cast<char*>(v.data()), sizeof(T) * n);
  if (!in) throw std::runtime_error("short input");
  return v;
}

int main(int argc, char** argv) {
  if (argc != 3) {
    std::cerr << "usage: facade_driver input.bin output.bin\n";
    return 2;
  }
  try {
    std::ifstream in(argv[1], std::ios::binary);
    const std::vector<int> h = take<int>(in, 9);
    const std::vector<double> hd = take<double>(in, 2);
    const int n = h[0], dim = h[1], sd = h[2], nt = h[3], nh = h[4];
    ArrayBoundary b;
    b.num_outer_nodes = h[5];
    b.points = take<double>(in, (size_t)dim * n);
    b.normals = take<double>(in, (size_t)dim * n);
    b.weights = take<double>(in, n);
    b.curvatures = take<double>(in, n);
    const std::vector<double> f = take<double>(in, (size_t)sd * n);
    const std::vector<double> targets = take<double>(in, (size_t)dim * nt);
    const std::vector<double> hc = take<double>(in, (size_t)dim * nh);
    const std::vector<int> hn = take<int>(in, nh);
    for (int q = 0; q < nh; q++) {
      Hole hole;
      hole.center = PointVec(std::vector<double>(hc.begin() + q * dim, hc.begin() + (q + 1) * dim));
      hole.num_nodes = hn[q];
      b.holes.push_back(hole);
    }
    b.boundary_values = ki_Mat(sd * n, 1);
    for (int i = 0; i < sd * n; i++) b.boundary_values.set(i, 0, f[i]);

    Kernel kernel(sd, dim, sd == 1 ? Kernel::LAPLACE : Kernel::STOKES, &b, targets);
    QuadTree quadtree;
    quadtree.initialize_tree(&b, sd, dim);
    SkelFactorization skel(hd[0], 4);
    skel.max_leaf_dofs = h[6];
    skel.num_proxy_points = h[7];
    skel.min_dofs_to_compress = h[8];
    skel.radius_ratio = hd[1];
    skel.skeletonize(kernel, &quadtree);
    ki_Mat mu, alpha;
    linear_solve(skel, quadtree, b.boundary_values, &mu, nh ? &alpha : nullptr);

    // the reference's one-call form on a fresh tree (its own tree/proxy
    // parameters are the reference defaults unless the problem is the same)
    QuadTree quadtree2;
    quadtree2.initialize_tree(&b, sd, dim);
    ki_Mat u = boundary_integral_solve(kernel, b, &quadtree2, hd[0], 4, kernel.domain_points);

    std::ofstream out(argv[2], std::ios::binary);
    out.write(reinterpret_cast<const char*>(mu.mat), sizeof(double) * mu.height());
    if (nh) out.write(reinterpret_cast<const char*>(alpha.mat), sizeof(double) * alpha.height());
    out.write(reinterpret_cast<const char*>(u.mat), sizeof(double) * u.height());

    // perturbation frames on the first tree (the boundaries outlive its use)
    int n_frames = 0;
    in.read(reinterpret_cast<char*>(&n_frames), sizeof(int));
    if (!in) n_frames = 0;
    std::vector<std::unique_ptr<ArrayBoundary>> frames;
    for (int fr = 0; fr < n_frames; fr++) {
      frames.emplace_back(new ArrayBoundary(b));
      ArrayBoundary& bf = *frames.back();
      bf.points = take<double>(in, (size_t)dim * n);
      const std::vector<double> c = take<double>(in, (size_t)dim * nh);
      for (int q = 0; q < nh; q++)
        bf.holes[q].center = PointVec(std::vector<double>(c.begin() + q * dim, c.begin() + (q + 1) * dim));
      quadtree.perturb(bf);
      Kernel kf(sd, dim, sd == 1 ? Kernel::LAPLACE : Kernel::STOKES, &bf, targets);
      skel.skeletonize(kf, &quadtree);
      ki_Mat muf, alf;
      linear_solve(skel, quadtree, bf.boundary_values, &muf, nh ? &alf : nullptr);
      out.write(reinterpret_cast<const char*>(muf.mat), sizeof(double) * muf.height());
      if (nh) out.write(reinterpret_cast<const char*>(alf.mat), sizeof(double) * alf.height());
    }
    return 0;
  } catch (const std::exception& e) {
    std::cerr << "facade_driver: " << e.what() << "\n";
    return 3;
  }
}
