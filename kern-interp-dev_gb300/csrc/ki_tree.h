// Host-side adaptive quadtree (2D) / octree (3D) over the boundary nodes.
//
// Restates the tree of the reference's QuadTree (kern_interp/quadtree/
// quadtree.cpp): the same root box (bounding square/cube of all coordinates
// +-0.01, :240-267), the same split rule (a box is subdivided while it holds
// more than max_leaf_dofs DOFs, :336-339 / :409-411), the same child
// numbering (coordinate d >= centre adds 2^(dim-1-d), :324-330 / :378-388)
// and the same neighbour relation (every box of the same level whose centre
// lies within side*sqrt(dim), plus, for the "near" set, touching leaves of
// coarser levels, :192-237 / :292-314).
//
// The layout differs on purpose: the tree is built top-down by stable
// partition instead of point-by-point insertion, boxes of a level are kept in
// depth-first (Morton) order, and every leaf's DOFs form one contiguous range
// of `dof_sorted` (ascending DOF index within a leaf, as the reference's
// original_box lists are).  The device code only ever sees these flat arrays.
#pragma once

#include <cstdint>
#include <utility>
#include <vector>

namespace ki {

constexpr int kMaxChildren = 8;

struct Box {
  int level = 0;
  int parent = -1;
  int child[kMaxChildren] = {-1, -1, -1, -1, -1, -1, -1, -1};
  bool leaf = true;
  double c[3] = {0, 0, 0};   // centre
  double side = 0;
  int orig_start = 0;   // leaf DOF range in dof_sorted (leaves only)
  int orig_count = 0;   // DOFs in the box (all boxes)
  int level_pos = 0;    // index within levels[level]
  std::vector<int> same_nbrs;    // neighbouring boxes of the same level
  std::vector<int> coarse_nbrs;  // touching leaves of coarser levels
};

struct Tree {
  int dim = 2, n_points = 0, sol_dim = 1, n_dofs = 0;
  int max_leaf_dofs = 64;
  std::vector<Box> boxes;
  std::vector<std::vector<int>> levels;   // box ids per level, Morton order
  std::vector<int> dof_sorted;            // leaves' DOFs, leaf after leaf

  int n_children() const { return 1 << dim; }
  // points: interleaved (x, y[, z]), n_points of them; dim 2 or 3.
  void build(const double* points, int n_points, int dim, int sol_dim, int max_leaf_dofs);
  // The same tree from the points' descent codes: code = the child indices
  // of the boxes containing the point at levels 1..depth, dim bits each,
  // level 1 most significant (computed with tree_root's box and the split
  // rule's centre arithmetic), sorted ascending with ties by point index,
  // `order` the point indices in that order.  Returns false (tree left
  // empty) when a box at level `depth` would still be split.
  // centre / side: the root box tree_root gave for these points.
  bool build_from_codes(int n_points, int dim, int sol_dim, int max_leaf_dofs,
                        const uint64_t* codes, const int* order, int depth, double centre,
                        double side);
  int num_levels() const { return (int)levels.size(); }

 private:
  void finish(const std::vector<int>& work, const std::vector<std::pair<int, int>>& range);
};

// Root box of the points: centre (all coordinates equal) and side, the
// bounding interval of every coordinate widened by 0.01 on both ends.
// Throws std::invalid_argument on a non-finite coordinate or no points.
void tree_root(const double* points, int n_points, int dim, double* centre, double* side);

// Deepest descent code the 64-bit codes hold: 30 levels in 2D, 21 in 3D.
inline int tree_code_depth(int dim) { return dim == 2 ? 30 : 21; }

}  // namespace ki
