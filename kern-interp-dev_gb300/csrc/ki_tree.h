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
};

// A box's neighbour list: a view into the tree's flat storage.
struct IdList {
  const int* p = nullptr;
  int n = 0;
  const int* begin() const { return p; }
  const int* end() const { return p + n; }
  int size() const { return n; }
};

// Neighbours per box are bounded by the 3^dim - 1 cells around it: the
// same-level ones within side*sqrt(dim), and the touching coarser leaves
// (each larger than the box, so one per direction).
inline int tree_nbr_cap(int dim) { return dim == 2 ? 8 : 26; }

struct Tree {
  int dim = 2, n_points = 0, sol_dim = 1, n_dofs = 0;
  int max_leaf_dofs = 64;
  std::vector<Box> boxes;
  std::vector<std::vector<int>> levels;   // box ids per level, Morton order
  std::vector<int> dof_sorted;            // leaves' DOFs, leaf after leaf
  // neighbour lists, tree_nbr_cap(dim) slots per box: same-level
  // neighbours and touching leaves of coarser levels, with their counts
  std::vector<int> nbr_same, nbr_coarse;
  std::vector<int> n_same, n_coarse;

  int n_children() const { return 1 << dim; }
  // neighbouring boxes of the same level
  IdList same_nbrs(int b) const {
    return IdList{nbr_same.data() + (size_t)b * tree_nbr_cap(dim), n_same[b]};
  }
  // touching leaves of coarser levels
  IdList coarse_nbrs(int b) const {
    return IdList{nbr_coarse.data() + (size_t)b * tree_nbr_cap(dim), n_coarse[b]};
  }
  // points: interleaved (x, y[, z]), n_points of them; dim 2 or 3.
  void build(const double* points, int n_points, int dim, int sol_dim, int max_leaf_dofs);
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
