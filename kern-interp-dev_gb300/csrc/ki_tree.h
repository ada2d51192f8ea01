// Host-side adaptive quadtree over the boundary nodes.
//
// Restates the tree of the reference's QuadTree (kern_interp/quadtree/
// quadtree.cpp): the same root box (bounding square of all coordinates
// +-0.01, :240-267), the same split rule (a box is subdivided while it holds
// more than max_leaf_dofs DOFs, :336-339 / :409-411), the same child
// numbering (x >= centre adds 2, y >= centre adds 1, :324-330) and the same
// neighbour relation (every touching box of the same level plus, for the
// "near" set, touching leaves of coarser levels, :192-237 / :292-314).
//
// The layout differs on purpose: the tree is built top-down by stable
// partition instead of point-by-point insertion, boxes of a level are kept in
// depth-first (Morton) order, and every leaf's DOFs form one contiguous range
// of `dof_sorted` (ascending DOF index within a leaf, as the reference's
// original_box lists are).  The device code only ever sees these flat arrays.
#pragma once

#include <cstdint>
#include <vector>

namespace ki {

struct Box {
  int level = 0;
  int parent = -1;
  int child[4] = {-1, -1, -1, -1};
  bool leaf = true;
  double cx = 0, cy = 0, side = 0;
  int orig_start = 0;   // leaf DOF range in dof_sorted (leaves only)
  int orig_count = 0;   // DOFs in the box (all boxes)
  int level_pos = 0;    // index within levels[level]
  std::vector<int> same_nbrs;    // touching boxes of the same level
  std::vector<int> coarse_nbrs;  // touching leaves of coarser levels
};

struct Tree {
  int n_points = 0, sol_dim = 1, n_dofs = 0;
  int max_leaf_dofs = 64;
  std::vector<Box> boxes;
  std::vector<std::vector<int>> levels;   // box ids per level, Morton order
  std::vector<int> dof_sorted;            // leaves' DOFs, leaf after leaf

  // points: interleaved (x, y), n_points of them.
  void build(const double* points, int n_points, int sol_dim, int max_leaf_dofs);
  int num_levels() const { return (int)levels.size(); }
};

}  // namespace ki
