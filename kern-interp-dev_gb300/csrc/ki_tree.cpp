#include "ki_tree.h"

#include <algorithm>
#include <cmath>
#include <stdexcept>

namespace ki {

namespace {

// Touching test of the reference's get_descendent_neighbors
// (kern_interp/quadtree/quadtree.cpp:292-314): |dc_d| <= (s_a + s_b)/2 + 1e-9.
bool touching(const Box& a, const Box& b) {
  double pred = (a.side + b.side) / 2.;
  return !(std::fabs(a.cx - b.cx) - pred > 1e-9) && !(std::fabs(a.cy - b.cy) - pred > 1e-9);
}

}  // namespace

void Tree::build(const double* pts, int n_points_, int sol_dim_, int max_leaf_dofs_) {
  n_points = n_points_;
  sol_dim = sol_dim_;
  n_dofs = n_points * sol_dim;
  max_leaf_dofs = max_leaf_dofs_;
  if (n_points <= 0) throw std::invalid_argument("no boundary points");
  if (max_leaf_dofs < 1) throw std::invalid_argument("max_leaf_dofs must be positive");
  boxes.clear();
  levels.clear();

  double mn = pts[0], mx = pts[0];
  for (int i = 0; i < 2 * n_points; i++) {
    if (!std::isfinite(pts[i])) throw std::invalid_argument("non-finite boundary coordinate");
    mn = std::min(mn, pts[i]);
    mx = std::max(mx, pts[i]);
  }
  double tmin = mn - 0.01, tmax = mx + 0.01;

  // Top-down construction.  Each box owns a range [lo, hi) of `work`, a
  // permutation of point indices kept ascending within every box (stable
  // partition), so a leaf's DOFs are ascending like the reference's
  // original_box.
  std::vector<int> work(n_points), tmp(n_points);
  for (int i = 0; i < n_points; i++) work[i] = i;
  struct Range { int lo, hi; };
  std::vector<Range> range;

  Box root;
  root.level = 0;
  root.cx = root.cy = (tmin + tmax) / 2.0;
  root.side = tmax - tmin;
  root.orig_count = n_dofs;
  boxes.push_back(root);
  range.push_back({0, n_points});
  levels.push_back({0});

  for (size_t l = 0; l < levels.size(); l++) {
    std::vector<int> next;
    for (int b : levels[l]) {
      if (boxes[b].orig_count <= max_leaf_dofs) continue;
      boxes[b].leaf = false;
      Range r = range[b];
      double cx = boxes[b].cx, cy = boxes[b].cy, side = boxes[b].side;
      int cnt[4] = {0, 0, 0, 0};
      for (int i = r.lo; i < r.hi; i++) {
        int p = work[i];
        int ci = (pts[2 * p] >= cx ? 2 : 0) + (pts[2 * p + 1] >= cy ? 1 : 0);
        cnt[ci]++;
      }
      int start[4];
      start[0] = r.lo;
      for (int c = 1; c < 4; c++) start[c] = start[c - 1] + cnt[c - 1];
      int pos[4] = {start[0], start[1], start[2], start[3]};
      for (int i = r.lo; i < r.hi; i++) {
        int p = work[i];
        int ci = (pts[2 * p] >= cx ? 2 : 0) + (pts[2 * p + 1] >= cy ? 1 : 0);
        tmp[pos[ci]++] = p;
      }
      std::copy(tmp.begin() + r.lo, tmp.begin() + r.hi, work.begin() + r.lo);
      for (int ci = 0; ci < 4; ci++) {
        Box ch;
        ch.level = (int)l + 1;
        ch.parent = b;
        // child centre exactly as QuadTree::node_subdivide (quadtree.cpp:377-388)
        ch.cx = cx + ((ci & 2) ? side / 4. : -side / 4.);
        ch.cy = cy + ((ci & 1) ? side / 4. : -side / 4.);
        ch.side = side / 2.0;
        ch.orig_count = cnt[ci] * sol_dim;
        int id = (int)boxes.size();
        boxes.push_back(ch);
        range.push_back({start[ci], start[ci] + cnt[ci]});
        boxes[b].child[ci] = id;
        next.push_back(id);
      }
    }
    if (!next.empty()) levels.push_back(next);
  }

  // Leaf DOF ranges in depth-first order.
  dof_sorted.clear();
  dof_sorted.reserve(n_dofs);
  std::vector<int> stack = {0};
  while (!stack.empty()) {
    int b = stack.back();
    stack.pop_back();
    Box& bx = boxes[b];
    if (bx.leaf) {
      bx.orig_start = (int)dof_sorted.size();
      for (int i = range[b].lo; i < range[b].hi; i++)
        for (int s = 0; s < sol_dim; s++) dof_sorted.push_back(work[i] * sol_dim + s);
    } else {
      for (int ci = 3; ci >= 0; ci--) stack.push_back(bx.child[ci]);
    }
  }

  // Levels in depth-first order (children of consecutive parents stay
  // consecutive, matching the BFS construction above), positions.
  for (auto& lv : levels)
    for (size_t i = 0; i < lv.size(); i++) boxes[lv[i]].level_pos = (int)i;

  // Neighbours (quadtree.cpp:192-237): same-level touching boxes come from the
  // parent's same-level neighbours' children; a box's coarser touching leaves
  // are found among the parent's coarser leaves and the parent's same-level
  // neighbours that are leaves.
  for (size_t l = 1; l < levels.size(); l++) {
    for (int b : levels[l]) {
      Box& bx = boxes[b];
      const Box& par = boxes[bx.parent];
      for (int ci = 0; ci < 4; ci++)
        if (par.child[ci] != b) bx.same_nbrs.push_back(par.child[ci]);
      for (int pn : par.same_nbrs) {
        const Box& pb = boxes[pn];
        if (pb.leaf) {
          if (touching(bx, pb)) bx.coarse_nbrs.push_back(pn);
          continue;
        }
        for (int ci = 0; ci < 4; ci++) {
          const Box& cb = boxes[pb.child[ci]];
          double dx = bx.cx - cb.cx, dy = bx.cy - cb.cy;
          if (std::sqrt(dx * dx + dy * dy) < bx.side * std::sqrt(2.0) + 1e-9)
            bx.same_nbrs.push_back(pb.child[ci]);
        }
      }
      for (int pn : par.coarse_nbrs)
        if (touching(bx, boxes[pn])) bx.coarse_nbrs.push_back(pn);
    }
  }
}

}  // namespace ki
