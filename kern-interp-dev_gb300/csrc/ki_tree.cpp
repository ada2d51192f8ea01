#include "ki_tree.h"

#include "ki_parallel.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <stdexcept>
#include <thread>
#include <vector>

namespace ki {

namespace {

// Touching test of the reference's get_descendent_neighbors
// (kern_interp/quadtree/quadtree.cpp:292-314): |dc_d| <= (s_a + s_b)/2 + 1e-9
// in every coordinate.
bool touching(const Box& a, const Box& b, int dim) {
  double pred = (a.side + b.side) / 2.;
  for (int d = 0; d < dim; d++)
    if (std::fabs(a.c[d] - b.c[d]) - pred > 1e-9) return false;
  return true;
}

// Child index of a point (QuadTree::recursive_add / node_subdivide,
// quadtree.cpp:324-330, 398-405): coordinate d at or above the centre adds
// 2^(dim-1-d).
inline int child_of(const double* p, const double* c, int dim) {
  int ci = 0;
  for (int d = 0; d < dim; d++)
    if (p[d] >= c[d]) ci += 1 << (dim - 1 - d);
  return ci;
}

}  // namespace

void tree_root(const double* pts, int n_points, int dim, double* centre, double* side) {
  if (n_points <= 0) throw std::invalid_argument("no boundary points");
  // min and max over every coordinate, in parallel chunks (exact, so the
  // result does not depend on the split)
  const int n = dim * n_points;
  const int chunk = 1 << 16, nchunk = (n + chunk - 1) / chunk;
  std::vector<double> cmn(nchunk), cmx(nchunk);
  std::atomic<bool> bad(false);
  parallel_ranges(nchunk, [&](int c0, int c1) {
    for (int c = c0; c < c1; c++) {
      double mn = pts[(size_t)c * chunk], mx = mn;
      const int e = std::min(n, (c + 1) * chunk);
      for (int i = c * chunk; i < e; i++) {
        if (!std::isfinite(pts[i])) bad = true;
        mn = std::min(mn, pts[i]);
        mx = std::max(mx, pts[i]);
      }
      cmn[c] = mn;
      cmx[c] = mx;
    }
  }, 2);
  if (bad) throw std::invalid_argument("non-finite boundary coordinate");
  const double mn = *std::min_element(cmn.begin(), cmn.end());
  const double mx = *std::max_element(cmx.begin(), cmx.end());
  const double tmin = mn - 0.01, tmax = mx + 0.01;
  *centre = (tmin + tmax) / 2.0;
  *side = tmax - tmin;
}

namespace {

void check_args(int dim, int n_points, int max_leaf_dofs) {
  if (dim != 2 && dim != 3) throw std::invalid_argument("domain dimension must be 2 or 3");
  if (n_points <= 0) throw std::invalid_argument("no boundary points");
  if (max_leaf_dofs < 1) throw std::invalid_argument("max_leaf_dofs must be positive");
}

// Child ci of box b (centre exactly as QuadTree::node_subdivide,
// quadtree.cpp:377-388), appended to the box list.
int add_child(std::vector<Box>* boxes, int b, int ci, int level, int dim, int count) {
  const Box& par = (*boxes)[b];
  Box ch;
  ch.level = level;
  ch.parent = b;
  for (int d = 0; d < dim; d++)
    ch.c[d] = par.c[d] + ((ci >> (dim - 1 - d)) & 1 ? par.side / 4. : -par.side / 4.);
  ch.side = par.side / 2.0;
  ch.orig_count = count;
  const int id = (int)boxes->size();
  boxes->push_back(ch);
  (*boxes)[b].child[ci] = id;
  return id;
}

}  // namespace

void Tree::build(const double* pts, int n_points_, int dim_, int sol_dim_, int max_leaf_dofs_) {
  check_args(dim_, n_points_, max_leaf_dofs_);
  dim = dim_;
  n_points = n_points_;
  sol_dim = sol_dim_;
  n_dofs = n_points * sol_dim;
  max_leaf_dofs = max_leaf_dofs_;
  boxes.clear();
  levels.clear();
  const int nch = 1 << dim;
  double c0, side0;
  tree_root(pts, n_points, dim, &c0, &side0);

  // Top-down construction.  Each box owns a range [lo, hi) of `work`, a
  // permutation of point indices kept ascending within every box (stable
  // partition), so a leaf's DOFs are ascending like the reference's
  // original_box.
  std::vector<int> work(n_points), tmp(n_points);
  for (int i = 0; i < n_points; i++) work[i] = i;
  std::vector<std::pair<int, int>> range;

  Box root;
  root.level = 0;
  for (int d = 0; d < dim; d++) root.c[d] = c0;
  root.side = side0;
  root.orig_count = n_dofs;
  boxes.push_back(root);
  range.push_back({0, n_points});
  levels.push_back({0});

  for (size_t l = 0; l < levels.size(); l++) {
    std::vector<int> next;
    for (int b : levels[l]) {
      if (boxes[b].orig_count <= max_leaf_dofs) continue;
      boxes[b].leaf = false;
      const int lo = range[b].first, hi = range[b].second;
      double c[3] = {boxes[b].c[0], boxes[b].c[1], boxes[b].c[2]};
      int cnt[kMaxChildren] = {};
      for (int i = lo; i < hi; i++) cnt[child_of(pts + (size_t)dim * work[i], c, dim)]++;
      int start[kMaxChildren];
      start[0] = lo;
      for (int ci = 1; ci < nch; ci++) start[ci] = start[ci - 1] + cnt[ci - 1];
      int pos[kMaxChildren];
      for (int ci = 0; ci < nch; ci++) pos[ci] = start[ci];
      for (int i = lo; i < hi; i++) {
        int p = work[i];
        tmp[pos[child_of(pts + (size_t)dim * p, c, dim)]++] = p;
      }
      std::copy(tmp.begin() + lo, tmp.begin() + hi, work.begin() + lo);
      for (int ci = 0; ci < nch; ci++) {
        const int id = add_child(&boxes, b, ci, (int)l + 1, dim, cnt[ci] * sol_dim);
        range.push_back({start[ci], start[ci] + cnt[ci]});
        next.push_back(id);
      }
    }
    if (!next.empty()) levels.push_back(next);
  }
  finish(work, range);
}

void Tree::finish(const std::vector<int>& work, const std::vector<std::pair<int, int>>& range) {
  const int nch = 1 << dim;
  // Leaf DOF ranges in depth-first order.  Both builds keep `work` in that
  // order (children in child order inside their parent's range), so a leaf's
  // DOFs start at its range's first point: the list is `work` expanded by
  // the solution dimension, filled in parallel.
  dof_sorted.assign((size_t)n_dofs, 0);
  parallel_ranges(n_points, [&](int lo, int hi) {
    for (int i = lo; i < hi; i++)
      for (int s = 0; s < sol_dim; s++) dof_sorted[(size_t)i * sol_dim + s] = work[i] * sol_dim + s;
  });
  parallel_ranges((int)boxes.size(), [&](int b0, int b1) {
    for (int b = b0; b < b1; b++)
      if (boxes[b].leaf) boxes[b].orig_start = range[b].first * sol_dim;
  });

  // Levels in depth-first order (children of consecutive parents stay
  // consecutive, matching the BFS construction above), positions.
  for (auto& lv : levels)
    for (size_t i = 0; i < lv.size(); i++) boxes[lv[i]].level_pos = (int)i;

  // Neighbours (quadtree.cpp:192-237): same-level neighbours come from the
  // parent's same-level neighbours' children (centre distance below
  // side*sqrt(dim)); a box's coarser touching leaves are found among the
  // parent's coarser leaves and the parent's same-level neighbours that are
  // leaves.  Flat storage, tree_nbr_cap(dim) slots per box.
  const int cap = tree_nbr_cap(dim);
  nbr_same.assign(boxes.size() * (size_t)cap, -1);
  nbr_coarse.assign(boxes.size() * (size_t)cap, -1);
  n_same.assign(boxes.size(), 0);
  n_coarse.assign(boxes.size(), 0);
  const double sq = std::sqrt((double)dim);
  std::atomic<bool> overflow(false);
  for (size_t l = 1; l < levels.size(); l++) {
    const std::vector<int>& lv = levels[l];
    parallel_ranges((int)lv.size(), [&](int i0, int i1) {
    for (int i = i0; i < i1; i++) {
      const int b = lv[i];
      const Box& bx = boxes[b];
      const Box& par = boxes[bx.parent];
      int* same = nbr_same.data() + (size_t)b * cap;
      int* coarse = nbr_coarse.data() + (size_t)b * cap;
      int ns = 0, nc = 0;
      auto push = [&](int* list, int* cnt, int v) {
        if (*cnt < cap) list[(*cnt)++] = v;
        else overflow = true;
      };
      for (int ci = 0; ci < nch; ci++)
        if (par.child[ci] != b) push(same, &ns, par.child[ci]);
      for (int pn : same_nbrs(bx.parent)) {
        const Box& pb = boxes[pn];
        if (pb.leaf) {
          if (touching(bx, pb, dim)) push(coarse, &nc, pn);
          continue;
        }
        for (int ci = 0; ci < nch; ci++) {
          const Box& cb = boxes[pb.child[ci]];
          double d2 = 0;
          for (int d = 0; d < dim; d++) d2 += (bx.c[d] - cb.c[d]) * (bx.c[d] - cb.c[d]);
          if (std::sqrt(d2) < bx.side * sq + 1e-9) push(same, &ns, pb.child[ci]);
        }
      }
      for (int pn : coarse_nbrs(bx.parent))
        if (touching(bx, boxes[pn], dim)) push(coarse, &nc, pn);
      n_same[b] = ns;
      n_coarse[b] = nc;
    }
    });
  }
  if (overflow) throw std::logic_error("tree: more neighbours than 3^dim - 1");
}

}  // namespace ki
