// GPU part of the tree build (see ki_tree.h): every point's descent code
// and the stable sort of the points by it.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace ki {

struct Tree;

// The whole tree on the GPU (the host Tree::build's boxes, numbering, leaf
// DOF lists and neighbour lists, bit for bit): every point's descent code
// below the root box (centre on every axis, side) to `depth` levels -- at
// each level the child index of the reference's split rule, the child centre
// c +- side/4 and side/2 as the host build computes them -- a stable radix
// sort of the points by it, then level by level the boxes that split (more
// than max_leaf_dofs DOFs) cut by binary search on the level's digit, the
// neighbour lists from the parents' (host order), each leaf's points
// ascending by index; one copy of the result into *tree.  Returns false
// when a box at level `depth` would still split, a leaf holds more than
// 1,024 points, or a neighbour list overflows: the caller then builds by
// partition on the host (Tree::build, which rewrites every field).  Stream-ordered; returns after the
// copies have completed.  Throws std::runtime_error on a CUDA error.
bool tree_build_gpu(const double* d_points, int n, int dim, int sol_dim, int max_leaf_dofs,
                    double centre, double side, int depth, Tree* tree, cudaStream_t s);

}  // namespace ki
