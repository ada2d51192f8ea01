// GPU part of the tree build (see ki_tree.h): every point's descent code
// and the stable sort of the points by it.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace ki {

// Descent codes of n points (device, interleaved dim per point) below the
// root box (centre on every axis, side) to `depth` levels -- at each level
// the child index of the reference's split rule (coordinate d >= centre
// adds 2^(dim-1-d)), the child centre c +- side/4 and side/2 as the host
// build computes them -- sorted ascending with ties in point order.
// Writes the sorted codes and point indices to host arrays of n entries.
// Stream-ordered; returns after the copies have completed.  Throws
// std::runtime_error on a CUDA error.
void tree_codes_sorted(const double* d_points, int n, int dim, double centre, double side,
                       int depth, uint64_t* h_codes, int* h_order, cudaStream_t s);

}  // namespace ki
