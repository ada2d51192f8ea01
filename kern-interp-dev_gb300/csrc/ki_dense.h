// Dense LU (partial pivoting) and solves on the GPU, column-major, ld = n.
#pragma once

#include <cuda_runtime.h>

namespace ki {

// In-place LU of A (n x n); piv[i] = row swapped with row i (0-based);
// a zero pivot sets *err to 2 (device word).
template <typename T>
void dense_lu(T* A, int n, int* piv, int* err, cudaStream_t s);

// B (n x nrhs, ldb) <- A^-1 B, or A^-T B when trans.
template <typename T>
void dense_lu_solve(const T* LU, int n, const int* piv, T* B, int ldb, int nrhs, bool trans,
                    cudaStream_t s);

}  // namespace ki
