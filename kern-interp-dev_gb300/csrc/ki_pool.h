// Stream-ordered device allocation from the library's own memory pool.
//
// One pool per device, created on first use, that keeps the memory freed
// into it for reuse (release threshold: unlimited).  Repeated
// factorizations and solves of similar sizes then reuse the same physical
// pages instead of mapping fresh memory after every synchronization, which
// the device's default pool (release threshold 0) would do.  The default
// pool of the process is left untouched; pool_trim() hands the cached memory
// back.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace ki {

cudaError_t pool_malloc(void** p, size_t bytes, cudaStream_t s);

// Release the cached (currently unused) memory of every device's pool.
cudaError_t pool_trim();

}  // namespace ki
