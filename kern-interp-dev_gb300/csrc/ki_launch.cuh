// Kernel launches through one helper, so that the library can report how
// many kernels it has launched (ki_launch_count).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <utility>

namespace ki {

// Kernels launched by this library since it was loaded.
std::atomic<long long>& launch_counter();

// kernel<<<grid, block, smem, stream>>>(args...), counted.
template <typename... P, typename... A>
inline void launch(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                   A&&... args) {
  launch_counter().fetch_add(1, std::memory_order_relaxed);
  kernel<<<grid, block, smem, stream>>>(std::forward<A>(args)...);
}

}  // namespace ki
