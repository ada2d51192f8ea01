#include "ki_pool.h"
#include "ki_launch.cuh"

#include <cstdint>
#include <mutex>

namespace ki {

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_pool_mutex;
cudaMemPool_t g_pool[kMaxDevices] = {};

cudaError_t pool_for_current_device(cudaMemPool_t* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_pool_mutex);
  if (!g_pool[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    e = cudaMemPoolCreate(&pool, &props);
    if (e != cudaSuccess) return e;
    uint64_t keep = UINT64_MAX;
    e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    if (e != cudaSuccess) {
      cudaMemPoolDestroy(pool);
      return e;
    }
    g_pool[dev] = pool;
  }
  *out = g_pool[dev];
  return cudaSuccess;
}

}  // namespace

std::atomic<long long>& launch_counter() {
  static std::atomic<long long> count(0);
  return count;
}

cudaError_t pool_malloc(void** p, size_t bytes, cudaStream_t s) {
  cudaMemPool_t pool = nullptr;
  cudaError_t e = pool_for_current_device(&pool);
  if (e != cudaSuccess) return e;
  return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

cudaError_t pool_trim() {
  std::lock_guard<std::mutex> lock(g_pool_mutex);
  for (int d = 0; d < kMaxDevices; d++)
    if (g_pool[d]) {
      cudaError_t e = cudaMemPoolTrimTo(g_pool[d], 0);
      if (e != cudaSuccess) return e;
    }
  return cudaSuccess;
}

}  // namespace ki
