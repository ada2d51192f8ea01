// Blackwell (sm_103a) tensor-core primitives: tcgen05 MMA with TMEM
// accumulators, shared-memory matrix descriptors, mbarrier completion.
//
// Operand tiles live in shared memory in the canonical K-major layout without
// swizzling: the matrix is cut into core matrices of 8 rows x 16 bytes (8 x 4
// TF32 values), each stored as 128 contiguous bytes (row r of the core matrix
// at byte 16 r).  Core matrices adjacent along K are kLbo = 128 bytes apart,
// core matrices adjacent along M (or N) are `sbo` bytes apart.  One
// kind::tf32 MMA consumes K = 8 (two core matrices along K); the k-th step of
// a tile starts 256 k bytes after the tile.
//
// Accumulators: an M = 128 MMA (cta_group::1) writes row i of D to TMEM lane
// i and column j to TMEM column base + j (32-bit).  Warp w may read lanes
// 32 (w % 4) .. 32 (w % 4) + 31 only.
#pragma once

#include <cstdint>

namespace ki {
namespace tc {

constexpr uint32_t kLbo = 128;   // bytes between core matrices adjacent along K

// Byte offset of element (row, k) in a K-major tile whose 8-row groups are
// `sbo` bytes apart.
__host__ __device__ __forceinline__ uint32_t kmajor_offset(int row, int k, uint32_t sbo) {
  return (uint32_t)(row >> 3) * sbo + (uint32_t)(k >> 2) * kLbo + (uint32_t)(row & 7) * 16u +
         (uint32_t)(k & 3) * 4u;
}

// Start of core matrix (rb, kb): a warp writing it maps lane -> (row 8 rb +
// lane / 4, k 4 kb + lane % 4), i.e. byte 4 lane of the core matrix, so its
// 32 stores fill 128 contiguous bytes (no bank conflicts).
__device__ __forceinline__ uint32_t core_offset(int rb, int kb, uint32_t sbo) {
  return (uint32_t)rb * sbo + (uint32_t)kb * kLbo;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor (tcgen05): start address, leading byte
// offset (K direction), stride byte offset (M/N direction), descriptor
// version 1 (bit 46), no swizzle, base offset 0.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of a dense kind::tf32 MMA: D in FP32 (bits 4-5 = 1),
// A and B TF32 (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// Instruction descriptor of a dense kind::f16 MMA with BF16 operands: D in
// FP32 (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12 = 1), both K-major.
// One MMA consumes K = 16 BF16 values, again two core matrices of 16 bytes
// per row, so the tile layout and the 256-byte K steps are those of TF32.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// Byte offset of BF16 element (row, k) in a K-major tile whose 8-row groups
// are `sbo` bytes apart (core matrix: 8 rows x 8 values).
__host__ __device__ __forceinline__ uint32_t kmajor_offset_bf16(int row, int k, uint32_t sbo) {
  return (uint32_t)(row >> 3) * sbo + (uint32_t)(k >> 3) * kLbo + (uint32_t)(row & 7) * 16u +
         (uint32_t)(k & 7) * 2u;
}

// Round to the nearest TF32 value (ties away from zero), returned in an FP32
// container with the low 13 bits clear, so the tensor core reads it exactly.
__device__ __forceinline__ float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// ------------------------------------------------------------------ mbarrier
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits until the phase of parity `parity` has completed, for at most about
// `limit_cycles` SM clock cycles; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit_cycles) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > limit_cycles) return false;
  return true;
}

// ---------------------------------------------------------------- fences
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// ------------------------------------------------------------------- TMEM
// Allocation by one full warp: the TMEM address is written to *dst (shared).
// ncols: a power of two, 32 .. 512.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 32 lanes x 16 consecutive 32-bit columns: lane t of the warp receives
// TMEM lane (lane field of taddr) + t, columns col .. col + 15.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// --------------------------------------------------------------------- MMA
// D[tmem] (+)= A[smem] * B[smem]^T (both K-major), issued by one thread.
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// The same with BF16 operands (kind::f16).
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// Arrives on *bar once every MMA this thread issued before has completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

}  // namespace tc
}  // namespace ki
