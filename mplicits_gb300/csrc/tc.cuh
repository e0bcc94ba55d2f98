// tcgen05 (5th-generation tensor core) and TMEM primitives for sm_103a,
// written as inline PTX.  Only what the level kernels use: cta_group::1,
// kind::f16 with BF16 operands from shared memory, FP32 accumulators in
// tensor memory, no swizzle (K-major core-matrix tiles).
#pragma once

#include <stdint.h>

namespace mpl {
namespace tc {

// Shared-memory matrix descriptor (64 bit) for a K-major operand tiled in
// 8-row x 16-byte core matrices without swizzle:
//   bits  0-13  start address >> 4
//   bits 16-29  leading-dimension byte offset >> 4 (next core matrix along K)
//   bits 32-45  stride-dimension byte offset >> 4 (next 8-row group along M/N)
//   bits 46-47  descriptor version (1 on sm_100 family)
//   bits 61-63  layout (0: no swizzle)
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= 1ull << 46;
  return d;
}

// Instruction descriptor of kind::f16 with FP32 accumulation, A and B of the
// same 16-bit type (fmt 1: bf16, 0: f16), both K-major:
//   bits 4-5 D format (1: f32), 7-9 A format, 10-12 B format, 15/16 A/B
//   major (0: K), 17-22 N >> 3, 24-28 M >> 4.
__host__ __device__ constexpr uint32_t idesc_f16kind_f32(int M, int N, uint32_t fmt) {
  return (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// The same with either operand MN-major (bit 15: A, bit 16: B).  An
// MN-major operand without swizzle is tiled in core matrices of 8 K-rows x
// 16 bytes (8 consecutive M/N elements per row); in its descriptor the
// leading-dimension offset steps along K and the stride offset along M/N.
__host__ __device__ constexpr uint32_t idesc_f16kind_f32_major(int M, int N, uint32_t fmt,
                                                               bool a_mn, bool b_mn) {
  return idesc_f16kind_f32(M, N, fmt) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16);
}

__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return idesc_f16kind_f32(M, N, 1u);
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}

// Arrive (once) on an mbarrier when every MMA issued so far by this thread
// has completed.
__device__ __forceinline__ void commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          (uint32_t)__cvta_generic_to_shared(bar))
      : "memory");
}

// 32 lanes x 32 consecutive 32-bit columns: lane i of the warp receives
// row (lane base + i), columns col..col+31.
__device__ __forceinline__ void ld_32x32b_x32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr)
      : "memory");
}

// 32 lanes x 16 consecutive 32-bit columns.
__device__ __forceinline__ void ld_32x32b_x16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
}

template <int U>
__device__ __forceinline__ void ld_32x32b(uint32_t taddr, uint32_t (&r)[U]);
template <>
__device__ __forceinline__ void ld_32x32b<16>(uint32_t taddr, uint32_t (&r)[16]) {
  ld_32x32b_x16(taddr, r);
}
template <>
__device__ __forceinline__ void ld_32x32b<32>(uint32_t taddr, uint32_t (&r)[32]) {
  ld_32x32b_x32(taddr, r);
}

__device__ __forceinline__ void wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

}  // namespace tc
}  // namespace mpl
