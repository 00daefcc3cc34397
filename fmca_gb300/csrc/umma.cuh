// Fifth-generation tensor core (tcgen05) and tensor-memory helpers for
// sm_103a, as inline PTX.
//
// Conventions used by the kernels of this library:
//   * one CTA (cta_group::1), kind::f16 with FP16 A and B and FP32 D;
//   * D (M = 128 rows x N columns, FP32) lives in tensor memory: row m in
//     lane m, column n in 32-bit column n;
//   * A (M = 128 x K = 16, FP16) lives in tensor memory: row m in lane m,
//     elements k = 2j (low half) and 2j + 1 (high half) in column j;
//   * B (N x K = 16, FP16, K-major) lives in shared memory as core matrices
//     of 8 rows (n) x 16 bytes (8 consecutive k), stored contiguously
//     (128 B); core matrices adjacent in n are SBO bytes apart, those
//     adjacent in k LBO bytes apart (no swizzle).
// A warp may access only its lane quarter of tensor memory: lanes
// 32 (warp % 4) .. 32 (warp % 4) + 31.
#pragma once

#include <stdint.h>

namespace fmca {
namespace gpu {

__device__ __forceinline__ uint32_t umma_smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// allocation of ncols (power of two, 32..512) tensor-memory columns by one
// whole warp; the base address is written to *dst (shared memory)
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   umma_smem_u32(dst)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr),
               "r"(ncols)
               : "memory");
}

// ordering of tcgen05 operations around thread synchronisation
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// instruction descriptor of kind::f16: FP16 A and B, both K-major, FP32 D,
// M x N (bits 4-5 D type, 7-9 / 10-12 A / B type, 15 / 16 majors,
// 17-22 N >> 3, 24-28 M >> 4)
__host__ __device__ constexpr uint32_t umma_idesc_f16(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// shared-memory matrix descriptor without swizzle: start address, LBO
// (k direction) and SBO (n direction) in bytes, all multiples of 16;
// bits 46-48 hold the fixed value 0b001
__device__ __forceinline__ uint64_t umma_desc(const void* p, uint32_t lbo, uint32_t sbo) {
  const uint32_t a = umma_smem_u32(p);
  return (uint64_t)((a & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// D[d] = A[a] * B (+ D[d] if accumulate), A in tensor memory; issued by one
// thread, completes asynchronously (track with umma_commit)
__device__ __forceinline__ void umma_f16_ts(uint32_t d, uint32_t a, uint64_t bdesc,
                                            uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}" ::"r"(d),
      "r"(a), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// the mbarrier receives one arrival when all tcgen05.mma operations issued
// so far by this thread have completed
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          umma_smem_u32(bar))
      : "memory");
}

// 8 consecutive 32-bit columns of this thread's lane (taddr: lane quarter
// base in bits 16-31, first column in bits 0-15)
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t* v) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(
          taddr),
      "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
      : "memory");
}
// 16 consecutive columns of this warp's lanes: columns 0..7 from a, 8..15
// from b
__device__ __forceinline__ void tmem_st8x2(uint32_t taddr, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15, %16};" ::"r"(taddr),
      "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]),
      "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7])
      : "memory");
}
__device__ __forceinline__ void tmem_wait_st() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// 16 consecutive 32-bit columns of this thread's lane; the values are valid
// after tmem_wait_ld16 on the same array (which also keeps the compiler
// from reading them earlier)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* v) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, "
      "%10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
        "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr)
      : "memory");
}
__device__ __forceinline__ void tmem_wait_ld16(uint32_t* v) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]),
                 "+r"(v[6]), "+r"(v[7]), "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]),
                 "+r"(v[12]), "+r"(v[13]), "+r"(v[14]), "+r"(v[15])
               :
               : "memory");
}

}  // namespace gpu
}  // namespace fmca
