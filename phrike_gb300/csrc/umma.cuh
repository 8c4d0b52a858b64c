// 5th-generation tensor core (tcgen05) building blocks for sm_100-family
// GPUs: tensor-memory (TMEM) allocation, shared-memory matrix descriptors,
// the bf16 MMA with float32 accumulation in TMEM, commit-to-mbarrier and
// TMEM loads.  Inline PTX only; the layouts follow the PTX ISA's tcgen05
// "shared memory descriptor" and "instruction descriptor" formats.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "tma.cuh"

namespace ps {

// TMEM: `ncols` 32-bit columns x 128 lanes; the base address is written to
// shared memory at `dst`.  Executed by one full warp.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory descriptor of a K-major operand tile stored in the 128-byte
// swizzle layout that a TMA load with CU_TENSOR_MAP_SWIZZLE_128B writes: rows
// of 64 bf16 (128 bytes), 8-row groups 1024 bytes apart (stride byte offset),
// the tile base 1024-byte aligned.  Advancing along K inside the 128-byte
// row is done by adding the byte offset to the start address.
__device__ __forceinline__ uint64_t sw128_kmajor_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address >> 4      (bits 0-13)
  d |= (uint64_t)1 << 16;                     // leading byte offset 16 B (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;           // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;                     // descriptor version (sm_100 family)
  d |= (uint64_t)2 << 61;                     // layout: 128-byte swizzle
  return d;
}

// Instruction descriptor of kind::f16 with bf16 A and B (both K-major) and
// a float32 accumulator, shape M x N.
__host__ __device__ constexpr uint32_t bf16_idesc(int M, int N) {
  return (1u << 4)                        // D format: f32
         | (1u << 7)                      // A format: bf16
         | (1u << 10)                     // B format: bf16
         | ((uint32_t)(N >> 3) << 17)     // N >> 3
         | ((uint32_t)(M >> 4) << 24);    // M >> 4
}

// D (TMEM) = A * B^T (+ D if accumulate), issued by one thread.
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive on `bar` once all tcgen05 operations issued so far by this thread
// have completed.
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_addr(bar))
               : "memory");
}

// 16 consecutive float32 columns of this thread's TMEM lane (warp w reads
// lanes 32w..32w+31; taddr carries the lane base in its upper 16 bits).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace ps
