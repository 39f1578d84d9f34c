// Fifth-generation tensor cores (tcgen05) from inline PTX: tensor-memory allocation, the
// single-thread MMA issue with shared-memory operand descriptors, completion through an mbarrier,
// and accumulator reads from tensor memory.
//
// Operands use the no-swizzle K-major canonical layout: an R x K BF16 tile is a grid of 8-row x
// 16-byte core matrices, element (r, k) at byte
//     (r % 8) * 16 + (r / 8) * SBO + (k % 8) * 2 + (k / 8) * LBO,
// with LBO = 128 (core matrices adjacent along K) and SBO = (K / 8) * 128 (adjacent 8-row groups).
// A K = 16 step of the MMA advances both descriptors' start addresses by 2 * LBO = 256 bytes.
#pragma once

#include <stdint.h>

#include "fit_tma.cuh"

namespace fit {

// Byte offset of element (r, k) in the canonical layout of a tile with K columns.
FIT_D uint32_t umma_off(int r, int k, int K) {
  return (uint32_t)((r & 7) * 16 + (r >> 3) * (K / 8) * 128 + (k & 7) * 2 + (k >> 3) * 128);
}

// Shared-memory matrix descriptor: start address, leading / stride byte offsets (16-byte units),
// descriptor version 1 (bits 46-47), base offset 0, layout type 0 (no swizzle, bits 61-63).
FIT_D uint64_t umma_desc(uint32_t smem_addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((smem_addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A and B (bits 7-9 and
// 10-12 = 1), both K-major (bits 15, 16 = 0), N / 8 at bits 17-22, M / 16 at bits 24-28.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Tensor-memory allocation of ncols columns (a power of two >= 32) by one whole warp; the base
// address is written to *dst in shared memory.
FIT_D void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
               : "memory");
}
FIT_D void tmem_relinquish() { asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory"); }
FIT_D void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

FIT_D void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
FIT_D void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, one M x N x 16 step (issued by one thread).
FIT_D void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}

// One arrival on the mbarrier once every MMA this thread issued before has completed.
FIT_D void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 16 consecutive FP32 columns of this thread's tensor-memory lane (warp w reads lanes 32w..32w+31:
// taddr carries the warp's lane base in its upper half), waited for in the same statement.
FIT_D void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace fit
