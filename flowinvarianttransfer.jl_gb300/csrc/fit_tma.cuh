// Bulk asynchronous copies (the TMA engine's non-tensor form) and mbarrier helpers, inline PTX.
//
// A copy global -> shared is issued by one thread: mbarrier.arrive.expect_tx announces the byte
// count, cp.async.bulk moves the bytes and completes them on the mbarrier. Every waiter polls
// mbarrier.try_wait.parity with a clock-bounded loop: a wait that does not finish within the
// bound reports failure instead of spinning forever, and the caller aborts the block uniformly
// (all threads reach the same __syncthreads_or) and records an error the host reads back.
#pragma once

#include <stdint.h>

#include "fit_common.cuh"

namespace fit {

FIT_D uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

FIT_D void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

FIT_D void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Order earlier generic-proxy accesses of shared memory before later async-proxy writes.
FIT_D void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

FIT_D void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// dst and src 16-byte aligned, bytes a multiple of 16.
FIT_D void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

FIT_D bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Non-blocking probe of phase `parity` (mbarrier.test_wait never suspends the thread).
FIT_D bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait on phase `parity`: false after max_cycles SM clocks (about 1 s at 2 GHz for the
// default FIT_WAIT_CYCLES). try_wait may suspend the thread for a while inside one probe, so a
// bound below FIT_WAIT_POLL_MIN cycles polls with the non-blocking test_wait instead: such a
// short bound then runs out whenever the phase is still pending at the first probes.
FIT_D bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, long long max_cycles) {
  const long long t0 = clock64();
  if (max_cycles < FIT_WAIT_POLL_MIN) {
    while (!mbar_test_wait(bar, parity)) {
      if (clock64() - t0 > max_cycles) return false;
    }
    return true;
  }
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > max_cycles) return false;
  }
  return true;
}

// Wait whose bound `lim` may run out: a wait that gives up marks `failed` (the launch's result is
// then discarded by the host) and waits again on the same phase with the full bound, so that the
// barrier's phases stay in step with the copies or tensor-core commits already issued. Returns
// false only when that second wait gives up as well.
FIT_D bool mbar_wait_or_flag(uint64_t* bar, uint32_t parity, long long lim, bool& failed) {
  if (mbar_wait_bounded(bar, parity, lim)) return true;
  failed = true;
  return mbar_wait_bounded(bar, parity, FIT_WAIT_CYCLES);
}

}  // namespace fit
