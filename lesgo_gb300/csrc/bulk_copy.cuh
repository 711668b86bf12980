// Bulk global->shared copies through the tensor memory accelerator (the
// untiled cp.async.bulk form) completing on a shared-memory mbarrier, with
// waits that give up after a bounded number of polls.
//
// Rules the callers keep: source, destination and size are multiples of 16
// bytes; one thread arms the barrier with the byte count of the copies of a
// phase (arrive.expect_tx) and issues them; every thread waits on the
// phase's parity.  A wait that runs out of polls reports false, and the
// kernel records the failure in a device flag and returns instead of
// spinning on.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace lesgo {

constexpr unsigned kMbarPollLimit = 1u << 22;

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes initialised barriers visible to the async proxy that the copies
// complete on (then a block barrier makes them visible to the threads).
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// bytes from global `src` to shared `dst`, completing on `bar`
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Polls until the phase with parity `parity` of `bar` has completed; false
// after kMbarPollLimit polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
  const unsigned a = smem_addr(bar);
  for (unsigned it = 0; it < kMbarPollLimit; ++it) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

}  // namespace lesgo
