// Asynchronous global -> shared copies on sm_100+: bulk copies by the TMA unit
// (cp.async.bulk, 1-D, 16-byte aligned addresses and sizes) completing on an
// mbarrier in shared memory, and a bounded wait on that barrier.
#pragma once

#include <cstdint>

namespace gb {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// one-time setup of a barrier that completes a phase after `count` arrivals
// (plus the transaction bytes announced for that phase)
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// makes the initialised barriers visible to the async proxy (the TMA unit)
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// orders this thread's earlier shared-memory accesses (generic proxy) before
// later async-proxy writes to the same buffers
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// arrive once on the barrier and announce `bytes` of copies completing on it
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// arrive once on the barrier (release: this thread's earlier shared-memory
// writes are visible to threads that observe the phase completing)
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// named barrier `id` over `nthreads` threads (a multiple of 32) that also
// returns whether `v` holds in every participating thread
__device__ __forceinline__ bool named_bar_all(int id, int nthreads, bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "bar.red.and.pred p, %2, %3, q;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(id), "r"(nthreads)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ void named_bar(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// bulk copy global -> shared (both 16-byte aligned, bytes a multiple of 16)
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// wait until the barrier's phase with the given parity has completed; gives up
// (returns false) after limit_ns nanoseconds.  Each try_wait may suspend the
// thread for up to kSuspendNs until the phase completes, so waiting warps do
// not take issue slots from working ones.
constexpr uint32_t kSuspendNs = 100000;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
  const uint32_t a = smem_u32(bar);
  uint64_t t0 = 0;
  for (int k = 0;; ++k) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity), "r"(kSuspendNs)
        : "memory");
    if (done) return true;
    if (k == 0) t0 = global_ns();
    else if (global_ns() - t0 > limit_ns) return false;
  }
}

}  // namespace gb
