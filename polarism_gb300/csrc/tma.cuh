// Inline-PTX helpers for mbarriers and 1-D bulk (TMA) copies, sm_90+ / sm_103a.
#pragma once
#include <cstdint>

namespace pg {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

// Make mbarrier initialisation visible to the async proxy (bulk copies).
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

// Global -> shared bulk copy completing on an mbarrier (16-byte aligned, size % 16 == 0).
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

// Non-blocking test: has the phase of parity `parity` completed?
__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Plain arrival (release semantics at CTA scope).
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// One poll: suspends the thread until the phase completes or a system-dependent time limit
// passes (no suspend-time hint: with a 20 us hint the full-width RK4 kernel ran 0.8% slower).
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// --- thread-block clusters (distributed shared memory) ---------------------------------
__device__ __forceinline__ uint32_t cluster_ctarank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// Every thread of every CTA of the cluster; orders shared-memory accesses across it.
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n"
               "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// The address of the same shared-memory location in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t map_shared_rank(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}

// Asynchronous store of two floats into another CTA's shared memory, completing 8 bytes of
// transactions on that CTA's mbarrier (both addresses from map_shared_rank, same CTA).
__device__ __forceinline__ void st_async_f2(uint32_t cluster_addr, float2 v, uint32_t cluster_bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f32 [%0], {%1, %2}, [%3];"
               ::"r"(cluster_addr), "f"(v.x), "f"(v.y), "r"(cluster_bar)
               : "memory");
}

// Bounded wait: gives up after `limit` polls (none when limit is 0) and reports failure
// instead of spinning forever.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, int limit) {
  for (int k = 0; k < limit; ++k)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Failure handling of the streaming kernels' waits.  Each wait polls at most kWaitPolls
// times, a bound compiled into the loop above: the wait sites keep exactly the shape
// `if (!mbar_wait_bounded(...)) timed_out = true;`, because anything more at them (a flag
// tested before the wait, a flag read between polls, a jump out of the row loop, even as a
// cold branch) measured 4-7% slower on the full-width RK4 kernel, whose warps spend part of
// every row in these polls.  What makes a failure end quickly lives in the one thread that
// feeds the ring: once its own wait has given up, it completes each later ring slot with an
// empty arrival instead of a copy (mbar_fill_empty), so every later wait on the ring passes at
// once on whatever the slot holds, the kernel runs to its end in about the time of one full
// wait, and the call reports the timeout.
constexpr int kWaitPolls = 100000;
// After a timeout, before the block exits, each ring use that may still have a copy in flight
// is waited for with this fixed bound (a copy that was issued lands within microseconds; the
// bound only keeps the exit from hanging should one never land).
constexpr int kDrainPolls = 100000;

// Completes ring use u of slot barrier `bar` (a ring of `ring` slots, count 1) with an empty
// arrival -- once the slot's previous use has completed: a slot whose copy never landed is left
// as it is (a second arrival in an open phase is not allowed), and its later waits give up.
__device__ __forceinline__ void mbar_fill_empty(uint32_t bar, unsigned u, unsigned ring) {
  if (u >= ring && !mbar_test(bar, ((u - ring) / ring) & 1u)) return;
  mbar_arrive(bar);
}

// Waits, bounded by kDrainPolls each, for the ring copies of global ring uses [lo, hi) (use u
// fills slot u % ring, phase parity (u / ring) & 1).
__device__ __forceinline__ void drain_ring(const uint64_t* mbar, int ring, unsigned lo, unsigned hi) {
  for (unsigned u = lo; u < hi; ++u)
    mbar_wait_bounded(smem_u32(&mbar[u % ring]), (u / ring) & 1u, kDrainPolls);
}

}  // namespace pg
