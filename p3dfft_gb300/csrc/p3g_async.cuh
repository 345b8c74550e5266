// Asynchronous global -> shared copies for the pipelined passes:
//   * TMA tensor tile loads (cp.async.bulk.tensor) completing on an mbarrier,
//   * per-thread cp.async (LDGSTS) with zero fill, tracked by commit groups.
// Every wait on an mbarrier is bounded: after a second (kMbarWaitNs) the
// waiting thread records an error in the plan's device flag and gives up, so
// a mis-sized transaction can never hang the GPU.
#pragma once

#include <cuda.h>

#include <cstdint>

#include "p3g_arith.cuh"

namespace p3g {

// A wait gives up after kMbarWaitNs of the global timer (try_wait suspends
// the thread for a hardware-chosen time on each poll, so a poll count alone
// is a poor clock), or after kMbarSpinLimit polls at the latest.
constexpr uint64_t kMbarWaitNs = 1000000000ull;  // 1 s
constexpr uint32_t kMbarSpinLimit = 1u << 24;
constexpr int kErrMbarTimeout = 1;

P3G_D uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

P3G_D uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// ------------------------------------------------------------------ cp.async
// src_bytes < size zero-fills the rest of the destination (0 = all zeros).
P3G_D void cp_async16(void* dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_u32(dst)), "l"(src), "r"(src_bytes)
               : "memory");
}
P3G_D void cp_async8(void* dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(smem_u32(dst)), "l"(src), "r"(src_bytes)
               : "memory");
}
P3G_D void cp_async4(void* dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(smem_u32(dst)), "l"(src), "r"(src_bytes)
               : "memory");
}
P3G_D void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
P3G_D void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// ------------------------------------------------------------------ mbarrier
P3G_D void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
P3G_D void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
P3G_D void mbar_arrive_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(b)), "r"(bytes)
               : "memory");
}
P3G_D bool mbar_try_wait(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for phase `parity` of the barrier; false (and the error flag
// set) if it did not complete within the limit.
P3G_D bool mbar_wait_bounded(uint64_t* b, uint32_t parity, int* err) {
  if (mbar_try_wait(b, parity)) return true;
  const uint64_t t0 = global_ns();
  for (uint32_t i = 0; i < kMbarSpinLimit; ++i) {
    if (mbar_try_wait(b, parity)) return true;
    if ((i & 15) == 15 && global_ns() - t0 > kMbarWaitNs) break;
    if (i > 16) __nanosleep(32);
  }
  if (err) atomicExch(err, kErrMbarTimeout);
  return false;
}
// Orders this thread's generic-proxy shared-memory accesses before later
// async-proxy (TMA) writes to the same buffer.
P3G_D void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// ------------------------------------------------------------------ TMA
// 4-D tiled tensor load into shared memory, completing tx bytes on `bar`.
P3G_D void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
      "%5}], [%6];\n" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}

// 4-D tiled tensor store from shared memory (bulk async group).  The
// threads that wrote the tile fence it to the async proxy and synchronise
// before one thread issues the store.
P3G_D void tma_store_4d(const CUtensorMap* map, const void* src, int c0, int c1, int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3, %4}], [%5];\n" ::"l"(map),
      "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(src))
      : "memory");
}
P3G_D void bulk_commit_group() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }
// Waits until at most N of this thread's bulk groups still read shared memory.
template <int N>
P3G_D void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;\n" ::"n"(N) : "memory");
}
// Waits until every bulk group of this thread has completed.
P3G_D void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }

// 1-D bulk copy of `bytes` (a multiple of 16, both addresses 16-byte
// aligned) from global into shared memory, completing on `bar`.
P3G_D void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

}  // namespace p3g
