// pfa_tma.cuh -- tensor-memory-accelerator (TMA) tile loads into shared
// memory, completed on mbarriers, for sm_103a kernels (inline PTX).
//
// One thread of a CTA arms a barrier with the bytes a plane's copies deliver
// and issues the tiled copies; every thread that reads the plane waits on
// the barrier's phase.  Waits are bounded: after kWaitNs (one second of the
// global timer) or kWaitLimit polls the wait gives up and reports it, so a
// copy that never lands cannot hold the GPU.
#pragma once

#include <cstdint>

namespace pfa {
namespace tma {

constexpr uint32_t kWaitLimit = 1u << 22;       // polls of mbarrier.try_wait before giving up
constexpr uint64_t kWaitNs = 1000000000ull;     // or this long (ns), whichever comes first

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return uint32_t(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void bar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}

// make barrier initialisation visible to the async proxy (the TMA unit)
__device__ __forceinline__ void bar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

// order this thread's earlier shared-memory accesses before its later
// async-proxy (TMA) writes to the same memory
__device__ __forceinline__ void proxy_fence() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// one arrival that also expects `bytes` of copy transactions on the phase
__device__ __forceinline__ void bar_arrive_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes)
               : "memory");
}

// nanoseconds of the GPU's global timer
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool bar_try(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n"
      ".reg .pred P;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n"
      "selp.u32 %0, 1, 0, P;\n"
      "}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

// true once the phase with this parity has completed; false when it has not
// after limit_ns of the global timer or kWaitLimit polls, whichever comes
// first (limit_ns 0: after the first 64 polls)
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity,
                                         uint64_t limit_ns = kWaitNs) {
  // a copy in flight usually lands within these polls: the clock is read
  // only for waits that outlast them
  for (int i = 0; i < 64; i++)
    if (bar_try(bar, parity)) return true;
  if (limit_ns == 0) return false;
  const uint64_t t0 = global_ns();
  for (uint32_t i = 0; i < kWaitLimit; i++) {
    if (bar_try(bar, parity)) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
  return false;
}

// tiled 3D copy of the box at (x, y, z) of `map` into shared memory at dst,
// completing `bar`'s transaction count; x is in elements of the map's type
// and x * element size must be a multiple of 16 bytes
__device__ __forceinline__ void load3(uint32_t dst, const void* map, int x, int y, int z,
                                      uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void prefetch_map(const void* map) {
  asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

}  // namespace tma
}  // namespace pfa
