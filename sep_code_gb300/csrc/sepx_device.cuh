// sepx_device.cuh -- sm_103a device helpers: mbarrier, TMA tensor loads,
// bounded waits, streaming stores.  Every spin on an mbarrier gives up after a
// wall-clock budget, records where it gave up in an error word and returns
// false, so that a bug can never hang the GPU.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace sepx {

// error codes written into the per-context device error word
enum DevErr : int {
  kErrNone = 0,
  kErrFullWait = 1,    // consumer gave up waiting for a TMA stage
  kErrEmptyWait = 2,   // producer gave up waiting for consumers to free a stage
  kErrDrainWait = 3,   // exit-time wait for in-flight copies gave up
  kErrMmaWait = 4,     // wait for tensor-core MMAs to finish gave up
  kErrAdamStep = 5,    // Adam read a step count below 1 from device memory (no update made)
};

constexpr unsigned long long kWaitBudgetNs = 2000000000ull;  // 2 s

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t addr, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(addr), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_inval(uint32_t addr) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(addr) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t addr, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(addr), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t addr) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(addr) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t addr, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(addr), "r"(parity)
      : "memory");
  return ok != 0;
}

// try_wait with a suspend-time hint: the warp may sleep in hardware until
// the phase completes or the hint (ns) elapses, instead of spinning
#ifndef SEPX_WAIT_HINT_NS
#define SEPX_WAIT_HINT_NS 20000
#endif
__device__ __forceinline__ bool mbar_try_wait_hint(uint32_t addr, uint32_t parity) {
#if SEPX_WAIT_HINT_NS > 0
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(addr), "r"(parity), "n"(SEPX_WAIT_HINT_NS)
      : "memory");
  return ok != 0;
#else
  return mbar_try_wait(addr, parity);
#endif
}

// Wait for the phase with the given parity to complete.  Returns false (and
// records `code`) when the budget runs out.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t addr, uint32_t parity, int *err,
                                                  int code) {
  if (mbar_try_wait(addr, parity)) return true;
  const unsigned long long t0 = globaltimer_ns();
  while (true) {
    if (mbar_try_wait_hint(addr, parity)) return true;
    if (globaltimer_ns() - t0 > kWaitBudgetNs) {
      if (err) atomicCAS(err, 0, code);
      return false;
    }
  }
}

// 3-D tiled TMA load of one box into shared memory, completing on `mbar`.
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int x, int y,
                                            int z, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(mbar)
      : "memory");
}

// 5-D tiled TMA load (coordinates innermost first), completing on `mbar`.
__device__ __forceinline__ void tma_load_5d(uint32_t dst, const CUtensorMap *map, int c0, int c1,
                                            int c2, int c3, int c4, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(mbar)
      : "memory");
}

// Plain bulk copy global -> shared (16-byte aligned addresses, size a
// multiple of 16), completing on `mbar`.
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes,
                                          uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(mbar)
      : "memory");
}

__device__ __forceinline__ void prefetch_tmap(const CUtensorMap *map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

__device__ __forceinline__ float4 lds4(const float *p) { return *reinterpret_cast<const float4 *>(p); }

__device__ __forceinline__ void stcs4(float *p, float4 v) { __stcs(reinterpret_cast<float4 *>(p), v); }

__device__ __forceinline__ float4 ldg4(const float *p) { return __ldg(reinterpret_cast<const float4 *>(p)); }

__device__ __forceinline__ float comp(const float4 &v, int c) {
  return c == 0 ? v.x : (c == 1 ? v.y : (c == 2 ? v.z : v.w));
}

}  // namespace sepx
