// tma.cuh -- tensor-memory-accelerator (TMA) copies and mbarriers for the
// stencil kernels: host-side tensor-map encoding (through the driver entry
// point, no link against the driver library) and device-side inline PTX.
//
// Every wait on an mbarrier is bounded: a waiting thread sleeps in
// try_wait (up to kSuspendNs per poll, woken early when the phase
// completes) and after kWaitPolls polls raises *err and stops waiting, so a
// copy that never completes ends the kernel with an error status the host
// reads, not a hang.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace om {
namespace tma {

// ---------------------------------------------------------------------------
// host
// ---------------------------------------------------------------------------

// cuTensorMapEncodeTiled through cudaGetDriverEntryPointByVersion (looked up
// once per process).  Returns false (and leaves *map untouched) when the
// driver does not provide it or rejects the description.
bool encode_tiled(CUtensorMap *map, CUtensorMapDataType type, int rank, void *base,
                  const uint64_t *dims, const uint64_t *strides_bytes, const uint32_t *box,
                  CUtensorMapSwizzle swizzle);

// ---------------------------------------------------------------------------
// device
// ---------------------------------------------------------------------------

constexpr uint32_t kSuspendNs = 20000;  // at most 20 us asleep per poll
constexpr uint32_t kWaitPolls = 50000;  // at most about one second in all

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

// make initialised mbarriers visible to the async proxy (TMA)
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// order this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (TMA) accesses of the same memory
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// one arrival on *bar (release: this thread's earlier shared-memory writes,
// and those ordered before them, are visible to a thread whose wait sees
// the phase complete)
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// wait until the phase with parity `parity` of *bar has completed; false
// (and *err raised) when `polls` polls ran out
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t *err,
                                          uint32_t polls = kWaitPolls) {
  const uint32_t a = smem_addr(bar);
  for (uint32_t i = 0; i < polls; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity), "r"(kSuspendNs)
        : "memory");
    if (done) return true;
  }
  if (err) atomicOr(err, 1u);
  return false;
}

// 3-D tiled load of the box at (c0, c1, c2) into shared memory, completing
// on *bar (the caller posts the expected bytes)
__device__ __forceinline__ void load_3d(void *dst, const CUtensorMap *map, int c0, int c1, int c2,
                                        uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
      "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
      : "memory");
}

// 2-D tiled load of the box at (c0, c1)
__device__ __forceinline__ void load_2d(void *dst, const CUtensorMap *map, int c0, int c1,
                                        uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(dst)),
      "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(smem_addr(bar))
      : "memory");
}

}  // namespace tma
}  // namespace om
