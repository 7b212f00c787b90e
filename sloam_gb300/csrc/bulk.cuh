// bulk.cuh — shared-memory mbarriers and the untiled bulk copy
// (cp.async.bulk, the TMA unit's 1-D form), used by the tensor-core proposal
// kernel to stage its weights.
//
// A bulk copy moves a contiguous range global -> shared and completes on an
// mbarrier's transaction count.  Both addresses must be 16-byte aligned and
// the size a multiple of 16; callers check this and take plain loads where
// it does not hold.
#pragma once
#include <stdint.h>

namespace sg {

__device__ __forceinline__ uint32_t saddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* m, uint32_t n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(m)), "r"(n) : "memory");
}
// the initialised barriers visible to the async proxy
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* m, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(saddr(m)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* m, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(m)),
               "r"(bytes)
               : "memory");
}
// generic-proxy accesses of shared memory ordered before later async-proxy
// ones (a bulk copy that overwrites what was just read)
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// bulk copy global -> shared (16-byte aligned, size a multiple of 16),
// completing on the mbarrier's transaction count
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes,
                                          uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(dst),
      "l"((uint64_t)__cvta_generic_to_global(src)), "r"(bytes), "r"(saddr(bar))
      : "memory");
}

}  // namespace sg
