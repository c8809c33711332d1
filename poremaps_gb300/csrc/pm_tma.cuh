// TMA and mbarrier helpers shared by the TMA-fed correction sweeps
// (inline PTX for sm_103a; bounded waits only).
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>

#include "pm_internal.h"

namespace pm {
namespace tma {

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count));
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect(unsigned long long* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(b)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try(unsigned long long* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: false once about `budget` clock cycles have passed.
__device__ __forceinline__ bool mbar_wait(unsigned long long* b, unsigned parity,
                                          long long budget) {
  long long t0 = clock64();
  for (unsigned i = 0;; ++i) {
    if (mbar_try(b, parity)) return true;
    if ((i & 255) == 255 && clock64() - t0 > budget) return false;
  }
}

__device__ __forceinline__ void mbar_arrive(unsigned long long* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(b)) : "memory");
}

// Untiled bulk copy global -> shared (cp.async.bulk): both addresses 16-byte
// aligned, bytes a multiple of 16; completes bytes on the barrier's tx count.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes,
                                         unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_addr(dst)), "l"((unsigned long long)src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void load3(void* dst, const CUtensorMap* map, int x, int y, int z,
                                      unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
      "l"((unsigned long long)map), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no -lcuda).
PFN_cuTensorMapEncodeTiled_v12000 encode_fn();

// 3-D map over a padded array: dims {pitch elements, NY, NZ}, box {bx, by, bz}.
bool encode(CUtensorMap* m, CUtensorMapDataType t, int esize, void* base, const Grid& g,
            long long pitch, unsigned bx, unsigned by, unsigned bz);

}  // namespace tma
}  // namespace pm
