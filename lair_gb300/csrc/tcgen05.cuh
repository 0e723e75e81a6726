// Device helpers shared by the tcgen05 kernels (mbarriers, shared-memory
// matrix descriptors) and the host's tensor-map encoder.
#pragma once

#include <cuda.h>
#include <stdint.h>

#include "common.cuh"

namespace luhot {

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, unsigned long long limit_ns) {
  const unsigned long long t0 = global_timer_ns();
  for (;;) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (global_timer_ns() - t0 > limit_ns) return false;
  }
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart.
__device__ __forceinline__ unsigned long long sw128_desc(unsigned addr) {
  unsigned long long d = 0;
  d |= (unsigned long long)((addr >> 4) & 0x3FFF);
  d |= (unsigned long long)1 << 16;            // leading byte offset (unused when swizzled)
  d |= (unsigned long long)(1024 >> 4) << 32;  // stride byte offset
  d |= (unsigned long long)1 << 46;            // descriptor version
  d |= (unsigned long long)2 << 61;            // 128-byte swizzle
  return d;
}

__device__ __forceinline__ void mbar_arrive(unsigned bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// cuTensorMapEncodeTiled, looked up once through the runtime's driver entry
// point (nullptr when the driver lacks it).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_fn();

}  // namespace luhot
