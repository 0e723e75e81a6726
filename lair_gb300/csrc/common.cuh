// Shared device/host helpers for the LU kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>

#include "luhot.h"

namespace luhot {

constexpr int kNumSmsGB300 = 152;

// Device-side error flags (written by kernels, read by the host after a call).
enum DeviceError : int {
  kDevOk = 0,
  kDevBarrierTimeout = 1,  // a bounded spin on a grid barrier ran out
  kDevBadArgument = 2,     // a kernel's own bounds check refused its input
};

// Per-context scratch that kernels use for grid barriers and error reporting.
struct DeviceStatus {
  unsigned int barrier;  // monotonically increasing arrive counter
  int error;             // DeviceError, first writer wins
  int singular;          // last zero-pivot step, -1 = none (atomicMax)
  int abort;             // set once any wait times out; later waits return at once
  unsigned long long timeout_where;  // step at which a wait gave up
  unsigned long long timeout_ns;     // limit of one wait (global-timer ns)
};

// ---------------------------------------------------------------------------
// Bounded grid barrier.  All CTAs of a cooperative launch (co-residency is
// guaranteed by cudaLaunchCooperativeKernel) call it with the same target.
// A wait gives up after st->timeout_ns of global time, records the error
// and sets `abort`, so every later wait of the launch returns at once and the
// kernel finishes; the host then turns the flag into LUHOT_ERR_TIMEOUT.
// ---------------------------------------------------------------------------
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull;  // default: 2 s

__device__ __forceinline__ unsigned long long global_timer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ int ld_relaxed_i32(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Returns false when the barrier was abandoned (timeout or earlier abort).
__device__ __forceinline__ bool grid_barrier(DeviceStatus* st, unsigned int target,
                                             unsigned long long where) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();
    atomicAdd(&st->barrier, 1u);
    if (ld_relaxed_i32(&st->abort)) {
      ok = 0;
    } else {
      const unsigned long long t0 = global_timer_ns();
      const unsigned long long limit = st->timeout_ns;
      unsigned int spins = 0;
      while (ld_acquire_u32(&st->barrier) < target) {
        if ((++spins & 63u) == 0) {
          if (ld_relaxed_i32(&st->abort)) {
            ok = 0;
            break;
          }
          if (global_timer_ns() - t0 > limit) {
            atomicCAS(&st->error, kDevOk, kDevBarrierTimeout);
            atomicExch(&st->timeout_where, where);
            atomicExch(&st->abort, 1);
            ok = 0;
            break;
          }
        }
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Loads that bypass L1 (data written by other CTAs during the same launch).
template <typename T>
__device__ __forceinline__ T ld_cg(const T* p) {
  return __ldcg(p);
}

}  // namespace luhot

// Host-side CUDA error check used inside functions returning a luhot status.
#define LUHOT_CUDA_TRY(ctx, expr)                                                   \
  do {                                                                              \
    cudaError_t _e = (expr);                                                        \
    if (_e != cudaSuccess) {                                                        \
      return ::luhot::set_error((ctx), LUHOT_ERR_CUDA,                              \
                                std::string(#expr " failed: ") + cudaGetErrorString(_e)); \
    }                                                                               \
  } while (0)
