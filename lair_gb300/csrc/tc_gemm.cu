// Tensor-core Schur update for the mixed-precision LU (tcgen05 + TMA).
//
//   C (M x N, FP32, row-major, ldc)  +=  alpha * A (M x K) * Bt (N x K)^T
//
// A and Bt are K-major operand copies in BF16, FP16 or TF32 (FP32 words rounded to TF32),
// made per panel by tc_convert_kernel from the FP32 matrix being factored
// (A = L21, Bt = U12^T), each scaled by a power of two so that its largest
// magnitude sits at 2^14 (per-panel scaling: no FP16 overflow, few
// subnormals); alpha = -1 / (scale_A * scale_B) undoes the scaling exactly.
//
// One CTA computes a 128 x 128 tile: one thread loads all K of the A and B
// tiles with TMA (128-byte swizzle, 16 KB boxes of 128 rows x 128 bytes)
// onto an mbarrier, then issues the K/16 (K/8 for TF32) tcgen05.mma
// instructions with the FP32 accumulator in TMEM (128 columns) and commits
// to a second mbarrier; the four warps then read their 32 TMEM lanes
// (tcgen05.ld 32x32b) and update C.  Every mbarrier wait is bounded by the
// global timer; on expiry the kernel records the error, waits a bounded time
// for its copies, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "common.cuh"
#include "luhot_internal.h"
#include "tc_gemm.cuh"
#include "tcgen05.cuh"

namespace luhot {

template <int KIND>
__global__ void __launch_bounds__(128) tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA,
                                                      const __grid_constant__ CUtensorMap tmB, float* C, int64_t ldc,
                                                      int M, int N, int K, const float* alpha_ptr,
                                                      DeviceStatus* st) {
  constexpr int ES = KIND == kTcTF32 ? 4 : 2;
  constexpr int KBOX = 128 / ES;
  constexpr int KSTEP = KIND == kTcTF32 ? 8 : 16;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int nbox = (K + KBOX - 1) / KBOX;
  unsigned char* sA = base;
  unsigned char* sB = base + nbox * 16384;
  __shared__ __align__(8) unsigned long long bar_tma, bar_mma;
  __shared__ unsigned tmem_base;
  __shared__ int s_ok;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * 128, n0 = blockIdx.x * 128;
  const unsigned long long limit = st->timeout_ns;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(smem_u32(&tmem_base)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar_tma)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar_mma)));
    asm volatile("fence.mbarrier_init.release.cluster;");
    asm volatile("fence.proxy.async.shared::cta;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const unsigned tmem = tmem_base;
  if (threadIdx.x == 0) {
    bool ok = true;
    const unsigned bytes = (unsigned)nbox * 2u * 16384u;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&bar_tma)), "r"(bytes)
                 : "memory");
    for (int bx = 0; bx < nbox; ++bx) {
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
              smem_u32(sA + bx * 16384)),
          "l"(&tmA), "r"(bx * KBOX), "r"(m0), "r"(smem_u32(&bar_tma))
          : "memory");
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
              smem_u32(sB + bx * 16384)),
          "l"(&tmB), "r"(bx * KBOX), "r"(n0), "r"(smem_u32(&bar_tma))
          : "memory");
    }
    ok = mbar_wait(smem_u32(&bar_tma), 0, limit);
    if (ok) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const unsigned fmt = KIND == kTcTF32 ? 2u : (KIND == kTcBF16 ? 1u : 0u);
      const unsigned idesc = (1u << 4) | (fmt << 7) | (fmt << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);
      const int ksteps = (K + KSTEP - 1) / KSTEP;
      for (int ks = 0; ks < ksteps; ++ks) {
        const int byte_k = ks * 32;
        const int bx = byte_k >> 7, within = byte_k & 127;
        const unsigned long long da = sw128_desc(smem_u32(sA + bx * 16384 + within));
        const unsigned long long db = sw128_desc(smem_u32(sB + bx * 16384 + within));
        const unsigned acc = ks > 0 ? 1u : 0u;
        if (KIND == kTcTF32)
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
                  tmem),
              "l"(da), "l"(db), "r"(idesc), "r"(acc));
        else
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
                  tmem),
              "l"(da), "l"(db), "r"(idesc), "r"(acc));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&bar_mma))
                   : "memory");
    } else {
      atomicCAS(&st->error, kDevOk, kDevBarrierTimeout);
      atomicExch(&st->abort, 1);
      mbar_wait(smem_u32(&bar_tma), 0, limit);  // bounded: let copies in flight land
    }
    s_ok = ok ? 1 : 0;
  }
  __syncthreads();
  if (s_ok) {
    const bool mma_ok = mbar_wait(smem_u32(&bar_mma), 0, limit);
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (!mma_ok) {
      atomicCAS(&st->error, kDevOk, kDevBarrierTimeout);
      atomicExch(&st->abort, 1);
    } else {
      const float alpha = *alpha_ptr;
      const int row = m0 + warp * 32 + lane;
      float* crow = C + (int64_t)row * ldc;
      const bool vec = ((ldc & 3) == 0) && ((reinterpret_cast<uintptr_t>(C) & 15) == 0);
#pragma unroll 1
      for (int cb = 0; cb < 4; ++cb) {
        unsigned r[32];
        const unsigned taddr = tmem + ((unsigned)(warp * 32) << 16) + (unsigned)(cb * 32);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,"
            "%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
              "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;");
        if (row < M) {
          const int c0 = n0 + cb * 32;
          if (vec && c0 + 32 <= N) {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              float4 v = *reinterpret_cast<const float4*>(crow + c0 + 4 * q);
              v.x = fmaf(alpha, __uint_as_float(r[4 * q + 0]), v.x);
              v.y = fmaf(alpha, __uint_as_float(r[4 * q + 1]), v.y);
              v.z = fmaf(alpha, __uint_as_float(r[4 * q + 2]), v.z);
              v.w = fmaf(alpha, __uint_as_float(r[4 * q + 3]), v.w);
              *reinterpret_cast<float4*>(crow + c0 + 4 * q) = v;
            }
          } else {
            for (int j = 0; j < 32; ++j)
              if (c0 + j < N) crow[c0 + j] = fmaf(alpha, __uint_as_float(r[j]), crow[c0 + j]);
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem));
}

// ---------------------------------------------------------------------------
// FP32-accurate variant on the BF16 tensor cores (kTcBF16x3).  Every FP32
// operand x is split into three BF16 pieces x0 + x1 + x2 (8 significant bits
// each, 24 together, each remainder exact in FP32), and the product is
// a0 b0 + a0 b1 + a1 b0 + a0 b2 + a1 b1 + a2 b0 (the terms down to 2^-16 of
// the leading one; the dropped ones are below FP32's unit roundoff),
// accumulated in FP32 in TMEM.  K runs in chunks of 64: per chunk one thread
// loads the six 128 x 64 tiles (96 KB) with TMA, issues 4 k-steps x 6
// products, commits, and waits before the next chunk reuses the tiles.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) tc_gemm_x3_kernel(const __grid_constant__ CUtensorMap tmA,
                                                         const __grid_constant__ CUtensorMap tmB, float* C,
                                                         int64_t ldc, int M, int N, int K, const float* alpha_ptr,
                                                         DeviceStatus* st) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* sA = base;               // 3 pieces x 16 KB
  unsigned char* sB = base + 3 * 16384;   // 3 pieces x 16 KB
  __shared__ __align__(8) unsigned long long bar_tma, bar_mma;
  __shared__ unsigned tmem_base;
  __shared__ int s_ok;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * 128, n0 = blockIdx.x * 128;
  const unsigned long long limit = st->timeout_ns;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(smem_u32(&tmem_base)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar_tma)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar_mma)));
    asm volatile("fence.mbarrier_init.release.cluster;");
    asm volatile("fence.proxy.async.shared::cta;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const unsigned tmem = tmem_base;
  if (threadIdx.x == 0) {
    bool ok = true;
    // Operand copies hold the three pieces side by side along K: piece p of
    // chunk c sits at x = p * kalloc + c * 64 (kalloc = padded K).
    const int kalloc = (K + 63) / 64 * 64;
    const int nchunk = kalloc / 64;
    const unsigned idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);
    const int pa[6] = {0, 0, 1, 0, 1, 2}, pb[6] = {0, 1, 0, 2, 1, 0};
    for (int c = 0; c < nchunk && ok; ++c) {
      const unsigned parity = (unsigned)(c & 1);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&bar_tma)), "r"(6u * 16384u)
                   : "memory");
      for (int p = 0; p < 3; ++p) {
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
                smem_u32(sA + p * 16384)),
            "l"(&tmA), "r"(p * kalloc + c * 64), "r"(m0), "r"(smem_u32(&bar_tma))
            : "memory");
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
                smem_u32(sB + p * 16384)),
            "l"(&tmB), "r"(p * kalloc + c * 64), "r"(n0), "r"(smem_u32(&bar_tma))
            : "memory");
      }
      ok = mbar_wait(smem_u32(&bar_tma), parity, limit);
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      for (int ks = 0; ks < 4; ++ks) {
        for (int t = 0; t < 6; ++t) {
          const unsigned long long da = sw128_desc(smem_u32(sA + pa[t] * 16384 + ks * 32));
          const unsigned long long db = sw128_desc(smem_u32(sB + pb[t] * 16384 + ks * 32));
          const unsigned acc = (c > 0 || ks > 0 || t > 0) ? 1u : 0u;
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
                  tmem),
              "l"(da), "l"(db), "r"(idesc), "r"(acc));
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&bar_mma))
                   : "memory");
      ok = mbar_wait(smem_u32(&bar_mma), parity, limit);  // tiles are reused by the next chunk
    }
    if (!ok) {
      atomicCAS(&st->error, kDevOk, kDevBarrierTimeout);
      atomicExch(&st->abort, 1);
    }
    s_ok = ok ? 1 : 0;
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (s_ok) {
    const float alpha = *alpha_ptr;
    const int row = m0 + warp * 32 + lane;
    float* crow = C + (int64_t)row * ldc;
    const bool vec = ((ldc & 3) == 0) && ((reinterpret_cast<uintptr_t>(C) & 15) == 0);
#pragma unroll 1
    for (int cb = 0; cb < 4; ++cb) {
      unsigned r[32];
      const unsigned taddr = tmem + ((unsigned)(warp * 32) << 16) + (unsigned)(cb * 32);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,"
          "%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
            "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
            "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;");
      if (row < M) {
        const int c0 = n0 + cb * 32;
        if (vec && c0 + 32 <= N) {
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            float4 v = *reinterpret_cast<const float4*>(crow + c0 + 4 * q);
            v.x = fmaf(alpha, __uint_as_float(r[4 * q + 0]), v.x);
            v.y = fmaf(alpha, __uint_as_float(r[4 * q + 1]), v.y);
            v.z = fmaf(alpha, __uint_as_float(r[4 * q + 2]), v.z);
            v.w = fmaf(alpha, __uint_as_float(r[4 * q + 3]), v.w);
            *reinterpret_cast<float4*>(crow + c0 + 4 * q) = v;
          }
        } else {
          for (int j = 0; j < 32; ++j)
            if (c0 + j < N) crow[c0 + j] = fmaf(alpha, __uint_as_float(r[j]), crow[c0 + j]);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem));
}

// ---------------------------------------------------------------------------
// Persistent, warp-specialised form (all kinds).  One CTA per SM walks a
// contiguous range of 128 x 128 tiles.  Six warps:
//   warp 0      TMA producer: per tile and 128-byte K box, the A and B boxes
//               (three pieces each for kTcBF16x3) into a ring of stages;
//   warp 1      TMEM owner and MMA issuer: two 128-column FP32 accumulators,
//               so one tile's MMAs overlap the previous tile's epilogue
//               (BF16x3: two pairs, the leading product a0 b0 in one, the
//               five smaller products in the other, added in the epilogue:
//               the tensor core's accumulation then never rounds the small
//               terms against the large running sum);
//   warps 2-5   epilogue: tcgen05.ld of their 32 TMEM lanes, scale by alpha,
//               stage 128 x 32 FP32 blocks in shared memory (128-byte
//               swizzle) and add them into C with TMA reduce-add, so C is
//               never read by the SM and its HBM traffic streams behind the
//               tensor cores.
// Stage ring: full[s] (TMA bytes landed) / empty[s] (MMAs that read the stage
// completed, via tcgen05.commit); accumulators: tfull[b] / tempty[b].  All
// mbarrier waits are bounded; on expiry a role records the error, raises the
// abort flag and stops, and before exit the CTA waits (bounded) for its
// copies and MMAs in flight and for its reductions to read their staging.
// ---------------------------------------------------------------------------
constexpr int kTcEpiWarps = 4;
constexpr int kTcThreads = 64 + 32 * kTcEpiWarps;

template <int KIND>
struct TcShape {
  static constexpr int kPieces = KIND == kTcBF16x3 ? 3 : 1;
  static constexpr int kES = KIND == kTcTF32 ? 4 : 2;
  static constexpr int kKBox = 128 / kES;
  static constexpr int kStageBytes = 2 * kPieces * 16384;
  static constexpr int kStages = KIND == kTcBF16x3 ? 2 : 4;
  static constexpr int kStagingBytes = 2 * 16384;
  static constexpr size_t kSmem = 1024 + (size_t)kStages * kStageBytes + kStagingBytes;
};

// 32 consecutive 32-bit TMEM columns of the warp's 32 lanes (completed by
// tcgen05.wait::ld).
__device__ __forceinline__ void tc_ld32(unsigned taddr, unsigned (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,"
      "%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}

__device__ __forceinline__ void tc_abort(DeviceStatus* st, int* s_abort) {
  atomicCAS(&st->error, kDevOk, kDevBarrierTimeout);
  atomicExch(&st->abort, 1);
  atomicExch(s_abort, 1);
}

template <int KIND>
__global__ void __launch_bounds__(kTcThreads, 1)
    tc_gemm_persistent_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                              const __grid_constant__ CUtensorMap tmC, int M, int N, int kalloc,
                              const float* alpha_ptr, DeviceStatus* st) {
  using Sh = TcShape<KIND>;
  constexpr int S = Sh::kStages;
  constexpr int PIECES = Sh::kPieces;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* ring = base;
  unsigned char* staging = base + (size_t)S * Sh::kStageBytes;
  __shared__ __align__(8) unsigned long long full[S], empty[S], tfull[2], tempty[2];
  __shared__ unsigned tmem_base;
  __shared__ int s_abort, s_issued, s_consumed, s_epi_stop;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned long long limit = st->timeout_ns;
  const int tiles_n = (N + 127) / 128;
  const int tiles = ((M + 127) / 128) * tiles_n;
  const int G = gridDim.x;
  const int t_begin = (int)((int64_t)blockIdx.x * tiles / G);
  const int t_end = (int)((int64_t)(blockIdx.x + 1) * tiles / G);
  const int nkb = kalloc / Sh::kKBox;

  // BF16x3 keeps the leading product a0 b0 and the five smaller ones in
  // separate accumulators (added once, in the epilogue), so the small terms
  // are not rounded against the large running sum at every k-step.
  constexpr bool kSplitAcc = KIND == kTcBF16x3;
  constexpr unsigned kAccCols = kSplitAcc ? 256u : 128u;  // TMEM columns per accumulator buffer
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "n"(2 * kAccCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    for (int i = 0; i < S; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full[i])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty[i])));
    }
    for (int i = 0; i < 2; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&tfull[i])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&tempty[i])), "r"(kTcEpiWarps));
    }
    s_abort = 0;
    s_issued = 0;
    s_consumed = 0;
    s_epi_stop = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
    asm volatile("fence.proxy.async.shared::cta;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const unsigned tmem = tmem_base;

  if (warp == 0) {
    if (lane == 0) {
      // Producer.
      int it = 0;
      for (int t = t_begin; t < t_end && !s_abort; ++t) {
        const int tm = t / tiles_n, tn = t - tm * tiles_n;
        for (int kb = 0; kb < nkb; ++kb, ++it) {
          const int s = it % S;
          if (!mbar_wait(smem_u32(&empty[s]), (unsigned)((it / S) & 1) ^ 1u, limit)) {
            tc_abort(st, &s_abort);
            break;
          }
          unsigned char* sa = ring + (size_t)s * Sh::kStageBytes;
          unsigned char* sb = sa + PIECES * 16384;
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&full[s])),
                       "r"((unsigned)Sh::kStageBytes)
                       : "memory");
          for (int pc = 0; pc < PIECES; ++pc) {
            const int x = pc * kalloc + kb * Sh::kKBox;
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
                "[%4];" ::"r"(smem_u32(sa + pc * 16384)),
                "l"(&tmA), "r"(x), "r"(tm * 128), "r"(smem_u32(&full[s]))
                : "memory");
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
                "[%4];" ::"r"(smem_u32(sb + pc * 16384)),
                "l"(&tmB), "r"(x), "r"(tn * 128), "r"(smem_u32(&full[s]))
                : "memory");
          }
          s_issued = it + 1;
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer.
      constexpr unsigned fmt = KIND == kTcTF32 ? 2u : ((KIND == kTcBF16 || KIND == kTcBF16x3) ? 1u : 0u);
      constexpr unsigned idesc = (1u << 4) | (fmt << 7) | (fmt << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);
      constexpr int NPROD = KIND == kTcBF16x3 ? 6 : 1;
      const int pa[6] = {0, 0, 1, 0, 1, 2}, pb[6] = {0, 1, 0, 2, 1, 0};
      int it = 0, tc = 0;
      for (int t = t_begin; t < t_end && !s_abort; ++t, ++tc) {
        const int b = tc & 1;
        if (!mbar_wait(smem_u32(&tempty[b]), (unsigned)((tc >> 1) & 1) ^ 1u, limit)) {
          tc_abort(st, &s_abort);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const unsigned acc_addr = tmem + (unsigned)b * kAccCols;
        bool ok = true;
        for (int kb = 0; kb < nkb; ++kb, ++it) {
          const int s = it % S;
          if (!mbar_wait(smem_u32(&full[s]), (unsigned)((it / S) & 1), limit)) {
            ok = false;
            break;
          }
          s_consumed = it + 1;
          asm volatile("tcgen05.fence::after_thread_sync;");
          unsigned char* sa = ring + (size_t)s * Sh::kStageBytes;
          unsigned char* sb = sa + PIECES * 16384;
          for (int ks = 0; ks < 4; ++ks) {
            for (int pr = 0; pr < NPROD; ++pr) {
              const unsigned long long da = sw128_desc(smem_u32(sa + pa[pr] * 16384 + ks * 32));
              const unsigned long long db = sw128_desc(smem_u32(sb + pb[pr] * 16384 + ks * 32));
              const bool lo = kSplitAcc && pr > 0;
              const unsigned accf = (kb > 0 || ks > 0 || pr > (lo ? 1 : 0)) ? 1u : 0u;
              const unsigned acc = acc_addr + (lo ? 128u : 0u);
              if (KIND == kTcTF32)
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, "
                    "p;\n}\n" ::"r"(acc),
                    "l"(da), "l"(db), "r"(idesc), "r"(accf));
              else
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, "
                    "p;\n}\n" ::"r"(acc),
                    "l"(da), "l"(db), "r"(idesc), "r"(accf));
            }
          }
          // The stage is free once these MMAs have read it.
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                           smem_u32(&empty[s]))
                       : "memory");
        }
        if (!ok) {
          tc_abort(st, &s_abort);
          break;
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(&tfull[b]))
                     : "memory");
      }
    }
  } else {
    // Epilogue: warp w reads TMEM lanes 32 * (w % 4) .. + 31 = tile rows.
    const int quarter = warp & 3;
    const int row = quarter * 32 + lane;
    const bool leader = (warp == 2 && lane == 0);
    const float alpha = *alpha_ptr;
    int tc = 0, sbuf = 0;
    for (int t = t_begin; t < t_end; ++t, ++tc) {
      const int tm = t / tiles_n, tn = t - tm * tiles_n;
      const int b = tc & 1;
      const bool got = mbar_wait(smem_u32(&tfull[b]), (unsigned)((tc >> 1) & 1), limit);
      // One decision for all four epilogue warps (they meet at named
      // barriers below): any failed wait or an abort stops them together.
      const bool all_got = __all_sync(0xffffffffu, got);
      if (lane == 0 && (!all_got || s_abort)) s_epi_stop = 1;
      __syncwarp();
      asm volatile("bar.sync 1, %0;" ::"n"(32 * kTcEpiWarps) : "memory");
      if (s_epi_stop) {
        if (leader) tc_abort(st, &s_abort);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      for (int cb = 0; cb < 4; ++cb, sbuf ^= 1) {
        unsigned r[32];
        const unsigned taddr = tmem + ((unsigned)(quarter * 32) << 16) + (unsigned)b * kAccCols + (unsigned)(cb * 32);
        tc_ld32(taddr, r);
        if constexpr (kSplitAcc) {
          unsigned r2[32];
          tc_ld32(taddr + 128u, r2);
          asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
          for (int q = 0; q < 32; ++q) r[q] = __float_as_uint(__uint_as_float(r[q]) + __uint_as_float(r2[q]));
        } else {
          asm volatile("tcgen05.wait::ld.sync.aligned;");
        }
        if (cb == 3) {
          // This warp is done with the accumulator: the MMA warp may reuse it.
          asm volatile("tcgen05.fence::before_thread_sync;");
          __syncwarp();
          if (lane == 0) mbar_arrive(smem_u32(&tempty[b]));
        }
        // The staging block written two reductions ago must have been read.
        if (leader) asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
        asm volatile("bar.sync 1, %0;" ::"n"(32 * kTcEpiWarps));
        unsigned char* blk = staging + sbuf * 16384 + row * 128;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          float4 v;
          v.x = alpha * __uint_as_float(r[4 * q + 0]);
          v.y = alpha * __uint_as_float(r[4 * q + 1]);
          v.z = alpha * __uint_as_float(r[4 * q + 2]);
          v.w = alpha * __uint_as_float(r[4 * q + 3]);
          *reinterpret_cast<float4*>(blk + ((q ^ (row & 7)) << 4)) = v;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("bar.sync 1, %0;" ::"n"(32 * kTcEpiWarps));
        if (leader) {
          // Boxes past the last column are not issued; the (possibly empty)
          // group is committed either way so the staging rotation stays in
          // step with the groups.
          if (tn * 128 + cb * 32 < N)
            asm volatile(
                "cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                    &tmC),
                "r"(tn * 128 + cb * 32), "r"(tm * 128), "r"(smem_u32(staging + sbuf * 16384))
                : "memory");
          asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        }
      }
    }
    if (leader) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_abort) {
    // Copies still in flight (issued, never consumed) must land before exit.
    for (int i = s_consumed; i < s_issued; ++i) mbar_wait(smem_u32(&full[i % S]), (unsigned)((i / S) & 1), limit);
  }
  if (threadIdx.x == 32 && s_abort) {
    // MMAs still running: every stage's last commit has arrived once they end.
    for (int i = 0; i < S; ++i) {
      const int uses = s_consumed - i > 0 ? (s_consumed - i + S - 1) / S : 0;
      if (uses > 0) mbar_wait(smem_u32(&empty[i]), (unsigned)((uses - 1) & 1), limit);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(2 * kAccCols));
}

// ---------------------------------------------------------------------------
// Per-panel operand conversion.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void atomic_max_f32_nonneg(float* addr, float v) {
  atomicMax(reinterpret_cast<unsigned*>(addr), __float_as_uint(v));
}

// s[0] = max |L21|, s[1] = max |U12|.
__global__ void tc_absmax_kernel(const float* __restrict__ a, int64_t lda, int k0, int w, int r1, int m, int c1, int n,
                                 float* s) {
  float ml = 0.f, mu = 0.f;
  const int64_t nl = (int64_t)(m - r1) * w, nu = (int64_t)w * (n - c1);
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nl + nu; t += (int64_t)gridDim.x * blockDim.x) {
    if (t < nl) {
      const int i = (int)(t / w), k = (int)(t - (int64_t)i * w);
      ml = fmaxf(ml, fabsf(a[(int64_t)(r1 + i) * lda + k0 + k]));
    } else {
      const int64_t u = t - nl;
      const int k = (int)(u / (n - c1)), j = (int)(u - (int64_t)k * (n - c1));
      mu = fmaxf(mu, fabsf(a[(int64_t)(k0 + k) * lda + c1 + j]));
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    ml = fmaxf(ml, __shfl_xor_sync(0xffffffffu, ml, off));
    mu = fmaxf(mu, __shfl_xor_sync(0xffffffffu, mu, off));
  }
  if ((threadIdx.x & 31) == 0) {
    atomic_max_f32_nonneg(&s[0], ml);
    atomic_max_f32_nonneg(&s[1], mu);
  }
}

// Power-of-two scale that puts a maximum magnitude at 2^14.
__device__ __forceinline__ float pow2_scale(float mx) {
  if (!(mx > 0.f) || !isfinite(mx)) return 1.f;
  int e;
  frexpf(mx, &e);  // mx = f * 2^e, f in [0.5, 1)
  return ldexpf(1.f, 14 - e);
}

__global__ void tc_scales_kernel(float* s) {
  const float sa = pow2_scale(s[0]), sb = pow2_scale(s[1]);
  s[2] = sa;
  s[3] = sb;
  s[4] = -1.f / (sa * sb);  // exact: a power of two
}

// Element (row, k) of an operand copy with padded K kalloc.  kTcBF16x3 rows
// hold the three BF16 pieces side by side: [piece 0 | piece 1 | piece 2].
template <int KIND>
__device__ __forceinline__ void store_op(void* dst, int64_t row, int k, int kalloc, float v) {
  if (KIND == kTcBF16) {
    reinterpret_cast<__nv_bfloat16*>(dst)[row * kalloc + k] = __float2bfloat16_rn(v);
  } else if (KIND == kTcFP16) {
    reinterpret_cast<__half*>(dst)[row * kalloc + k] = __float2half_rn(v);
  } else if (KIND == kTcBF16x3) {
    __nv_bfloat16* r = reinterpret_cast<__nv_bfloat16*>(dst) + row * 3 * kalloc + k;
    const __nv_bfloat16 p0 = __float2bfloat16_rn(v);
    const float r1 = v - __bfloat162float(p0);  // exact
    const __nv_bfloat16 p1 = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(p1);  // exact
    r[0] = p0;
    r[kalloc] = p1;
    r[2 * kalloc] = __float2bfloat16_rn(r2);
  } else {
    // TF32: round to nearest here (the MMA would drop the low 13 bits), so
    // the operand's unit roundoff is 2^-11, not 2^-10.
    unsigned t;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v));
    reinterpret_cast<unsigned*>(dst)[row * kalloc + k] = t;
  }
}

// Aop[i][k] = L21[i][k] * sa (k < w; zero up to kalloc), Bop[j][k] = U12[k][j] * sb.
template <int KIND>
__global__ void tc_convert_kernel(const float* __restrict__ a, int64_t lda, int k0, int w, int r1, int m, int c1, int n,
                                  void* aop, void* bop, int kalloc, const float* s) {
  __shared__ float tile[32][33];
  const float sa = s[2], sb = s[3];
  const int rowsA = m - r1, rowsB = n - c1;
  const int tilesA = (rowsA + 31) / 32;
  const int kt = (kalloc + 31) / 32;
  const int bid = blockIdx.x;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  if (bid < tilesA * kt) {
    const int ti = bid / kt, tk = bid - ti * kt;
    for (int rr = ty; rr < 32; rr += 8) {
      const int i = ti * 32 + rr, k = tk * 32 + tx;
      if (i < rowsA && k < kalloc) {
        const float v = (k < w) ? a[(int64_t)(r1 + i) * lda + k0 + k] * sa : 0.f;
        store_op<KIND>(aop, i, k, kalloc, v);
      }
    }
    return;
  }
  const int b2 = bid - tilesA * kt;
  const int tj = b2 / kt, tk = b2 - tj * kt;
  // read U12[k][j] for a 32 x 32 (k, j) tile, coalesced along j
  for (int kk = ty; kk < 32; kk += 8) {
    const int k = tk * 32 + kk, j = tj * 32 + tx;
    tile[kk][tx] = (k < w && j < rowsB) ? a[(int64_t)(k0 + k) * lda + c1 + j] * sb : 0.f;
  }
  __syncthreads();
  // write Bop[j][k], coalesced along k
  for (int jj = ty; jj < 32; jj += 8) {
    const int j = tj * 32 + jj, k = tk * 32 + tx;
    if (j < rowsB && k < kalloc) store_op<KIND>(bop, j, k, kalloc, tile[tx][jj]);
  }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
EncodeTiledFn encode_fn() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

int tc_kalloc(int kind, int w) {
  const int kbox = kind == kTcTF32 ? 32 : 64;
  return (w + kbox - 1) / kbox * kbox;
}

size_t tc_operand_bytes(int kind, int rows, int w) {
  const int pieces = kind == kTcBF16x3 ? 3 : 1;
  return (size_t)rows * pieces * tc_kalloc(kind, w) * (kind == kTcTF32 ? 4 : 2);
}

static int make_map(luhot_ctx* ctx, CUtensorMap* m, void* ptr, int kind, int rows, int kalloc) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return set_error(ctx, LUHOT_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is unavailable");
  const int es = kind == kTcTF32 ? 4 : 2;
  const CUtensorMapDataType dt = kind == kTcTF32                        ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                 : (kind == kTcBF16 || kind == kTcBF16x3) ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                                                                        : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
  const int row_elems = kind == kTcBF16x3 ? 3 * kalloc : kalloc;
  cuuint64_t dims[2] = {(cuuint64_t)row_elems, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)row_elems * es};
  cuuint32_t box[2] = {(cuuint32_t)(128 / es), 128};
  cuuint32_t estr[2] = {1, 1};
  const CUresult r = enc(m, dt, 2, ptr, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                         CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(ctx, LUHOT_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return LUHOT_OK;
}

// C (M x N FP32, row stride ldc) as the target of 128-row x 32-column
// reduce-add boxes, 128-byte swizzled like the staging blocks.
static int make_c_map(luhot_ctx* ctx, CUtensorMap* m, float* c, int M, int N, int64_t ldc) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return set_error(ctx, LUHOT_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is unavailable");
  cuuint64_t dims[2] = {(cuuint64_t)N, (cuuint64_t)M};
  cuuint64_t strides[1] = {(cuuint64_t)ldc * 4};
  cuuint32_t box[2] = {32, 128};
  cuuint32_t estr[2] = {1, 1};
  const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, c, dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(ctx, LUHOT_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return LUHOT_OK;
}

// a[r1.., c1..] (M = m - r1 rows, N = n - c1 columns) -= a[r1.., k0..k0+w] a[k0..k0+w, c1..]
template <int KIND>
static int launch_tc(luhot_ctx* ctx, float* a, int64_t lda, int k0, int w, int r1, int m, int c1, int n, void* aop,
                     void* bop, float* scal, cudaStream_t stream) {
  const int M = m - r1, N = n - c1;
  if (M <= 0 || N <= 0 || w <= 0) return LUHOT_OK;
  const int kalloc = tc_kalloc(KIND, w);
  {
    // The one-tile fallback (unaligned C) stages all of K in shared memory:
    // past 128 it takes the update in two halves.
    float* cb = a + (int64_t)r1 * lda + c1;
    const bool aligned = (lda % 4 == 0) && (reinterpret_cast<uintptr_t>(cb) % 16 == 0);
    if (!(aligned && TcShape<KIND>::kSmem <= (size_t)ctx->max_smem_optin) && w > 128) {
      int rc = launch_tc<KIND>(ctx, a, lda, k0, 128, r1, m, c1, n, aop, bop, scal, stream);
      if (rc) return rc;
      return launch_tc<KIND>(ctx, a, lda, k0 + 128, w - 128, r1, m, c1, n, aop, bop, scal, stream);
    }
  }
  // scales
  LUHOT_CUDA_TRY(ctx, cudaMemsetAsync(scal, 0, 8 * sizeof(float), stream));
  prof_begin(ctx, kProfGemm);
  tc_absmax_kernel<<<std::min(ctx->num_sms * 4, (int)(((int64_t)M * w + (int64_t)w * N + 255) / 256)), 256, 0, stream>>>(
      a, lda, k0, w, r1, m, c1, n, scal);
  prof_end(ctx, kProfGemm, 0.0, 4.0 * ((double)M * w + (double)w * N));
  tc_scales_kernel<<<1, 1, 0, stream>>>(scal);
  count_launch(ctx);
  const int kt = (kalloc + 31) / 32;
  const int blocks = ((M + 31) / 32) * kt + ((N + 31) / 32) * kt;
  prof_begin(ctx, kProfGemm);
  tc_convert_kernel<KIND><<<blocks, 256, 0, stream>>>(a, lda, k0, w, r1, m, c1, n, aop, bop, kalloc, scal);
  prof_end(ctx, kProfGemm, 0.0, (4.0 + (KIND == kTcTF32 ? 4 : 2)) * ((double)M + N) * kalloc);
  LUHOT_CUDA_TRY(ctx, cudaGetLastError());
  CUtensorMap tA, tB;
  int rc = make_map(ctx, &tA, aop, KIND, M, kalloc);
  if (rc) return rc;
  rc = make_map(ctx, &tB, bop, KIND, N, kalloc);
  if (rc) return rc;
  float* cbase = a + (int64_t)r1 * lda + c1;
  const bool c_aligned = (lda % 4 == 0) && (reinterpret_cast<uintptr_t>(cbase) % 16 == 0);
  if (c_aligned && TcShape<KIND>::kSmem <= (size_t)ctx->max_smem_optin) {
    CUtensorMap tC;
    rc = make_c_map(ctx, &tC, cbase, M, N, lda);
    if (rc) return rc;
    auto kern = tc_gemm_persistent_kernel<KIND>;
    LUHOT_CUDA_TRY(ctx, allow_max_dynamic_smem(kern));
    const int tiles = ((M + 127) / 128) * ((N + 127) / 128);
    const int cap = ctx->tc_grid_cap > 0 ? std::min(ctx->tc_grid_cap, ctx->num_sms) : ctx->num_sms;
    prof_begin(ctx, kProfGemm);
    kern<<<std::min(tiles, cap), kTcThreads, TcShape<KIND>::kSmem, stream>>>(tA, tB, tC, M, N, kalloc, scal + 4,
                                                                           ctx->d_status);
  } else {
    const int kbox = KIND == kTcTF32 ? 32 : 64;
    const size_t smem = KIND == kTcBF16x3 ? 1024 + 6 * 16384 : 1024 + (size_t)(kalloc / kbox) * 2 * 16384;
    auto kern = KIND == kTcBF16x3 ? tc_gemm_x3_kernel : tc_gemm_kernel<KIND>;
    LUHOT_CUDA_TRY(ctx, allow_max_dynamic_smem(kern));
    dim3 grid((N + 127) / 128, (M + 127) / 128);
    prof_begin(ctx, kProfGemm);
    kern<<<grid, 128, smem, stream>>>(tA, tB, cbase, lda, M, N, w, scal + 4, ctx->d_status);
  }
  prof_end(ctx, kProfGemm, 2.0 * M * (double)N * w,
           8.0 * M * (double)N + (double)(M + N) * kalloc * (KIND == kTcTF32 ? 4 : KIND == kTcBF16x3 ? 6 : 2));
  LUHOT_CUDA_TRY(ctx, cudaGetLastError());
  return LUHOT_OK;
}

int tc_gemm_update(luhot_ctx* ctx, int kind, float* a, int64_t lda, int k0, int w, int r1, int m, int c1, int n,
                   void* aop, void* bop, float* scal, cudaStream_t stream) {
  switch (kind) {
    case kTcBF16: return launch_tc<kTcBF16>(ctx, a, lda, k0, w, r1, m, c1, n, aop, bop, scal, stream);
    case kTcFP16: return launch_tc<kTcFP16>(ctx, a, lda, k0, w, r1, m, c1, n, aop, bop, scal, stream);
    case kTcTF32: return launch_tc<kTcTF32>(ctx, a, lda, k0, w, r1, m, c1, n, aop, bop, scal, stream);
    case kTcBF16x3: return launch_tc<kTcBF16x3>(ctx, a, lda, k0, w, r1, m, c1, n, aop, bop, scal, stream);
    default: return set_error(ctx, LUHOT_ERR_INVALID_ARG, "unknown tensor-core operand kind");
  }
}

int tc_schur_update(luhot_ctx* ctx, int kind, float* a, int64_t lda, int k0, int w, int m, int n, void* aop, void* bop,
                    float* scal, cudaStream_t stream) {
  return tc_gemm_update(ctx, kind, a, lda, k0, w, k0 + w, m, k0 + w, n, aop, bop, scal, stream);
}

}  // namespace luhot
