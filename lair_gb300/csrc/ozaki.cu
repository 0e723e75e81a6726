// FP64 Schur update on the FP16 tensor cores (Ozaki scheme).
//
//   C (M x N, FP64, row-major, ldc)  -=  L (M x K) U (K x N),   K <= 64
//
// This part runs FP64 at about 2 FMA per clock per SM and FP16 tensor-core
// products at 4096 per clock, so fast-mode FP64 trailing updates are computed
// as exact integer products on the tensor cores:
//
// Split (oz_split_rows_kernel for L, oz_split_cols_kernel for U).  Row i of L
//   gets the exponent ea[i] with max_k |L(i,k)| < 2^ea[i], column j of U the
//   exponent eb[j].  Each element x of a row (column) with exponent e is
//   rounded to the 56-bit integer N = round(|x| 2^(56-e)) and written as seven
//   balanced base-256 digits, most significant first:
//       x = sign(x) 2^e sum_{p=0..6} d_p 2^(-8(p+1))    (error <= 2^(e-57)),
//   d_0 in [-256, 256], d_1..d_6 in [-128, 128], every digit exact in FP16.
//   The digits of L are stored K-major per slice, As[p][i][k], those of U
//   transposed, Bs[p][j][k] (one 128-byte row per i or j: one TMA box row).
// Products (oz_gemm_kernel).  With A_p, B_q the digit matrices,
//       L U = 2^(ea+eb) sum_G T_G 2^(-8(G+2)),   T_G = sum_{p+q=G} A_p B_q^T,
//   kept for G = 0..7 (34 slice products of the 49).  Every partial sum of
//   T_G is an integer of magnitude below 9 * 2^20 for K <= 64, so the FP32
//   accumulation in TMEM is exact.  Dropped groups (G >= 8) weigh less than
//   2^-57 of 2^(ea+eb), the element roundings 2^-57 of each operand's scale:
//   the product error is of order K 2^(ea+eb-56), inside FP64's own bound for
//   a K-term dot product (measured on N(0,1) factors: 2.3e-16 of |L||U|
//   against 4.2e-16 for a plain FP64 GEMM).
// Combine (epilogue).  R = sum_G T_G 2^(38-8G) in 64-bit fixed point, formed by
//   Horner from G = 7 down (each step truncates below 2^-38 of T_0's unit;
//   |R| < 2^62), then C = fma(R, -2^(ea+eb-54), C): one rounding of R to 53
//   bits and one of the subtraction.  Rows or columns holding Inf or NaN give
//   NaN in the elements they touch.
//
// oz_gemm_kernel: persistent, one CTA per SM, 128 x 64 output tiles in row
// order, a contiguous range per CTA.  Ten warps:
//   warp 0      TMA producer: the seven 128-row A slices of the CTA's current
//               row block (112 KB, reloaded when the row block changes) and a
//               two-stage ring of the seven 64-row B slices of each tile
//               (56 KB per stage), 3-D tensor maps (k, row, slice), 128-byte
//               swizzle, rows past M or N zero-filled;
//   warp 1      TMEM owner (512 columns: one 64-column FP32 accumulator per
//               group) and MMA issuer: per tile and group G (7 down to 0) the
//               group's slice products, 4 k-steps of M=128, N=64, K=16 each,
//               then a commit to that group's full barrier;
//   warps 2-9   epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (tile
//               rows) and 32 of the 64 columns ((w - 2) / 4); it drains each
//               group as soon as it is complete and releases it, so the next
//               tile's MMAs on that group overlap this tile's combine.
// All mbarrier waits are bounded by the context's wait limit; on expiry a role
// records the error and raises the CTA's abort flag, the others stop at their
// next wait, and before exit the CTA waits (bounded) for its copies and MMAs
// in flight and frees TMEM.
#include <cuda.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <string>

#include "common.cuh"
#include "luhot_internal.h"
#include "ozaki.cuh"
#include "tcgen05.cuh"

namespace luhot {

constexpr int kOzSlices = 7;
constexpr int kOzGroups = 8;   // G = p + q = 0 .. 7
constexpr int kOzK = 64;       // K of one update (one 128-byte box row of FP16)
constexpr int kOzBM = 128, kOzBN = 64;
constexpr int kOzFrac = 38;    // fractional bits of the fixed-point combine
constexpr int kOzEpiWarps = 8;
constexpr int kOzThreads = 64 + 32 * kOzEpiWarps;
constexpr int kOzABytes = kOzBM * 128;  // one A slice box: 128 rows x 128 B
constexpr int kOzBBytes = kOzBN * 128;  // one B slice box: 64 rows x 128 B
constexpr int kOzStages = 2;
constexpr size_t kOzSmem = 1024 + (size_t)kOzSlices * kOzABytes + (size_t)kOzStages * kOzSlices * kOzBBytes;
constexpr int kOzNonFinite = 1 << 20;  // exponent of a row / column that holds Inf or NaN
constexpr int kOzZero = -(1 << 20);    // exponent of a zero element
static_assert(kOzGroups * kOzBN <= 512, "one TMEM accumulator per group");

// ---------------------------------------------------------------------------
// Split.
// ---------------------------------------------------------------------------

// The e of frexp(x) (|x| < 2^e, |x| >= 2^(e-1)) from the bits; kOzZero for
// zeros, kOzNonFinite for Inf and NaN.
__device__ __forceinline__ int oz_exponent(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const int E = (int)((u >> 52) & 0x7ff);
  const unsigned long long m = u & 0xFFFFFFFFFFFFFull;
  if (E == 0x7ff) return kOzNonFinite;
  if (E != 0) return E - 1022;
  if (m == 0) return kOzZero;
  return (64 - __clzll((long long)m)) - 1074;
}

// Seven balanced base-256 digits of round(|x| 2^(56-e)), signed like x, most
// significant first; |x| < 2^e.  Integer arithmetic only.
__device__ __forceinline__ void oz_digits(double x, int e, int (&d)[kOzSlices]) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const int E = (int)((u >> 52) & 0x7ff);
  unsigned long long m = u & 0xFFFFFFFFFFFFFull;
  int ex = -1074;
  if (E != 0) {
    m |= 1ull << 52;
    ex = E - 1075;
  }
  // |x| = m 2^ex < 2^e, so m 2^(ex - e + 56) < 2^56.
  const int sh = ex - e + 56;
  unsigned long long N;
  if (m == 0 || sh <= -64)
    N = 0;
  else if (sh >= 0)
    N = m << sh;
  else
    N = (m + (1ull << (-sh - 1))) >> (-sh);  // round half up; m < 2^53, so no overflow
  int carry = 0;
#pragma unroll
  for (int p = kOzSlices - 1; p >= 1; --p) {
    const int v = (int)(N & 255u) + carry;
    N >>= 8;
    carry = v >= 128 ? 1 : 0;
    d[p] = v - (carry << 8);
  }
  d[0] = (int)N + carry;  // N < 2^8 here: d_0 <= 256
  if (u >> 63) {
#pragma unroll
    for (int p = 0; p < kOzSlices; ++p) d[p] = -d[p];
  }
}

// One warp writes the digits of a 64-element row (x0 = element lane, x1 =
// element lane + 32) with the warp-reduced exponent e into slice rows
// dst[p * slice + 0..63].
__device__ __forceinline__ void oz_emit_row(double x0, double x1, int e, __half* __restrict__ dst, int64_t slice,
                                            int lane) {
  int d0[kOzSlices], d1[kOzSlices];
  if (e == kOzZero || e >= kOzNonFinite) {
#pragma unroll
    for (int p = 0; p < kOzSlices; ++p) d0[p] = d1[p] = 0;
  } else {
    oz_digits(x0, e, d0);
    oz_digits(x1, e, d1);
  }
#pragma unroll
  for (int p = 0; p < kOzSlices; ++p) {
    dst[p * slice + lane] = __int2half_rn(d0[p]);
    dst[p * slice + lane + 32] = __int2half_rn(d1[p]);
  }
}

__device__ __forceinline__ int oz_warp_max(int v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, off));
  return v;
}

// Rows r1 .. r1 + M - 1, columns k0 .. k0 + w - 1 of the row-major a (w <= 64):
// As[p][i][k] (zero for k >= w), ea[i].  One warp per row.
__global__ void __launch_bounds__(256) oz_split_rows_kernel(const double* __restrict__ a, int64_t lda, int r1, int M,
                                                            int k0, int w, __half* __restrict__ as,
                                                            int* __restrict__ ea) {
  const int i = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (i >= M) return;
  const double* row = a + (int64_t)(r1 + i) * lda + k0;
  const double x0 = lane < w ? row[lane] : 0.0;
  const double x1 = lane + 32 < w ? row[lane + 32] : 0.0;
  const int e = oz_warp_max(max(oz_exponent(x0), oz_exponent(x1)));
  oz_emit_row(x0, x1, e, as + (int64_t)i * kOzK, (int64_t)M * kOzK, lane);
  if (lane == 0) ea[i] = e == kOzZero ? 0 : e;
}

// Rows k0 .. k0 + w - 1 (w <= 64), columns c1 .. c1 + N - 1 of the row-major
// a: Bs[p][j][k] (the transpose; zero for k >= w), eb[j].  A CTA stages 64 x 32
// elements through shared memory (coalesced reads along the rows), then each
// warp splits four columns.
__global__ void __launch_bounds__(256) oz_split_cols_kernel(const double* __restrict__ a, int64_t lda, int k0, int w,
                                                            int c1, int N, __half* __restrict__ bs,
                                                            int* __restrict__ eb) {
  __shared__ double tile[kOzK][33];
  const int j0 = blockIdx.x * 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = warp; k < kOzK; k += 8) {
    const int j = j0 + lane;
    tile[k][lane] = (k < w && j < N) ? a[(int64_t)(k0 + k) * lda + c1 + j] : 0.0;
  }
  __syncthreads();
  for (int jj = warp; jj < 32; jj += 8) {
    const int j = j0 + jj;
    if (j >= N) break;
    const double x0 = tile[lane][jj], x1 = tile[lane + 32][jj];
    const int e = oz_warp_max(max(oz_exponent(x0), oz_exponent(x1)));
    oz_emit_row(x0, x1, e, bs + (int64_t)j * kOzK, (int64_t)N * kOzK, lane);
    if (lane == 0) eb[j] = e == kOzZero ? 0 : e;
  }
}

// ---------------------------------------------------------------------------
// Products and combine.
// ---------------------------------------------------------------------------

__device__ __forceinline__ void oz_abort(DeviceStatus* st, int* s_abort) {
  atomicCAS(&st->error, kDevOk, kDevBarrierTimeout);
  atomicExch(&st->abort, 1);
  atomicExch(s_abort, 1);
}

// Bounded mbarrier wait that also gives up once the CTA's abort flag is up.
__device__ __forceinline__ bool oz_wait(unsigned bar, unsigned parity, unsigned long long limit_ns,
                                        const int* s_abort) {
  const unsigned long long t0 = global_timer_ns();
  for (unsigned spins = 0;; ++spins) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if ((spins & 15u) == 15u) {
      if (*reinterpret_cast<const volatile int*>(s_abort)) return false;
      if (global_timer_ns() - t0 > limit_ns) return false;
    }
  }
}

__device__ __forceinline__ void oz_tma3d(unsigned dst, const CUtensorMap* map, int y, int z, unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          dst),
      "l"(map), "r"(0), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void oz_commit(unsigned bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// C - R 2^s for the fixed-point R; NaN when a row or column held Inf / NaN.
__device__ __forceinline__ double oz_combine(long long R, int ea_i, int eb_j, double c) {
  if (ea_i >= kOzNonFinite || eb_j >= kOzNonFinite) return __longlong_as_double(0x7ff8000000000000ll);
  const int s = ea_i + eb_j - (kOzFrac + 16);
  const double r = __ll2double_rn(R);
  if (s >= -1022 && s <= 1023) return fma(r, -__longlong_as_double((long long)(s + 1023) << 52), c);
  return c - scalbn(r, s);
}

__global__ void __launch_bounds__(kOzThreads, 1)
    oz_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   double* __restrict__ c, int64_t ldc, int M, int N, const int* __restrict__ ea,
                   const int* __restrict__ eb, int vec, DeviceStatus* st) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* sA = base;
  unsigned char* sB = base + (size_t)kOzSlices * kOzABytes;
  __shared__ __align__(8) unsigned long long a_full, a_empty, b_full[kOzStages], b_empty[kOzStages],
      g_full[kOzGroups], g_empty[kOzGroups], mma_done;
  __shared__ unsigned tmem_base;
  __shared__ int s_abort, s_a_issued, s_a_consumed, s_b_issued, s_b_consumed;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned long long limit = st->timeout_ns;
  const int tiles_n = (N + kOzBN - 1) / kOzBN;
  const int tiles = ((M + kOzBM - 1) / kOzBM) * tiles_n;
  const int t_begin = (int)((int64_t)blockIdx.x * tiles / gridDim.x);
  const int t_end = (int)((int64_t)(blockIdx.x + 1) * tiles / gridDim.x);

  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&tmem_base)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&a_full)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&a_empty)));
    for (int s = 0; s < kOzStages; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&b_full[s])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&b_empty[s])));
    }
    for (int g = 0; g < kOzGroups; ++g) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&g_full[g])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&g_empty[g])), "r"(kOzEpiWarps));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mma_done)));
    s_abort = 0;
    s_a_issued = s_a_consumed = s_b_issued = s_b_consumed = 0;
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
      int cur_rb = -1, na = 0, nb = 0;
      for (int t = t_begin; t < t_end; ++t) {
        if (*reinterpret_cast<volatile int*>(&s_abort)) break;
        const int rb = t / tiles_n, cb = t - rb * tiles_n;
        if (rb != cur_rb) {
          // The previous row block's slices are free once its last MMAs end.
          if (na > 0 && !oz_wait(smem_u32(&a_empty), (unsigned)((na - 1) & 1), limit, &s_abort)) {
            oz_abort(st, &s_abort);
            break;
          }
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&a_full)),
                       "r"((unsigned)(kOzSlices * kOzABytes))
                       : "memory");
          for (int p = 0; p < kOzSlices; ++p)
            oz_tma3d(smem_u32(sA + p * kOzABytes), &tmA, rb * kOzBM, p, smem_u32(&a_full));
          s_a_issued = ++na;
          cur_rb = rb;
        }
        const int s = nb % kOzStages;
        if (!oz_wait(smem_u32(&b_empty[s]), (unsigned)((nb / kOzStages) & 1) ^ 1u, limit, &s_abort)) {
          oz_abort(st, &s_abort);
          break;
        }
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&b_full[s])),
                     "r"((unsigned)(kOzSlices * kOzBBytes))
                     : "memory");
        unsigned char* sb = sB + (size_t)s * kOzSlices * kOzBBytes;
        for (int p = 0; p < kOzSlices; ++p)
          oz_tma3d(smem_u32(sb + p * kOzBBytes), &tmB, cb * kOzBN, p, smem_u32(&b_full[s]));
        s_b_issued = ++nb;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer: D FP32 (bit 4), A and B FP16 (format 0), K-major, N = 64, M = 128.
      constexpr unsigned idesc = (1u << 4) | ((unsigned)(kOzBN >> 3) << 17) | ((unsigned)(kOzBM >> 4) << 24);
      int cur_rb = -1, na = 0, nb = 0, tc = 0;
      bool ok = true;
      for (int t = t_begin; t < t_end && ok; ++t, ++tc) {
        if (*reinterpret_cast<volatile int*>(&s_abort)) break;
        const int rb = t / tiles_n;
        if (rb != cur_rb) {
          if (!oz_wait(smem_u32(&a_full), (unsigned)(na & 1), limit, &s_abort)) {
            ok = false;
            break;
          }
          s_a_consumed = ++na;
          cur_rb = rb;
        }
        const int s = nb % kOzStages;
        if (!oz_wait(smem_u32(&b_full[s]), (unsigned)((nb / kOzStages) & 1), limit, &s_abort)) {
          ok = false;
          break;
        }
        s_b_consumed = ++nb;
        asm volatile("tcgen05.fence::after_thread_sync;");
        const unsigned char* sb = sB + (size_t)s * kOzSlices * kOzBBytes;
        for (int G = kOzGroups - 1; G >= 0; --G) {
          // The epilogue has drained this group of the previous tile.
          if (!oz_wait(smem_u32(&g_empty[G]), (unsigned)(tc & 1) ^ 1u, limit, &s_abort)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const unsigned acc_addr = tmem + (unsigned)(G * kOzBN);
          unsigned accf = 0;
          for (int p = max(0, G - (kOzSlices - 1)); p <= min(G, kOzSlices - 1); ++p) {
            const int q = G - p;
#pragma unroll
            for (int ks = 0; ks < kOzK / 16; ++ks) {
              const unsigned long long da = sw128_desc(smem_u32(sA + p * kOzABytes + ks * 32));
              const unsigned long long db = sw128_desc(smem_u32(sb + q * kOzBBytes + ks * 32));
              asm volatile(
                  "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, "
                  "p;\n}\n" ::"r"(acc_addr),
                  "l"(da), "l"(db), "r"(idesc), "r"(accf));
              accf = 1;
            }
          }
          oz_commit(smem_u32(&g_full[G]));
        }
        if (!ok) break;
        oz_commit(smem_u32(&b_empty[s]));
        const bool row_ends = (t + 1 >= t_end) || ((t + 1) / tiles_n != rb);
        if (row_ends) oz_commit(smem_u32(&a_empty));
      }
      if (!ok) oz_abort(st, &s_abort);
      // Arrives once every MMA issued above has completed.
      oz_commit(smem_u32(&mma_done));
      mbar_wait(smem_u32(&mma_done), 0u, limit);
    }
  } else {
    // Epilogue.
    const int quarter = warp & 3, half = (warp - 2) >> 2;
    int tc = 0;
    for (int t = t_begin; t < t_end; ++t, ++tc) {
      const int rb = t / tiles_n, cb = t - rb * tiles_n;
      long long R[32];
      bool ok = true;
      for (int G = kOzGroups - 1; G >= 0; --G) {
        const bool got = oz_wait(smem_u32(&g_full[G]), (unsigned)(tc & 1), limit, &s_abort);
        if (!__all_sync(0xffffffffu, got)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        unsigned r[32];
        const unsigned taddr = tmem + ((unsigned)(quarter * 32) << 16) + (unsigned)(G * kOzBN + half * 32);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,"
            "%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
              "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&g_empty[G]));
        if (G == kOzGroups - 1) {
#pragma unroll
          for (int j = 0; j < 32; ++j) R[j] = (long long)__float2int_rn(__uint_as_float(r[j])) << kOzFrac;
        } else {
#pragma unroll
          for (int j = 0; j < 32; ++j)
            R[j] = ((long long)__float2int_rn(__uint_as_float(r[j])) << kOzFrac) + (R[j] >> 8);
        }
      }
      if (!ok) {
        if (lane == 0) oz_abort(st, &s_abort);
        break;
      }
      const int row = rb * kOzBM + quarter * 32 + lane;
      const int col0 = cb * kOzBN + half * 32;
      if (row < M) {
        const int ea_i = ea[row];
        double* crow = c + (int64_t)row * ldc + col0;
        if (vec && col0 + 32 <= N) {
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            const int2 e2 = *reinterpret_cast<const int2*>(eb + col0 + 2 * q);
            double2 v = *reinterpret_cast<const double2*>(crow + 2 * q);
            v.x = oz_combine(R[2 * q], ea_i, e2.x, v.x);
            v.y = oz_combine(R[2 * q + 1], ea_i, e2.y, v.y);
            *reinterpret_cast<double2*>(crow + 2 * q) = v;
          }
        } else {
#pragma unroll
          for (int j = 0; j < 32; ++j)
            if (col0 + j < N) crow[j] = oz_combine(R[j], ea_i, eb[col0 + j], crow[j]);
        }
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_abort) {
    // Copies issued but never consumed must land before the CTA exits.
    if (s_a_issued > s_a_consumed) mbar_wait(smem_u32(&a_full), (unsigned)((s_a_issued - 1) & 1), limit);
    for (int i = s_b_consumed; i < s_b_issued; ++i)
      mbar_wait(smem_u32(&b_full[i % kOzStages]), (unsigned)((i / kOzStages) & 1), limit);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
static size_t oz_round(size_t b) { return (b + 1023) / 1024 * 1024; }

size_t ozaki_workspace_bytes(int m, int n) {
  return oz_round((size_t)kOzSlices * m * kOzK * 2) + oz_round((size_t)kOzSlices * n * kOzK * 2) +
         oz_round((size_t)m * 4) + oz_round((size_t)n * 4);
}

bool ozaki_available(luhot_ctx* ctx) { return kOzSmem <= (size_t)ctx->max_smem_optin && encode_fn() != nullptr; }

// Slices [7][rows][64] FP16 as a 3-D tensor map (k, row, slice) with boxes of
// 64 x box_rows x 1 (128-byte rows, 128-byte swizzle); rows past `rows` read
// as zero.
static int make_slice_map(luhot_ctx* ctx, CUtensorMap* map, void* ptr, int rows, int box_rows) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return set_error(ctx, LUHOT_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is unavailable");
  cuuint64_t dims[3] = {(cuuint64_t)kOzK, (cuuint64_t)rows, (cuuint64_t)kOzSlices};
  cuuint64_t strides[2] = {(cuuint64_t)kOzK * 2, (cuuint64_t)rows * kOzK * 2};
  cuuint32_t box[3] = {(cuuint32_t)kOzK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, ptr, dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(ctx, LUHOT_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return LUHOT_OK;
}

int ozaki_update(luhot_ctx* ctx, double* a, int64_t lda, int k0, int w, int r1, int m, int c1, int n, void* ws,
                 cudaStream_t stream) {
  const int M = m - r1, N = n - c1;
  if (M <= 0 || N <= 0 || w <= 0) return LUHOT_OK;
  if (w > kOzK) {
    int rc = ozaki_update(ctx, a, lda, k0, kOzK, r1, m, c1, n, ws, stream);
    if (rc) return rc;
    return ozaki_update(ctx, a, lda, k0 + kOzK, w - kOzK, r1, m, c1, n, ws, stream);
  }
  char* p = static_cast<char*>(ws);
  __half* as = reinterpret_cast<__half*>(p);
  p += oz_round((size_t)kOzSlices * M * kOzK * 2);
  __half* bs = reinterpret_cast<__half*>(p);
  p += oz_round((size_t)kOzSlices * N * kOzK * 2);
  int* ea = reinterpret_cast<int*>(p);
  p += oz_round((size_t)M * 4);
  int* eb = reinterpret_cast<int*>(p);

  prof_begin(ctx, kProfOther);
  oz_split_rows_kernel<<<(M + 7) / 8, 256, 0, stream>>>(a, lda, r1, M, k0, w, as, ea);
  prof_end(ctx, kProfOther, 0.0, (double)M * w * 8 + (double)M * kOzK * kOzSlices * 2);
  prof_begin(ctx, kProfOther);
  oz_split_cols_kernel<<<(N + 31) / 32, 256, 0, stream>>>(a, lda, k0, w, c1, N, bs, eb);
  prof_end(ctx, kProfOther, 0.0, (double)N * w * 8 + (double)N * kOzK * kOzSlices * 2);
  LUHOT_CUDA_TRY(ctx, cudaGetLastError());

  CUtensorMap tmA, tmB;
  int rc = make_slice_map(ctx, &tmA, as, M, kOzBM);
  if (!rc) rc = make_slice_map(ctx, &tmB, bs, N, kOzBN);
  if (rc) return rc;
  double* cb = a + (int64_t)r1 * lda + c1;
  const int vec = (lda % 2 == 0) && (reinterpret_cast<uintptr_t>(cb) % 16 == 0) ? 1 : 0;
  const int tiles = ((M + kOzBM - 1) / kOzBM) * ((N + kOzBN - 1) / kOzBN);
  LUHOT_CUDA_TRY(ctx, allow_max_dynamic_smem(oz_gemm_kernel));
  prof_begin(ctx, kProfGemm);
  oz_gemm_kernel<<<std::min(tiles, ctx->num_sms), kOzThreads, kOzSmem, stream>>>(tmA, tmB, cb, lda, M, N, ea, eb, vec,
                                                                                ctx->d_status);
  // algorithmic work: 2MNK FP64 flops; bytes: C read + written, the slices read once
  prof_end(ctx, kProfGemm, 2.0 * M * N * w,
           (double)M * N * 16 + (double)(M + N) * kOzK * kOzSlices * 2 + (double)(M + N) * 4);
  LUHOT_CUDA_TRY(ctx, cudaGetLastError());
  return LUHOT_OK;
}

}  // namespace luhot
