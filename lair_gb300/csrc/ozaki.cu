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
//   kept for G = 0..6 (28 slice products of the 49).  Every partial sum of
//   T_G is an integer of magnitude below 9 * 2^20 for K <= 64, so the FP32
//   accumulation in TMEM is exact.  The dropped groups (G >= 7) weigh at most
//   2^-49.4 of 2^(ea+eb) (typically 2^-55), the element roundings 2^-57 of
//   each operand's scale: the product error stays well inside FP64's own
//   bound for a K-term dot product (measured on N(0,1) factors: 1.1e-16 of
//   |C| + |L||U| against 4.7e-16 for the FP64 tensor cores).
// Combine (epilogue).  R = sum_G T_G 2^(38-8G) in 64-bit fixed point, formed by
//   Horner from G = 6 down (each step truncates below 2^-38 of T_0's unit;
//   |R| < 2^62), then C = C - R 2^(ea+eb-54): one rounding of R to 53 bits
//   (built with integer operations) and one of the subtraction.  Rows or columns holding Inf or NaN give
//   NaN in the elements they touch.
//
// oz_gemm_kernel: persistent, one CTA per SM, 128 x 128 output tiles, a
// contiguous range per CTA in column-block order.  An M = 128 MMA costs the
// tensor pipe about the same time for any N up to 256 (measured: ~128 cycles
// at N = 64), so the tile is as wide as TMEM allows: three 128-column FP32
// accumulators and the low words of the tile's 64-bit fixed-point sums
// (512 columns).  The MMAs compute C^T: TMEM lanes are C's columns, so a
// warp's accesses to one row of C are 32 consecutive doubles.  Eighteen warps:
//   warp 0      TMA producer: the seven U slices of the CTA's current column
//               block (112 KB, reloaded when the column block changes) and
//               the seven L slices of each tile (112 KB), one barrier pair
//               per slice: L slice p is last read by group G = p, so the
//               slices free up in the order the next tile needs them (6 .. 0);
//               3-D tensor maps (k, row, slice), 128-byte swizzle, rows past M
//               or N zero-filled;
//   warp 1      TMEM owner (512 columns) and MMA issuer: per tile, groups
//               G = 6 .. 0, taking the three accumulators in turn over the
//               launch: the group's slice products, 4 k-steps of M = 128,
//               N = 128, K = 16 each, then a commit to that accumulator's full
//               barrier;
//   warps 2-17  epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (32
//               columns of C) and 32 of the tile's 128 rows ((w - 2) / 4); its
//               thread keeps the high words of its column's 32 sums in
//               registers and the low words in TMEM; per group it folds the
//               accumulator in (Horner on word pairs) and releases it, so the
//               MMAs of the next group (and of the next tile) overlap the
//               epilogue; after group 0 it applies the sums to C (C prefetched
//               into L2 at the tile's start; one FP64 subtraction per element).
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
constexpr int kOzGroups = 7;   // G = p + q = 0 .. 6
constexpr int kOzK = 64;       // K of one update (one 128-byte box row of FP16)
constexpr int kOzBM = 128, kOzBN = 128;
constexpr int kOzFrac = 38;    // fractional bits of the fixed-point combine
constexpr int kOzEpiWarps = 16;
constexpr int kOzThreads = 64 + 32 * kOzEpiWarps;
constexpr int kOzSliceBytes = 128 * 128;  // one slice box: 128 rows x 128 B
constexpr int kOzAccBufs = 3;           // TMEM accumulators of 128 columns, used in turn by the groups
constexpr unsigned kOzLoCol = 384;      // TMEM columns 384-511: low words of the fixed-point sums
constexpr size_t kOzSmem = 1024 + 2 * (size_t)kOzSlices * kOzSliceBytes;
constexpr int kOzNonFinite = 1 << 20;  // exponent of a row / column that holds Inf or NaN
constexpr int kOzZero = -(1 << 20);    // exponent of a zero element
static_assert(kOzAccBufs * kOzBM <= (int)kOzLoCol && kOzLoCol + kOzBM <= 512, "accumulators and sums fit in TMEM");

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

// U12 = L11^-1 A12 as a product: U12 = A12 - N A12 with N = I - L11^-1
// (strictly lower).  oz_trsm_inverse_kernel forms N for the unit lower
// triangular L11 = a[k0.., k0..] (w x w, w <= 64) into nb (128 x 64,
// row-major; rows >= w and columns >= w zero), one CTA per column c: warp 0
// holds x = L11^-1 e_c (rows lane and lane + 32) and runs the column sweep
// x_i -= L(i,k) x_k for i > k, k = c, c + 1, ... (x_k by shuffle), so each
// step costs one shuffle and two FMAs on this part's thin FP64 pipe; the
// CTA's four warps first stage L11 in shared memory.  oz_split_rows_kernel
// then writes N's digit slices like any L21.
constexpr int kOzInvLds = 65;
constexpr int kOzMapRows = 128;  // rows of the L-slice tensor map of the triangular solve

__global__ void __launch_bounds__(128) oz_trsm_inverse_kernel(const double* __restrict__ a, int64_t lda, int k0, int w,
                                                              double* __restrict__ nb) {
  __shared__ double L[kOzK * kOzInvLds];  // L[i * kOzInvLds + k] = L11(i, k) for k < i < w, else 0
  const int c = blockIdx.x, tid = threadIdx.x;
  for (int idx = tid; idx < kOzK * kOzK; idx += blockDim.x) {
    const int i = idx >> 6, k = idx & 63;
    L[i * kOzInvLds + k] = (i < w && k < i && k >= c) ? a[(int64_t)(k0 + i) * lda + k0 + k] : 0.0;
  }
  __syncthreads();
  if (tid >= 32) return;
  const int lane = tid;
  double x0 = lane == c ? 1.0 : 0.0, x1 = lane + 32 == c ? 1.0 : 0.0;
  for (int k = c; k < w - 1; ++k) {
    const double xk = __shfl_sync(0xffffffffu, k < 32 ? x0 : x1, k & 31);
    if (lane > k) x0 = fma(-L[lane * kOzInvLds + k], xk, x0);
    if (lane + 32 > k) x1 = fma(-L[(lane + 32) * kOzInvLds + k], xk, x1);
  }
  // N(i, c) = -x_i below the diagonal (the unit diagonal cancels), zero elsewhere
  nb[lane * kOzK + c] = (lane > c && lane < w && c < w) ? -x0 : 0.0;
  nb[(lane + 32) * kOzK + c] = (lane + 32 > c && lane + 32 < w && c < w) ? -x1 : 0.0;
  nb[(lane + 64) * kOzK + c] = 0.0;
  nb[(lane + 96) * kOzK + c] = 0.0;
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

// TMEM loads and stores of one warp: its 32 lanes, 4 or 16 consecutive
// 32-bit columns from taddr (lane field in bits 16+).
__device__ __forceinline__ void tmem_ld16(unsigned taddr, unsigned (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld4(unsigned taddr, unsigned (&r)[4]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
}
__device__ __forceinline__ void tmem_st16(unsigned taddr, const unsigned (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};"
      ::"r"(taddr), "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]),
        "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
      : "memory");
}

__device__ __forceinline__ void oz_commit(unsigned bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// C - R 2^s for the fixed-point R = hi 2^32 + lo (s = ea + eb - 54); NaN
// when a row or column held Inf or NaN.  R 2^s is rounded to 53 bits (to
// nearest, ties to even, as a conversion of R would).  oz_combine_fast
// assembles it with 32-bit integer operations whenever it is a normal number
// and |R| >= 2^32, so the FP64 pipe runs one subtraction per element; the
// rest (zeros, small sums, subnormal and overflowing products, non-finite
// rows or columns) go through oz_combine, rarely.
__device__ __noinline__ double oz_combine_rare(long long R, int s, double c) {
  const unsigned long long neg = R < 0 ? (1ull << 63) : 0ull;
  const unsigned long long u = R < 0 ? 0ull - (unsigned long long)R : (unsigned long long)R;
  if (u == 0) return __dsub_rn(c, 0.0);
  const int lz = __clzll((long long)u);
  const unsigned long long un = u << lz;
  unsigned long long m = un >> 11;
  const unsigned rem = (unsigned)(un & 0x7FF);
  int t = 63 - lz;
  m += (rem > 0x400u || (rem == 0x400u && (m & 1))) ? 1ull : 0ull;
  if (m >> 53) {
    m >>= 1;
    ++t;
  }
  const int E = t + s + 1023;
  const unsigned long long frac = m & 0xFFFFFFFFFFFFFull;
  if (E >= 1 && E <= 2046)
    return __dsub_rn(c, __longlong_as_double((long long)(neg | ((unsigned long long)E << 52) | frac)));
  if (E > 2046) return __dsub_rn(c, __longlong_as_double((long long)(neg | 0x7FF0000000000000ull)));
  // Below the normal range: the 53-bit value at exponent -1000 (exact), then
  // one multiplication by 2^d rounds it once, to the subnormal grid.
  const int d = E - 23;  // the value is (that number) x 2^d, d < -22
  if (d < -1074) return __dsub_rn(c, __longlong_as_double((long long)neg));
  const double mid = __longlong_as_double((long long)(neg | (23ull << 52) | frac));
  const double p2 = d >= -1022 ? __longlong_as_double((long long)(d + 1023) << 52)
                               : __longlong_as_double((long long)(1ull << (d + 1074)));
  return __dsub_rn(c, __dmul_rn(mid, p2));
}

// The common case of oz_combine: |R| >= 2^32 and a normal product.  s
// already holds ea + eb - 54 (huge when a row or column is non-finite).
// Returns false, leaving c alone, when the element needs oz_combine.
__device__ __forceinline__ bool oz_combine_fast(unsigned hi, unsigned lo, int s, double& c) {
  const unsigned sgn = (unsigned)((int)hi >> 31);  // 0 or ~0
  // |R| = (hi, lo) negated when negative: one's complement plus one, with carry.
  const unsigned xl = lo ^ sgn, xh = hi ^ sgn;
  const unsigned ul = xl - sgn;
  const unsigned uh = xh + ((sgn != 0u && ul == 0u) ? 1u : 0u);  // uh < 2^30
  const int lz = __clz((int)uh);
  const unsigned nh = __funnelshift_l(ul, uh, lz);  // leading one at bit 31 (when uh != 0)
  const unsigned nl = ul << lz;
  unsigned mh = nh >> 11, ml = __funnelshift_r(nl, nh, 11);  // 53 bits: mh has 21
  const unsigned rem = nl & 0x7FFu;
  const unsigned inc = (rem > 0x400u || (rem == 0x400u && (ml & 1u))) ? 1u : 0u;
  ml += inc;
  mh += (inc != 0u && ml == 0u) ? 1u : 0u;
  const int E = 63 - lz + (int)(mh >> 21) + s + 1023;
  if (uh == 0u || (unsigned)(E - 1) >= 2046u) return false;
  const unsigned dh = (sgn & 0x80000000u) | ((unsigned)E << 20) | (mh & 0xFFFFFu);
  c = __dsub_rn(c, __hiloint2double((int)dh, (int)ml));
  return true;
}

__device__ __forceinline__ double oz_combine(unsigned hi, unsigned lo, int ea_i, int eb_j, double c) {
  if (ea_i >= kOzNonFinite || eb_j >= kOzNonFinite) return __longlong_as_double(0x7ff8000000000000ll);
  return oz_combine_rare((long long)(((unsigned long long)hi << 32) | lo), ea_i + eb_j - (kOzFrac + 16), c);
}

__global__ void __launch_bounds__(kOzThreads, 1)
    oz_gemm_kernel(const __grid_constant__ CUtensorMap tmL, const __grid_constant__ CUtensorMap tmU,
                   double* __restrict__ c, int64_t ldc, int M, int N, const int* __restrict__ ea,
                   const int* __restrict__ eb, DeviceStatus* st) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* sU = base;                                    // resident: U^T slices of the column block
  unsigned char* sL = base + (size_t)kOzSlices * kOzSliceBytes;  // streamed: L slices of each tile's rows
  __shared__ __align__(8) unsigned long long u_full, u_empty, l_full[kOzSlices], l_empty[kOzSlices],
      acc_full[kOzAccBufs], acc_empty[kOzAccBufs], mma_done;
  __shared__ unsigned tmem_base;
  __shared__ int s_abort, s_u_issued, s_u_consumed, s_l_issued;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned long long limit = st->timeout_ns;
  const int tiles_i = (M + kOzBM - 1) / kOzBM;
  const int tiles = tiles_i * ((N + kOzBN - 1) / kOzBN);
  const int t_begin = (int)((int64_t)blockIdx.x * tiles / gridDim.x);
  const int t_end = (int)((int64_t)(blockIdx.x + 1) * tiles / gridDim.x);

  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&tmem_base)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&u_full)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&u_empty)));
    for (int p = 0; p < kOzSlices; ++p) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&l_full[p])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&l_empty[p])));
    }
    for (int b = 0; b < kOzAccBufs; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&acc_full[b])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&acc_empty[b])), "r"(kOzEpiWarps));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mma_done)));
    s_abort = 0;
    s_u_issued = s_u_consumed = s_l_issued = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
    asm volatile("fence.proxy.async.shared::cta;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const unsigned tmem = tmem_base;

  if (warp == 0) {
    if (lane == 0) {
      // Producer.  L slices go in the order the MMAs free them (6 .. 0).
      int cur_jb = -1, nu = 0, tc = 0;
      for (int t = t_begin; t < t_end; ++t, ++tc) {
        if (*reinterpret_cast<volatile int*>(&s_abort)) break;
        const int jb = t / tiles_i, ib = t - jb * tiles_i;
        if (jb != cur_jb) {
          // The previous column block's slices are free once its last MMAs end.
          if (nu > 0 && !oz_wait(smem_u32(&u_empty), (unsigned)((nu - 1) & 1), limit, &s_abort)) {
            oz_abort(st, &s_abort);
            break;
          }
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&u_full)),
                       "r"((unsigned)(kOzSlices * kOzSliceBytes))
                       : "memory");
          for (int q = 0; q < kOzSlices; ++q)
            oz_tma3d(smem_u32(sU + q * kOzSliceBytes), &tmU, jb * kOzBN, q, smem_u32(&u_full));
          s_u_issued = ++nu;
          cur_jb = jb;
        }
        bool ok = true;
        for (int p = kOzSlices - 1; p >= 0; --p) {
          if (!oz_wait(smem_u32(&l_empty[p]), (unsigned)(tc & 1) ^ 1u, limit, &s_abort)) {
            ok = false;
            break;
          }
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&l_full[p])),
                       "r"((unsigned)kOzSliceBytes)
                       : "memory");
          oz_tma3d(smem_u32(sL + p * kOzSliceBytes), &tmL, ib * kOzBM, p, smem_u32(&l_full[p]));
          ++s_l_issued;
        }
        if (!ok) {
          oz_abort(st, &s_abort);
          break;
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer: D FP32 (bit 4), A and B FP16 (format 0), K-major, M = N = 128.
      // D[j][i] += sum_k U^T_q[j][k] L_p[i][k]: TMEM lanes are columns of C.
      constexpr unsigned idesc = (1u << 4) | ((unsigned)(kOzBM >> 3) << 17) | ((unsigned)(kOzBN >> 4) << 24);
      int cur_jb = -1, nu = 0, tc = 0;
      bool ok = true;
      for (int t = t_begin; t < t_end && ok; ++t, ++tc) {
        if (*reinterpret_cast<volatile int*>(&s_abort)) break;
        const int jb = t / tiles_i;
        if (jb != cur_jb) {
          if (!oz_wait(smem_u32(&u_full), (unsigned)(nu & 1), limit, &s_abort)) {
            ok = false;
            break;
          }
          s_u_consumed = ++nu;
          cur_jb = jb;
        }
        unsigned have = 0;  // L slices of this tile already waited for
        for (int G = kOzGroups - 1; G >= 0 && ok; --G) {
          // The groups take the accumulators in turn over the whole launch:
          // group number i = 8 tc + 7 - G uses accumulator i % 3 for its use
          // i / 3; wait for the epilogue's release of the previous use.
          const int gi = kOzGroups * tc + kOzGroups - 1 - G;
          const int buf = gi % kOzAccBufs;
          const unsigned use_parity = (unsigned)((gi / kOzAccBufs) & 1);
          if (!oz_wait(smem_u32(&acc_empty[buf]), use_parity ^ 1u, limit, &s_abort)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const unsigned acc_addr = tmem + (unsigned)(buf * kOzBM);
          unsigned accf = 0;
          for (int p = max(0, G - (kOzSlices - 1)); p <= min(G, kOzSlices - 1); ++p) {
            const int q = G - p;
            if (!(have & (1u << p))) {
              if (!oz_wait(smem_u32(&l_full[p]), (unsigned)(tc & 1), limit, &s_abort)) {
                ok = false;
                break;
              }
              asm volatile("tcgen05.fence::after_thread_sync;");
              have |= 1u << p;
            }
#pragma unroll
            for (int ks = 0; ks < kOzK / 16; ++ks) {
              const unsigned long long da = sw128_desc(smem_u32(sU + q * kOzSliceBytes + ks * 32));
              const unsigned long long db = sw128_desc(smem_u32(sL + p * kOzSliceBytes + ks * 32));
              asm volatile(
                  "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, "
                  "p;\n}\n" ::"r"(acc_addr),
                  "l"(da), "l"(db), "r"(idesc), "r"(accf));
              accf = 1;
            }
          }
          if (!ok) break;
          oz_commit(smem_u32(&acc_full[buf]));
          // L slice G is last used by group G.
          if (G < kOzSlices) oz_commit(smem_u32(&l_empty[G]));
        }
        if (!ok) break;
        const bool block_ends = (t + 1 >= t_end) || ((t + 1) / tiles_i != jb);
        if (block_ends) oz_commit(smem_u32(&u_empty));
      }
      if (!ok) oz_abort(st, &s_abort);
      // Arrives once every MMA issued above has completed.
      oz_commit(smem_u32(&mma_done));
      mbar_wait(smem_u32(&mma_done), 0u, limit);
    }
  } else {
    // Epilogue: warp w owns TMEM lanes 32 (w % 4) .. + 31 (32 columns of the
    // tile) and 32 of its 128 rows, g = (w - 2) / 4.  Its thread keeps the
    // high words of its column's 32 fixed-point sums in registers and the low
    // words in TMEM (tile row r: column kOzLoCol + r); 16 rows of an
    // accumulator at a time pass through registers.
    const int quarter = warp & 3, rq = (warp - 2) >> 2;
    const unsigned lane_base = tmem + ((unsigned)(quarter * 32) << 16);
    const unsigned lo_base = lane_base + kOzLoCol + (unsigned)(rq * 32);
    int tc = 0;
    for (int t = t_begin; t < t_end; ++t, ++tc) {
      const int jb = t / tiles_i, ib = t - jb * tiles_i;
      const int col = jb * kOzBN + quarter * 32 + lane;
      const int row0 = ib * kOzBM + rq * 32;
      const bool col_ok = col < N;
      {
        // Bring this warp's 32 rows x 32 columns of C into L2 while the
        // tile's products run (lane r: row r, 256 bytes).
        const int c0 = jb * kOzBN + quarter * 32;
        if (c0 < N && row0 + lane < M) {
          const double* pr = c + (int64_t)(row0 + lane) * ldc + c0;
          asm volatile("prefetch.global.L2 [%0];" ::"l"(pr));
          if (c0 + 16 < N) asm volatile("prefetch.global.L2 [%0];" ::"l"(pr + 16));
        }
      }
      unsigned rh[32];
      bool ok = true;
      for (int G = kOzGroups - 1; G >= 0; --G) {
        const int gi = kOzGroups * tc + kOzGroups - 1 - G;
        const int buf = gi % kOzAccBufs;
        const unsigned use_parity = (unsigned)((gi / kOzAccBufs) & 1);
        const bool got = oz_wait(smem_u32(&acc_full[buf]), use_parity, limit, &s_abort);
        if (!__all_sync(0xffffffffu, got)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const unsigned acc = lane_base + (unsigned)(buf * kOzBM + rq * 32);
        if (G == kOzGroups - 1) {
          // First group: R = T 2^38.
#pragma unroll
          for (int cc = 0; cc < 2; ++cc) {
            unsigned tv[16], lv[16];
            tmem_ld16(acc + (unsigned)(cc * 16), tv);
            asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
            for (int r = 0; r < 16; ++r) {
              rh[cc * 16 + r] = (unsigned)(__float2int_rn(__uint_as_float(tv[r])) << (kOzFrac - 32));
              lv[r] = 0u;
            }
            tmem_st16(lo_base + (unsigned)(cc * 16), lv);
          }
        } else {
          // R = T 2^38 + floor(R / 2^8) on (hi, lo) words: T 2^38 only
          // touches hi (|R| < 2^62), so no carry crosses the words.
#pragma unroll
          for (int cc = 0; cc < 2; ++cc) {
            unsigned tv[16], lv[16];
            tmem_ld16(acc + (unsigned)(cc * 16), tv);
            tmem_ld16(lo_base + (unsigned)(cc * 16), lv);
            asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
            for (int r = 0; r < 16; ++r) {
              const unsigned hi = rh[cc * 16 + r];
              lv[r] = __funnelshift_r(lv[r], hi, 8);
              rh[cc * 16 + r] =
                  (unsigned)(((int)hi >> 8) + (__float2int_rn(__uint_as_float(tv[r])) << (kOzFrac - 32)));
            }
            tmem_st16(lo_base + (unsigned)(cc * 16), lv);
          }
        }
        // This warp has read the accumulator: the MMA warp may reuse it.
        asm volatile("tcgen05.wait::st.sync.aligned;");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&acc_empty[buf]));
      }
      if (!ok) {
        if (lane == 0) oz_abort(st, &s_abort);
        break;
      }
      // C -= the sums: thread = one column of C, its 32 rows in chunks of 4;
      // a warp's loads and stores of one row are 32 consecutive doubles.
      // Lane r holds the exponent of row r.  Elements the fast path declines
      // (rare) are redone, warp-uniformly, by the general path.
      const int eb_j = col_ok ? eb[col] : 0;
      const int my_ea = row0 + lane < M ? ea[row0 + lane] : 0;
      const int s_col = eb_j >= kOzNonFinite ? (1 << 24) : eb_j - (kOzFrac + 16);
      const int s_row = my_ea >= kOzNonFinite ? (1 << 24) : my_ea;
      const bool whole = (jb * kOzBN + quarter * 32 + 32 <= N) && (row0 + 32 <= M);  // warp-uniform
      double* cptr = c + (int64_t)row0 * ldc + (col_ok ? col : 0);
#pragma unroll
      for (int cc = 0; cc < 8; ++cc) {
        unsigned lv[4];
        tmem_ld4(lo_base + (unsigned)(cc * 4), lv);
        double cv[4];
        if (whole) {
#pragma unroll
          for (int r = 0; r < 4; ++r) cv[r] = __ldcs(cptr + (int64_t)r * ldc);
        } else {
#pragma unroll
          for (int r = 0; r < 4; ++r)
            cv[r] = (col_ok && row0 + 4 * cc + r < M) ? __ldcs(cptr + (int64_t)r * ldc) : 0.0;
        }
        asm volatile("tcgen05.wait::ld.sync.aligned;");
        unsigned declined = 0;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int k = 4 * cc + r;
          const int s = s_col + __shfl_sync(0xffffffffu, s_row, k);
          if (!oz_combine_fast(rh[k], lv[r], s, cv[r])) declined |= 1u << r;
        }
        if (__any_sync(0xffffffffu, declined != 0u)) {
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            const int k = 4 * cc + r;
            const int ea_i = __shfl_sync(0xffffffffu, my_ea, k);
            if (declined & (1u << r)) cv[r] = oz_combine(rh[k], lv[r], ea_i, eb_j, cv[r]);
          }
        }
        if (whole) {
#pragma unroll
          for (int r = 0; r < 4; ++r) __stcs(cptr + (int64_t)r * ldc, cv[r]);
        } else {
#pragma unroll
          for (int r = 0; r < 4; ++r)
            if (col_ok && row0 + 4 * cc + r < M) __stcs(cptr + (int64_t)r * ldc, cv[r]);
        }
        cptr += 4 * ldc;
        asm volatile("" ::: "memory");  // keep the chunks' loads from being hoisted together
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_abort) {
    // Copies issued but never consumed must land before the CTA exits.
    if (s_u_issued > s_u_consumed) mbar_wait(smem_u32(&u_full), (unsigned)((s_u_issued - 1) & 1), limit);
    // L slices: every issued slice's barrier completes once its bytes land
    // (issue order 6 .. 0 per tile).
    for (int p = 0; p < kOzSlices; ++p) {
      const int uses = s_l_issued / kOzSlices + (kOzSlices - 1 - p < s_l_issued % kOzSlices ? 1 : 0);
      if (uses > 0) mbar_wait(smem_u32(&l_full[p]), (unsigned)((uses - 1) & 1), limit);
    }
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

// Workspace layout for an M x N product: A slices [7][M'][64], B slices
// [7][N][64], exponents ea[M'], eb[N], with M' = max(M, 128) (the triangular
// solve's L slices always have 128 rows).
struct OzWs {
  __half* as;
  __half* bs;
  int* ea;
  int* eb;
  double* nb;  // N = I - L11^-1 of the triangular solve (128 x 64)
};
static OzWs oz_layout(void* ws, int M, int N) {
  const size_t Mp = (size_t)std::max(M, kOzMapRows);
  char* p = static_cast<char*>(ws);
  OzWs w;
  w.as = reinterpret_cast<__half*>(p);
  p += oz_round((size_t)kOzSlices * Mp * kOzK * 2);
  w.bs = reinterpret_cast<__half*>(p);
  p += oz_round((size_t)kOzSlices * N * kOzK * 2);
  w.ea = reinterpret_cast<int*>(p);
  p += oz_round(Mp * 4);
  w.eb = reinterpret_cast<int*>(p);
  p += oz_round((size_t)N * 4);
  w.nb = reinterpret_cast<double*>(p);
  return w;
}

size_t ozaki_workspace_bytes(int m, int n) {
  const size_t mp = (size_t)std::max(m, kOzMapRows);
  return oz_round((size_t)kOzSlices * mp * kOzK * 2) + oz_round((size_t)kOzSlices * n * kOzK * 2) + oz_round(mp * 4) +
         oz_round((size_t)n * 4) + oz_round((size_t)kOzMapRows * kOzK * sizeof(double));
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

// C (M x N, ldc) -= the product of the slices in `w` (L map of map_rows
// rows); one persistent launch.
static int oz_launch_gemm(luhot_ctx* ctx, const OzWs& w, int map_rows, double* c, int64_t ldc, int M, int N,
                          cudaStream_t stream) {
  CUtensorMap tmL, tmU;
  int rc = make_slice_map(ctx, &tmL, w.as, map_rows, kOzBM);
  if (!rc) rc = make_slice_map(ctx, &tmU, w.bs, N, kOzBN);
  if (rc) return rc;
  const int tiles = ((M + kOzBM - 1) / kOzBM) * ((N + kOzBN - 1) / kOzBN);
  LUHOT_CUDA_TRY(ctx, allow_max_dynamic_smem(oz_gemm_kernel));
  oz_gemm_kernel<<<std::min(tiles, ctx->num_sms), kOzThreads, kOzSmem, stream>>>(tmL, tmU, c, ldc, M, N, w.ea, w.eb,
                                                                                ctx->d_status);
  LUHOT_CUDA_TRY(ctx, cudaGetLastError());
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
  const OzWs lay = oz_layout(ws, M, N);

  prof_begin(ctx, kProfOther);
  oz_split_rows_kernel<<<(M + 7) / 8, 256, 0, stream>>>(a, lda, r1, M, k0, w, lay.as, lay.ea);
  prof_end(ctx, kProfOther, 0.0, (double)M * w * 8 + (double)M * kOzK * kOzSlices * 2);
  prof_begin(ctx, kProfOther);
  oz_split_cols_kernel<<<(N + 31) / 32, 256, 0, stream>>>(a, lda, k0, w, c1, N, lay.bs, lay.eb);
  prof_end(ctx, kProfOther, 0.0, (double)N * w * 8 + (double)N * kOzK * kOzSlices * 2);
  LUHOT_CUDA_TRY(ctx, cudaGetLastError());

  prof_begin(ctx, kProfGemm);
  int rc = oz_launch_gemm(ctx, lay, M, a + (int64_t)r1 * lda + c1, lda, M, N, stream);
  // algorithmic work: 2MNK FP64 flops; bytes: C read + written, the slices read once
  prof_end(ctx, kProfGemm, 2.0 * M * N * w,
           (double)M * N * 16 + (double)(M + N) * kOzK * kOzSlices * 2 + (double)(M + N) * 4);
  return rc;
}

int ozaki_trsm(luhot_ctx* ctx, double* a, int64_t lda, int k0, int w, int c1, int n, void* ws, cudaStream_t stream) {
  const int N = n - c1;
  if (N <= 0 || w <= 1) return LUHOT_OK;
  if (w > kOzK || N < kOzBN) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "ozaki_trsm: w > 64 or fewer than 128 columns");
  const OzWs lay = oz_layout(ws, w, N);
  oz_trsm_inverse_kernel<<<kOzK, 128, 0, stream>>>(a, lda, k0, w, lay.nb);
  oz_split_rows_kernel<<<kOzMapRows / 8, 256, 0, stream>>>(lay.nb, kOzK, 0, kOzMapRows, 0, w, lay.as, lay.ea);
  oz_split_cols_kernel<<<(N + 31) / 32, 256, 0, stream>>>(a, lda, k0, w, c1, N, lay.bs, lay.eb);
  LUHOT_CUDA_TRY(ctx, cudaGetLastError());
  // rows [k0, k0 + w) of columns [c1, n): A12 -= N A12 (its slices were taken first)
  return oz_launch_gemm(ctx, lay, kOzMapRows, a + (int64_t)k0 * lda + c1, lda, w, N, stream);
}

}  // namespace luhot
