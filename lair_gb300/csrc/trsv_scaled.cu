// Single-right-hand-side triangular sweeps on block-scaled factors, for
// factors that stay on the device and are solved many times
// (lu::Factorized::solve, src/decomposition/lu.rs:87-98, through
// luhot_dfactor_solve).
//
// Cut a triangular factor T (L: unit lower; U: upper) into 64-row blocks with
// diagonal blocks D_I.  T x = b is
//     x(I) = D_I^-1 b(I) - sum_{J before I} W(I, J) x(J),   W(I, J) = D_I^-1 T(I, J),
// so once W is formed (scale_blocks_kernel: one 64 x 64 x 64 product per
// off-diagonal tile, stored beside the factor) no row needs the other rows of
// its block.  Each 64-row block is split over four CTAs of 16 rows, and the
// work that waits on x(I - 1) is one 16 x 64 tile per CTA (1024 FMAs) instead
// of a 64 x 64 tile plus the 64 x 64 diagonal inverse (8192 FMAs on one SM):
// at this part's FP64 rate (about 1.6 FMA per clock per SM) those FMAs, not
// the memory, bounded each step of the block chain.
//
// Order and publication follow the chained FP32 sweep (trsv_chain.cu): CTAs
// take (block, quarter) tickets in sweep order and wait only for blocks of
// earlier tickets, i.e. of CTAs already running; x(I) is published as
// epoch-tagged words (two per FP64 value, each carrying the launch's epoch in
// its top half), which each warp polls with one 32-byte load per lane and a
// vote, so the loop has no flags, fences or block barriers.
// Thread layout: 128 threads = 16 rows x 8 groups of 8 columns; each thread
// keeps one partial sum, reduced over the 8 lanes of its row once at the end.
// Every wait is bounded by the context's wait limit (LUHOT_ERR_TIMEOUT).
#include <algorithm>

#include "common.cuh"
#include "luhot_internal.h"
#include "trsv.cuh"

namespace luhot {

constexpr int kSB = 64;         // block rows (the diagonal-inverse blocks)
constexpr int kSParts = 4;      // CTAs per block
constexpr int kSRows = 16;      // rows per CTA
constexpr int kSThreads = 128;  // 16 rows x 8 column groups
constexpr int kSLd = kSB + 1;

// W(I, J) = D_I^-1 T(I, J) for every off-diagonal tile of one triangle, in
// FP64 arithmetic; T's tiles are read from the row-major factor a (storage
// TA), D_I^-1 from dinv (64 x 64 per block, zero past n), W written with
// leading dimension ldw in storage TW.  One CTA per tile of the grid's
// (J, I) square; tiles outside the triangle return at once.
template <typename TA, typename TW, bool kLower>
__global__ void __launch_bounds__(256) scale_blocks_kernel(const TA* __restrict__ a, int64_t lda,
                                                           const double* __restrict__ dinv, TW* __restrict__ w,
                                                           int64_t ldw, int n) {
  const int I = blockIdx.y, J = blockIdx.x;
  if (kLower ? (J >= I) : (J <= I)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* Ds = reinterpret_cast<double*>(smem_raw);  // [64][65] D_I^-1
  double* Ts = Ds + kSB * kSLd;                       // [64][65] T(I, J)
  const int i0 = I * kSB, j0 = J * kSB;
  const double* dsrc = dinv + (size_t)I * kSB * kSB;
  for (int idx = threadIdx.x; idx < kSB * kSB; idx += 256) {
    const int r = idx / kSB, c = idx - r * kSB;
    Ds[r * kSLd + c] = dsrc[idx];
    Ts[r * kSLd + c] = (i0 + r < n && j0 + c < n) ? static_cast<double>(a[(int64_t)(i0 + r) * lda + j0 + c]) : 0.0;
  }
  __syncthreads();
  const int r0 = (threadIdx.x >> 4) * 4, c0 = (threadIdx.x & 15) * 4;
  double acc[4][4] = {};
  for (int k = 0; k < kSB; ++k) {
    double d[4], t[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      d[q] = Ds[(r0 + q) * kSLd + k];
      t[q] = Ts[k * kSLd + c0 + q];
    }
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[p][q] = fma(d[p], t[q], acc[p][q]);
  }
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int r = i0 + r0 + p, c = j0 + c0 + q;
      if (r < n && c < n) w[(int64_t)r * ldw + c] = static_cast<TW>(acc[p][q]);
    }
}

__device__ __forceinline__ void scaled_ld_quad(const unsigned long long* p, unsigned long long* v) {
  asm volatile("ld.relaxed.gpu.global.v4.u64 {%0, %1, %2, %3}, [%4];"
               : "=l"(v[0]), "=l"(v[1]), "=l"(v[2]), "=l"(v[3])
               : "l"(p)
               : "memory");
}
__device__ __forceinline__ void scaled_st_word(unsigned long long* p, unsigned int bits, unsigned int tag) {
  const unsigned long long v = ((unsigned long long)tag << 32) | bits;
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Eight consecutive entries of row i of W from column j (zero past n); the
// whole-segment case as 16-byte loads (j is a multiple of 8 and rows start
// on 256-byte boundaries).
__device__ __forceinline__ void scaled_load_row8(double (&d)[8], const double* __restrict__ w, int64_t ldw, int i,
                                                 int j, int n) {
  const double* src = w + (int64_t)i * ldw + j;
  if (i < n && j + 8 <= n) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const double2 v = __ldg(reinterpret_cast<const double2*>(src) + q);
      d[2 * q] = v.x;
      d[2 * q + 1] = v.y;
    }
  } else {
#pragma unroll
    for (int e = 0; e < 8; ++e) d[e] = (i < n && j + e < n) ? __ldg(src + e) : 0.0;
  }
}

// Whether a lane's quad of tagged words (values 2L and 2L + 1 of a block of
// `count` published values) carries this launch's epoch.
__device__ __forceinline__ bool scaled_quad_ok(const unsigned long long (&q)[4], int lane, int count,
                                               unsigned int epoch) {
  const bool v0 = 2 * lane >= count || ((unsigned int)(q[0] >> 32) == epoch && (unsigned int)(q[1] >> 32) == epoch);
  const bool v1 = 2 * lane + 1 >= count || ((unsigned int)(q[2] >> 32) == epoch && (unsigned int)(q[3] >> 32) == epoch);
  return v0 && v1;
}
__device__ __forceinline__ double scaled_decode(unsigned long long hi, unsigned long long lo) {
  return __longlong_as_double((long long)(((unsigned long long)(unsigned int)hi << 32) | (unsigned int)lo));
}

// One sweep: y = T^-1 b (b and y are n-vectors with strides 1 and ldy; y may
// not alias b).  xt holds two tagged words per row (at least 2 * 64 * nblk).
// x(J) is fetched per warp: lane L loads the 32-byte quad of values 2L and
// 2L + 1, the warp votes on the tags, the values go through a per-warp
// shared buffer to the eight lanes of each row that use them; the next
// tile's quad is requested while the current tile is used.
template <typename TW, bool kLower>
__global__ void __launch_bounds__(kSThreads) trsv_scaled_kernel(const TW* __restrict__ w, int64_t ldw,
                                                                const double* __restrict__ dinv,
                                                                const double* __restrict__ b, double* y, int64_t ldy,
                                                                int n, unsigned long long* xt, unsigned int epoch,
                                                                int* ticket, DeviceStatus* st) {
  __shared__ int s_ticket;
  __shared__ double s_x[kSThreads / 32][2][kSB];
  if (threadIdx.x == 0) s_ticket = atomicAdd(ticket, 1);
  __syncthreads();
  const int nblk = (n + kSB - 1) / kSB;
  const int t = s_ticket;
  if (t >= nblk * kSParts) return;
  const int I = kLower ? t / kSParts : nblk - 1 - t / kSParts;
  const int part = t % kSParts;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = threadIdx.x >> 3, kp = threadIdx.x & 7;
  const int rb = part * kSRows + r;  // row within the block
  const int i = I * kSB + rb;        // this thread's row
  const int c8 = kp * 8;             // this thread's columns within a tile

  // D_I^-1 b(I): this thread's eight terms of its row.
  double acc = 0.0;
  {
    const double* drow = dinv + (size_t)I * kSB * kSB + rb * kSB + c8;
    const int ib = I * kSB + c8;
#pragma unroll
    for (int e = 0; e < 8; ++e)
      if (ib + e < n) acc = fma(drow[e], b[ib + e], acc);
  }

  const int nupd = kLower ? I : nblk - 1 - I;
  double cur[8], nxt[8];
  unsigned long long q[4];
  if (nupd > 0) {
    const int J0 = kLower ? 0 : nblk - 1;
    scaled_load_row8(nxt, w, ldw, i, J0 * kSB + c8, n);
    scaled_ld_quad(xt + 2 * (size_t)J0 * kSB + 4 * lane, q);
  }
  const unsigned long long limit = st->timeout_ns;
  // Every branch below is warp-uniform (votes and shuffles), so a wait that
  // gives up ends the loop for the whole warp and every lane still reaches
  // the shuffles after it.
  bool alive = true;
  for (int s = 0; s < nupd; ++s) {
    const int J = kLower ? s : nblk - 1 - s;
    const int j0 = J * kSB;
    const int count = min(kSB, n - j0);
#pragma unroll
    for (int e = 0; e < 8; ++e) cur[e] = nxt[e];
    if (s + 1 < nupd) scaled_load_row8(nxt, w, ldw, i, (kLower ? s + 1 : nblk - 2 - s) * kSB + c8, n);
    unsigned long long t0 = 0;
    unsigned int spins = 0;
    while (!__all_sync(0xffffffffu, scaled_quad_ok(q, lane, count, epoch))) {
      if (spins == 0) t0 = global_timer_ns();
      if ((++spins & 63u) == 0) {
        int stop = 0;
        if (lane == 0) {
          if (ld_relaxed_i32(&st->abort)) {
            stop = 1;
          } else if (global_timer_ns() - t0 > limit) {
            atomicCAS(&st->error, kDevOk, kDevBarrierTimeout);
            atomicExch(&st->timeout_where, (unsigned long long)J);
            atomicExch(&st->abort, 1);
            stop = 1;
          }
        }
        if (__shfl_sync(0xffffffffu, stop, 0)) {
          alive = false;
          break;
        }
      }
      scaled_ld_quad(xt + 2 * (size_t)j0 + 4 * lane, q);
    }
    if (!alive) break;
    double* xb = s_x[warp][s & 1];
    xb[2 * lane] = 2 * lane < count ? scaled_decode(q[0], q[1]) : 0.0;
    xb[2 * lane + 1] = 2 * lane + 1 < count ? scaled_decode(q[2], q[3]) : 0.0;
    if (s + 1 < nupd) scaled_ld_quad(xt + 2 * (size_t)(kLower ? s + 1 : nblk - 2 - s) * kSB + 4 * lane, q);
    __syncwarp();
#pragma unroll
    for (int e = 0; e < 8; ++e) acc = fma(-cur[e], xb[c8 + e], acc);
  }
  // Sum the row's eight partial sums (lanes 8r' .. 8r'+7 of the warp).
  acc += __shfl_xor_sync(0xffffffffu, acc, 1);
  acc += __shfl_xor_sync(0xffffffffu, acc, 2);
  acc += __shfl_xor_sync(0xffffffffu, acc, 4);
  if (alive && kp == 0 && i < n) {
    y[(int64_t)i * ldy] = acc;
    const unsigned long long bits = (unsigned long long)__double_as_longlong(acc);
    scaled_st_word(xt + 2 * (size_t)i, (unsigned int)(bits >> 32), epoch);
    scaled_st_word(xt + 2 * (size_t)i + 1, (unsigned int)bits, epoch);
  }
}

size_t trsv_scaled_tag_words(int n) { return (size_t)((n + kSB - 1) / kSB) * kSB * 2; }

template <typename TA, typename TW>
cudaError_t launch_scale_blocks(cudaStream_t stream, const TA* a, int64_t lda, const double* dinv_l,
                                const double* dinv_u, TW* w, int64_t ldw, int n) {
  if (n <= kSB) return cudaSuccess;  // one block: no off-diagonal tiles
  const int nblk = (n + kSB - 1) / kSB;
  const size_t smem = 2 * (size_t)kSB * kSLd * sizeof(double);
  cudaError_t e = allow_max_dynamic_smem(scale_blocks_kernel<TA, TW, true>);
  if (e == cudaSuccess) e = allow_max_dynamic_smem(scale_blocks_kernel<TA, TW, false>);
  if (e != cudaSuccess) return e;
  dim3 grid(nblk, nblk);
  scale_blocks_kernel<TA, TW, true><<<grid, 256, smem, stream>>>(a, lda, dinv_l, w, ldw, n);
  scale_blocks_kernel<TA, TW, false><<<grid, 256, smem, stream>>>(a, lda, dinv_u, w, ldw, n);
  return cudaGetLastError();
}

template <typename TW>
cudaError_t launch_trsv_scaled(cudaStream_t stream, const TW* w, int64_t ldw, const double* dinv, const double* b,
                               double* y, int64_t ldy, int n, bool lower, unsigned long long* xt, unsigned int epoch,
                               int* ticket, DeviceStatus* st) {
  if (n <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(ticket, 0, sizeof(int), stream);
  if (e != cudaSuccess) return e;
  const int grid = ((n + kSB - 1) / kSB) * kSParts;
  if (lower)
    trsv_scaled_kernel<TW, true><<<grid, kSThreads, 0, stream>>>(w, ldw, dinv, b, y, ldy, n, xt, epoch, ticket, st);
  else
    trsv_scaled_kernel<TW, false><<<grid, kSThreads, 0, stream>>>(w, ldw, dinv, b, y, ldy, n, xt, epoch, ticket, st);
  return cudaGetLastError();
}

template cudaError_t launch_scale_blocks<double, double>(cudaStream_t, const double*, int64_t, const double*,
                                                         const double*, double*, int64_t, int);
template cudaError_t launch_scale_blocks<float, double>(cudaStream_t, const float*, int64_t, const double*,
                                                        const double*, double*, int64_t, int);
template cudaError_t launch_trsv_scaled<double>(cudaStream_t, const double*, int64_t, const double*, const double*,
                                                double*, int64_t, int, bool, unsigned long long*, unsigned int, int*,
                                                DeviceStatus*);

}  // namespace luhot
