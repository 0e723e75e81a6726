// Chained triangular sweep for one right-hand side (fast mode, untransposed,
// FP32 factors, FP32 arithmetic): the corrections of the mixed-precision
// refinement.  (The kernels are written for FP64 arithmetic too, but with
// FP64 this slow the 128 x 128 tile on each chain step costs more than the
// 64-row sync-free sweeps, which GMRES-IR therefore keeps.)
//
// The rows are cut into 128-row blocks; CTAs take blocks by ticket in sweep
// order (top-down for L, bottom-up for U), so a CTA only waits for blocks of
// CTAs that are already running.  The CTA of block I streams its row tiles
// op(A)(I, J) (128 x 128, the next tile prefetched into registers while the
// current one waits), subtracts op(A)(I, J) x(J) as soon as x(J) is
// published, then forms x(I) = D_I^-1 (b(I) - sum) with the precomputed
// inverse of its diagonal block, and publishes x(I).
//
// Publication without flags or fences: x(I) is also written as step-tagged
// 8-byte words (payload in the low 32 bits, the launch's epoch in the high
// 32; two words per FP64 value).  A consumer's warp 0 polls exactly the words
// it needs with 32-byte loads (lane L takes columns 4L..4L+3 of the block,
// the columns its float4 loads of the factor cover) and accepts them when
// every tag is this launch's epoch; the epoch grows per launch, so words of
// an earlier sweep are never taken.  Within a launch every word is written
// once (by the CTA of its block), and launches on the context's stream do
// not overlap, so no word is rewritten while a reader may still want it.
// Every wait is bounded by the context's wait limit and reports
// LUHOT_ERR_TIMEOUT on expiry.
//
// Layout of the work: 16 warps x 8 rows; lane L holds per-row partial sums
// over its 4 columns of every tile, reduced once at the end with a 9-shuffle
// transpose reduction; the diagonal inverse (128 x 128, shared memory) is
// applied with lanes along k and the same reduction.
#include <algorithm>

#include "common.cuh"
#include "luhot_internal.h"
#include "trsv.cuh"

namespace luhot {

constexpr int kCB = 128;        // block rows
constexpr int kCThreads = 512;  // 16 warps
constexpr int kCRows = 8;       // rows per warp

__device__ __forceinline__ void chain_ld_quad(const unsigned long long* p, unsigned long long* v) {
  asm volatile("ld.relaxed.gpu.global.v4.u64 {%0, %1, %2, %3}, [%4];"
               : "=l"(v[0]), "=l"(v[1]), "=l"(v[2]), "=l"(v[3])
               : "l"(p)
               : "memory");
}
__device__ __forceinline__ void chain_st_word(unsigned long long* p, unsigned int bits, unsigned int tag) {
  const unsigned long long v = ((unsigned long long)tag << 32) | bits;
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

template <typename T>
struct ChainVal;
template <>
struct ChainVal<float> {
  static constexpr int kW = 1;
  __device__ static float decode(const unsigned long long* w) { return __uint_as_float((unsigned int)w[0]); }
  __device__ static void publish(unsigned long long* p, float v, unsigned int tag) {
    chain_st_word(p, __float_as_uint(v), tag);
  }
};
template <>
struct ChainVal<double> {
  static constexpr int kW = 2;
  __device__ static double decode(const unsigned long long* w) {
    return __longlong_as_double(
        (long long)(((unsigned long long)(unsigned int)w[0] << 32) | (unsigned int)w[1]));
  }
  __device__ static void publish(unsigned long long* p, double v, unsigned int tag) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    chain_st_word(p, (unsigned int)(b >> 32), tag);
    chain_st_word(p + 1, (unsigned int)b, tag);
  }
};

// Sum of v[0..7] over the 32 lanes of a warp, row k of 8: after the
// reduction lane L holds the total of row 4*b4(L) + 2*b3(L) + b2(L) (bits 4,
// 3, 2 of L); 9 shuffles instead of 40.
template <typename T>
__device__ __forceinline__ T reduce8_transpose(const T (&v)[8], int lane, int& row) {
  const int h16 = (lane >> 4) & 1, h8 = (lane >> 3) & 1, h4 = (lane >> 2) & 1;
  T a4[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const T keep = h16 ? v[k + 4] : v[k];
    const T send = h16 ? v[k] : v[k + 4];
    a4[k] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
  T a2[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const T keep = h8 ? a4[k + 2] : a4[k];
    const T send = h8 ? a4[k] : a4[k + 2];
    a2[k] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
  T a1;
  {
    const T keep = h4 ? a2[1] : a2[0];
    const T send = h4 ? a2[0] : a2[1];
    a1 = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  }
  a1 += __shfl_xor_sync(0xffffffffu, a1, 2);
  a1 += __shfl_xor_sync(0xffffffffu, a1, 1);
  row = 4 * h16 + 2 * h8 + h4;
  return a1;
}

// Rows [i0 + r0, +8) x columns [j0 + c4, +4) of the FP32 factor; zero outside
// rows x cols.  16-byte loads when the row segment is whole and aligned.
__device__ __forceinline__ void chain_load_tile(float (&d)[kCRows][4], const float* __restrict__ a, int64_t lda,
                                                int i0, int r0, int rows, int j0, int c4, int cols, bool vec) {
#pragma unroll
  for (int r = 0; r < kCRows; ++r) {
    const int rr = r0 + r;
    const float* src = a + (int64_t)(i0 + rr) * lda + j0 + c4;
    if (rr < rows && vec && c4 + 4 <= cols) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(src));
      d[r][0] = v.x;
      d[r][1] = v.y;
      d[r][2] = v.z;
      d[r][3] = v.w;
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e) d[r][e] = (rr < rows && c4 + e < cols) ? __ldg(src + e) : 0.f;
    }
  }
}

template <typename T, bool kLower>
__global__ void __launch_bounds__(kCThreads, 1)
    trsv_chain_kernel(const float* __restrict__ a, int64_t lda, T* x, int n, const T* __restrict__ dinv,
                      unsigned long long* xt, unsigned int epoch, int* ticket, DeviceStatus* st) {
  constexpr int kW = ChainVal<T>::kW;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* D = reinterpret_cast<T*>(smem_raw);  // [128][128] inverse of the diagonal block
  T* xs = D + kCB * kCB;                   // [2][128] x(J), double-buffered by tile
  T* ys = xs + 2 * kCB;                    // [128] b(I) - sum over the tiles
  __shared__ int s_ticket, s_ok;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    s_ticket = atomicAdd(ticket, 1);
    s_ok = 1;
  }
  __syncthreads();
  const int nblk = (n + kCB - 1) / kCB;
  const int t = s_ticket;
  if (t >= nblk) return;
  const int I = kLower ? t : nblk - 1 - t;
  const int i0 = I * kCB;
  const int rows = min(kCB, n - i0);
  const int r0 = warp * kCRows;  // this warp's rows of the block
  const int c4 = lane * 4;       // this lane's columns of every tile
  const bool vec = (lda % 4 == 0) && ((reinterpret_cast<uintptr_t>(a) & 15) == 0);

  // b(I) for the row this lane will hold after the reductions.
  const int my_row = r0 + 4 * ((lane >> 4) & 1) + 2 * ((lane >> 3) & 1) + ((lane >> 2) & 1);
  const T b_mine = ((lane & 3) == 0 && my_row < rows) ? x[i0 + my_row] : T(0);
  // The diagonal block's inverse (used last; its loads overlap the waits).
  {
    const T* src = dinv + (size_t)I * kCB * kCB;
    for (int idx = tid; idx < kCB * kCB; idx += kCThreads) D[idx] = src[idx];
  }

  T acc[kCRows];
#pragma unroll
  for (int r = 0; r < kCRows; ++r) acc[r] = T(0);
  const int nupd = kLower ? I : nblk - 1 - I;
  float cur[kCRows][4], nxt[kCRows][4];
  if (nupd > 0) {
    const int J0 = kLower ? 0 : nblk - 1;
    chain_load_tile(nxt, a, lda, i0, r0, rows, J0 * kCB, c4, min(kCB, n - J0 * kCB), vec);
  }
  for (int s = 0; s < nupd; ++s) {
    const int J = kLower ? s : nblk - 1 - s;
    const int j0 = J * kCB;
#pragma unroll
    for (int r = 0; r < kCRows; ++r)
#pragma unroll
      for (int e = 0; e < 4; ++e) cur[r][e] = nxt[r][e];
    if (s + 1 < nupd) {  // the next tile's loads overlap this tile's wait
      const int Jn = kLower ? s + 1 : nblk - 2 - s;
      chain_load_tile(nxt, a, lda, i0, r0, rows, Jn * kCB, c4, min(kCB, n - Jn * kCB), vec);
    }
    T* xb = xs + (s & 1) * kCB;
    if (warp == 0) {
      // x(J): this lane's four values, as tagged words.
      const unsigned long long* src = xt + ((size_t)j0 + c4) * kW;
      unsigned long long wd[4 * kW];
      const unsigned long long t0 = global_timer_ns();
      unsigned int spins = 0;
      bool ok = true;
      while (true) {
#pragma unroll
        for (int q = 0; q < kW; ++q) chain_ld_quad(src + 4 * q, wd + 4 * q);
        bool cur_ok = true;
#pragma unroll
        for (int e = 0; e < 4 * kW; ++e) cur_ok = cur_ok && (unsigned int)(wd[e] >> 32) == epoch;
        if (__all_sync(0xffffffffu, cur_ok)) break;
        if ((++spins & 15u) == 0) {
          const int late = (global_timer_ns() - t0 > st->timeout_ns) ? 1 : 0;
          const int stop = __shfl_sync(0xffffffffu, late, 0) | __any_sync(0xffffffffu, ld_relaxed_i32(&st->abort));
          if (stop) {
            if (lane == 0 && late) {
              atomicCAS(&st->error, kDevOk, kDevBarrierTimeout);
              atomicExch(&st->timeout_where, (unsigned long long)J);
              atomicExch(&st->abort, 1);
            }
            ok = false;
            break;
          }
        }
      }
      if (!ok) {
        if (lane == 0) s_ok = 0;
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) xb[c4 + e] = ChainVal<T>::decode(wd + e * kW);
      }
    }
    __syncthreads();
    if (!s_ok) return;
    T xv[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) xv[e] = xb[c4 + e];
#pragma unroll
    for (int r = 0; r < kCRows; ++r)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[r] = fma(-static_cast<T>(cur[r][e]), xv[e], acc[r]);
  }

  // y = b(I) - sum, into shared memory.
  {
    int rr;
    const T sum = reduce8_transpose(acc, lane, rr);
    if ((lane & 3) == 0) ys[r0 + rr] = (r0 + rr < rows) ? b_mine + sum : T(0);
  }
  __syncthreads();
  // x(I) = D^-1 y: warp w takes outputs r0..r0+7, lanes along k.
  T part[kCRows];
  {
    T yk[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) yk[m] = ys[lane + 32 * m];
#pragma unroll
    for (int r = 0; r < kCRows; ++r) {
      const T* drow = D + (r0 + r) * kCB;
      T v = T(0);
#pragma unroll
      for (int m = 0; m < 4; ++m) v = fma(drow[lane + 32 * m], yk[m], v);
      part[r] = v;
    }
  }
  int rr;
  const T xi = reduce8_transpose(part, lane, rr);
  if ((lane & 3) == 0) {
    const int o = r0 + rr;  // every row of the block is published, padding as 0
    ChainVal<T>::publish(xt + ((size_t)i0 + o) * kW, o < rows ? xi : T(0), epoch);
    if (o < rows) x[i0 + o] = xi;
  }
}

// Inverse of every 128 x 128 diagonal block of the FP32 factor (lower unit
// or upper non-unit) in the arithmetic type T, row-major per block,
// zero-padded past n.  One CTA per block, one thread per column of the
// inverse (substitution on the unit vector), in shared memory.
template <typename T, bool kLower>
__global__ void __launch_bounds__(kCB) trsv_chain_invert_kernel(const float* __restrict__ a, int64_t lda, int n,
                                                                T* dinv) {
  constexpr int kL = kCB + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* Y = reinterpret_cast<T*>(smem_raw);               // [128][129] inverse, column c owned by thread c
  float* S = reinterpret_cast<float*>(Y + kCB * kL);   // [128][129] diagonal block
  const int i0 = blockIdx.x * kCB;
  const int rows = min(kCB, n - i0);
  for (int idx = threadIdx.x; idx < kCB * kCB; idx += kCB) {
    const int r = idx / kCB, c = idx - r * kCB;
    S[r * kL + c] = (r < rows && c < rows) ? a[(int64_t)(i0 + r) * lda + i0 + c] : 0.f;
  }
  __syncthreads();
  const int c = threadIdx.x;
  if (kLower) {
    for (int i = 0; i < kCB; ++i) {
      T v = T(0);
      if (c < rows && i < rows && i >= c) {
        v = (i == c) ? T(1) : T(0);
        for (int k = c; k < i; ++k) v = fma(-static_cast<T>(S[i * kL + k]), Y[k * kL + c], v);
      }
      Y[i * kL + c] = v;
    }
  } else {
    for (int i = kCB - 1; i >= 0; --i) {
      T v = T(0);
      if (c < rows && i < rows && i <= c) {
        v = (i == c) ? T(1) : T(0);
        for (int k = i + 1; k <= c; ++k) v = fma(-static_cast<T>(S[i * kL + k]), Y[k * kL + c], v);
        v = v / static_cast<T>(S[i * kL + i]);
      }
      Y[i * kL + c] = v;
    }
  }
  __syncthreads();
  T* out = dinv + (size_t)blockIdx.x * kCB * kCB;
  for (int idx = threadIdx.x; idx < kCB * kCB; idx += kCB) out[idx] = Y[(idx / kCB) * kL + idx % kCB];
}

int trsv_chain_blocks(int n) { return (n + kCB - 1) / kCB; }
size_t trsv_chain_inverse_elems(int n) { return (size_t)trsv_chain_blocks(n) * kCB * kCB; }
size_t trsv_chain_tag_words(int n) { return (size_t)trsv_chain_blocks(n) * kCB * 2; }

template <typename T>
cudaError_t launch_trsv_chain_invert(cudaStream_t stream, const float* a, int64_t lda, int n, bool lower, T* dinv) {
  if (n <= 0) return cudaSuccess;
  const size_t smem = (size_t)kCB * (kCB + 1) * (sizeof(T) + sizeof(float));
  auto k = lower ? trsv_chain_invert_kernel<T, true> : trsv_chain_invert_kernel<T, false>;
  cudaError_t e = allow_max_dynamic_smem(k);
  if (e != cudaSuccess) return e;
  k<<<trsv_chain_blocks(n), kCB, smem, stream>>>(a, lda, n, dinv);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_trsv_chain(cudaStream_t stream, const float* a, int64_t lda, T* x, int n, bool lower,
                              const T* dinv, unsigned long long* xt, unsigned int epoch, int* ticket,
                              DeviceStatus* st) {
  if (n <= 0) return cudaSuccess;
  const size_t smem = ((size_t)kCB * kCB + 3 * (size_t)kCB) * sizeof(T);
  auto k = lower ? trsv_chain_kernel<T, true> : trsv_chain_kernel<T, false>;
  cudaError_t e = allow_max_dynamic_smem(k);
  if (e == cudaSuccess) e = cudaMemsetAsync(ticket, 0, sizeof(int), stream);
  if (e != cudaSuccess) return e;
  k<<<trsv_chain_blocks(n), kCThreads, smem, stream>>>(a, lda, x, n, dinv, xt, epoch, ticket, st);
  return cudaGetLastError();
}

template cudaError_t launch_trsv_chain_invert<float>(cudaStream_t, const float*, int64_t, int, bool, float*);
template cudaError_t launch_trsv_chain<float>(cudaStream_t, const float*, int64_t, float*, int, bool, const float*,
                                              unsigned long long*, unsigned int, int*, DeviceStatus*);

}  // namespace luhot
