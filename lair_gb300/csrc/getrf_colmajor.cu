// lair's left-looking (Crout) LU for non-standard layouts, bit for bit.
//
// lair's getrf dispatcher (src/lapack/getrf.rs:12-27) factors every array
// that is not in ndarray's standard (C-contiguous) layout -- F order, sliced
// views with padded rows, negative strides -- with getrf_col_major
// (getrf.rs:128-213).  Its rounding sequence differs from the row-major
// elimination's, so exact mode reproduces it here, for m <= 4096 rows, on a
// column-major copy of the matrix in HBM (element (i, j) at a[j * ld + i]).
//
// Per column ul (one CTA of 1024 threads walks the columns in order):
//   1. the earlier interchanges are applied to the column (getrf.rs:139-145);
//   2. rows 1..min(ul, m) become x_i = a_i - dot(L[i, 0..i], x[0..i])
//      (getrf.rs:147-151) with lair's dot order (src/blas/dot.rs:39-133):
//      four partial sums over the complete groups of four, added as
//      ((s0 + s1) + s2) + s3, then the remaining one to three terms in order,
//      every product and sum rounded apart.  Rows are finalised 32 at a time
//      by one warp (lane j owns row 32I + j; x_k is broadcast by shuffle);
//      once a block of 32 is final, all threads add its terms into the
//      partial sums of the rows below, in increasing k;
//   3. rows ul..m: y_r += (-x_k) * L[r][k] for k = 0..ul-1 in order, the
//      gemv::notrans column-axpy order (src/blas/gemv.rs:6-47), one thread
//      per row;
//   4. pivot search with iamax's strict `>` from 0 (src/blas/iamax.rs:6-21);
//      the step is singular when the pivot *value* is zero (getrf.rs:167),
//      otherwise rows ul and pr swap their first ul+1 entries and the column
//      below the pivot is multiplied by the rounded reciprocal.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "luhot_internal.h"

namespace luhot {
namespace {

constexpr int kCmThreads = 1024;
constexpr int kCmMaxRows = 4096;

template <typename T>
__device__ __forceinline__ T mul_rn_cm(T a, T b);
template <>
__device__ __forceinline__ double mul_rn_cm<double>(double a, double b) {
  return __dmul_rn(a, b);
}
template <>
__device__ __forceinline__ float mul_rn_cm<float>(float a, float b) {
  return __fmul_rn(a, b);
}
template <typename T>
__device__ __forceinline__ T add_rn_cm(T a, T b);
template <>
__device__ __forceinline__ double add_rn_cm<double>(double a, double b) {
  return __dadd_rn(a, b);
}
template <>
__device__ __forceinline__ float add_rn_cm<float>(float a, float b) {
  return __fadd_rn(a, b);
}
template <typename T>
__device__ __forceinline__ T sub_rn_cm(T a, T b);
template <>
__device__ __forceinline__ double sub_rn_cm<double>(double a, double b) {
  return __dsub_rn(a, b);
}
template <>
__device__ __forceinline__ float sub_rn_cm<float>(float a, float b) {
  return __fsub_rn(a, b);
}

template <typename T>
__global__ void __launch_bounds__(kCmThreads) getrf_colmajor_kernel(T* a, int64_t ld, int m, int n, int* piv,
                                                                    DeviceStatus* st) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* col = reinterpret_cast<T*>(smem_raw);  // [m] column ul
  T* ps = col + m;                          // [4][m] dot partial sums of the rows above ul
  __shared__ T red_v[32];
  __shared__ int red_i[32];
  __shared__ int s_pr;
  __shared__ T s_pivot;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  for (int ul = 0; ul < n; ++ul) {
    T* gcol = a + (int64_t)ul * ld;
    for (int r = tid; r < m; r += kCmThreads) col[r] = gcol[r];
    const int nu = min(ul, m);
    for (int r = tid; r < 4 * nu; r += kCmThreads) ps[(r / nu) * m + r % nu] = T(0);
    __syncthreads();
    // 1. earlier interchanges, in order
    if (tid == 0)
      for (int i = 0; i < nu; ++i) {
        const int ip = piv[i];
        if (ip != i) {
          const T t = col[i];
          col[i] = col[ip];
          col[ip] = t;
        }
      }
    __syncthreads();
    // 2. x_i = a_i - dot(L[i, 0..i], x[0..i]) for i = 1..nu-1
    for (int i0 = 0; i0 < nu; i0 += 32) {
      if (warp == 0) {
        const int i = i0 + lane;
        const bool own = i < nu && i > 0;
        const int q4 = 4 * (i / 4);
        T p0 = own ? ps[i] : T(0), p1 = own ? ps[m + i] : T(0), p2 = own ? ps[2 * m + i] : T(0),
          p3 = own ? ps[3 * m + i] : T(0);
        T s = T(0);
        bool combined = false;
        T xi = (i < nu) ? col[i] : T(0);
        const int kend = min(i0 + 32, nu);
        if (own && i == i0) {
          // The block's first row has no terms inside the block: all its terms
          // (a multiple of four) are already in the partial sums.
          xi = sub_rn_cm(xi, add_rn_cm(add_rn_cm(add_rn_cm(p0, p1), p2), p3));
        }
        for (int k = i0; k < kend; ++k) {
          const T xk = __shfl_sync(0xffffffffu, xi, k - i0);
          if (own && k < i) {
            const T prod = mul_rn_cm(a[(int64_t)k * ld + i], xk);
            if (k < q4) {
              T& pk = (k & 3) == 0 ? p0 : (k & 3) == 1 ? p1 : (k & 3) == 2 ? p2 : p3;
              pk = add_rn_cm(pk, prod);
            } else {
              if (!combined) {
                s = i >= 4 ? add_rn_cm(add_rn_cm(add_rn_cm(p0, p1), p2), p3) : T(0);
                combined = true;
              }
              s = add_rn_cm(s, prod);
            }
            if (k == i - 1) {
              if (!combined) s = i >= 4 ? add_rn_cm(add_rn_cm(add_rn_cm(p0, p1), p2), p3) : T(0);
              xi = sub_rn_cm(xi, s);
            }
          }
        }
        if (i < nu) col[i] = xi;
      }
      __syncthreads();
      // The finished block's terms into the partial sums of the rows below.
      const int kend = min(i0 + 32, nu);
      for (int i = i0 + 32 + tid; i < nu; i += kCmThreads) {
        T p0 = ps[i], p1 = ps[m + i], p2 = ps[2 * m + i], p3 = ps[3 * m + i];
        for (int k = i0; k < kend; k += 4) {
          // i >= i0 + 32 > k: every k of the block lies in i's complete groups of four
          p0 = add_rn_cm(p0, mul_rn_cm(a[(int64_t)k * ld + i], col[k]));
          if (k + 1 < kend) p1 = add_rn_cm(p1, mul_rn_cm(a[(int64_t)(k + 1) * ld + i], col[k + 1]));
          if (k + 2 < kend) p2 = add_rn_cm(p2, mul_rn_cm(a[(int64_t)(k + 2) * ld + i], col[k + 2]));
          if (k + 3 < kend) p3 = add_rn_cm(p3, mul_rn_cm(a[(int64_t)(k + 3) * ld + i], col[k + 3]));
        }
        ps[i] = p0;
        ps[m + i] = p1;
        ps[2 * m + i] = p2;
        ps[3 * m + i] = p3;
      }
      __syncthreads();
    }
    if (ul < m) {
      // 3. rows ul..m-1: y_r += (-x_k) * L[r][k], k increasing
      for (int r = ul + tid; r < m; r += kCmThreads) {
        T y = col[r];
        for (int k = 0; k < ul; ++k) y = add_rn_cm(y, mul_rn_cm(-col[k], a[(int64_t)k * ld + r]));
        col[r] = y;
      }
      __syncthreads();
      // 4. pivot: first index of the largest |x| (strict >, from 0)
      T bv = T(0);
      int bi = INT_MAX;
      for (int r = ul + tid; r < m; r += kCmThreads) {
        const T v = fabs(col[r]);
        if (v > bv) {
          bv = v;
          bi = r;
        }
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const T v2 = __shfl_down_sync(0xffffffffu, bv, off);
        const int i2 = __shfl_down_sync(0xffffffffu, bi, off);
        if (v2 > bv || (v2 == bv && i2 < bi)) {
          bv = v2;
          bi = i2;
        }
      }
      if (lane == 0) {
        red_v[warp] = bv;
        red_i[warp] = bi;
      }
      __syncthreads();
      if (tid == 0) {
        T v = red_v[0];
        int i = red_i[0];
        for (int w = 1; w < kCmThreads / 32; ++w)
          if (red_v[w] > v || (red_v[w] == v && red_i[w] < i)) {
            v = red_v[w];
            i = red_i[w];
          }
        const int pr = (i == INT_MAX) ? ul : i;
        piv[ul] = pr;
        s_pr = pr;
        s_pivot = col[pr];
        if (col[pr] == T(0)) atomicMax(&st->singular, ul);
      }
      __syncthreads();
      const int pr = s_pr;
      const T pivot = s_pivot;
      if (pivot != T(0)) {
        const T recip = T(1) / pivot;
        if (pr != ul) {
          // rows ul and pr, columns 0..ul (column ul lives in smem)
          for (int j = tid; j < ul; j += kCmThreads) {
            T* cj = a + (int64_t)j * ld;
            const T t = cj[ul];
            cj[ul] = cj[pr];
            cj[pr] = t;
          }
          __syncthreads();
          if (tid == 0) {
            const T t = col[ul];
            col[ul] = col[pr];
            col[pr] = t;
          }
          __syncthreads();
        }
        for (int r = ul + 1 + tid; r < m; r += kCmThreads) col[r] = mul_rn_cm(col[r], recip);
      }
    }
    __syncthreads();
    for (int r = tid; r < m; r += kCmThreads) gcol[r] = col[r];
    __syncthreads();
  }
}

// ndarray 0.17 ArrayBase::is_standard_layout for two axes (the dispatch
// predicate of lair's getrf): empty arrays are standard; otherwise every
// axis of length != 1 must have the C-order stride.
bool standard_layout(int64_t m, int64_t n, int64_t rs, int64_t cs) {
  if (m == 0 || n == 0) return true;
  int64_t contig = 1;
  if (n != 1) {
    if (cs != contig) return false;
    contig *= n;
  }
  if (m != 1 && rs != contig) return false;
  return true;
}

}  // namespace

bool getrf_uses_colmajor(int64_t m, int64_t n, int64_t rs, int64_t cs) { return !standard_layout(m, n, rs, cs); }

template <typename T>
int getrf_colmajor_host(luhot_ctx* ctx, int64_t m, int64_t n, T* a, int64_t rs, int64_t cs, uint64_t* piv,
                        int64_t* singular) {
  const int64_t k = std::min(m, n);
  if (singular) *singular = -1;
  if (k == 0) return LUHOT_OK;
  if (m > kCmMaxRows)
    return set_error(ctx, LUHOT_ERR_UNSUPPORTED,
                     "exact mode on a non-standard layout (lair's column-major order) takes at most " +
                         std::to_string(kCmMaxRows) + " rows; use fast mode or a C-order array");
  const int64_t ld = (m + 31) / 32 * 32;
  int rc = ensure_buf(ctx, ctx->work[0], (size_t)ld * n * sizeof(T));
  if (rc) return rc;
  rc = ensure_buf(ctx, ctx->piv_buf, (size_t)k * sizeof(int));
  if (rc) return rc;
  T* d_a = static_cast<T*>(ctx->work[0].ptr);
  int* d_piv = static_cast<int*>(ctx->piv_buf.ptr);
  // Column-major copy: the transpose (n x m, row-major) of the caller's array.
  rc = stage_in<T>(ctx, a, n, m, cs, rs, d_a, ld, ctx->work[1]);
  if (rc) return rc;
  std::vector<int> hp((size_t)k);
  for (int64_t i = 0; i < k; ++i) hp[(size_t)i] = (int)i;  // getrf.rs:14: pivots start as 0..min(m, n)
  LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(d_piv, hp.data(), (size_t)k * sizeof(int), cudaMemcpyHostToDevice,
                                      ctx->stream));
  rc = reset_status(ctx);
  if (rc) return rc;
  const size_t smem = (size_t)5 * m * sizeof(T);
  LUHOT_CUDA_TRY(ctx, allow_max_dynamic_smem(getrf_colmajor_kernel<T>));
  prof_begin(ctx, kProfPanel);
  getrf_colmajor_kernel<T><<<1, kCmThreads, smem, ctx->stream>>>(d_a, ld, (int)m, (int)n, d_piv, ctx->d_status);
  prof_end(ctx, kProfPanel, 2.0 / 3.0 * (double)k * k * k, 2.0 * m * n * sizeof(T));
  LUHOT_CUDA_TRY(ctx, cudaGetLastError());
  int64_t sing = -1;
  rc = finish_status(ctx, &sing);
  if (rc) return rc;
  rc = stage_out<T>(ctx, d_a, ld, a, n, m, cs, rs, ctx->work[1]);
  if (rc) return rc;
  LUHOT_CUDA_TRY(ctx, cudaMemcpy(hp.data(), d_piv, (size_t)k * sizeof(int), cudaMemcpyDeviceToHost));
  for (int64_t i = 0; i < k; ++i) piv[i] = (uint64_t)hp[(size_t)i];
  if (singular) *singular = sing;
  return LUHOT_OK;
}

template int getrf_colmajor_host<double>(luhot_ctx*, int64_t, int64_t, double*, int64_t, int64_t, uint64_t*,
                                         int64_t*);
template int getrf_colmajor_host<float>(luhot_ctx*, int64_t, int64_t, float*, int64_t, int64_t, uint64_t*,
                                        int64_t*);

}  // namespace luhot
