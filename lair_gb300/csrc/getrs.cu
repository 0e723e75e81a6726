// Triangular solves with the LU factors (getrs) on one GB300.
//
// Layout: LU row-major (lda), right-hand sides row-major n x nrhs (ld).
// A = P L U with P the product of the sequential interchanges in piv.
//
//   trans = 0:  x = U^-1 L^-1 P^T b   (lair's getrs, src/lapack/getrs.rs:12-38)
//   trans = 1:  x = P L^-T U^-T b     (for the adjoint; no lair counterpart)
//
// P^T b is one gather through the permutation that the interchanges compose
// to (computed once by perm_kernel); P w is the matching scatter.
//
// Triangular sweeps run as one sync-free launch each (trsv.cu).  In exact mode
// the forward sweep keeps lair's order (each row subtracts l[i][k] * x[k] for
// increasing k, multiply and subtract rounded apart).  The backward sweep in
// lair subtracts u[i][k] * x[k] for k = i+1 .. n-1 in increasing k, which
// makes every row wait for the row below it and the whole sweep one dependent
// chain of n^2/2 subtractions; exact mode runs that chain literally
// (back_exact_kernel, one warp per right-hand side).  Fast mode sweeps both
// triangles sync-free with FMA.
//
// The allocation-free entry point at the end of this file uses the simpler
// blocked kernels below (a diagonal-block kernel, sequential per right-hand
// side, and an update kernel for the rows outside the block), which need no
// scratch besides the permutation and the right-hand-side copy.
#include <cuda.h>

#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "luhot_internal.h"
#include "trsv.cuh"

namespace luhot {

__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }

template <bool kExact>
__device__ __forceinline__ double sub_prod(double c, double l, double u) {
  if (kExact) return __dsub_rn(c, __dmul_rn(l, u));
  return fma(-l, u, c);
}
template <bool kExact>
__device__ __forceinline__ float sub_prod(float c, float l, float u) {
  if (kExact) return __fsub_rn(c, __fmul_rn(l, u));
  return fmaf(-l, u, c);
}

// perm[i] = row of the original vector that lands at position i once the
// interchanges piv[0..n) are applied in order (the effect of
// src/lapack/laswp.rs:11-40 on an index vector).
__global__ void perm_kernel(const int* piv_in, int n, int* perm_out, int use_smem) {
  extern __shared__ int sbuf[];
  int* perm = use_smem ? sbuf : perm_out;
  const int* piv = piv_in;
  if (use_smem) {
    int* spiv = sbuf + n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) spiv[i] = piv_in[i];
    piv = spiv;
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = i;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 0; i < n; ++i) {
      const int p = piv[i];
      if (p != i && p >= 0 && p < n) {
        const int t = perm[i];
        perm[i] = perm[p];
        perm[p] = t;
      }
    }
  }
  __syncthreads();
  if (use_smem)
    for (int i = threadIdx.x; i < n; i += blockDim.x) perm_out[i] = perm[i];
}

// x[i][r] = b[perm[i]][r] (gather) or x[perm[i]][r] = b[i][r] (scatter).
template <typename T, bool kScatter>
__global__ void permute_rows_kernel(const T* b, int64_t ldb, T* x, int64_t ldx, const int* perm,
                                    int n, int nrhs) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * nrhs) return;
  const int i = (int)(t / nrhs), r = (int)(t - (int64_t)i * nrhs);
  if (kScatter)
    x[(int64_t)perm[i] * ldx + r] = b[(int64_t)i * ldb + r];
  else
    x[(int64_t)i * ldx + r] = b[(int64_t)perm[i] * ldb + r];
}

constexpr int kTrsvBlock = 64;

// Element (i, k) of op(A): A itself or its transpose.
template <typename T, bool kTrans>
__device__ __forceinline__ T op_at(const T* a, int64_t lda, int i, int k) {
  return kTrans ? a[(int64_t)k * lda + i] : a[(int64_t)i * lda + k];
}

// Solve the diagonal block [j0, j0+bs) of a triangular op(A) in place in x.
// kLower: forward, rows ascending; otherwise backward, rows descending.
// kUnit: unit diagonal (L); otherwise divide by the diagonal (U).
template <typename T, bool kExact, bool kLower, bool kUnit, bool kTrans>
__global__ void trsv_diag_kernel(const T* a, int64_t lda, T* x, int64_t ldx, int j0, int bs,
                                 int nrhs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* A = reinterpret_cast<T*>(smem_raw);  // [bs][bs]
  for (int idx = threadIdx.x; idx < bs * bs; idx += blockDim.x) {
    const int i = idx / bs, k = idx - i * bs;
    A[idx] = op_at<T, kTrans>(a, lda, j0 + i, j0 + k);
  }
  __syncthreads();
  for (int r = threadIdx.x; r < nrhs; r += blockDim.x) {
    if (kLower) {
      for (int i = 0; i < bs; ++i) {
        T acc = x[(int64_t)(j0 + i) * ldx + r];
        for (int k = 0; k < i; ++k) acc = sub_prod<kExact>(acc, A[i * bs + k], x[(int64_t)(j0 + k) * ldx + r]);
        if (!kUnit) acc = acc / A[i * bs + i];
        x[(int64_t)(j0 + i) * ldx + r] = acc;
      }
    } else {
      for (int i = bs - 1; i >= 0; --i) {
        T acc = x[(int64_t)(j0 + i) * ldx + r];
        for (int k = i + 1; k < bs; ++k)
          acc = sub_prod<kExact>(acc, A[i * bs + k], x[(int64_t)(j0 + k) * ldx + r]);
        if (!kUnit) acc = acc / A[i * bs + i];
        x[(int64_t)(j0 + i) * ldx + r] = acc;
      }
    }
  }
}

// x[i] -= sum_{k in [j0, j0+bs)} op(A)(i, k) x[k] for rows i in [i_begin, i_end),
// k increasing.  Each CTA stages a 64-row slice of op(A)(:, J) in shared memory.
template <typename T, bool kExact, bool kTrans>
__global__ void __launch_bounds__(256) trsv_update_kernel(const T* a, int64_t lda, T* x, int64_t ldx,
                                                          int j0, int bs, int i_begin, int i_end,
                                                          int nrhs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* As = reinterpret_cast<T*>(smem_raw);  // [64][bs + 1]
  T* Xs = As + 64 * (bs + 1);              // [bs][nrhs]
  const int row0 = i_begin + blockIdx.x * 64;
  const int rows = min(64, i_end - row0);
  if (rows <= 0) return;
  for (int idx = threadIdx.x; idx < rows * bs; idx += blockDim.x) {
    int i, k;
    if (kTrans) {  // coalesce along i: element (i, k) = a[k][i]
      k = idx / rows;
      i = idx - k * rows;
    } else {
      i = idx / bs;
      k = idx - i * bs;
    }
    As[i * (bs + 1) + k] = op_at<T, kTrans>(a, lda, row0 + i, j0 + k);
  }
  for (int idx = threadIdx.x; idx < bs * nrhs; idx += blockDim.x) {
    const int k = idx / nrhs, r = idx - k * nrhs;
    Xs[idx] = x[(int64_t)(j0 + k) * ldx + r];
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < rows * nrhs; idx += blockDim.x) {
    const int i = idx / nrhs, r = idx - i * nrhs;
    T acc = x[(int64_t)(row0 + i) * ldx + r];
    for (int k = 0; k < bs; ++k) acc = sub_prod<kExact>(acc, As[i * (bs + 1) + k], Xs[k * nrhs + r]);
    x[(int64_t)(row0 + i) * ldx + r] = acc;
  }
}

// lair's backward substitution, literally (src/lapack/getrs.rs:30-36):
// for i = n-1 .. 0: for k = i+1 .. n-1: x[i] -= u[i][k] * x[k]; x[i] /= u[i][i].
// One warp per right-hand side: the lanes form the products of a 32-wide
// chunk, lane 0 subtracts them in order.  x lives in shared memory when it
// fits, else in place in global memory.
template <typename T>
__global__ void back_exact_kernel(const T* u, int64_t lda, T* x, int64_t ldx, int n, int use_smem) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T prod[32];
  T* xs = reinterpret_cast<T*>(smem_raw);
  const int r = blockIdx.x;
  const int lane = threadIdx.x;
  T* xg = x + r;  // column r, stride ldx
  if (use_smem) {
    for (int i = lane; i < n; i += 32) xs[i] = xg[(int64_t)i * ldx];
    __syncwarp();
  }
  for (int i = n - 1; i >= 0; --i) {
    const T* urow = u + (int64_t)i * lda;
    T acc = use_smem ? xs[i] : xg[(int64_t)i * ldx];
    for (int k0 = i + 1; k0 < n; k0 += 32) {
      const int k = k0 + lane;
      if (k < n) prod[lane] = mul_rn(urow[k], use_smem ? xs[k] : xg[(int64_t)k * ldx]);
      __syncwarp();
      if (lane == 0) {
        const int cnt = min(32, n - k0);
        for (int q = 0; q < cnt; ++q) acc = acc - prod[q];
      }
      __syncwarp();
    }
    if (lane == 0) {
      acc = acc / urow[i];
      if (use_smem)
        xs[i] = acc;
      else
        xg[(int64_t)i * ldx] = acc;
    }
    __syncwarp();
  }
  if (use_smem) {
    for (int i = lane; i < n; i += 32) xg[(int64_t)i * ldx] = xs[i];
  }
}

int getrs_perm(luhot_ctx* ctx, const int* piv, int n, int* perm) {
  const size_t bytes = 2 * (size_t)n * sizeof(int);  // permutation + pivots
  const int use_smem = bytes <= (size_t)ctx->max_smem_optin ? 1 : 0;
  const size_t smem = use_smem ? bytes : 0;
  LUHOT_CUDA_TRY(ctx, allow_max_dynamic_smem(perm_kernel));
  prof_begin(ctx, kProfPermute);
  perm_kernel<<<1, 1024, smem, ctx->stream>>>(piv, n, perm, use_smem);
  prof_end(ctx, kProfPermute, 0.0, 2.0 * n * sizeof(int));
  LUHOT_CUDA_TRY(ctx, cudaGetLastError());
  return LUHOT_OK;
}

int trsv_scratch(luhot_ctx* ctx, int n, int** flags, int** ticket) {
  const int nblk = trsv_syncfree_blocks(n);
  // ready flags of up to four chains of right-hand sides, then the ticket
  int rc = ensure_buf(ctx, ctx->trsv_buf, (4 * (size_t)nblk + 64) * sizeof(int));
  if (rc) return rc;
  *flags = static_cast<int*>(ctx->trsv_buf.ptr);
  *ticket = *flags + ((4 * nblk + 31) / 32) * 32;
  return LUHOT_OK;
}

// Tagged-word scratch of the chained and block-scaled sweeps (the context's
// chain buffer: words, then the ticket) and a fresh epoch for one launch.  A
// grown buffer is cleared, and so is every word when the 32-bit epoch wraps,
// so no word ever carries the epoch of a later launch.
static int sweep_tags(luhot_ctx* ctx, size_t words, unsigned long long** xt, int** ticket, unsigned int* epoch) {
  const size_t bytes = words * sizeof(unsigned long long) + 256;
  if (ctx->chain_buf.bytes < bytes) {
    int rc = ensure_buf(ctx, ctx->chain_buf, bytes);
    if (rc) return rc;
    LUHOT_CUDA_TRY(ctx, cudaMemsetAsync(ctx->chain_buf.ptr, 0, ctx->chain_buf.bytes, ctx->stream));
    ctx->chain_epoch = 0;
  }
  const size_t have = (ctx->chain_buf.bytes - 256) / sizeof(unsigned long long);
  *xt = static_cast<unsigned long long*>(ctx->chain_buf.ptr);
  *ticket = reinterpret_cast<int*>(*xt + have);
  if (++ctx->chain_epoch == 0) {  // the tag wrapped: clear every word once
    LUHOT_CUDA_TRY(ctx, cudaMemsetAsync(*xt, 0, have * sizeof(unsigned long long), ctx->stream));
    ctx->chain_epoch = 1;
  }
  *epoch = ctx->chain_epoch;
  return LUHOT_OK;
}

template <typename T>
int trsv_chain_sweep(luhot_ctx* ctx, const float* lu, int64_t lda, T* x, int n, bool lower, const T* dinv) {
  unsigned long long* xt = nullptr;
  int* ticket = nullptr;
  unsigned int epoch = 0;
  int rc = sweep_tags(ctx, trsv_chain_tag_words(n), &xt, &ticket, &epoch);
  if (rc) return rc;
  prof_begin(ctx, kProfTrsv);
  cudaError_t e = launch_trsv_chain<T>(ctx->stream, lu, lda, x, n, lower, dinv, xt, epoch, ticket, ctx->d_status);
  prof_end(ctx, kProfTrsv, (double)n * n, (double)n * n / 2 * sizeof(float) + 2.0 * n * sizeof(T));
  count_launch(ctx);
  if (e != cudaSuccess) return set_error(ctx, LUHOT_ERR_CUDA, std::string("chained sweep: ") + cudaGetErrorString(e));
  return LUHOT_OK;
}

template <typename T>
int chain_invert_blocks(luhot_ctx* ctx, int n, const float* lu, int64_t lda, T* dinv_l, T* dinv_u) {
  prof_begin(ctx, kProfTrsv);
  cudaError_t e = launch_trsv_chain_invert<T>(ctx->stream, lu, lda, n, true, dinv_l);
  if (e == cudaSuccess) e = launch_trsv_chain_invert<T>(ctx->stream, lu, lda, n, false, dinv_u);
  prof_end(ctx, kProfTrsv, 2.0 * 128.0 * 128.0 * 128.0 / 3.0 * trsv_chain_blocks(n),
           4.0 * (double)trsv_chain_inverse_elems(n) * sizeof(T));
  count_launch(ctx, 2);
  if (e != cudaSuccess) return set_error(ctx, LUHOT_ERR_CUDA, std::string("diagonal inverses: ") + cudaGetErrorString(e));
  return LUHOT_OK;
}

template int trsv_chain_sweep<float>(luhot_ctx*, const float*, int64_t, float*, int, bool, const float*);

template <typename TA, typename TW>
int scale_factor_blocks(luhot_ctx* ctx, int n, const TA* lu, int64_t lda, const double* dinv_l, const double* dinv_u,
                        TW* w, int64_t ldw) {
  prof_begin(ctx, kProfTrsv);
  cudaError_t e = launch_scale_blocks<TA, TW>(ctx->stream, lu, lda, dinv_l, dinv_u, w, ldw, n);
  const double nblk = (n + 63) / 64;
  prof_end(ctx, kProfTrsv, 2.0 * 64.0 * 64.0 * 64.0 * nblk * (nblk - 1),
           (double)n * n * (sizeof(TA) + sizeof(TW)));
  count_launch(ctx);
  if (e != cudaSuccess) return set_error(ctx, LUHOT_ERR_CUDA, std::string("block scaling: ") + cudaGetErrorString(e));
  return LUHOT_OK;
}
template int scale_factor_blocks<double, double>(luhot_ctx*, int, const double*, int64_t, const double*,
                                                 const double*, double*, int64_t);
template int scale_factor_blocks<float, double>(luhot_ctx*, int, const float*, int64_t, const double*, const double*,
                                                double*, int64_t);

template <typename TW>
int scaled_sweep(luhot_ctx* ctx, const TW* w, int64_t ldw, const double* dinv, const double* b, double* y,
                 int64_t ldy, int n, bool lower) {
  unsigned long long* xt = nullptr;
  int* ticket = nullptr;
  unsigned int epoch = 0;
  int rc = sweep_tags(ctx, trsv_scaled_tag_words(n), &xt, &ticket, &epoch);
  if (rc) return rc;
  prof_begin(ctx, kProfTrsv);
  cudaError_t e = launch_trsv_scaled<TW>(ctx->stream, w, ldw, dinv, b, y, ldy, n, lower, xt, epoch, ticket,
                                         ctx->d_status);
  prof_end(ctx, kProfTrsv, (double)n * n, (double)n * n / 2 * sizeof(TW) + 32.0 * n);
  count_launch(ctx);
  if (e != cudaSuccess) return set_error(ctx, LUHOT_ERR_CUDA, std::string("scaled sweep: ") + cudaGetErrorString(e));
  return LUHOT_OK;
}
template int scaled_sweep<double>(luhot_ctx*, const double*, int64_t, const double*, const double*, double*, int64_t,
                                  int, bool);

int getrs_scaled_apply(luhot_ctx* ctx, int n, const double* w, int64_t ldw, const int* perm, const double* b,
                       int64_t ldb, double* x, int64_t ldx, const double* dinv_l, const double* dinv_u, double* v1,
                       double* v2) {
  const int pblocks = (n + 255) / 256;
  prof_begin(ctx, kProfPermute);
  permute_rows_kernel<double, false><<<pblocks, 256, 0, ctx->stream>>>(b, ldb, v1, 1, perm, n, 1);
  prof_end(ctx, kProfPermute, 0.0, 16.0 * n);
  LUHOT_CUDA_TRY(ctx, cudaGetLastError());
  int rc = scaled_sweep<double>(ctx, w, ldw, dinv_l, v1, v2, 1, n, true);
  if (!rc) rc = scaled_sweep<double>(ctx, w, ldw, dinv_u, v2, x, ldx, n, false);
  return rc;
}
template int chain_invert_blocks<float>(luhot_ctx*, int, const float*, int64_t, float*, float*);

template <typename T>
int getrs_apply(luhot_ctx* ctx, int n, int nrhs, const T* lu, int64_t lda, const int* perm, const T* b,
                int64_t ldb, T* x, int64_t ldx, int trans, int mode, T* w, const T* dinv_l, const T* dinv_u) {
  cudaStream_t stream = ctx->stream;
  int* flags = nullptr;
  int* ticket = nullptr;
  int rc = trsv_scratch(ctx, n, &flags, &ticket);
  if (rc) return rc;
  const int64_t ldw = nrhs;
  const int64_t total = (int64_t)n * nrhs;
  const int pblocks = (int)((total + 255) / 256);
  const bool exact = (mode == LUHOT_MODE_EXACT);
  // One triangular sweep of the LU factor over w (sync-free, one launch per
  // 16 right-hand sides).
  auto sweep = [&](bool lower, bool unit, bool tr, bool ex) -> int {
    prof_begin(ctx, kProfTrsv);
    // op(A) lower: L, or U^T whose diagonal blocks invert to (D_U^-1)^T;
    // op(A) upper: U, or L^T (the kernel reads a given inverse transposed).
    const T* dinv = ex ? nullptr : ((lower != tr) ? dinv_l : dinv_u);
    cudaError_t e = launch_trsv_syncfree<T>(stream, lu, lda, w, ldw, n, nrhs, lower, unit, tr, ex, flags, ticket,
                                            ctx->d_status, dinv);
    prof_end(ctx, kProfTrsv, (double)n * n * nrhs, ((double)n * n / 2 + 2.0 * total) * sizeof(T));
    if (e != cudaSuccess) return set_error(ctx, LUHOT_ERR_CUDA, std::string("getrs sweep: ") + cudaGetErrorString(e));
    return LUHOT_OK;
  };
  if (!trans) {
    prof_begin(ctx, kProfPermute);
    permute_rows_kernel<T, false><<<pblocks, 256, 0, stream>>>(b, ldb, w, ldw, perm, n, nrhs);
    prof_end(ctx, kProfPermute, 0.0, 2.0 * total * sizeof(T));
    rc = sweep(true, true, false, exact);
    if (rc) return rc;
    if (exact) {
      const size_t xs = (size_t)n * sizeof(T);
      const int use_smem = xs <= (size_t)ctx->max_smem_optin - 1024 ? 1 : 0;
      LUHOT_CUDA_TRY(ctx, allow_max_dynamic_smem(back_exact_kernel<T>));
      prof_begin(ctx, kProfTrsv);
      back_exact_kernel<T><<<nrhs, 32, use_smem ? xs : 0, stream>>>(lu, lda, w, ldw, n, use_smem);
      prof_end(ctx, kProfTrsv, (double)n * n * nrhs, ((double)n * n / 2 + 2.0 * total) * sizeof(T));
    } else {
      rc = sweep(false, false, false, false);
      if (rc) return rc;
    }
    {
      int rc_ = copy_2d(ctx, x, ldx * sizeof(T), w, ldw * sizeof(T), nrhs * sizeof(T), n,
                                          cudaMemcpyDeviceToDevice);
      if (rc_) return rc_;
    }
  } else {
    // A^T x = b:  U^T z = b (lower, non-unit), L^T y = z (upper, unit), x = P y.
    {
      int rc_ = copy_2d(ctx, w, ldw * sizeof(T), b, ldb * sizeof(T), nrhs * sizeof(T), n,
                                          cudaMemcpyDeviceToDevice);
      if (rc_) return rc_;
    }
    rc = sweep(true, false, true, false);
    if (rc) return rc;
    rc = sweep(false, true, true, false);
    if (rc) return rc;
    prof_begin(ctx, kProfPermute);
    permute_rows_kernel<T, true><<<pblocks, 256, 0, stream>>>(w, ldw, x, ldx, perm, n, nrhs);
    prof_end(ctx, kProfPermute, 0.0, 2.0 * total * sizeof(T));
  }
  LUHOT_CUDA_TRY(ctx, cudaGetLastError());
  return LUHOT_OK;
}

template <typename T>
int getrs_device(luhot_ctx* ctx, int n, int nrhs, const T* lu, int64_t lda, const int* piv,
                 const T* b, int64_t ldb, T* x, int64_t ldx, int trans, int mode) {
  if (n < 0 || nrhs < 0 || lda < std::max(1, n) || ldb < std::max(1, nrhs) || ldx < std::max(1, nrhs))
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrs: bad shape or leading dimension");
  if (n == 0 || nrhs == 0) return LUHOT_OK;
  int rc = reset_status(ctx);
  if (rc) return rc;
  rc = ensure_buf(ctx, ctx->perm_buf, (size_t)n * sizeof(int));
  if (rc) return rc;
  int* perm = static_cast<int*>(ctx->perm_buf.ptr);
  rc = getrs_perm(ctx, piv, n, perm);
  if (rc) return rc;
  // Work in a private buffer so that x may alias b.
  rc = ensure_buf(ctx, ctx->work[3], (size_t)n * nrhs * sizeof(T));
  if (rc) return rc;
  // Fast solves use the inverses of the diagonal blocks (read transposed by
  // the transposed sweeps); one small launch (64 threads per block) against
  // two n^2 sweeps.
  T* dinv_l = nullptr;
  T* dinv_u = nullptr;
  if (mode == LUHOT_MODE_FAST) {
    const size_t ne = trsv_inverse_elems(n);
    rc = ensure_buf(ctx, ctx->dinv_buf, 2 * ne * sizeof(T));
    if (rc) return rc;
    dinv_l = static_cast<T*>(ctx->dinv_buf.ptr);
    dinv_u = dinv_l + ne;
    rc = invert_diag_blocks<T, T>(ctx, n, lu, lda, dinv_l, dinv_u);
    if (rc) return rc;
  }
  rc = getrs_apply<T>(ctx, n, nrhs, lu, lda, perm, b, ldb, x, ldx, trans, mode, static_cast<T*>(ctx->work[3].ptr),
                      dinv_l, dinv_u);
  if (rc) return rc;
  return finish_status(ctx, nullptr);
}

template <typename T, typename TA>
int invert_diag_blocks(luhot_ctx* ctx, int n, const TA* lu, int64_t lda, T* dinv_l, T* dinv_u) {
  prof_begin(ctx, kProfTrsv);
  cudaError_t e = launch_trsv_invert_diag<T, TA>(ctx->stream, lu, lda, n, true, dinv_l);
  if (e == cudaSuccess) e = launch_trsv_invert_diag<T, TA>(ctx->stream, lu, lda, n, false, dinv_u);
  prof_end(ctx, kProfTrsv, 2.0 * 64.0 * 64.0 * 64.0 / 3.0 * ((n + 63) / 64),
           4.0 * (double)trsv_inverse_elems(n) * sizeof(T));
  count_launch(ctx);
  if (e != cudaSuccess) return set_error(ctx, LUHOT_ERR_CUDA, std::string("diagonal inverses: ") + cudaGetErrorString(e));
  return LUHOT_OK;
}

template int getrs_apply<double>(luhot_ctx*, int, int, const double*, int64_t, const int*, const double*, int64_t,
                                 double*, int64_t, int, int, double*, const double*, const double*);
template int getrs_apply<float>(luhot_ctx*, int, int, const float*, int64_t, const int*, const float*, int64_t,
                                float*, int64_t, int, int, float*, const float*, const float*);
template int invert_diag_blocks<double, double>(luhot_ctx*, int, const double*, int64_t, double*, double*);
template int invert_diag_blocks<float, float>(luhot_ctx*, int, const float*, int64_t, float*, float*);
template int invert_diag_blocks<double, float>(luhot_ctx*, int, const float*, int64_t, double*, double*);
template int getrs_device<double>(luhot_ctx*, int, int, const double*, int64_t, const int*,
                                  const double*, int64_t, double*, int64_t, int, int);
template int getrs_device<float>(luhot_ctx*, int, int, const float*, int64_t, const int*,
                                 const float*, int64_t, float*, int64_t, int, int);

// ---------------------------------------------------------------------------
// Allocation-free solve (luhot_dgetrs_dev_noalloc).
//
// Some callers cannot call cudaMalloc: a host program whose device memory is
// all owned by its own pool or caching allocator (a raw cudaMalloc there
// either fails because the pool reserved the memory up front, or escapes the
// pool's accounting), and latency-critical solve loops where the implicit
// device-wide synchronisation of cudaMalloc/cudaFree is not acceptable.  A
// luhot context allocates its workspace, so this path needs no context: the
// scratch it needs (the row permutation and a copy of the right-hand sides)
// lives in the file-scope array below, which every GPU that loads this
// library holds until the process exits.  Every call uses the same array;
// calls that overlap on the GPU (different streams, or other host threads)
// race on it.  Each call writes every scratch byte it reads first (the
// permutation kernel fills all n entries, the gather all n x nrhs values), so
// nothing in it needs clearing between calls.
// ---------------------------------------------------------------------------
constexpr size_t kNoAllocScratchBytes = (size_t)LUHOT_NOALLOC_SCRATCH_BYTES;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_addr[kNoAllocMaxDevices] = {};            // device address of g_noalloc_scratch, per device
unsigned long long g_noalloc_ctx[kNoAllocMaxDevices] = {};  // id of the context that address belongs to
int g_noalloc_smem[kNoAllocMaxDevices] = {};

// Unique id of the calling thread's current CUDA context (cuCtxGetId, reached
// through the runtime's driver entry points), 0 when there is none or the
// driver cannot tell.  A context made after a cudaDeviceReset has a new id.
unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(p);
    cudaGetLastError();
  });
  if (!get_current || !get_id) return 0;
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (get_current(&c) != CUDA_SUCCESS || !c) return 0;
  if (get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Set-up, once per device with that device current: look up the device
// address of the scratch array.  In host code `g_noalloc_scratch` names a
// host-side stand-in, never the device memory, so kernels only ever get this
// address.  The address belongs to the device's context: when the context
// changes (a cudaDeviceReset ends it, the next call gets a new one), the
// set-up runs again, so no call launches with an address of a context that
// is gone.
int noalloc_setup(void** scratch, int* max_smem) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return LUHOT_ERR_CUDA;
  }
  if (dev < 0 || dev >= kNoAllocMaxDevices) return LUHOT_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  const unsigned long long ctx_id = current_context_id();
  if (!g_noalloc_addr[dev] || ctx_id == 0 || ctx_id != g_noalloc_ctx[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress((void**)&p, g_noalloc_scratch) != cudaSuccess || !p) {
      cudaGetLastError();
      return LUHOT_ERR_CUDA;
    }
    int smem = 0;
    if (cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
      cudaGetLastError();
      return LUHOT_ERR_CUDA;
    }
    g_noalloc_smem[dev] = smem;
    g_noalloc_addr[dev] = p;
    g_noalloc_ctx[dev] = current_context_id();  // the lookup made the context current if none was
  }
  *scratch = g_noalloc_addr[dev];
  *max_smem = g_noalloc_smem[dev];
  return LUHOT_OK;
}

// Right-hand sides per update launch: the update kernel stages its block of
// x (64 rows x chunk) in shared memory.
constexpr int kNoAllocRhsChunk = 256;

template <typename T, bool kExact, bool kLower, bool kUnit, bool kTrans>
cudaError_t trsv_noalloc(const T* a, int64_t lda, T* x, int64_t ldx, int n, int nrhs, cudaStream_t stream) {
  const int bsz = kTrsvBlock;
  auto dk = trsv_diag_kernel<T, kExact, kLower, kUnit, kTrans>;
  auto uk = trsv_update_kernel<T, kExact, kTrans>;
  cudaError_t e = allow_max_dynamic_smem(dk);
  if (e != cudaSuccess) return e;
  e = allow_max_dynamic_smem(uk);
  if (e != cudaSuccess) return e;
  const int nblk = (n + bsz - 1) / bsz;
  for (int s = 0; s < nblk; ++s) {
    const int blk = kLower ? s : (nblk - 1 - s);
    const int j0 = blk * bsz;
    const int bs = std::min(bsz, n - j0);
    dk<<<1, 128, (size_t)bs * bs * sizeof(T), stream>>>(a, lda, x, ldx, j0, bs, nrhs);
    const int i_begin = kLower ? j0 + bs : 0;
    const int i_end = kLower ? n : j0;
    for (int c0 = 0; i_end > i_begin && c0 < nrhs; c0 += kNoAllocRhsChunk) {
      const int nc = std::min(kNoAllocRhsChunk, nrhs - c0);
      const size_t sm = ((size_t)64 * (bs + 1) + (size_t)bs * nc) * sizeof(T);
      uk<<<(i_end - i_begin + 63) / 64, 256, sm, stream>>>(a, lda, x + c0, ldx, j0, bs, i_begin, i_end, nc);
    }
  }
  return cudaGetLastError();
}
}  // namespace

}  // namespace luhot

extern "C" int luhot_dgetrs_dev_noalloc(int64_t n, int64_t nrhs, const double* d_lu, int64_t lda,
                                        const int32_t* d_piv, double* d_b, int64_t ldb, int trans,
                                        int mode, void* cuda_stream) {
  LUHOT_NVTX_FN();
  using namespace luhot;
  if (n < 0 || nrhs < 0 || n >= INT32_MAX || nrhs >= INT32_MAX) return LUHOT_ERR_INVALID_ARG;
  if (mode != LUHOT_MODE_FAST && mode != LUHOT_MODE_EXACT) return LUHOT_ERR_INVALID_ARG;
  if (n == 0 || nrhs == 0) return LUHOT_OK;
  if (!d_lu || !d_piv || !d_b || lda < n || ldb < nrhs) return LUHOT_ERR_INVALID_ARG;
  const size_t perm_bytes = ((size_t)n * sizeof(int) + 255) / 256 * 256;
  const size_t work_bytes = (size_t)n * (size_t)nrhs * sizeof(double);
  if (perm_bytes + work_bytes > kNoAllocScratchBytes) return LUHOT_ERR_UNSUPPORTED;
  void* scratch = nullptr;
  int max_smem = 0;
  int rc = noalloc_setup(&scratch, &max_smem);
  if (rc) return rc;
  cudaStream_t stream = static_cast<cudaStream_t>(cuda_stream);
  int* perm = static_cast<int*>(scratch);
  double* w = reinterpret_cast<double*>(static_cast<unsigned char*>(scratch) + perm_bytes);
  const int nn = (int)n, nr = (int)nrhs;
  const int64_t ldw = nrhs;
  const int64_t total = n * nrhs;
  const int pblocks = (int)((total + 255) / 256);
  const int use_smem = 2 * (size_t)n * sizeof(int) <= (size_t)max_smem ? 1 : 0;
  if (allow_max_dynamic_smem(perm_kernel) != cudaSuccess) {
    cudaGetLastError();
    return LUHOT_ERR_CUDA;
  }
  perm_kernel<<<1, 1024, use_smem ? 2 * n * sizeof(int) : 0, stream>>>(d_piv, nn, perm, use_smem);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && !trans) {
    permute_rows_kernel<double, false><<<pblocks, 256, 0, stream>>>(d_b, ldb, w, ldw, perm, nn, nr);
    if (mode == LUHOT_MODE_EXACT) {
      e = trsv_noalloc<double, true, true, true, false>(d_lu, lda, w, ldw, nn, nr, stream);
      const size_t xs = (size_t)n * sizeof(double);
      const int xs_smem = xs <= (size_t)max_smem - 1024 ? 1 : 0;
      if (e == cudaSuccess) e = allow_max_dynamic_smem(back_exact_kernel<double>);
      if (e == cudaSuccess)
        back_exact_kernel<double><<<nr, 32, xs_smem ? xs : 0, stream>>>(d_lu, lda, w, ldw, nn, xs_smem);
    } else {
      e = trsv_noalloc<double, false, true, true, false>(d_lu, lda, w, ldw, nn, nr, stream);
      if (e == cudaSuccess) e = trsv_noalloc<double, false, false, false, false>(d_lu, lda, w, ldw, nn, nr, stream);
    }
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(d_b, ldb * sizeof(double), w, ldw * sizeof(double), nrhs * sizeof(double), n,
                            cudaMemcpyDeviceToDevice, stream);
  } else if (e == cudaSuccess) {
    e = cudaMemcpy2DAsync(w, ldw * sizeof(double), d_b, ldb * sizeof(double), nrhs * sizeof(double), n,
                          cudaMemcpyDeviceToDevice, stream);
    if (e == cudaSuccess) e = trsv_noalloc<double, false, true, false, true>(d_lu, lda, w, ldw, nn, nr, stream);
    if (e == cudaSuccess) e = trsv_noalloc<double, false, false, true, true>(d_lu, lda, w, ldw, nn, nr, stream);
    if (e == cudaSuccess)
      permute_rows_kernel<double, true><<<pblocks, 256, 0, stream>>>(w, ldw, d_b, ldb, perm, nn, nr);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    cudaGetLastError();
    return LUHOT_ERR_CUDA;
  }
  return LUHOT_OK;
}
