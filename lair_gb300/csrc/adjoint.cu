// Adjoint (backward) of the linear solve X = A^-1 B.
//
// For a scalar loss L with upstream gradient W = dL/dX:
//   lambda = A^-T W      (transposed getrs on the stored LU factors and pivots)
//   dL/dB  = lambda
//   dL/dA  = -lambda X^T (a rank-nrhs outer product, written once: 8 n^2 bytes)
// The mixed-precision form obtains lambda by iterative refinement on A^T
// with the low-precision factors (FP64 residual), then forms dA in FP64.
// lair has no differentiation; this is an added capability of the solve.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "luhot_internal.h"

namespace luhot {

// dA[i][j] = -sum_c lambda[i][c] x[j][c]; 32 x 32 output tiles, lambda and x
// rows of the tile staged in shared memory (nrhs <= 64 per pass, accumulated).
__global__ void __launch_bounds__(256) outer_grad_kernel(const double* __restrict__ lam, int64_t ldl,
                                                         const double* __restrict__ x, int64_t ldx, double* da,
                                                         int64_t ldda, int n, int nrhs) {
  __shared__ double L[32][65];
  __shared__ double X[32][65];
  const int i0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 8 rows of threads
  double acc[4] = {0, 0, 0, 0};
  for (int c0 = 0; c0 < nrhs; c0 += 64) {
    const int nc = min(64, nrhs - c0);
    __syncthreads();
    for (int idx = threadIdx.x; idx < 32 * 64; idx += 256) {
      const int r = idx / 64, c = idx - r * 64;
      L[r][c] = (i0 + r < n && c < nc) ? lam[(int64_t)(i0 + r) * ldl + c0 + c] : 0.0;
      X[r][c] = (j0 + r < n && c < nc) ? x[(int64_t)(j0 + r) * ldx + c0 + c] : 0.0;
    }
    __syncthreads();
    for (int c = 0; c < nc; ++c) {
      const double xv = X[tx][c];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] = fma(L[ty + 8 * q][c], xv, acc[q]);
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = i0 + ty + 8 * q, j = j0 + tx;
    if (i < n && j < n) da[(int64_t)i * ldda + j] = -acc[q];
  }
}

static int launch_outer(luhot_ctx* ctx, const double* lam, int64_t ldl, const double* x, int64_t ldx, double* da,
                        int64_t ldda, int n, int nrhs) {
  dim3 grid((n + 31) / 32, (n + 31) / 32);
  prof_begin(ctx, kProfOther);
  outer_grad_kernel<<<grid, 256, 0, ctx->stream>>>(lam, ldl, x, ldx, da, ldda, n, nrhs);
  prof_end(ctx, kProfOther, 2.0 * n * (double)n * nrhs, 8.0 * n * (double)n + 16.0 * n * nrhs);
  LUHOT_CUDA_TRY(ctx, cudaGetLastError());
  return LUHOT_OK;
}

int solve_backward_device(luhot_ctx* ctx, int n, int nrhs, const double* lu, int64_t lda, const int* piv,
                          const double* x, int64_t ldx, const double* w, int64_t ldw, double* db, int64_t lddb,
                          double* da, int64_t ldda, int mode) {
  if (n < 0 || nrhs < 0 || lda < std::max(1, n) || ldx < std::max(1, nrhs) || ldw < std::max(1, nrhs) ||
      lddb < std::max(1, nrhs) || ldda < std::max(1, n))
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "backward: bad shape or leading dimension");
  if (n == 0 || nrhs == 0) return LUHOT_OK;
  // lambda = A^-T W, written straight into dB.
  int rc = getrs_device<double>(ctx, n, nrhs, lu, lda, piv, w, ldw, db, lddb, 1, mode);
  if (rc) return rc;
  if (da) {
    rc = launch_outer(ctx, db, lddb, x, ldx, da, ldda, n, nrhs);
    if (rc) return rc;
  }
  LUHOT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return LUHOT_OK;
}

int solve_backward_ir_device(luhot_ctx* ctx, int n, int nrhs, const double* a, int64_t lda, const double* x,
                             int64_t ldx, const double* w, int64_t ldw, double* db, int64_t lddb, double* da,
                             int64_t ldda, int precision, int solver, double tol, int max_iter, luhot_ir_info* info) {
  if (n < 0 || nrhs < 0 || lda < std::max(1, n) || ldx < std::max(1, nrhs) || ldw < std::max(1, nrhs) ||
      lddb < std::max(1, nrhs) || ldda < std::max(1, n))
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "backward: bad shape or leading dimension");
  if (n == 0 || nrhs == 0) {
    *info = luhot_ir_info{};
    info->converged = 1;
    info->singular = -1;
    return LUHOT_OK;
  }
  // A^T, row-major, in a private buffer; then lambda by refinement on A^T.
  const int64_t ldt = ((int64_t)n + 31) / 32 * 32;
  int rc = ensure_buf(ctx, ctx->adj_buf, (size_t)n * ldt * sizeof(double));
  if (rc) return rc;
  double* at = static_cast<double*>(ctx->adj_buf.ptr);
  rc = launch_transpose<double>(ctx, a, lda, at, ldt, n, n);
  if (rc) return rc;
  rc = gesv_ir_device(ctx, n, nrhs, at, ldt, w, ldw, db, lddb, precision, solver, tol, max_iter, info);
  if (rc) return rc;
  if (da) {
    rc = launch_outer(ctx, db, lddb, x, ldx, da, ldda, n, nrhs);
    if (rc) return rc;
  }
  LUHOT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return LUHOT_OK;
}

}  // namespace luhot

using namespace luhot;

extern "C" {

int luhot_dgesv_backward_dev(luhot_ctx* ctx, int64_t n, int64_t nrhs, const double* d_lu, int64_t lda,
                             const int32_t* d_piv, const double* d_x, int64_t ldx, const double* d_w, int64_t ldw,
                             double* d_db, int64_t lddb, double* d_da, int64_t ldda, int mode) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  CtxGuard g(ctx);
  if (n < 0 || nrhs < 0 || n >= INT32_MAX || nrhs >= INT32_MAX)
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "backward: invalid dimensions");
  if (n > 0 && nrhs > 0 && (!d_lu || !d_piv || !d_w || !d_db || (d_da && !d_x)))
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "backward: null pointer");
  return solve_backward_device(ctx, (int)n, (int)nrhs, d_lu, lda, d_piv, d_x, ldx, d_w, ldw, d_db, lddb, d_da, ldda,
                               mode);
}

int luhot_dgesv_backward_ir_dev(luhot_ctx* ctx, int64_t n, int64_t nrhs, const double* d_a, int64_t lda,
                                const double* d_x, int64_t ldx, const double* d_w, int64_t ldw, double* d_db,
                                int64_t lddb, double* d_da, int64_t ldda, int precision, int solver, double tol,
                                int max_iter, luhot_ir_info* info) {
  LUHOT_NVTX_FN();
  if (!ctx || !info) return LUHOT_ERR_INVALID_ARG;
  CtxGuard g(ctx);
  if (n < 0 || nrhs < 0 || n >= INT32_MAX || nrhs >= INT32_MAX)
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "backward: invalid dimensions");
  if (n > 0 && nrhs > 0 && (!d_a || !d_w || !d_db || (d_da && !d_x)))
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "backward: null pointer");
  return solve_backward_ir_device(ctx, (int)n, (int)nrhs, d_a, lda, d_x, ldx, d_w, ldw, d_db, lddb, d_da, ldda,
                                  precision, solver, tol, max_iter, info);
}

}  // extern "C"

extern "C" int luhot_dgesv_backward(luhot_ctx* ctx, int64_t n, int64_t nrhs, const double* lu, int64_t lu_rs,
                                    int64_t lu_cs, const uint64_t* piv, const double* x, int64_t x_rs, int64_t x_cs,
                                    const double* w, int64_t w_rs, int64_t w_cs, double* db, int64_t db_rs,
                                    int64_t db_cs, double* da, int64_t da_rs, int64_t da_cs, int mode) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  CtxGuard g(ctx);
  if (n < 0 || nrhs < 0 || n >= INT32_MAX || nrhs >= INT32_MAX)
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "backward: invalid dimensions");
  if (n == 0 || nrhs == 0) return LUHOT_OK;
  if (!lu || !piv || !w || !db || (da && !x)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "backward: null pointer");
  for (int64_t i = 0; i < n; ++i)
    if (piv[i] >= (uint64_t)n) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "backward: pivot index out of range");
  const int64_t lda = ((int64_t)n + 31) / 32 * 32;
  const size_t vec = (size_t)n * nrhs;
  int rc = ensure_buf(ctx, ctx->work[0], (size_t)n * lda * sizeof(double));
  if (!rc) rc = ensure_buf(ctx, ctx->work[2], 3 * vec * sizeof(double));
  if (!rc) rc = ensure_buf(ctx, ctx->piv_buf, (size_t)n * sizeof(int));
  if (!rc && da) rc = ensure_buf(ctx, ctx->adj_buf, (size_t)n * lda * sizeof(double));
  if (rc) return rc;
  double* d_lu = static_cast<double*>(ctx->work[0].ptr);
  double* d_x = static_cast<double*>(ctx->work[2].ptr);
  double* d_w = d_x + vec;
  double* d_db = d_w + vec;
  double* d_da = da ? static_cast<double*>(ctx->adj_buf.ptr) : nullptr;
  int* d_piv = static_cast<int*>(ctx->piv_buf.ptr);
  rc = stage_in<double>(ctx, lu, n, n, lu_rs, lu_cs, d_lu, lda, ctx->work[1]);
  if (!rc) rc = stage_in<double>(ctx, w, n, nrhs, w_rs, w_cs, d_w, nrhs, ctx->work[1]);
  if (!rc && da) rc = stage_in<double>(ctx, x, n, nrhs, x_rs, x_cs, d_x, nrhs, ctx->work[1]);
  if (rc) return rc;
  std::vector<int> hp((size_t)n);
  for (int64_t i = 0; i < n; ++i) hp[(size_t)i] = (int)piv[i];
  LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(d_piv, hp.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  rc = solve_backward_device(ctx, (int)n, (int)nrhs, d_lu, lda, d_piv, d_x, nrhs, d_w, nrhs, d_db, nrhs, d_da, lda,
                             mode);
  if (rc) return rc;
  rc = stage_out<double>(ctx, d_db, nrhs, db, n, nrhs, db_rs, db_cs, ctx->work[1]);
  if (!rc && da) rc = stage_out<double>(ctx, d_da, lda, da, n, n, da_rs, da_cs, ctx->work[1]);
  return rc;
}
