// Device-resident LU factors: factor once, solve many times, read back lazily.
//
// lair's lu::Factorized (src/decomposition/lu.rs:12-20, 156-171) owns the
// factored array and its pivots; Factorized::solve (lu.rs:87-98) runs getrs
// on them for each right-hand side.  Here the factor stays in HBM between
// solves together with everything a solve derives from it once: the row
// permutation composed from the pivots and the inverses of the 64 x 64
// diagonal blocks of L and U (fast mode).  A solve then moves only b and x
// across PCIe/C2C and runs two triangular sweeps.  The host copy of the
// factored array is written only when luhot_factor_read asks for it, which is
// what p()/l()/u() (lu.rs:28-72) need.
#include <algorithm>
#include <string>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "luhot_internal.h"
#include "trsv.cuh"

struct luhot_factor {
  luhot_ctx* ctx = nullptr;
  int dtype = 0;  // 0 = f64, 1 = f32
  int mode = LUHOT_MODE_FAST;
  int64_t m = 0, n = 0, lda = 0;
  void* d_lu = nullptr;   // m x n row-major, leading dimension lda
  int* d_piv = nullptr;   // min(m, n) int32 pivots
  int* d_perm = nullptr;  // m composed row order (m <= n only)
  void* d_dinv = nullptr; // inverses of the diagonal blocks of L then U (fast mode, m <= n)
  size_t dinv_elems = 0;  // per triangle
  // Block-scaled off-diagonal tiles of L and U (FP64 fast mode, square),
  // formed by the first single-right-hand-side solve; no_scaled once that
  // allocation failed (later solves keep the plain sweeps).
  double* d_w = nullptr;
  bool no_scaled = false;
};

namespace luhot {
namespace {

int64_t round_up(int64_t v, int64_t m) { return (v + m - 1) / m * m; }

void free_factor(luhot_factor* f) {
  if (!f) return;
  if (f->d_lu) cudaFree(f->d_lu);
  if (f->d_piv) cudaFree(f->d_piv);
  if (f->d_perm) cudaFree(f->d_perm);
  if (f->d_dinv) cudaFree(f->d_dinv);
  if (f->d_w) cudaFree(f->d_w);
  delete f;
}

int factor_alloc(luhot_ctx* ctx, void** p, size_t bytes, const char* what) {
  if (cudaMalloc(p, std::max<size_t>(bytes, 256)) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return set_error(ctx, LUHOT_ERR_ALLOC, std::string("factor: cannot allocate ") + what);
  }
  return LUHOT_OK;
}

template <typename T>
int factor_create(luhot_ctx* ctx, int64_t m, int64_t n, const T* a, int64_t rs, int64_t cs, const T* d_a,
                  int64_t ld_in, int mode, uint64_t* piv, int64_t* singular, luhot_factor** out) {
  if (!out) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "factor: null output handle");
  *out = nullptr;
  if (m < 0 || n < 0 || m >= (int64_t)INT32_MAX || n >= (int64_t)INT32_MAX)
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "factor: invalid dimensions");
  if (mode != LUHOT_MODE_FAST && mode != LUHOT_MODE_EXACT)
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "factor: unknown mode");
  const int64_t k = std::min(m, n);
  if ((m * n > 0 && !a && !d_a) || (k > 0 && !piv))
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "factor: null pointer");
  if (d_a && ld_in < std::max<int64_t>(1, n))
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "factor: leading dimension below n");
  if (singular) *singular = -1;

  luhot_factor* f = new luhot_factor();
  f->ctx = ctx;
  f->dtype = sizeof(T) == 8 ? 0 : 1;
  f->mode = mode;
  f->m = m;
  f->n = n;
  f->lda = round_up(std::max<int64_t>(n, 1), 256 / (int64_t)sizeof(T));
  const bool solvable = m <= n && m > 0;
  int rc = factor_alloc(ctx, &f->d_lu, (size_t)m * f->lda * sizeof(T), "the factor");
  if (!rc) rc = factor_alloc(ctx, reinterpret_cast<void**>(&f->d_piv), (size_t)k * sizeof(int), "the pivots");
  if (!rc && solvable)
    rc = factor_alloc(ctx, reinterpret_cast<void**>(&f->d_perm), (size_t)m * sizeof(int), "the permutation");
  if (!rc && solvable && mode == LUHOT_MODE_FAST) {
    f->dinv_elems = trsv_inverse_elems((int)m);
    rc = factor_alloc(ctx, &f->d_dinv, 2 * f->dinv_elems * sizeof(T), "the diagonal inverses");
  }
  if (rc) {
    free_factor(f);
    return rc;
  }
  T* lu = static_cast<T*>(f->d_lu);
  if (k > 0) {
    HostPin pin_a(ctx, d_a ? nullptr : a, m, n, rs, cs, sizeof(T));
    int64_t sing = -1;
    if (!d_a && mode == LUHOT_MODE_EXACT && getrf_uses_colmajor(m, n, rs, cs)) {
      // lair factors a non-standard layout in its column-major order
      // (src/lapack/getrf.rs:20-26, 128-213): run that order on an F-order
      // copy, then keep the factored copy on the device.
      std::vector<T> colmajor((size_t)m * n);
      for (int64_t j = 0; j < n; ++j)
        for (int64_t i = 0; i < m; ++i) colmajor[(size_t)j * m + i] = a[i * rs + j * cs];
      rc = getrf_colmajor_host<T>(ctx, m, n, colmajor.data(), 1, m, piv, &sing);
      if (!rc) rc = stage_in<T>(ctx, colmajor.data(), m, n, 1, m, lu, f->lda, ctx->work[1]);
      if (!rc) {
        std::vector<int> hp((size_t)k);
        for (int64_t i = 0; i < k; ++i) hp[(size_t)i] = (int)piv[i];
        if (cudaMemcpyAsync(f->d_piv, hp.data(), (size_t)k * sizeof(int), cudaMemcpyHostToDevice, ctx->stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(ctx->stream) != cudaSuccess)
          rc = set_error(ctx, LUHOT_ERR_CUDA, std::string("factor: ") + cudaGetErrorString(cudaGetLastError()));
      }
    } else {
      if (d_a) {
        rc = copy_2d(ctx, lu, f->lda * sizeof(T), d_a, ld_in * sizeof(T), n * sizeof(T), m,
                     cudaMemcpyDeviceToDevice);
      } else {
        rc = stage_in<T>(ctx, a, m, n, rs, cs, lu, f->lda, ctx->work[1]);
      }
      if (!rc) rc = getrf_device<T>(ctx, (int)m, (int)n, lu, f->lda, f->d_piv, mode, &sing);
    }
    if (!rc && solvable) rc = getrs_perm(ctx, f->d_piv, (int)m, f->d_perm);
    if (!rc && f->d_dinv) {
      T* dl = static_cast<T*>(f->d_dinv);
      rc = invert_diag_blocks<T, T>(ctx, (int)m, lu, f->lda, dl, dl + f->dinv_elems);
    }
    if (!rc) {
      std::vector<int> hp((size_t)k);
      if (cudaMemcpyAsync(hp.data(), f->d_piv, (size_t)k * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream) !=
              cudaSuccess ||
          cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        rc = set_error(ctx, LUHOT_ERR_CUDA, std::string("factor: ") + cudaGetErrorString(cudaGetLastError()));
      } else {
        for (int64_t i = 0; i < k; ++i) piv[i] = (uint64_t)hp[(size_t)i];
        if (singular) *singular = sing;
      }
    }
  }
  if (rc) {
    free_factor(f);
    return rc;
  }
  *out = f;
  return LUHOT_OK;
}

template <typename T>
int factor_solve(luhot_factor* f, int64_t nrhs, const T* b, int64_t b_rs, int64_t b_cs, T* x, int64_t x_rs,
                 int64_t x_cs, T* d_b, int64_t ldb, int trans) {
  luhot_ctx* ctx = f->ctx;
  const int64_t n = f->m;
  if (f->m > f->n)
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "factor solve: the factor has more rows than columns");
  if (nrhs < 0 || nrhs >= (int64_t)INT32_MAX || n * nrhs / std::max<int64_t>(nrhs, 1) != n)
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "factor solve: invalid number of right-hand sides");
  if (n == 0 || nrhs == 0) return LUHOT_OK;
  const bool host = (d_b == nullptr);
  if (host && (!b || !x)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "factor solve: null pointer");
  if (!host && ldb < nrhs) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "factor solve: ldb below nrhs");
  int rc = LUHOT_OK;
  if (host) {
    ldb = nrhs;
    rc = ensure_buf(ctx, ctx->work[2], (size_t)n * ldb * sizeof(T));
    if (rc) return rc;
    d_b = static_cast<T*>(ctx->work[2].ptr);
    rc = stage_in<T>(ctx, b, n, nrhs, b_rs, b_cs, d_b, ldb, ctx->work[1]);
    if (rc) return rc;
  }
  rc = ensure_buf(ctx, ctx->work[3], (size_t)n * nrhs * sizeof(T));
  if (rc) return rc;
  rc = reset_status(ctx);
  if (rc) return rc;
  const T* dl = f->d_dinv ? static_cast<const T*>(f->d_dinv) : nullptr;
  const T* du = f->d_dinv ? dl + f->dinv_elems : nullptr;
  if constexpr (std::is_same<T, double>::value) {
    // One right-hand side, fast mode: the block-scaled sweeps (W formed once,
    // n^2 more doubles on the device).
    if (nrhs == 1 && !trans && dl && f->m == f->n && !f->no_scaled) {
      if (!f->d_w) {
        if (cudaMalloc(reinterpret_cast<void**>(&f->d_w), (size_t)n * f->lda * sizeof(double)) != cudaSuccess) {
          cudaGetLastError();
          f->d_w = nullptr;
          f->no_scaled = true;
        } else {
          rc = scale_factor_blocks(ctx, (int)n, static_cast<const double*>(f->d_lu), f->lda, dl, du, f->d_w, f->lda);
          if (rc) return rc;
        }
      }
      if (f->d_w) {
        rc = ensure_buf(ctx, ctx->work[3], 2 * (size_t)n * sizeof(double));
        if (rc) return rc;
        double* v1 = static_cast<double*>(ctx->work[3].ptr);
        rc = getrs_scaled_apply(ctx, (int)n, f->d_w, f->lda, f->d_perm, d_b, ldb, d_b, ldb, dl, du, v1, v1 + n);
        if (rc) return rc;
        rc = finish_status(ctx, nullptr);
        if (rc) return rc;
        if (host) rc = stage_out<T>(ctx, d_b, ldb, x, n, nrhs, x_rs, x_cs, ctx->work[1]);
        return rc;
      }
    }
  }
  rc = getrs_apply<T>(ctx, (int)n, (int)nrhs, static_cast<const T*>(f->d_lu), f->lda, f->d_perm, d_b, ldb, d_b,
                      ldb, trans, f->mode, static_cast<T*>(ctx->work[3].ptr), dl, du);
  if (rc) return rc;
  rc = finish_status(ctx, nullptr);
  if (rc) return rc;
  if (host) rc = stage_out<T>(ctx, d_b, ldb, x, n, nrhs, x_rs, x_cs, ctx->work[1]);
  return rc;
}

template <typename T>
int factor_check(const luhot_factor* f) {
  if (!f) return LUHOT_ERR_INVALID_ARG;
  if (f->dtype != (sizeof(T) == 8 ? 0 : 1))
    return set_error(f->ctx, LUHOT_ERR_INVALID_ARG, "factor: element type does not match the factor");
  return LUHOT_OK;
}

}  // namespace
}  // namespace luhot

using namespace luhot;

extern "C" {

int luhot_dfactor_create(luhot_ctx* ctx, int64_t m, int64_t n, const double* a, int64_t rs, int64_t cs, int mode,
                         uint64_t* piv, int64_t* singular, luhot_factor** out) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  CtxGuard g(ctx);
  return factor_create<double>(ctx, m, n, a, rs, cs, nullptr, 0, mode, piv, singular, out);
}

int luhot_sfactor_create(luhot_ctx* ctx, int64_t m, int64_t n, const float* a, int64_t rs, int64_t cs, int mode,
                         uint64_t* piv, int64_t* singular, luhot_factor** out) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  CtxGuard g(ctx);
  return factor_create<float>(ctx, m, n, a, rs, cs, nullptr, 0, mode, piv, singular, out);
}

int luhot_dfactor_create_dev(luhot_ctx* ctx, int64_t m, int64_t n, const double* d_a, int64_t lda, int mode,
                             uint64_t* piv, int64_t* singular, luhot_factor** out) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  CtxGuard g(ctx);
  if (m * n > 0 && !d_a) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "factor: null pointer");
  return factor_create<double>(ctx, m, n, nullptr, 0, 0, d_a, lda, mode, piv, singular, out);
}

int luhot_dfactor_solve(luhot_factor* f, int64_t nrhs, const double* b, int64_t b_rs, int64_t b_cs, double* x,
                        int64_t x_rs, int64_t x_cs, int trans) {
  LUHOT_NVTX_FN();
  if (!f) return LUHOT_ERR_INVALID_ARG;
  CtxGuard g(f->ctx);
  int rc = factor_check<double>(f);
  if (rc) return rc;
  return factor_solve<double>(f, nrhs, b, b_rs, b_cs, x, x_rs, x_cs, nullptr, 0, trans);
}

int luhot_sfactor_solve(luhot_factor* f, int64_t nrhs, const float* b, int64_t b_rs, int64_t b_cs, float* x,
                        int64_t x_rs, int64_t x_cs, int trans) {
  LUHOT_NVTX_FN();
  if (!f) return LUHOT_ERR_INVALID_ARG;
  CtxGuard g(f->ctx);
  int rc = factor_check<float>(f);
  if (rc) return rc;
  return factor_solve<float>(f, nrhs, b, b_rs, b_cs, x, x_rs, x_cs, nullptr, 0, trans);
}

int luhot_dfactor_solve_dev(luhot_factor* f, int64_t nrhs, double* d_b, int64_t ldb, int trans) {
  LUHOT_NVTX_FN();
  if (!f) return LUHOT_ERR_INVALID_ARG;
  CtxGuard g(f->ctx);
  int rc = factor_check<double>(f);
  if (rc) return rc;
  if (f->m * nrhs > 0 && !d_b) return set_error(f->ctx, LUHOT_ERR_INVALID_ARG, "factor solve: null pointer");
  if (f->m * nrhs == 0) return LUHOT_OK;
  return factor_solve<double>(f, nrhs, nullptr, 0, 0, nullptr, 0, 0, d_b, ldb, trans);
}

int luhot_factor_read(luhot_factor* f, void* a, int64_t rs, int64_t cs) {
  LUHOT_NVTX_FN();
  if (!f) return LUHOT_ERR_INVALID_ARG;
  CtxGuard g(f->ctx);
  if (f->m * f->n == 0) return LUHOT_OK;
  if (!a) return set_error(f->ctx, LUHOT_ERR_INVALID_ARG, "factor read: null pointer");
  if (f->dtype == 0)
    return stage_out<double>(f->ctx, static_cast<const double*>(f->d_lu), f->lda, static_cast<double*>(a), f->m,
                             f->n, rs, cs, f->ctx->work[1]);
  return stage_out<float>(f->ctx, static_cast<const float*>(f->d_lu), f->lda, static_cast<float*>(a), f->m, f->n,
                          rs, cs, f->ctx->work[1]);
}

int luhot_factor_device(const luhot_factor* f, const void** d_lu, int64_t* lda, const int32_t** d_piv) {
  if (!f) return LUHOT_ERR_INVALID_ARG;
  if (d_lu) *d_lu = f->d_lu;
  if (lda) *lda = f->lda;
  if (d_piv) *d_piv = f->d_piv;
  return LUHOT_OK;
}

void luhot_factor_destroy(luhot_factor* f) {
  if (!f) return;
  CtxGuard g(f->ctx);
  cudaStreamSynchronize(f->ctx->stream);
  free_factor(f);
}

}  // extern "C"
