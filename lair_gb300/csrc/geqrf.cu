// Householder QR (lair's lapack::geqrf, src/lapack/geqrf.rs:9-27) and the Q
// of qr::Factorized (src/decomposition/qr.rs:26-60) on one GB300.
//
// Matrix layout: row-major in HBM with leading dimension lda.  Per column i
// three launches:
//   qr_reflector_kernel  (1 CTA)  larfg (src/lapack/larfg.rs:9-43): ||x||,
//                        beta, tau, the scaling of x by 1/(alpha - beta);
//                        copies v = [1, x] and finds its last non-zero entry;
//   qr_w_kernel          (grid over the columns of C = A[i.., i+1..])
//                        w = C^T v over rows 0..=last_v, and the last column
//                        of C with a non-zero in those rows (ilalc,
//                        src/lapack/ilal.rs:6-22);
//   qr_ger_kernel        (2-D grid) C[r][j] += ((-tau) v_r) w_j for
//                        r <= last_v, j <= last_c (larf::left + gerc,
//                        src/lapack/larf.rs:10-52, src/blas/gerc.rs).
// Exact mode follows lair's arithmetic: nrm2's sequential sum of squares,
// the dot of each column of C with v summed in increasing row order, every
// product and sum rounded apart (results are bit-identical to lair).  Fast
// mode sums in trees and uses FMA.  This level-2 form reads the trailing
// block twice and writes it once per column (~24 bytes per element); a
// blocked (compact-WY) form would move the two updates onto the FP64 tensor
// pipe.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "common.cuh"
#include "luhot_internal.h"

namespace luhot {
namespace {

constexpr int kQrThreads = 256;

template <typename T>
struct QrScalars {
  T tau;
  int last_v;  // last non-zero entry of v
  int last_c;  // last column of C with a non-zero entry in rows 0..=last_v (-1: none)
};

template <typename T>
__device__ __forceinline__ T q_mul(T a, T b);
template <>
__device__ __forceinline__ double q_mul<double>(double a, double b) {
  return __dmul_rn(a, b);
}
template <>
__device__ __forceinline__ float q_mul<float>(float a, float b) {
  return __fmul_rn(a, b);
}
template <typename T>
__device__ __forceinline__ T q_add(T a, T b);
template <>
__device__ __forceinline__ double q_add<double>(double a, double b) {
  return __dadd_rn(a, b);
}
template <>
__device__ __forceinline__ float q_add<float>(float a, float b) {
  return __fadd_rn(a, b);
}

// src/scalar.rs:393-402
template <typename T>
__device__ __forceinline__ T lair_eps() {
  return sizeof(T) == 8 ? T(1.1102230246251565e-16) : T(5.9604645e-08f);
}
template <typename T>
__device__ __forceinline__ T lair_sfmin() {
  return sizeof(T) == 8 ? T(2.2250738585072014e-308) : T(1.17549435e-38f);
}

// Rust's powi: repeated squaring in the order of compiler-rt's powi.
template <typename T>
__device__ T powi_rt(T a, int b) {
  const bool recip = b < 0;
  T r = T(1);
  for (;;) {
    if (b & 1) r = q_mul(r, a);
    b /= 2;
    if (b == 0) break;
    a = q_mul(a, a);
  }
  return recip ? T(1) / r : r;
}

// Sum of squares of x[0..n) (stride inc): sequentially in exact mode
// (nrm2's fold, src/blas/nrm2.rs:6-15), as a tree otherwise.  Result in
// thread 0 (exact) or all threads (fast, via shared memory).
template <typename T, bool kExact>
__device__ T sum_squares(const T* x, int64_t inc, int n, T* red) {
  if (kExact) {
    T s = -T(0);
    if (threadIdx.x == 0)
      for (int r = 0; r < n; ++r) {
        const T v = x[(int64_t)r * inc];
        s = q_add(s, q_add(q_mul(v, v), T(0)));
      }
    return s;
  }
  T s = T(0);
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    const T v = x[(int64_t)r * inc];
    s = fma(v, v, s);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  T t = T(0);
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
  __syncthreads();
  return t;
}

// larfg on alpha = a[i][i], x = a[i+1.., i]; v = [1, x'] to vbuf; a[i][i] = beta.
template <typename T, bool kExact>
__global__ void __launch_bounds__(kQrThreads) qr_reflector_kernel(T* a, int64_t lda, int m, int i, T* tau_out,
                                                                  T* vbuf, QrScalars<T>* sc) {
  __shared__ T red[kQrThreads / 32];
  __shared__ T s_alpha, s_beta, s_tau, s_scale;
  __shared__ int s_knt, s_zero, s_lastv;
  const int nx = m - i - 1;
  T* x = a + (int64_t)(i + 1) * lda + i;
  const T alpha0 = a[(int64_t)i * lda + i];
  T ss = sum_squares<T, kExact>(x, lda, nx, red);
  if (threadIdx.x == 0) {
    const T x_norm = sqrt(ss);
    s_lastv = 0;
    if (x_norm == T(0)) {
      s_zero = 1;
      s_beta = alpha0;
      s_tau = T(0);
    } else {
      s_zero = 0;
      // lapy3(alpha, 0, x_norm) = sqrt((alpha*alpha + 0*0) + x_norm*x_norm)
      const T r = sqrt(q_add(q_add(q_mul(alpha0, alpha0), q_mul(T(0), T(0))), q_mul(x_norm, x_norm)));
      T beta = -copysign(r, alpha0);
      T alpha = alpha0;
      const T safe_min = lair_sfmin<T>() / lair_eps<T>();
      int knt = 0;
      if (fabs(beta) < safe_min) {
        const T rcp = T(1) / safe_min;
        for (;;) {
          ++knt;
          beta = q_mul(beta, rcp);
          alpha = q_mul(alpha, rcp);
          if (fabs(beta) >= safe_min || knt >= 20) break;
        }
      }
      s_knt = knt;
      s_alpha = alpha;
      s_beta = beta;
    }
  }
  __syncthreads();
  if (!s_zero) {
    const int knt = s_knt;
    if (knt > 0) {
      // x scaled knt times by 1/safe_min, then the norm and beta again
      const T rcp = T(1) / (lair_sfmin<T>() / lair_eps<T>());
      for (int r = threadIdx.x; r < nx; r += blockDim.x) {
        T v = x[(int64_t)r * lda];
        for (int k = 0; k < knt; ++k) v = q_mul(v, rcp);
        x[(int64_t)r * lda] = v;
      }
      __syncthreads();
      ss = sum_squares<T, kExact>(x, lda, nx, red);
      if (threadIdx.x == 0) {
        const T x_norm = sqrt(ss);
        const T alpha = s_alpha;
        s_beta = -copysign(q_add(q_mul(alpha, alpha), q_mul(x_norm, x_norm)), alpha);
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      const T alpha = s_alpha, beta = s_beta;
      s_tau = (beta - alpha) / beta;
      s_scale = T(1) / (alpha - beta);
      s_beta = q_mul(beta, powi_rt(lair_sfmin<T>() / lair_eps<T>(), knt));
    }
    __syncthreads();
    const T scale = s_scale;
    for (int r = threadIdx.x; r < nx; r += blockDim.x) x[(int64_t)r * lda] = q_mul(x[(int64_t)r * lda], scale);
  }
  __syncthreads();
  // v = a[i.., i] with a[i][i] = 1, and its last non-zero entry
  int lastv = 0;
  for (int r = threadIdx.x; r < nx; r += blockDim.x) {
    const T v = x[(int64_t)r * lda];
    vbuf[r + 1] = v;
    if (v != T(0)) lastv = max(lastv, r + 1);
  }
  if (lastv > 0) atomicMax(&s_lastv, lastv);
  __syncthreads();
  if (threadIdx.x == 0) {
    vbuf[0] = T(1);
    a[(int64_t)i * lda + i] = s_beta;
    tau_out[i] = s_tau;
    sc->tau = s_tau;
    sc->last_v = s_lastv;
    sc->last_c = -1;
  }
}

// w_j = 0 + sum_r C[r][j] v_r over r <= last_v (increasing r in exact mode),
// and the last column with a non-zero entry in those rows.  Block: 32
// columns x 8 row groups (fast mode splits the rows; exact mode uses the
// first group only, one sequential sum per column).
template <typename T, bool kExact>
__global__ void __launch_bounds__(256) qr_w_kernel(const T* c, int64_t ldc, int ncols, const T* v, T* w,
                                                   QrScalars<T>* sc) {
  __shared__ T part[8][33];
  __shared__ int nzs[8][33];
  const T tau = sc->tau;
  if (tau == T(0)) return;
  const int last_v = sc->last_v;
  const int j = blockIdx.x * 32 + threadIdx.x;
  const int g = threadIdx.y;
  T sum = T(0);
  int nz = 0;
  if (j < ncols) {
    if (kExact) {
      if (g == 0)
        for (int r = 0; r <= last_v; ++r) {
          const T cv = c[(int64_t)r * ldc + j];
          sum = q_add(sum, q_mul(cv, v[r]));
          nz |= cv != T(0);
        }
    } else {
      for (int r = g; r <= last_v; r += 8) {
        const T cv = c[(int64_t)r * ldc + j];
        sum = fma(cv, v[r], sum);
        nz |= cv != T(0);
      }
    }
  }
  part[g][threadIdx.x] = sum;
  nzs[g][threadIdx.x] = nz;
  __syncthreads();
  if (g == 0 && j < ncols) {
    T s = part[0][threadIdx.x];
    int any = nzs[0][threadIdx.x];
    if (!kExact)
      for (int q = 1; q < 8; ++q) {
        s += part[q][threadIdx.x];
        any |= nzs[q][threadIdx.x];
      }
    w[j] = q_add(T(0), s);  // conjtrans: y = 0, then y += 1 * sum
    if (any) atomicMax(&sc->last_c, j);
  }
}

// C[r][j] += ((-tau) v_r) w_j for r <= last_v, j <= last_c.
template <typename T, bool kExact>
__global__ void __launch_bounds__(256) qr_ger_kernel(T* c, int64_t ldc, const T* v, const T* w, QrScalars<T>* sc) {
  const T tau = sc->tau;
  const int last_v = sc->last_v, last_c = sc->last_c;
  if (tau == T(0) || last_c < 0) return;
  const int j = blockIdx.x * 32 + threadIdx.x;
  if (j > last_c) return;
  const T wj = w[j];
  for (int r = blockIdx.y * 8 + threadIdx.y; r <= last_v; r += gridDim.y * 8) {
    const T factor = q_mul(-tau, v[r]);
    T* e = c + (int64_t)r * ldc + j;
    *e = kExact ? q_add(*e, q_mul(factor, wj)) : fma(factor, wj, *e);
  }
}

// One larf::left(v, tau, C) with v already in vbuf and the scalars set.
template <typename T, bool kExact>
int apply_reflector(luhot_ctx* ctx, T* c, int64_t ldc, int rows, int cols, const T* v, T* w, QrScalars<T>* sc) {
  if (rows <= 0 || cols <= 0) return LUHOT_OK;
  dim3 blk(32, 8);
  prof_begin(ctx, kProfOther);
  qr_w_kernel<T, kExact><<<(cols + 31) / 32, blk, 0, ctx->stream>>>(c, ldc, cols, v, w, sc);
  prof_end(ctx, kProfOther, 2.0 * rows * cols, 8.0 * rows * cols);
  const int gy = std::max(1, std::min((rows + 7) / 8, std::max(1, 4 * ctx->num_sms / ((cols + 31) / 32))));
  prof_begin(ctx, kProfOther);
  qr_ger_kernel<T, kExact><<<dim3((cols + 31) / 32, gy), blk, 0, ctx->stream>>>(c, ldc, v, w, sc);
  prof_end(ctx, kProfOther, 2.0 * rows * cols, 16.0 * rows * cols);
  LUHOT_CUDA_TRY(ctx, cudaGetLastError());
  return LUHOT_OK;
}

template <typename T>
struct QrWork {
  T* v;
  T* w;
  QrScalars<T>* sc;
};

template <typename T>
int qr_work(luhot_ctx* ctx, int m, int n, QrWork<T>* out) {
  const size_t vbytes = ((size_t)std::max(m, 1) * sizeof(T) + 255) / 256 * 256;
  const size_t wbytes = ((size_t)std::max(n, std::max(m, 1)) * sizeof(T) + 255) / 256 * 256;
  int rc = ensure_buf(ctx, ctx->work[2], vbytes + wbytes + 256);
  if (rc) return rc;
  char* base = static_cast<char*>(ctx->work[2].ptr);
  out->v = reinterpret_cast<T*>(base);
  out->w = reinterpret_cast<T*>(base + vbytes);
  out->sc = reinterpret_cast<QrScalars<T>*>(base + vbytes + wbytes);
  return LUHOT_OK;
}

template <typename T, bool kExact>
int geqrf_impl(luhot_ctx* ctx, int m, int n, T* a, int64_t lda, T* tau) {
  const int k = std::min(m, n);
  QrWork<T> wk;
  int rc = qr_work<T>(ctx, m, n, &wk);
  if (rc) return rc;
  for (int i = 0; i < k; ++i) {
    prof_begin(ctx, kProfPanel);
    qr_reflector_kernel<T, kExact><<<1, kQrThreads, 0, ctx->stream>>>(a, lda, m, i, tau, wk.v, wk.sc);
    prof_end(ctx, kProfPanel, 4.0 * (m - i), 16.0 * (m - i));
    LUHOT_CUDA_TRY(ctx, cudaGetLastError());
    rc = apply_reflector<T, kExact>(ctx, a + (int64_t)i * lda + i + 1, lda, m - i, n - i - 1, wk.v, wk.w, wk.sc);
    if (rc) return rc;
  }
  return LUHOT_OK;
}

// Q (m x m) from the factored array: lair's backward accumulation.
template <typename T, bool kExact>
__global__ void qr_q_init_kernel(const T* qr, int64_t ldqr, int m, int ntau, T* q, int64_t ldq) {
  const int64_t total = (int64_t)m * m;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t / m), c = (int)(t - (int64_t)r * m);
    q[(int64_t)r * ldq + c] = c < ntau ? qr[(int64_t)r * ldqr + c] : (r == c ? T(1) : T(0));
  }
}

// Column i of Q before its reflector: q[i][i] = 1, v = q[i.., i], last_v.
template <typename T>
__global__ void __launch_bounds__(kQrThreads) qr_q_vector_kernel(T* q, int64_t ldq, int m, int i, const T* tau,
                                                                 T* vbuf, QrScalars<T>* sc) {
  __shared__ int s_lastv;
  if (threadIdx.x == 0) s_lastv = 0;
  __syncthreads();
  int lastv = 0;
  for (int r = i + 1 + threadIdx.x; r < m; r += blockDim.x) {
    const T v = q[(int64_t)r * ldq + i];
    vbuf[r - i] = v;
    if (v != T(0)) lastv = max(lastv, r - i);
  }
  if (lastv > 0) atomicMax(&s_lastv, lastv);
  __syncthreads();
  if (threadIdx.x == 0) {
    q[(int64_t)i * ldq + i] = T(1);
    vbuf[0] = T(1);
    sc->tau = tau[i];
    sc->last_v = s_lastv;
    sc->last_c = -1;
  }
}

// After the reflector: q[i+1.., i] *= -tau (blas::scal), q[i][i] = 1 - tau,
// q[0..i, i] = 0.
template <typename T>
__global__ void qr_q_column_kernel(T* q, int64_t ldq, int m, int i, const T* tau) {
  const T t = tau[i];
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
    T* e = q + (int64_t)r * ldq + i;
    if (r < i)
      *e = T(0);
    else if (r == i)
      *e = T(1) - t;
    else if (i < m - 1)
      *e = q_mul(*e, -t);
  }
}

template <typename T, bool kExact>
int qr_q_impl(luhot_ctx* ctx, int m, int n, const T* qr, int64_t ldqr, const T* tau, T* q, int64_t ldq) {
  const int ntau = std::min(m, n);
  QrWork<T> wk;
  int rc = qr_work<T>(ctx, m, m, &wk);
  if (rc) return rc;
  const int64_t total = (int64_t)m * m;
  qr_q_init_kernel<T, kExact><<<(int)std::min<int64_t>((total + 255) / 256, 4 * ctx->num_sms), 256, 0,
                                ctx->stream>>>(qr, ldqr, m, ntau, q, ldq);
  count_launch(ctx);
  for (int i = ntau - 1; i >= 0; --i) {
    if (i < m - 1) {
      qr_q_vector_kernel<T><<<1, kQrThreads, 0, ctx->stream>>>(q, ldq, m, i, tau, wk.v, wk.sc);
      count_launch(ctx);
      rc = apply_reflector<T, kExact>(ctx, q + (int64_t)i * ldq + i + 1, ldq, m - i, m - i - 1, wk.v, wk.w, wk.sc);
      if (rc) return rc;
    }
    qr_q_column_kernel<T><<<(m + 255) / 256, 256, 0, ctx->stream>>>(q, ldq, m, i, tau);
    count_launch(ctx);
  }
  LUHOT_CUDA_TRY(ctx, cudaGetLastError());
  return LUHOT_OK;
}

template <typename T>
int64_t qr_ld(int64_t n) {
  return (std::max<int64_t>(n, 1) + 31) / 32 * 32;
}

template <typename T>
int geqrf_device(luhot_ctx* ctx, int m, int n, T* d_a, int64_t lda, T* d_tau, int mode) {
  if (m < 0 || n < 0 || lda < std::max(1, n)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "geqrf: bad shape or lda");
  if (mode != LUHOT_MODE_FAST && mode != LUHOT_MODE_EXACT)
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "geqrf: unknown mode");
  if (m == 0 || n == 0) return LUHOT_OK;
  return mode == LUHOT_MODE_EXACT ? geqrf_impl<T, true>(ctx, m, n, d_a, lda, d_tau)
                                  : geqrf_impl<T, false>(ctx, m, n, d_a, lda, d_tau);
}

template <typename T>
int geqrf_host(luhot_ctx* ctx, int64_t m, int64_t n, T* a, int64_t rs, int64_t cs, T* tau, int mode) {
  if (m < 0 || n < 0 || m >= INT32_MAX || n >= INT32_MAX) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "geqrf: invalid dimensions");
  const int64_t k = std::min(m, n);
  if (k == 0) return LUHOT_OK;
  if (!a || !tau) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "geqrf: null pointer");
  const int64_t lda = qr_ld<T>(n);
  HostPin pin_a(ctx, a, m, n, rs, cs, sizeof(T));
  int rc = ensure_buf(ctx, ctx->work[0], (size_t)m * lda * sizeof(T) + (size_t)k * sizeof(T) + 256);
  if (rc) return rc;
  T* d_a = static_cast<T*>(ctx->work[0].ptr);
  T* d_tau = d_a + m * lda;
  rc = stage_in<T>(ctx, a, m, n, rs, cs, d_a, lda, ctx->work[1]);
  if (rc) return rc;
  rc = geqrf_device<T>(ctx, (int)m, (int)n, d_a, lda, d_tau, mode);
  if (rc) return rc;
  rc = stage_out<T>(ctx, d_a, lda, a, m, n, rs, cs, ctx->work[1]);
  if (rc) return rc;
  LUHOT_CUDA_TRY(ctx, cudaMemcpy(tau, d_tau, (size_t)k * sizeof(T), cudaMemcpyDeviceToHost));
  return LUHOT_OK;
}

template <typename T>
int qr_q_host(luhot_ctx* ctx, int64_t m, int64_t n, const T* qr, int64_t rs, int64_t cs, const T* tau, T* q,
              int64_t q_rs, int64_t q_cs, int mode) {
  if (m < 0 || n < 0 || m >= INT32_MAX || n >= INT32_MAX) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "qr q: invalid dimensions");
  if (mode != LUHOT_MODE_FAST && mode != LUHOT_MODE_EXACT) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "qr q: unknown mode");
  if (m == 0) return LUHOT_OK;
  const int64_t k = std::min(m, n);
  if (!qr || !q || (k > 0 && !tau)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "qr q: null pointer");
  const int64_t ldqr = qr_ld<T>(n), ldq = qr_ld<T>(m);
  int rc = ensure_buf(ctx, ctx->work[0], ((size_t)m * ldqr + (size_t)m * ldq + (size_t)k) * sizeof(T) + 512);
  if (rc) return rc;
  T* d_qr = static_cast<T*>(ctx->work[0].ptr);
  T* d_q = d_qr + m * ldqr;
  T* d_tau = d_q + m * ldq;
  if (n > 0) {
    rc = stage_in<T>(ctx, qr, m, n, rs, cs, d_qr, ldqr, ctx->work[1]);
    if (rc) return rc;
  }
  if (k > 0)
    LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(d_tau, tau, (size_t)k * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
  rc = mode == LUHOT_MODE_EXACT ? qr_q_impl<T, true>(ctx, (int)m, (int)n, d_qr, ldqr, d_tau, d_q, ldq)
                                : qr_q_impl<T, false>(ctx, (int)m, (int)n, d_qr, ldqr, d_tau, d_q, ldq);
  if (rc) return rc;
  return stage_out<T>(ctx, d_q, ldq, q, m, m, q_rs, q_cs, ctx->work[1]);
}

}  // namespace
}  // namespace luhot

using namespace luhot;

extern "C" {

int luhot_dgeqrf(luhot_ctx* ctx, int64_t m, int64_t n, double* a, int64_t rs, int64_t cs, double* tau, int mode) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  CtxGuard g(ctx);
  return geqrf_host<double>(ctx, m, n, a, rs, cs, tau, mode);
}

int luhot_sgeqrf(luhot_ctx* ctx, int64_t m, int64_t n, float* a, int64_t rs, int64_t cs, float* tau, int mode) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  CtxGuard g(ctx);
  return geqrf_host<float>(ctx, m, n, a, rs, cs, tau, mode);
}

int luhot_dgeqrf_dev(luhot_ctx* ctx, int64_t m, int64_t n, double* d_a, int64_t lda, double* d_tau, int mode) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  CtxGuard g(ctx);
  if (m >= INT32_MAX || n >= INT32_MAX) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "geqrf: invalid dimensions");
  return geqrf_device<double>(ctx, (int)m, (int)n, d_a, lda, d_tau, mode);
}

int luhot_dqr_q(luhot_ctx* ctx, int64_t m, int64_t n, const double* qr, int64_t rs, int64_t cs, const double* tau,
                double* q, int64_t q_rs, int64_t q_cs, int mode) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  CtxGuard g(ctx);
  return qr_q_host<double>(ctx, m, n, qr, rs, cs, tau, q, q_rs, q_cs, mode);
}

int luhot_sqr_q(luhot_ctx* ctx, int64_t m, int64_t n, const float* qr, int64_t rs, int64_t cs, const float* tau,
                float* q, int64_t q_rs, int64_t q_cs, int mode) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  CtxGuard g(ctx);
  return qr_q_host<float>(ctx, m, n, qr, rs, cs, tau, q, q_rs, q_cs, mode);
}

}  // extern "C"
