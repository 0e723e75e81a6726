// Mixed-precision LU with iterative refinement (plain IR and GMRES-IR).
//
// The factorization runs in a low precision; FP64 is used only for the
// residual r = b - A x, the update x += d and the backward-error test
//   berr = ||r||_inf / (||A||_inf ||x||_inf + ||b||_inf)  <= tol (n * 2^-53 by default).
//
// Plain IR (Wilkinson / Moler): d = (LU)^-1 r in the low precision, x += d.
// Converges when kappa(A) * u_low < 1 (FP32: kappa up to ~1e6).
// GMRES-IR (Carson & Higham, SIAM J. Sci. Comput. 2017/2018): the correction
// equation A d = r is solved by restarted GMRES in FP64 on the left-
// preconditioned system (LU)^-1 A d = (LU)^-1 r; the low-precision factors
// are applied to FP64 vectors in FP64 arithmetic (their storage stays FP32),
// so each preconditioner application is accurate to the factors themselves;
// classical Gram-Schmidt with one reorthogonalisation pass; Givens rotations
// and the small least-squares problem on the host.  It converges for much
// larger kappa * u_low.
//
// Every plain-IR correction solve scales its right-hand side by its
// infinity norm first (the scale stays on the device), so tiny residuals
// neither underflow nor lose relative accuracy in the low precision.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "common.cuh"
#include "luhot_internal.h"
#include "tc_gemm.cuh"
#include "trsv.cuh"

namespace luhot {

__device__ __forceinline__ void atomic_max_nonneg(double* addr, double v) {
  // Non-negative doubles order like their bit patterns; NaN sorts above inf.
  atomicMax(reinterpret_cast<unsigned long long*>(addr), (unsigned long long)__double_as_longlong(v));
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
  return v;
}

template <typename Tlo>
__device__ __forceinline__ Tlo to_low(double v) {
  return static_cast<Tlo>(v);
}

// lo = A (rounded), anorm = max_i sum_j |a_ij|.  One warp per row.
template <typename Tlo>
__global__ void ir_convert_kernel(const double* __restrict__ a, int64_t lda, Tlo* lo, int64_t ldlo, int n,
                                  double* anorm) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n) return;
  const double* row = a + (int64_t)warp * lda;
  Tlo* out = lo + (int64_t)warp * ldlo;
  double s = 0.0;
  for (int c = lane; c < n; c += 32) {
    const double v = row[c];
    s += fabs(v);
    out[c] = to_low<Tlo>(v);
  }
  s = warp_sum(s);
  if (lane == 0) atomic_max_nonneg(anorm, s);
}

// kResidual: r = b - A x and rnorm = max |r_i|;  otherwise r = A x.
// One warp per row, FP64 FMA, x read through L1/L2 (n doubles).
template <bool kResidual>
__global__ void ir_matvec_kernel(const double* __restrict__ a, int64_t lda, const double* __restrict__ x,
                                 const double* __restrict__ b, double* r, int n, double* rnorm) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n) return;
  const double* row = a + (int64_t)warp * lda;
  double s0 = 0.0, s1 = 0.0;
  int c = lane * 2;
  if ((reinterpret_cast<uintptr_t>(row) & 15) == 0) {
    for (; c + 1 < n; c += 64) {
      const double2 v = *reinterpret_cast<const double2*>(row + c);
      s0 = fma(v.x, x[c], s0);
      s1 = fma(v.y, x[c + 1], s1);
    }
    if (c < n) s0 = fma(row[c], x[c], s0);
  } else {
    for (int cc = lane; cc < n; cc += 32) s0 = fma(row[cc], x[cc], s0);
  }
  const double s = warp_sum(s0 + s1);
  if (lane == 0) {
    if (kResidual) {
      const double ri = b[warp] - s;
      r[warp] = ri;
      atomic_max_nonneg(rnorm, fabs(ri));
    } else {
      r[warp] = s;
    }
  }
}

// out[i] = v[perm[i]] (P^T v).
template <typename T>
__global__ void ir_gather_kernel(const T* __restrict__ v, const int* __restrict__ perm, T* out, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = v[perm[i]];
}

__global__ void ir_infnorm_kernel(const double* __restrict__ v, int n, double* out) {
  double m = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) m = fmax(m, fabs(v[i]));
  m = warp_max(m);
  if ((threadIdx.x & 31) == 0) atomic_max_nonneg(out, m);
}

// lo = v / scale (scale = *sc, or 1 when it is 0).
template <typename Tlo>
__global__ void ir_to_low_kernel(const double* __restrict__ v, Tlo* lo, int n, const double* sc) {
  const double s = *sc;
  const double inv = (s > 0.0 && isfinite(s)) ? 1.0 / s : 1.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    lo[i] = to_low<Tlo>(v[i] * inv);
}

// out = lo * scale   or (kAdd) x += lo * scale with xnorm = max |x|.
template <typename Tlo, bool kAdd>
__global__ void ir_from_low_kernel(const Tlo* __restrict__ lo, double* out, int n, const double* sc, double* xnorm) {
  const double s = *sc;
  const double mul = (s > 0.0 && isfinite(s)) ? s : 1.0;
  double m = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double d = static_cast<double>(lo[i]) * mul;
    if (kAdd) {
      const double xi = out[i] + d;
      out[i] = xi;
      m = fmax(m, fabs(xi));
    } else {
      out[i] = d;
    }
  }
  if (kAdd) {
    m = warp_max(m);
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(xnorm, m);
  }
}

// h[j] += sum_i V_j[i] w[i] for j < k  (V_j contiguous, n each).
__global__ void ir_dots_kernel(const double* __restrict__ V, int k, const double* __restrict__ w, double* h, int n) {
  __shared__ double part[32][8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int j0 = 0; j0 < k; j0 += 8) {
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      const double wi = w[i];
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (j0 + q < k) acc[q] = fma(V[(int64_t)(j0 + q) * n + i], wi, acc[q]);
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const double s = warp_sum(acc[q]);
      if (lane == 0) part[wid][q] = s;
    }
    __syncthreads();
    if (threadIdx.x < 8 && j0 + threadIdx.x < k) {
      double s = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += part[q][threadIdx.x];
      atomicAdd(&h[j0 + threadIdx.x], s);
    }
    __syncthreads();
  }
}

// w -= sum_j V_j h_j (j < k);  if nrm2 != nullptr, also nrm2 += sum w_i^2.
__global__ void ir_orth_kernel(const double* __restrict__ V, int k, const double* __restrict__ h, double* w, int n,
                               double* nrm2) {
  double sq = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double wi = w[i];
    for (int j = 0; j < k; ++j) wi = fma(-V[(int64_t)j * n + i], h[j], wi);
    w[i] = wi;
    sq = fma(wi, wi, sq);
  }
  if (nrm2) {
    sq = warp_sum(sq);
    if ((threadIdx.x & 31) == 0) atomicAdd(nrm2, sq);
  }
}

// dst = src * (1 / *den)   (den = a 2-norm, taken as sqrt here when kSqrt).
template <bool kSqrt>
__global__ void ir_scale_kernel(const double* src, double* dst, int n, const double* den) {
  const double d = kSqrt ? sqrt(*den) : *den;
  const double inv = d > 0.0 ? 1.0 / d : 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[i] * inv;
}

// x += sum_j V_j y_j, xnorm = max |x|.
__global__ void ir_combine_kernel(const double* __restrict__ V, int k, const double* __restrict__ y, double* x, int n,
                                  double* xnorm) {
  double m = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double xi = x[i];
    for (int j = 0; j < k; ++j) xi = fma(V[(int64_t)j * n + i], y[j], xi);
    x[i] = xi;
    m = fmax(m, fabs(xi));
  }
  m = warp_max(m);
  if ((threadIdx.x & 31) == 0) atomic_max_nonneg(xnorm, m);
}

// ---------------------------------------------------------------------------
// Driver.
// ---------------------------------------------------------------------------
namespace {

// Krylov dimension before a restart.  For the kappa = 1e4 systems of the
// benchmark with 11-bit (TF32 / FP16) factors, unrestarted GMRES needs about
// 25, 35, 51 and 88 iterations at n = 512 ... 4096 (it grows like n^0.7), so
// about 250 at n = 16384; restarting every 120 iterations stalled there.
constexpr int kGmresRestart = 400;
constexpr double kGmresTol = 1e-6;  // relative reduction of the preconditioned residual per solve
// Preconditioner applications in one solve before the block-scaled tiles are
// formed: the forming costs about as much as 24 plain applications at large n.
constexpr int kScaledAfter = 24;

// Device scalars.
enum Sc : int { kAnorm = 0, kBnorm, kRnorm, kXnorm, kVscale, kNrm2, kH = 8 };
static_assert(kH + kGmresRestart + 1 <= kIrScalarSlots, "scalar slots hold one Hessenberg column");

template <typename Tlo>
struct IrRun {
  luhot_ctx* ctx;
  int n;
  const double* a;
  int64_t lda;
  Tlo* lu;
  int64_t ldlo;
  int* piv;
  int* perm;
  Tlo* lo1;
  Tlo* lo2;
  double* r;   // residual / Arnoldi work
  double* t;   // second FP64 work vector
  double* u;   // third FP64 work vector (block-scaled preconditioner sweeps)
  double* w64 = nullptr; // block-scaled tiles of the factors, once formed
  int minv_calls = 0;    // preconditioner applications of this solve
  double* V;   // (restart + 1) x n
  double* sc;  // device scalars
  double* hsc; // pinned host mirror of sc
  double* dl64 = nullptr;  // inverses of the diagonal blocks of L and U, FP64 ...
  double* du64 = nullptr;
  Tlo* dl = nullptr;       // ... and in the low precision
  Tlo* du = nullptr;
  int grid_vec;

  int launch_check(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(ctx, LUHOT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return LUHOT_OK;
  }

  int zero_scalar(int idx, int count = 1) {
    LUHOT_CUDA_TRY(ctx, cudaMemsetAsync(sc + idx, 0, sizeof(double) * count, ctx->stream));
    return LUHOT_OK;
  }

  int read_scalars(int count) {
    LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(hsc, sc, sizeof(double) * count, cudaMemcpyDeviceToHost, ctx->stream));
    LUHOT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return LUHOT_OK;
  }

  // out (FP64) = (LU)^-1 v with the low-precision factors applied in FP64
  // arithmetic on FP64 vectors (no rounding of the Krylov vectors): the
  // preconditioner of GMRES-IR, whose accuracy then depends only on the
  // factors, not on u_low * kappa of each application.
  // FP64 arithmetic is slow on this part, so these sweeps keep 64-row
  // blocks (a quarter of the per-step FP64 work of the chained 128-row form).
  int lo_solve64(const double* v, double* out, bool cycle_start) {
    // A long GMRES run (more than kScaledAfter applications) switches to the
    // block-scaled sweeps, whose critical path per 64-row block is a quarter
    // of the FMAs: the tiles W = D^-1 T of the factors are formed once, in
    // FP64 arithmetic and FP64 storage.  The switch happens only where a
    // restart cycle begins, so every Krylov basis is built with one operator:
    // the two forms agree only to rounding (relative 2^-53 cond(D)), and a
    // mid-cycle change breaks the Arnoldi relation that the cycle's residual
    // estimate rests on.
    ++minv_calls;
    if (!w64 && cycle_start && minv_calls > kScaledAfter && n > 64) {
      if (ensure_buf(ctx, ctx->scaled_buf, (size_t)n * ldlo * sizeof(double)) == LUHOT_OK) {
        double* w = static_cast<double*>(ctx->scaled_buf.ptr);
        int rc = scale_factor_blocks(ctx, n, lu, ldlo, dl64, du64, w, ldlo);
        if (rc) return rc;
        w64 = w;
      } else {
        ctx->last_error.clear();  // no room: keep the plain sweeps
        minv_calls = INT32_MIN;
      }
    }
    if (w64) {
      prof_begin(ctx, kProfRefine);
      ir_gather_kernel<double><<<grid_vec, 256, 0, ctx->stream>>>(v, perm, out, n);
      prof_end(ctx, kProfRefine, 0.0, 20.0 * n);
      int rc = scaled_sweep<double>(ctx, w64, ldlo, dl64, out, u, 1, n, true);
      if (!rc) rc = scaled_sweep<double>(ctx, w64, ldlo, du64, u, out, 1, n, false);
      return rc;
    }
    int* flags = nullptr;
    int* ticket = nullptr;
    int rc = trsv_scratch(ctx, n, &flags, &ticket);
    if (rc) return rc;
    prof_begin(ctx, kProfRefine);
    ir_gather_kernel<double><<<grid_vec, 256, 0, ctx->stream>>>(v, perm, out, n);
    prof_end(ctx, kProfRefine, 0.0, 20.0 * n);
    prof_begin(ctx, kProfTrsv);
    cudaError_t e = launch_trsv_syncfree<double, Tlo>(ctx->stream, lu, ldlo, out, 1, n, 1, true, true, false, false,
                                                      flags, ticket, ctx->d_status, dl64);
    if (e == cudaSuccess)
      e = launch_trsv_syncfree<double, Tlo>(ctx->stream, lu, ldlo, out, 1, n, 1, false, false, false, false, flags,
                                            ticket, ctx->d_status, du64);
    prof_end(ctx, kProfTrsv, 2.0 * n * (double)n, (double)n * n * sizeof(Tlo) + 32.0 * n);
    if (e != cudaSuccess) return set_error(ctx, LUHOT_ERR_CUDA, std::string("ir sweep: ") + cudaGetErrorString(e));
    return LUHOT_OK;
  }

  // out (FP64) = (LU)^-1 v through the low precision with infinity-norm
  // scaling (the plain-IR correction), or out += it: v scaled and rounded to
  // FP32, permuted, the chained FP32 sweeps, widened back.
  int lo_solve(const double* v, double* out, bool add_into_out) {
    int rc = zero_scalar(kVscale);
    if (rc) return rc;
    prof_begin(ctx, kProfRefine);
    ir_infnorm_kernel<<<grid_vec, 256, 0, ctx->stream>>>(v, n, sc + kVscale);
    prof_end(ctx, kProfRefine, 0.0, 8.0 * n);
    prof_begin(ctx, kProfRefine);
    ir_to_low_kernel<Tlo><<<grid_vec, 256, 0, ctx->stream>>>(v, lo1, n, sc + kVscale);
    prof_end(ctx, kProfRefine, 0.0, (8.0 + sizeof(Tlo)) * n);
    rc = launch_check("ir to-low");
    if (rc) return rc;
    // lo2 = P lo1, then L and U sweeps in place (chained, 128-row blocks).
    prof_begin(ctx, kProfPermute);
    ir_gather_kernel<Tlo><<<grid_vec, 256, 0, ctx->stream>>>(lo1, perm, lo2, n);
    prof_end(ctx, kProfPermute, 0.0, (4.0 + 2.0 * sizeof(Tlo)) * n);
    rc = launch_check("ir gather");
    if (!rc) rc = trsv_chain_sweep<Tlo>(ctx, lu, ldlo, lo2, n, true, dl);
    if (!rc) rc = trsv_chain_sweep<Tlo>(ctx, lu, ldlo, lo2, n, false, du);
    if (rc) return rc;
    prof_begin(ctx, kProfRefine);
    if (add_into_out) {
      ir_from_low_kernel<Tlo, true><<<grid_vec, 256, 0, ctx->stream>>>(lo2, out, n, sc + kVscale, sc + kXnorm);
    } else {
      ir_from_low_kernel<Tlo, false><<<grid_vec, 256, 0, ctx->stream>>>(lo2, out, n, sc + kVscale, nullptr);
    }
    prof_end(ctx, kProfRefine, (double)n, (sizeof(Tlo) + 16.0) * n);
    return launch_check("ir from-low");
  }

  int residual(const double* b, const double* x) {
    int rc = zero_scalar(kRnorm);
    if (rc) return rc;
    const int blocks = (n + 7) / 8;
    prof_begin(ctx, kProfRefine);
    ir_matvec_kernel<true><<<blocks, 256, 0, ctx->stream>>>(a, lda, x, b, r, n, sc + kRnorm);
    prof_end(ctx, kProfRefine, 2.0 * n * n, 8.0 * n * (double)n + 24.0 * n);
    return launch_check("ir residual");
  }

  int matvec(const double* x, double* y) {
    const int blocks = (n + 7) / 8;
    prof_begin(ctx, kProfRefine);
    ir_matvec_kernel<false><<<blocks, 256, 0, ctx->stream>>>(a, lda, x, nullptr, y, n, nullptr);
    prof_end(ctx, kProfRefine, 2.0 * n * n, 8.0 * n * (double)n + 16.0 * n);
    return launch_check("ir matvec");
  }

  // One GMRES cycle for A d = r (left-preconditioned), x += d.  Returns the
  // number of inner iterations through *inner.
  int gmres_cycle(double* x, int* inner) {
    const int m = kGmresRestart;
    // v0 = M^-1 r / ||M^-1 r||_2
    int rc = lo_solve64(r, t, true);
    if (rc) return rc;
    rc = zero_scalar(kNrm2);
    if (rc) return rc;
    ir_orth_kernel<<<grid_vec, 256, 0, ctx->stream>>>(V, 0, sc + kH, t, n, sc + kNrm2);
    ir_scale_kernel<true><<<grid_vec, 256, 0, ctx->stream>>>(t, V, n, sc + kNrm2);
    count_launch(ctx, 2);
    rc = read_scalars(kH);
    if (rc) return rc;
    const double beta = std::sqrt(hsc[kNrm2]);
    if (!(beta > 0.0) || !std::isfinite(beta)) {
      *inner = 0;
      return LUHOT_OK;
    }
    std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1, 0.0);
    g[0] = beta;
    int k = 0;
    for (; k < m; ++k) {
      double* vk = V + (int64_t)k * n;
      double* vk1 = V + (int64_t)(k + 1) * n;
      rc = matvec(vk, r);  // r is free as scratch inside the cycle
      if (rc) return rc;
      rc = lo_solve64(r, vk1, false);
      if (rc) return rc;
      // Two passes of classical Gram-Schmidt against v_0..v_k.
      std::vector<double> hcol(k + 2, 0.0);
      for (int pass = 0; pass < 2; ++pass) {
        rc = zero_scalar(kH, k + 1);
        if (rc) return rc;
        if (pass == 1) {
          rc = zero_scalar(kNrm2);
          if (rc) return rc;
        }
        ir_dots_kernel<<<std::min(grid_vec, 256), 256, 0, ctx->stream>>>(V, k + 1, vk1, sc + kH, n);
        ir_orth_kernel<<<grid_vec, 256, 0, ctx->stream>>>(V, k + 1, sc + kH, vk1, n, pass == 1 ? sc + kNrm2 : nullptr);
        count_launch(ctx, 2);
        rc = read_scalars(kH + k + 1);
        if (rc) return rc;
        for (int j = 0; j <= k; ++j) hcol[j] += hsc[kH + j];
      }
      const double hnext = std::sqrt(hsc[kNrm2]);
      hcol[k + 1] = hnext;
      // v_{k+1} = w / ||w||_2 (sc[kNrm2] holds sum w_i^2 of the second pass)
      ir_scale_kernel<true><<<grid_vec, 256, 0, ctx->stream>>>(vk1, vk1, n, sc + kNrm2);
      count_launch(ctx);
      // Givens rotations on column k.
      for (int j = 0; j < k; ++j) {
        const double t0 = cs[j] * hcol[j] + sn[j] * hcol[j + 1];
        hcol[j + 1] = -sn[j] * hcol[j] + cs[j] * hcol[j + 1];
        hcol[j] = t0;
      }
      const double den = std::hypot(hcol[k], hcol[k + 1]);
      cs[k] = den > 0.0 ? hcol[k] / den : 1.0;
      sn[k] = den > 0.0 ? hcol[k + 1] / den : 0.0;
      hcol[k] = den;
      hcol[k + 1] = 0.0;
      g[k + 1] = -sn[k] * g[k];
      g[k] = cs[k] * g[k];
      for (int j = 0; j <= k; ++j) H[(size_t)j * m + k] = hcol[j];
      if (std::fabs(g[k + 1]) <= kGmresTol * beta || !(hnext > 0.0)) {
        ++k;
        break;
      }
    }
    // Solve the k x k upper-triangular system H y = g.
    std::vector<double> y(k, 0.0);
    for (int i = k - 1; i >= 0; --i) {
      double s = g[i];
      for (int j = i + 1; j < k; ++j) s -= H[(size_t)i * m + j] * y[j];
      y[i] = H[(size_t)i * m + i] != 0.0 ? s / H[(size_t)i * m + i] : 0.0;
    }
    for (int i = 0; i < k; ++i) hsc[kH + i] = y[i];
    LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(sc + kH, hsc + kH, sizeof(double) * k, cudaMemcpyHostToDevice, ctx->stream));
    rc = zero_scalar(kXnorm);
    if (rc) return rc;
    ir_combine_kernel<<<grid_vec, 256, 0, ctx->stream>>>(V, k, sc + kH, x, n, sc + kXnorm);
    count_launch(ctx);
    *inner = k;
    return launch_check("gmres combine");
  }
};

}  // namespace

// Refinement state shared by every right-hand side of one call.
static int ir_setup(luhot_ctx* ctx, int n, const double* a, int64_t lda, IrRun<float>& s) {
  const int64_t ldlo = ((int64_t)n + 63) / 64 * 64;
  int rc = ensure_buf(ctx, ctx->ir_buf[0], (size_t)n * ldlo * sizeof(float));
  if (rc) return rc;
  const size_t vecs = (size_t)n * sizeof(double);
  rc = ensure_buf(ctx, ctx->ir_buf[1], vecs * (3 + kGmresRestart + 1) + 3 * (size_t)n * sizeof(float) + 4096);
  if (rc) return rc;
  const size_t idx_ints = (2 * (size_t)n + 63) / 64 * 64;  // pivots + permutation, 256-byte aligned end
  rc = ensure_buf(ctx, ctx->ir_buf[2], idx_ints * sizeof(int) + kIrScalarSlots * sizeof(double));
  if (rc) return rc;
  s.ctx = ctx;
  s.n = n;
  s.a = a;
  s.lda = lda;
  s.lu = static_cast<float*>(ctx->ir_buf[0].ptr);
  s.ldlo = ldlo;
  char* base = static_cast<char*>(ctx->ir_buf[1].ptr);
  s.r = reinterpret_cast<double*>(base);
  s.t = s.r + n;
  s.u = s.t + n;
  s.V = s.u + n;
  s.lo1 = reinterpret_cast<float*>(s.V + (size_t)(kGmresRestart + 1) * n);
  s.lo2 = s.lo1 + n;
  s.piv = static_cast<int*>(ctx->ir_buf[2].ptr);
  s.perm = s.piv + n;
  s.sc = reinterpret_cast<double*>(s.piv + idx_ints);
  s.hsc = ctx->h_scalars;
  s.grid_vec = std::min(ctx->num_sms * 4, (n + 255) / 256);
  return LUHOT_OK;
}

// FP64 -> FP32 copy with ||A||_inf, then the low-precision LU: FP32 on the
// CUDA cores, or FP32 storage with tensor-core Schur updates (TF32, or BF16 /
// FP16 operands with per-panel scaling).
static int ir_factor(IrRun<float>& s, int precision, luhot_ir_info* info) {
  luhot_ctx* ctx = s.ctx;
  const int n = s.n;
  LUHOT_CUDA_TRY(ctx, cudaMemsetAsync(s.sc, 0, 64 * sizeof(double), ctx->stream));
  prof_begin(ctx, kProfRefine);
  ir_convert_kernel<float><<<(n + 7) / 8, 256, 0, ctx->stream>>>(s.a, s.lda, s.lu, s.ldlo, n, s.sc + kAnorm);
  prof_end(ctx, kProfRefine, (double)n * n, 12.0 * n * (double)n);
  int rc = s.launch_check("ir convert");
  if (rc) return rc;
  int64_t sing = -1;
  rc = getrf_mixed_device(ctx, n, n, s.lu, s.ldlo, s.piv, precision, &sing);
  if (rc) return rc;
  info->singular = sing;
  if (sing >= 0) return set_error(ctx, LUHOT_ERR_SINGULAR, "the low-precision factor is singular");
  // Inverses of the diagonal blocks for the sweeps of every later solve: the
  // 128 x 128 blocks of the chained FP32 sweeps (plain IR) and the 64 x 64
  // blocks widened to FP64 (GMRES-IR's preconditioner).
  const size_t ne64 = trsv_inverse_elems(n), ne = trsv_chain_inverse_elems(n);
  rc = ensure_buf(ctx, ctx->dinv_buf, 2 * ne64 * sizeof(double) + 2 * ne * sizeof(float));
  if (rc) return rc;
  s.dl64 = static_cast<double*>(ctx->dinv_buf.ptr);
  s.du64 = s.dl64 + ne64;
  s.dl = reinterpret_cast<float*>(s.du64 + ne64);
  s.du = s.dl + ne;
  rc = invert_diag_blocks<double, float>(ctx, n, s.lu, s.ldlo, s.dl64, s.du64);
  if (!rc) rc = chain_invert_blocks<float>(ctx, n, s.lu, s.ldlo, s.dl, s.du);
  if (rc) return rc;
  return getrs_perm(ctx, s.piv, n, s.perm);
}

// Refine one right-hand side (contiguous b, x) with the factors in s.
static int ir_refine(IrRun<float>& s, const double* b, double* x, int solver, double tol, int max_iter,
                     luhot_ir_info* info) {
  luhot_ctx* ctx = s.ctx;
  cudaStream_t stream = ctx->stream;
  const int n = s.n;
  int rc = s.zero_scalar(kBnorm);
  if (rc) return rc;
  prof_begin(ctx, kProfRefine);
  ir_infnorm_kernel<<<s.grid_vec, 256, 0, stream>>>(b, n, s.sc + kBnorm);
  prof_end(ctx, kProfRefine, 0.0, 8.0 * n);
  rc = s.lo_solve(b, x, false);
  if (rc) return rc;
  const double tol_eff = tol > 0.0 ? tol : n * std::ldexp(1.0, -53);
  int it = 0, inner_total = 0;
  double berr = INFINITY, prev = INFINITY;
  bool converged = false;
  int stall = 0;
  for (;;) {
    rc = s.zero_scalar(kXnorm);
    if (rc) return rc;
    prof_begin(ctx, kProfRefine);
    ir_infnorm_kernel<<<s.grid_vec, 256, 0, stream>>>(x, n, s.sc + kXnorm);
    prof_end(ctx, kProfRefine, 0.0, 8.0 * n);
    rc = s.residual(b, x);
    if (rc) return rc;
    rc = s.read_scalars(kVscale);
    if (rc) return rc;
    const double anorm = s.hsc[kAnorm], bnorm = s.hsc[kBnorm], rnorm = s.hsc[kRnorm], xnorm = s.hsc[kXnorm];
    berr = rnorm / (anorm * xnorm + bnorm);
    if (!std::isfinite(berr)) berr = INFINITY;
    if (ctx->trace) fprintf(stderr, "luhot ir: step %d berr %.3e inner %d\n", it, berr, inner_total);
    if (berr <= tol_eff) {
      converged = true;
      break;
    }
    if (it >= max_iter) break;
    // Stop when the iteration no longer contracts (plain IR diverging, or
    // stagnation at the attainable accuracy).
    if (berr > 0.9 * prev) {
      if (++stall >= 3) break;
    } else {
      stall = 0;
    }
    prev = std::min(prev, berr);
    if (solver == LUHOT_REFINE_GMRES) {
      int inner = 0;
      rc = s.gmres_cycle(x, &inner);
      if (rc) return rc;
      inner_total += inner;
    } else {
      rc = s.lo_solve(s.r, x, true);
      if (rc) return rc;
    }
    ++it;
  }
  info->iterations = std::max(info->iterations, it);
  info->inner_iterations += inner_total;
  info->backward_error = std::max(info->backward_error, berr);
  info->converged = info->converged && converged;
  return LUHOT_OK;
}

int getrf_mixed_device(luhot_ctx* ctx, int m, int n, float* a, int64_t lda, int* piv, int precision,
                       int64_t* singular) {
  if (m < 0 || n < 0 || lda < std::max(1, n)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrf: bad shape or lda");
  if (precision == LUHOT_PREC_FP32) return getrf_device<float>(ctx, m, n, a, lda, piv, LUHOT_MODE_FAST, singular);
  if (precision != LUHOT_PREC_BF16 && precision != LUHOT_PREC_FP16 && precision != LUHOT_PREC_TF32 &&
      precision != LUHOT_PREC_BF16X3)
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrf: unknown precision");
  const int kind = precision == LUHOT_PREC_BF16     ? kTcBF16
                   : precision == LUHOT_PREC_FP16   ? kTcFP16
                   : precision == LUHOT_PREC_BF16X3 ? kTcBF16x3
                                                    : kTcTF32;
  return getrf_device_tc(ctx, m, n, a, lda, piv, kind, singular);
}

int gesv_ir_device(luhot_ctx* ctx, int n, int nrhs, const double* a, int64_t lda, const double* b, int64_t ldb,
                   double* x, int64_t ldx, int precision, int solver, double tol, int max_iter,
                   luhot_ir_info* info) {
  if (n < 0 || nrhs < 0 || lda < std::max(1, n) || ldb < std::max(1, nrhs) || ldx < std::max(1, nrhs))
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "gesv_ir: bad shape or leading dimension");
  if (solver != LUHOT_REFINE_IR && solver != LUHOT_REFINE_GMRES)
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "gesv_ir: unknown solver");
  if (precision != LUHOT_PREC_FP32 && precision != LUHOT_PREC_BF16 && precision != LUHOT_PREC_FP16 &&
      precision != LUHOT_PREC_TF32 && precision != LUHOT_PREC_BF16X3)
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "gesv_ir: unknown precision");
  if (max_iter < 0) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "gesv_ir: negative max_iter");
  *info = luhot_ir_info{};
  info->converged = 1;
  info->precision = precision;
  info->solver = solver;
  info->singular = -1;
  if (n == 0 || nrhs == 0) return LUHOT_OK;
  int rc = reset_status(ctx);
  if (rc) return rc;
  // Columns of b and x are strided (ld); the refinement works on contiguous vectors.
  rc = ensure_buf(ctx, ctx->ir_buf[3], (size_t)n * 2 * sizeof(double));
  if (rc) return rc;
  double* bc = static_cast<double*>(ctx->ir_buf[3].ptr);
  double* xc = bc + n;
  IrRun<float> s;
  rc = ir_setup(ctx, n, a, lda, s);
  if (rc) return rc;
  cudaEvent_t e0, e1, e2;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventCreate(&e2);
  struct EvGuard {
    cudaEvent_t a, b, c;
    ~EvGuard() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      cudaEventDestroy(c);
    }
  } guard{e0, e1, e2};
  cudaEventRecord(e0, ctx->stream);
  {
    NvtxRange range("luhot ir: low-precision factorization");
    rc = ir_factor(s, precision, info);
  }
  if (rc) return rc;
  cudaEventRecord(e1, ctx->stream);
  for (int c = 0; c < nrhs; ++c) {
    rc = copy_2d(ctx, bc, sizeof(double), b + c, ldb * sizeof(double), sizeof(double), n, cudaMemcpyDeviceToDevice);
    if (rc) return rc;
    {
      NvtxRange range("luhot ir: refinement");
      rc = ir_refine(s, bc, xc, solver, tol, max_iter, info);
    }
    if (rc) return rc;
    rc = copy_2d(ctx, x + c, ldx * sizeof(double), xc, sizeof(double), sizeof(double), n, cudaMemcpyDeviceToDevice);
    if (rc) return rc;
  }
  cudaEventRecord(e2, ctx->stream);
  LUHOT_CUDA_TRY(ctx, cudaEventSynchronize(e2));
  float f_ms = 0.f, r_ms = 0.f;
  cudaEventElapsedTime(&f_ms, e0, e1);
  cudaEventElapsedTime(&r_ms, e1, e2);
  info->factor_ms = f_ms;
  info->refine_ms = r_ms;
  rc = finish_status(ctx, nullptr);
  if (rc) return rc;
  if (!info->converged)
    return set_error(ctx, LUHOT_ERR_NOT_CONVERGED,
                     "refinement stopped at backward error " + std::to_string(info->backward_error));
  return LUHOT_OK;
}

}  // namespace luhot
