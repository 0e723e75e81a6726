// Blocked right-looking LU with partial pivoting on one GB300 (sm_103a).
//
// Matrix layout in HBM: row-major, leading dimension lda >= n (elements).
// Pivots: int32 on the device, LAPACK-style sequential interchanges
// (step i swapped row i with row piv[i]), the convention of lair's
// src/lapack/getrf.rs:12-27.
//
// One block step k0 (panel width w) runs four kernels:
//   1. panel_kernel   cooperative; factors rows [k0, m) x cols [k0, k0+w) held
//                     in shared memory across all CTAs; one bounded grid
//                     barrier per column for the pivot search (warp-shuffle
//                     iamax, then a deterministic reduce over CTAs).
//   2. laswp_kernel   applies the w interchanges to the columns left and
//                     right of the panel (coalesced 16-byte row moves).
//   3. trsm_kernel    U12 <- L11^-1 A12 (unit lower).
//   4. gemm_*_kernel  A22 <- A22 - L21 U12 (the Schur complement).
//
// Two arithmetic modes:
//   exact: every update is a separately rounded multiply then subtract, in
//          increasing elimination-step order, which is exactly the sequence
//          of lair's getrf_row_major (src/lapack/getrf.rs:76-89).  Blocking
//          only moves data, so results are bit-identical to lair.
//   fast:  the Schur update runs on the FP64 tensor cores (DMMA,
//          mma.sync m8n8k4) and the other kernels use FMA.
#include <cooperative_groups.h>

#include <algorithm>

#include "common.cuh"
#include "luhot_internal.h"
#include "tc_gemm.cuh"

namespace luhot {

// ---------------------------------------------------------------------------
// Arithmetic of one elimination update: c - l*u.
// ---------------------------------------------------------------------------
template <bool kExact>
__device__ __forceinline__ double upd(double c, double l, double u) {
  if (kExact) return __dsub_rn(c, __dmul_rn(l, u));
  return fma(-l, u, c);
}
template <bool kExact>
__device__ __forceinline__ float upd(float c, float l, float u) {
  if (kExact) return __fsub_rn(c, __fmul_rn(l, u));
  return fmaf(-l, u, c);
}
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }

// ---------------------------------------------------------------------------
// 1. Panel factorization.
// ---------------------------------------------------------------------------
template <typename T>
struct PanelArgs {
  T* a;
  int64_t lda;
  int m;          // rows of the whole matrix
  int k0;         // first row/column of the panel
  int w;          // panel width == elimination steps in this panel
  int rows_per;   // panel rows owned by each CTA
  int lds;        // shared-memory row stride (elements)
  int* piv;       // device pivots (global row index per step)
  T* cand_val;    // [2][P]
  int* cand_idx;  // [2][P]
  T* cand_row;    // [2][P][w]   row segment of each CTA's candidate
  T* row_ul;      // [2][w]      segment of row ul before the swap
  DeviceStatus* st;
  unsigned int bar_base;
};

// First index of the largest |x| with lair's strict `>` (src/blas/iamax.rs:6-21):
// larger value wins, equal values keep the smaller row.  NaN never compares
// greater, so it never wins.  (0, INT_MAX) means "no positive entry".
template <typename T>
__device__ __forceinline__ void iamax_combine(T& v, int& i, T v2, int i2) {
  if (v2 > v || (v2 == v && i2 < i)) {
    v = v2;
    i = i2;
  }
}

template <typename T, bool kExact>
__global__ void __launch_bounds__(256) panel_kernel(PanelArgs<T> p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* S = reinterpret_cast<T*>(smem_raw);              // [rows_per][lds]
  T* seg = S + (size_t)p.rows_per * p.lds;            // [w] pivot row segment
  __shared__ T red_v[32];
  __shared__ int red_i[32];
  __shared__ int s_piv;
  __shared__ T s_max;
  __shared__ int s_win;

  const int P = gridDim.x;
  const int b = blockIdx.x;
  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = nthr >> 5;
  const int r_begin = p.k0 + b * p.rows_per;
  const int r_end = min(p.m, r_begin + p.rows_per);
  const int nloc = max(0, r_end - r_begin);
  const int w = p.w;

  // Stage this CTA's rows of the panel in shared memory.
  for (int idx = tid; idx < nloc * w; idx += nthr) {
    const int r = idx / w, c = idx - r * w;
    S[r * p.lds + c] = p.a[(int64_t)(r_begin + r) * p.lda + p.k0 + c];
  }
  __syncthreads();

  unsigned int target = p.bar_base;
  for (int j = 0; j < w; ++j) {
    const int ul = p.k0 + j;
    const int par = j & 1;
    // Local pivot search over owned rows >= ul in column j.
    T bv = T(0);
    int bi = INT_MAX;
    for (int r = max(0, ul - r_begin) + tid; r < nloc; r += nthr) {
      const T v = fabs(S[r * p.lds + j]);
      if (v > bv) {  // rows visited in increasing order per thread
        bv = v;
        bi = r_begin + r;
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const T v2 = __shfl_down_sync(0xffffffffu, bv, off);
      const int i2 = __shfl_down_sync(0xffffffffu, bi, off);
      iamax_combine(bv, bi, v2, i2);
    }
    if (lane == 0) {
      red_v[warp] = bv;
      red_i[warp] = bi;
    }
    __syncthreads();
    if (tid == 0) {
      for (int q = 1; q < nwarps; ++q) iamax_combine(bv, bi, red_v[q], red_i[q]);
      s_max = bv;
      s_win = bi;
    }
    __syncthreads();
    // Publish the candidate, its row segment, and (owner only) row ul.
    const int cbi = s_win;
    if (tid == 0) {
      p.cand_val[par * P + b] = s_max;
      p.cand_idx[par * P + b] = cbi;
    }
    if (cbi != INT_MAX) {
      const int r = cbi - r_begin;
      for (int c = tid; c < w; c += nthr) p.cand_row[((size_t)par * P + b) * w + c] = S[r * p.lds + c];
    }
    if (ul >= r_begin && ul < r_end) {
      const int r = ul - r_begin;
      for (int c = tid; c < w; c += nthr) p.row_ul[(size_t)par * w + c] = S[r * p.lds + c];
    }
    target += P;
    if (!grid_barrier(p.st, target, (unsigned long long)ul)) return;

    // Every CTA reduces the P candidates in the same order: same answer.
    if (warp == 0) {
      T v = T(0);
      int i = INT_MAX, win = -1;
      for (int q = lane; q < P; q += 32) {
        const T v2 = ld_cg(&p.cand_val[par * P + q]);
        const int i2 = ld_cg(&p.cand_idx[par * P + q]);
        if (v2 > v || (v2 == v && i2 < i)) {
          v = v2;
          i = i2;
          win = q;
        }
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const T v2 = __shfl_down_sync(0xffffffffu, v, off);
        const int i2 = __shfl_down_sync(0xffffffffu, i, off);
        const int w2 = __shfl_down_sync(0xffffffffu, win, off);
        if (v2 > v || (v2 == v && i2 < i)) {
          v = v2;
          i = i2;
          win = w2;
        }
      }
      if (lane == 0) {
        s_max = v;
        s_piv = (v > T(0)) ? i : ul;
        s_win = win;
      }
    }
    __syncthreads();
    const T maxv = s_max;
    const int pr = s_piv;
    if (!(maxv > T(0))) {
      // lair: max == 0 -> record the step as singular, no swap, no update
      // (src/lapack/getrf.rs:72-73).  The last such step wins.
      if (b == 0 && tid == 0) {
        p.piv[ul] = ul;
        atomicMax(&p.st->singular, ul);
      }
      continue;
    }
    const int win = s_win;
    for (int c = tid; c < w; c += nthr) seg[c] = ld_cg(&p.cand_row[((size_t)par * P + win) * w + c]);
    __syncthreads();
    if (pr != ul) {
      if (ul >= r_begin && ul < r_end) {
        const int r = ul - r_begin;
        for (int c = tid; c < w; c += nthr) S[r * p.lds + c] = seg[c];
      }
      if (pr >= r_begin && pr < r_end) {
        const int r = pr - r_begin;
        for (int c = tid; c < w; c += nthr) S[r * p.lds + c] = ld_cg(&p.row_ul[(size_t)par * w + c]);
      }
    }
    if (b == 0 && tid == 0) p.piv[ul] = pr;
    __syncthreads();
    // Scale the column below the pivot by the reciprocal (1/pivot rounded,
    // then a rounded multiply: src/lapack/getrf.rs:76-81).
    const T recip = T(1) / seg[j];
    const int r0 = max(0, ul + 1 - r_begin);
    for (int r = r0 + tid; r < nloc; r += nthr) S[r * p.lds + j] = mul_rn(S[r * p.lds + j], recip);
    __syncthreads();
    // Rank-1 update of the panel columns right of j.
    const int wr = w - j - 1;
    if (wr > 0) {
      const int total = (nloc - r0) * wr;
      for (int idx = tid; idx < total; idx += nthr) {
        const int r = r0 + idx / wr;
        const int c = j + 1 + idx % wr;
        S[r * p.lds + c] = upd<kExact>(S[r * p.lds + c], S[r * p.lds + j], seg[c]);
      }
    }
    __syncthreads();
  }
  __syncthreads();
  for (int idx = tid; idx < nloc * w; idx += nthr) {
    const int r = idx / w, c = idx - r * w;
    p.a[(int64_t)(r_begin + r) * p.lda + p.k0 + c] = S[r * p.lds + c];
  }
}

// ---------------------------------------------------------------------------
// 2. Row interchanges outside the panel.  Each thread owns one column (or a
//    16-byte pair/quad) and replays the w swaps in order, as
//    src/lapack/laswp.rs:11-40 does row by row.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void laswp_kernel(T* a, int64_t lda, const int* piv, int k0, int w, int c_left_end,
                             int c_right_begin, int n) {
  const int nleft = c_left_end;
  const int nright = max(0, n - c_right_begin);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nleft + nright) return;
  const int c = (t < nleft) ? t : (c_right_begin + t - nleft);
  for (int s = 0; s < w; ++s) {
    const int i = k0 + s;
    const int pr = piv[i];
    if (pr != i) {
      T* x = a + (int64_t)i * lda + c;
      T* y = a + (int64_t)pr * lda + c;
      const T tmp = *x;
      *x = *y;
      *y = tmp;
    }
  }
}

// ---------------------------------------------------------------------------
// 3. U12 <- L11^-1 A12 for rows [k0, k0+w), columns [c0, n).  One thread per
//    column; each row i subtracts l[i][k]*u[k][c] for k = 0..i-1 in order,
//    the order in which lair's elimination steps reach these entries.
// ---------------------------------------------------------------------------
constexpr int kTrsmCols = 64;

template <typename T, bool kExact>
__global__ void __launch_bounds__(kTrsmCols) trsm_kernel(T* a, int64_t lda, int k0, int w, int c0,
                                                         int n) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* L = reinterpret_cast<T*>(smem_raw);  // [w][w]
  T* X = L + w * w;                       // [w][kTrsmCols]
  const int cb = c0 + blockIdx.x * kTrsmCols;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < w * w; idx += blockDim.x) {
    const int i = idx / w, k = idx - i * w;
    L[idx] = a[(int64_t)(k0 + i) * lda + k0 + k];
  }
  const int c = cb + tid;
  const bool active = c < n;
  if (active)
    for (int i = 0; i < w; ++i) X[i * kTrsmCols + tid] = a[(int64_t)(k0 + i) * lda + c];
  __syncthreads();
  if (!active) return;
  for (int i = 1; i < w; ++i) {
    T acc = X[i * kTrsmCols + tid];
    for (int k = 0; k < i; ++k) acc = upd<kExact>(acc, L[i * w + k], X[k * kTrsmCols + tid]);
    X[i * kTrsmCols + tid] = acc;
  }
  for (int i = 1; i < w; ++i) a[(int64_t)(k0 + i) * lda + c] = X[i * kTrsmCols + tid];
}

// ---------------------------------------------------------------------------
// 4a. Schur update on the CUDA cores (exact mode and FP32): C -= A B with a
//     64x64 tile per CTA, 4x4 per thread, K <= 64 staged in shared memory.
//     Each C entry starts from its old value and takes the K updates one at a
//     time in increasing k, which is lair's order.
// ---------------------------------------------------------------------------
constexpr int kGemmTile = 64;
constexpr int kGemmKC = 32;  // K chunk staged per pass (static smem stays < 48 KB)

template <typename T, bool kExact>
__global__ void __launch_bounds__(256) gemm_cuda_kernel(T* a, int64_t lda, int r0, int c0, int kk0,
                                                        int K, int M, int N) {
  __shared__ T As[kGemmKC][kGemmTile + 1];  // As[k][i] = L21[i][k]
  __shared__ T Bs[kGemmKC][kGemmTile];      // Bs[k][j] = U12[k][j]
  const int tile_r = r0 + blockIdx.y * kGemmTile;
  const int tile_c = c0 + blockIdx.x * kGemmTile;
  const int tid = threadIdx.x;
  const int tr = (tid / 16) * 4, tc = (tid % 16);
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const int r = tile_r + tr + i, c = tile_c + tc + 16 * jj;
      acc[i][jj] = (r < r0 + M && c < c0 + N) ? a[(int64_t)r * lda + c] : T(0);
    }
  for (int kb = 0; kb < K; kb += kGemmKC) {
    const int kc = min(kGemmKC, K - kb);
    __syncthreads();
    for (int idx = tid; idx < kc * kGemmTile; idx += 256) {
      const int i = idx / kc, k = idx - i * kc;
      const int r = tile_r + i;
      As[k][i] = (r < r0 + M) ? a[(int64_t)r * lda + kk0 + kb + k] : T(0);
    }
    for (int idx = tid; idx < kc * kGemmTile; idx += 256) {
      const int k = idx / kGemmTile, j = idx - k * kGemmTile;
      const int c = tile_c + j;
      Bs[k][j] = (c < c0 + N) ? a[(int64_t)(kk0 + kb + k) * lda + c] : T(0);
    }
    __syncthreads();
    for (int k = 0; k < kc; ++k) {
      T av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = As[k][tr + i];
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) bv[jj] = Bs[k][tc + 16 * jj];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) acc[i][jj] = upd<kExact>(acc[i][jj], av[i], bv[jj]);
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const int r = tile_r + tr + i, c = tile_c + tc + 16 * jj;
      if (r < r0 + M && c < c0 + N) a[(int64_t)r * lda + c] = acc[i][jj];
    }
}

// ---------------------------------------------------------------------------
// 4b. Schur update on the FP64 tensor cores: mma.sync.m8n8k4 (DMMA).
//     CTA tile 128x128, 8 warps as 4 (rows) x 2 (cols), warp tile 32x64 =
//     4 x 8 MMA tiles.  L21/U12 slices (K <= 64) are staged in shared memory
//     once; C is read, updated and written once.
// ---------------------------------------------------------------------------
constexpr int kDmmaBM = 128, kDmmaBN = 128;

__device__ __forceinline__ void dmma_8x8x4(double& d0, double& d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
               : "+d"(d0), "+d"(d1)
               : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(256) gemm_dmma_kernel(double* a, int64_t lda, int r0, int c0,
                                                        int kk0, int K, int M, int N) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // As: [kDmmaBM][Kp] (row i, col k), Kp = Kpad + 4 keeps the fragment loads
  // free of bank conflicts; Bs: [Kpad][kDmmaBN + 4] likewise.
  const int Kpad = (K + 15) & ~15;
  const int Kp = Kpad + 4;
  double* As = reinterpret_cast<double*>(smem_raw);
  double* Bs = As + kDmmaBM * Kp;
  const int ldb = kDmmaBN + 4;
  const int tile_r = r0 + blockIdx.y * kDmmaBM;
  const int tile_c = c0 + blockIdx.x * kDmmaBN;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < kDmmaBM * Kpad; idx += 256) {
    const int i = idx / Kpad, k = idx - i * Kpad;
    const int r = tile_r + i;
    As[i * Kp + k] = (r < r0 + M && k < K) ? a[(int64_t)r * lda + kk0 + k] : 0.0;
  }
  for (int idx = tid; idx < Kpad * kDmmaBN; idx += 256) {
    const int k = idx / kDmmaBN, j = idx - k * kDmmaBN;
    const int c = tile_c + j;
    Bs[k * ldb + j] = (c < c0 + N && k < K) ? a[(int64_t)(kk0 + k) * lda + c] : 0.0;
  }
  __syncthreads();
  const int lane = tid & 31, warp = tid >> 5;
  const int wr = (warp >> 1) * 32;  // warp row offset in tile
  const int wc = (warp & 1) * 64;   // warp col offset in tile
  const int g = lane >> 2, t4 = lane & 3;
  double acc[4][8][2];
#pragma unroll
  for (int mi = 0; mi < 4; ++mi)
#pragma unroll
    for (int ni = 0; ni < 8; ++ni)
#pragma unroll
      for (int e = 0; e < 2; ++e) acc[mi][ni][e] = 0.0;
  const int Kmma = (K + 3) & ~3;
  for (int k = 0; k < Kmma; k += 4) {
    double af[4], bf[8];
#pragma unroll
    for (int mi = 0; mi < 4; ++mi) af[mi] = As[(wr + mi * 8 + g) * Kp + k + t4];
#pragma unroll
    for (int ni = 0; ni < 8; ++ni) bf[ni] = Bs[(k + t4) * ldb + wc + ni * 8 + g];
#pragma unroll
    for (int mi = 0; mi < 4; ++mi)
#pragma unroll
      for (int ni = 0; ni < 8; ++ni) dmma_8x8x4(acc[mi][ni][0], acc[mi][ni][1], af[mi], bf[ni]);
  }
#pragma unroll
  for (int mi = 0; mi < 4; ++mi) {
    const int r = tile_r + wr + mi * 8 + g;
    if (r >= r0 + M) continue;
#pragma unroll
    for (int ni = 0; ni < 8; ++ni) {
      const int c = tile_c + wc + ni * 8 + t4 * 2;
      double* dst = a + (int64_t)r * lda + c;
      if (c + 1 < c0 + N && (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
        double2 v = *reinterpret_cast<double2*>(dst);
        v.x -= acc[mi][ni][0];
        v.y -= acc[mi][ni][1];
        *reinterpret_cast<double2*>(dst) = v;
      } else {
        if (c < c0 + N) dst[0] -= acc[mi][ni][0];
        if (c + 1 < c0 + N) dst[1] -= acc[mi][ni][1];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Host driver.
// ---------------------------------------------------------------------------
template <typename T>
static size_t panel_smem_bytes(int rows_per, int w) {
  return ((size_t)rows_per * (w + 1) + w) * sizeof(T);
}

template <typename T, bool kExact>
static int launch_panel(luhot_ctx* ctx, T* a, int64_t lda, int m, int k0, int w, int* piv,
                        unsigned int* bar_count, cudaStream_t stream) {
  const int rows = m - k0;
  const int max_smem = ctx->max_smem_optin;
  // CTAs: enough that each owns >= 32 rows, at most the SM count, and with
  // the rows of one CTA fitting in shared memory.
  int P = std::min(ctx->num_sms, std::max(1, (rows + 31) / 32));
  int rows_per = (rows + P - 1) / P;
  while (panel_smem_bytes<T>(rows_per, w) > (size_t)max_smem && P < ctx->num_sms) {
    P = std::min(ctx->num_sms, P * 2);
    rows_per = (rows + P - 1) / P;
  }
  if (panel_smem_bytes<T>(rows_per, w) > (size_t)max_smem)
    return set_error(ctx, LUHOT_ERR_UNSUPPORTED, "panel does not fit in shared memory");
  const size_t smem = panel_smem_bytes<T>(rows_per, w);
  auto kern = panel_kernel<T, kExact>;
  LUHOT_CUDA_TRY(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
  int per_sm = 0;
  LUHOT_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem));
  if (per_sm * ctx->num_sms < P)
    return set_error(ctx, LUHOT_ERR_UNSUPPORTED, "panel grid cannot be co-resident");
  PanelArgs<T> args;
  args.a = a;
  args.lda = lda;
  args.m = m;
  args.k0 = k0;
  args.w = w;
  args.rows_per = rows_per;
  args.lds = w + 1;
  args.piv = piv;
  T* scratch = reinterpret_cast<T*>(ctx->panel_scratch);
  args.cand_val = scratch;
  args.cand_row = scratch + 2 * kMaxPanelCtas;
  args.row_ul = args.cand_row + 2 * (size_t)kMaxPanelCtas * kMaxPanelWidth;
  args.cand_idx = reinterpret_cast<int*>(args.row_ul + 2 * kMaxPanelWidth);
  args.st = ctx->d_status;
  args.bar_base = *bar_count;
  void* kargs[] = {&args};
  prof_begin(ctx, kProfPanel);
  LUHOT_CUDA_TRY(ctx, cudaLaunchCooperativeKernel((void*)kern, dim3(P), dim3(256), kargs, smem,
                                                  stream));
  // panel flops: sum over steps of (rows below) * (1 + 2 * cols right)
  double fl = 0.0;
  for (int j = 0; j < w; ++j) fl += (double)(rows - j - 1) * (1.0 + 2.0 * (w - j - 1));
  prof_end(ctx, kProfPanel, fl, 2.0 * rows * w * sizeof(T));
  *bar_count += (unsigned int)P * (unsigned int)w;
  return LUHOT_OK;
}

template <typename T, bool kExact>
static int launch_gemm(luhot_ctx* ctx, T* a, int64_t lda, int r0, int c0, int kk0, int K, int M,
                       int N, cudaStream_t stream) {
  if (M <= 0 || N <= 0 || K <= 0) return LUHOT_OK;
  if constexpr (std::is_same<T, double>::value && !kExact) {
    const int Kpad = (K + 15) & ~15;
    const size_t smem = ((size_t)kDmmaBM * (Kpad + 4) + (size_t)Kpad * (kDmmaBN + 4)) * sizeof(double);
    LUHOT_CUDA_TRY(ctx, cudaFuncSetAttribute(gemm_dmma_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((N + kDmmaBN - 1) / kDmmaBN, (M + kDmmaBM - 1) / kDmmaBM);
    prof_begin(ctx, kProfGemm);
    gemm_dmma_kernel<<<grid, 256, smem, stream>>>(a, lda, r0, c0, kk0, K, M, N);
  } else {
    dim3 grid((N + kGemmTile - 1) / kGemmTile, (M + kGemmTile - 1) / kGemmTile);
    prof_begin(ctx, kProfGemm);
    gemm_cuda_kernel<T, kExact><<<grid, 256, 0, stream>>>(a, lda, r0, c0, kk0, K, M, N);
  }
  // algorithmic work: 2MNK flops; bytes: C read + written, L21 and U12 read once
  prof_end(ctx, kProfGemm, 2.0 * M * N * K,
           ((double)2 * M * N + (double)M * K + (double)K * N) * sizeof(T));
  LUHOT_CUDA_TRY(ctx, cudaGetLastError());
  return LUHOT_OK;
}

template <typename T, bool kExact>
static int getrf_impl(luhot_ctx* ctx, int m, int n, T* a, int64_t lda, int* piv, int nb,
                      cudaStream_t stream, int tc_kind = -1, void* tc_a = nullptr, void* tc_b = nullptr,
                      float* tc_scal = nullptr) {
  const int dim_min = std::min(m, n);
  unsigned int bar_count = 0;
  for (int k0 = 0; k0 < dim_min; k0 += nb) {
    const int w = std::min(nb, dim_min - k0);
    int rc = launch_panel<T, kExact>(ctx, a, lda, m, k0, w, piv, &bar_count, stream);
    if (rc != LUHOT_OK) return rc;
    const int c_right = k0 + w;
    const int ncols_swap = k0 + std::max(0, n - c_right);
    if (ncols_swap > 0) {
      prof_begin(ctx, kProfLaswp);
      laswp_kernel<T><<<(ncols_swap + 255) / 256, 256, 0, stream>>>(a, lda, piv, k0, w, k0, c_right,
                                                                    n);
      prof_end(ctx, kProfLaswp, 0.0, 4.0 * w * ncols_swap * sizeof(T));
      LUHOT_CUDA_TRY(ctx, cudaGetLastError());
    }
    if (c_right < n) {
      const size_t smem = ((size_t)w * w + (size_t)w * kTrsmCols) * sizeof(T);
      auto kern = trsm_kernel<T, kExact>;
      LUHOT_CUDA_TRY(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem));
      prof_begin(ctx, kProfTrsm);
      kern<<<(n - c_right + kTrsmCols - 1) / kTrsmCols, kTrsmCols, smem, stream>>>(a, lda, k0, w,
                                                                                   c_right, n);
      prof_end(ctx, kProfTrsm, (double)w * (w - 1) * (n - c_right),
               ((double)w * w + 2.0 * w * (n - c_right)) * sizeof(T));
      LUHOT_CUDA_TRY(ctx, cudaGetLastError());
      if constexpr (std::is_same<T, float>::value) {
        if (tc_kind >= 0) {
          rc = tc_schur_update(ctx, tc_kind, a, lda, k0, w, m, n, tc_a, tc_b, tc_scal, stream);
          if (rc != LUHOT_OK) return rc;
          continue;
        }
      }
      rc = launch_gemm<T, kExact>(ctx, a, lda, k0 + w, c_right, k0, w, m - (k0 + w), n - c_right,
                                  stream);
      if (rc != LUHOT_OK) return rc;
    }
  }
  return LUHOT_OK;
}

template <typename T>
int getrf_device(luhot_ctx* ctx, int m, int n, T* a, int64_t lda, int* piv, int mode,
                 int64_t* singular) {
  if (m < 0 || n < 0 || lda < std::max(1, n)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrf: bad shape or lda");
  if (singular) *singular = -1;
  if (m == 0 || n == 0) return LUHOT_OK;
  cudaStream_t stream = ctx->stream;
  int rc = reset_status(ctx);
  if (rc != LUHOT_OK) return rc;
  const int nb = ctx->nb_override > 0 ? std::min(ctx->nb_override, kDefaultPanelWidth) : kDefaultPanelWidth;
  if (mode == LUHOT_MODE_EXACT)
    rc = getrf_impl<T, true>(ctx, m, n, a, lda, piv, nb, stream);
  else
    rc = getrf_impl<T, false>(ctx, m, n, a, lda, piv, nb, stream);
  if (rc != LUHOT_OK) return rc;
  return finish_status(ctx, singular);
}

template int getrf_device<double>(luhot_ctx*, int, int, double*, int64_t, int*, int, int64_t*);
template int getrf_device<float>(luhot_ctx*, int, int, float*, int64_t, int*, int, int64_t*);

int getrf_device_tc(luhot_ctx* ctx, int m, int n, float* a, int64_t lda, int* piv, int tc_kind, int64_t* singular) {
  if (m < 0 || n < 0 || lda < std::max(1, n)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrf: bad shape or lda");
  if (singular) *singular = -1;
  if (m == 0 || n == 0) return LUHOT_OK;
  const int nb = kTcPanelWidth;
  const size_t bytes = tc_operand_bytes(tc_kind, m, nb) + tc_operand_bytes(tc_kind, n, nb) + 4096;
  int rc = ensure_buf(ctx, ctx->tc_buf, bytes);
  if (rc) return rc;
  char* base = static_cast<char*>(ctx->tc_buf.ptr);
  void* tc_a = base;
  void* tc_b = base + (tc_operand_bytes(tc_kind, m, nb) + 1023) / 1024 * 1024;
  float* tc_scal = reinterpret_cast<float*>(base + bytes - 1024);
  rc = reset_status(ctx);
  if (rc != LUHOT_OK) return rc;
  rc = getrf_impl<float, false>(ctx, m, n, a, lda, piv, nb, ctx->stream, tc_kind, tc_a, tc_b, tc_scal);
  if (rc != LUHOT_OK) return rc;
  return finish_status(ctx, singular);
}

}  // namespace luhot
