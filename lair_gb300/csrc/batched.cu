// Batched LU + solve of thousands of small uneven systems in one persistent
// launch (replayed from a CUDA graph).
//
// Packed layout: system i is an n_i x n_i row-major matrix at element offset
// a_off[i] = sum_{j<i} n_j^2 and a right-hand side (overwritten by x) and
// int32 pivots at b_off[i] = sum_{j<i} n_j.  info[i] = last all-zero pivot
// step of system i (lair's Option<usize>) or -1.
//
// One CTA (256 threads) per system at a time; CTAs draw systems from an
// atomic counter in largest-first order (longest-processing-time first
// keeps the tail short).  Two per-system algorithms:
//   * shared-memory path (n <= smem_n): the whole matrix and x live in
//     shared memory; unblocked right-looking elimination (warp-shuffle
//     pivot search, row swap, reciprocal scale, rank-1 update), then the
//     two triangular sweeps, all in shared memory;
//   * blocked path: panels of nb columns are factored in shared memory, the
//     interchanges, U12 and the Schur update run on the L2-resident matrix.
// Which path and which nb each size bucket uses is chosen by the autotuner
// (luhot_batch_autotune), which times the candidates on sample systems of
// the batch.  In exact mode every update is lair's separately rounded
// multiply and subtract in elimination order (src/lapack/getrf.rs:76-89),
// and the solve follows src/lapack/getrs.rs:24-36, so each system's LU,
// pivots and x are bit-identical to lair's.
#include <algorithm>
#include <climits>
#include <cstring>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "luhot_internal.h"

namespace luhot {

constexpr int kBatchThreads = 256;
constexpr int kBatchMaxN = 256;
constexpr int kBuckets = 9;         // n in (0,16], (16,32], (32,64], (64,96], ..., (224,256]
constexpr size_t kBatchSmem = 76 * 1024;

__host__ __device__ inline int batch_bucket(int n) {
  if (n <= 16) return 0;
  if (n <= 32) return 1;
  if (n <= 64) return 2;
  return min(kBuckets - 1, 3 + (n - 65) / 32);
}

struct BatchMeta {
  const int* sizes;
  const int64_t* aoff;
  const int64_t* boff;
  const int* order;
  const int* tune;  // [kBuckets]: 0 = shared-memory path, else the panel width
  int count;
  int smem_n;
};

template <bool kExact>
__device__ __forceinline__ double bupd(double c, double l, double u) {
  if (kExact) return __dsub_rn(c, __dmul_rn(l, u));
  return fma(-l, u, c);
}
template <bool kExact>
__device__ __forceinline__ float bupd(float c, float l, float u) {
  if (kExact) return __fsub_rn(c, __fmul_rn(l, u));
  return fmaf(-l, u, c);
}
__device__ __forceinline__ double bmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float bmul(float a, float b) { return __fmul_rn(a, b); }

// Block-wide pivot search over rows [r0, r1) of column c of S (stride ld):
// strict '>' first-index semantics of src/blas/iamax.rs:6-21.  Returns the
// pivot row (r0 when the column is all zero or NaN) and the max in *maxv.
template <typename T>
__device__ __forceinline__ int block_iamax(const T* S, int ld, int c, int r0, int r1, T* maxv, T* red_v,
                                           int* red_i) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  T bv = T(0);
  int bi = INT_MAX;
  for (int r = r0 + tid; r < r1; r += kBatchThreads) {
    const T v = fabs(S[r * ld + c]);
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
    for (int q = 1; q < kBatchThreads / 32; ++q)
      if (red_v[q] > bv || (red_v[q] == bv && red_i[q] < bi)) {
        bv = red_v[q];
        bi = red_i[q];
      }
    red_v[0] = bv;
    red_i[0] = (bv > T(0)) ? bi : r0;
  }
  __syncthreads();
  const int p = red_i[0];
  *maxv = red_v[0];
  __syncthreads();  // red_* reused by the next search
  return p;
}

// Unblocked elimination of columns [c0, c0 + w) of S (rows [c0, nrow) active),
// row swaps across columns [0, ncol).  Pivots are recorded as absolute rows
// (row offset `roff` added).  Returns the last singular step (+roff) or -1.
template <typename T, bool kExact>
__device__ int eliminate(T* S, int ld, int nrow, int ncol, int c0, int w, int roff, int* piv, T* red_v, int* red_i) {
  const int tid = threadIdx.x;
  int sing = -1;
  for (int j = 0; j < w; ++j) {
    const int k = c0 + j;
    T maxv;
    const int p = block_iamax<T>(S, ld, k, k, nrow, &maxv, red_v, red_i);
    if (!(maxv > T(0))) {
      sing = k + roff;
      if (tid == 0) piv[k] = k + roff;
      continue;
    }
    if (tid == 0) piv[k] = p + roff;
    if (p != k)
      for (int c = tid; c < ncol; c += kBatchThreads) {
        const T t = S[k * ld + c];
        S[k * ld + c] = S[p * ld + c];
        S[p * ld + c] = t;
      }
    __syncthreads();
    const T recip = T(1) / S[k * ld + k];
    for (int r = k + 1 + tid; r < nrow; r += kBatchThreads) S[r * ld + k] = bmul(S[r * ld + k], recip);
    __syncthreads();
    const int cols = c0 + w - k - 1;  // update only the columns of this panel
    if (cols > 0 && k + 1 < nrow) {
      // Fixed column per thread, rows strided: one division per step.
      const int rstep = kBatchThreads / cols;  // >= 1 since cols < 256
      const int tr = tid / cols, tc = tid - tr * cols;
      if (tr < rstep) {
        const int c = k + 1 + tc;
        const T u = S[k * ld + c];
        for (int r = k + 1 + tr; r < nrow; r += rstep) S[r * ld + c] = bupd<kExact>(S[r * ld + c], S[r * ld + k], u);
      }
    }
    __syncthreads();
  }
  return sing;
}

// x <- U^-1 L^-1 P^T x for factors in M (stride ld, may be shared or global).
template <typename T, bool kExact>
__device__ void solve_factored(const T* M, int ld, int n, const int* piv, int poff, T* x) {
  const int tid = threadIdx.x;
  if (tid == 0)
    for (int i = 0; i < n; ++i) {
      const int p = piv[i] - poff;
      if (p != i) {
        const T t = x[i];
        x[i] = x[p];
        x[p] = t;
      }
    }
  __syncthreads();
  // Forward (unit L), column-oriented: x[i] takes its updates in increasing k.
  for (int k = 0; k < n - 1; ++k) {
    const T xk = x[k];
    for (int i = k + 1 + tid; i < n; i += kBatchThreads) x[i] = bupd<kExact>(x[i], M[i * ld + k], xk);
    __syncthreads();
  }
  if (kExact) {
    // lair's backward order: x[i] -= u[i][k] * x[k] for k = i+1.. in increasing k.
    if (tid == 0)
      for (int i = n - 1; i >= 0; --i) {
        T acc = x[i];
        for (int k = i + 1; k < n; ++k) acc = bupd<true>(acc, M[i * ld + k], x[k]);
        x[i] = acc / M[i * ld + i];
      }
    __syncthreads();
  } else {
    for (int k = n - 1; k >= 0; --k) {
      const T xk = x[k] / M[k * ld + k];
      __syncthreads();
      if (tid == 0) x[k] = xk;
      for (int i = tid; i < k; i += kBatchThreads) x[i] = bupd<false>(x[i], M[i * ld + k], xk);
      __syncthreads();
    }
  }
}

template <typename T, bool kExact>
__device__ int lu_solve_smem(T* A, T* xg, int* piv, int n, T* sm, T* red_v, int* red_i) {
  const int tid = threadIdx.x;
  const int ld = n + 1;
  T* S = sm;
  T* xs = sm + n * ld;
  for (int idx = tid; idx < n * n; idx += kBatchThreads) S[(idx / n) * ld + idx % n] = A[idx];
  for (int i = tid; i < n; i += kBatchThreads) xs[i] = xg[i];
  __syncthreads();
  const int sing = eliminate<T, kExact>(S, ld, n, n, 0, n, 0, piv, red_v, red_i);
  solve_factored<T, kExact>(S, ld, n, piv, 0, xs);
  for (int idx = tid; idx < n * n; idx += kBatchThreads) A[idx] = S[(idx / n) * ld + idx % n];
  for (int i = tid; i < n; i += kBatchThreads) xg[i] = xs[i];
  __syncthreads();
  return sing;
}

template <typename T, bool kExact>
__device__ int lu_solve_blocked(T* A, T* xg, int* piv, int n, int nb, T* sm, T* red_v, int* red_i) {
  const int tid = threadIdx.x;
  int sing = -1;
  for (int k0 = 0; k0 < n; k0 += nb) {
    const int w = min(nb, n - k0);
    const int prow = n - k0;
    const int ld = w + 1;
    T* P = sm;  // panel rows [k0, n), columns [k0, k0+w)
    for (int idx = tid; idx < prow * w; idx += kBatchThreads) {
      const int r = idx / w, c = idx - r * w;
      P[r * ld + c] = A[(k0 + r) * n + k0 + c];
    }
    __syncthreads();
    // piv entries k0.. are written relative to the panel, then made absolute.
    const int s = eliminate<T, kExact>(P, ld, prow, w, 0, w, k0, piv + k0, red_v, red_i);
    if (s >= 0) sing = s;
    for (int idx = tid; idx < prow * w; idx += kBatchThreads) {
      const int r = idx / w, c = idx - r * w;
      A[(k0 + r) * n + k0 + c] = P[r * ld + c];
    }
    __syncthreads();
    // Interchanges on the columns outside the panel, in order.
    const int nout = n - w;
    for (int c2 = tid; c2 < nout; c2 += kBatchThreads) {
      const int c = (c2 < k0) ? c2 : c2 + w;
      for (int j = 0; j < w; ++j) {
        const int r = k0 + j, p = piv[k0 + j];
        if (p != r) {
          const T t = A[r * n + c];
          A[r * n + c] = A[p * n + c];
          A[p * n + c] = t;
        }
      }
    }
    __syncthreads();
    const int c1 = k0 + w;
    if (c1 < n) {
      // U12 <- L11^-1 A12, one column per thread, increasing elimination step.
      for (int c = c1 + tid; c < n; c += kBatchThreads)
        for (int r = 1; r < w; ++r) {
          T acc = A[(k0 + r) * n + c];
          for (int q = 0; q < r; ++q) acc = bupd<kExact>(acc, P[r * ld + q], A[(k0 + q) * n + c]);
          A[(k0 + r) * n + c] = acc;
        }
      __syncthreads();
      // A22 <- A22 - L21 U12, each element's updates in increasing step.
      const int rows = n - c1, cols = n - c1;
      for (int idx = tid; idx < rows * cols; idx += kBatchThreads) {
        const int r = idx / cols, c = idx - r * cols;
        T acc = A[(c1 + r) * n + c1 + c];
        for (int q = 0; q < w; ++q) acc = bupd<kExact>(acc, P[(w + r) * ld + q], A[(k0 + q) * n + c1 + c]);
        A[(c1 + r) * n + c1 + c] = acc;
      }
      __syncthreads();
    }
  }
  solve_factored<T, kExact>(A, n, n, piv, 0, xg);
  return sing;
}

template <typename T, bool kExact>
__global__ void __launch_bounds__(kBatchThreads) batched_lu_kernel(BatchMeta m, T* a, T* b, int* piv, int* info,
                                                                   int* counter) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  __shared__ T red_v[kBatchThreads / 32];
  __shared__ int red_i[kBatchThreads / 32];
  __shared__ int s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int item = s_item;
    __syncthreads();
    if (item >= m.count) break;
    const int sys = m.order[item];
    const int n = m.sizes[sys];
    if (n <= 0 || n > kBatchMaxN) {
      if (threadIdx.x == 0) info[sys] = -2;  // rejected on the host; never reached
      continue;
    }
    T* A = a + m.aoff[sys];
    T* x = b + m.boff[sys];
    int* p = piv + m.boff[sys];
    const int nb = m.tune[batch_bucket(n)];
    int sing;
    if ((nb == 0 && n <= m.smem_n) || n <= 8)
      sing = lu_solve_smem<T, kExact>(A, x, p, n, sm, red_v, red_i);
    else
      sing = lu_solve_blocked<T, kExact>(A, x, p, n, nb > 0 ? nb : 32, sm, red_v, red_i);
    if (threadIdx.x == 0) info[sys] = sing;
  }
}

}  // namespace luhot

// ---------------------------------------------------------------------------
// Plan object (host).
// ---------------------------------------------------------------------------
struct luhot_batch {
  luhot_ctx* ctx = nullptr;
  int dtype = 0;  // 0 f64, 1 f32
  int mode = LUHOT_MODE_FAST;
  int64_t count = 0;
  int64_t a_elems = 0, b_elems = 0;
  std::vector<int> sizes;
  std::vector<int64_t> aoff, boff;
  std::vector<int> order;
  int tune[luhot::kBuckets];
  int smem_n = 0;
  int grid = 0;
  // device metadata: sizes, aoff, boff, order, tune, counter
  void* d_meta = nullptr;
  int* d_counter = nullptr;
  luhot::BatchMeta meta{};
  // cached graph
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  void* g_ptrs[4] = {nullptr, nullptr, nullptr, nullptr};
};

namespace luhot {

static size_t elem_size(int dtype) { return dtype == 0 ? sizeof(double) : sizeof(float); }

static int smem_n_for(size_t budget, size_t es) {
  int n = 8;
  while ((size_t)((n + 1) * (n + 2) + (n + 1)) * es <= budget && n + 1 <= kBatchMaxN) ++n;
  return n;
}

template <typename T, bool kExact>
static cudaError_t launch_batched(luhot_ctx* ctx, const BatchMeta& m, int grid, void* a, void* b, int* piv, int* info,
                                  int* counter, cudaStream_t stream) {
  // The shared-memory attribute was set when the plan was created (grid_for),
  // outside any stream capture.
  auto k = batched_lu_kernel<T, kExact>;
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(int), stream);
  if (e != cudaSuccess) return e;
  k<<<grid, kBatchThreads, kBatchSmem, stream>>>(m, static_cast<T*>(a), static_cast<T*>(b), piv, info, counter);
  (void)ctx;
  return cudaGetLastError();
}

static cudaError_t launch_plan(luhot_batch* p, const BatchMeta& m, int grid, void* a, void* b, int* piv, int* info,
                               int* counter, cudaStream_t stream) {
  const bool ex = p->mode == LUHOT_MODE_EXACT;
  if (p->dtype == 0)
    return ex ? launch_batched<double, true>(p->ctx, m, grid, a, b, piv, info, counter, stream)
              : launch_batched<double, false>(p->ctx, m, grid, a, b, piv, info, counter, stream);
  return ex ? launch_batched<float, true>(p->ctx, m, grid, a, b, piv, info, counter, stream)
            : launch_batched<float, false>(p->ctx, m, grid, a, b, piv, info, counter, stream);
}

static int grid_for(luhot_ctx* ctx, int dtype, int mode) {
  int per_sm = 0;
  const void* k;
  if (dtype == 0)
    k = mode == LUHOT_MODE_EXACT ? (const void*)batched_lu_kernel<double, true> : (const void*)batched_lu_kernel<double, false>;
  else
    k = mode == LUHOT_MODE_EXACT ? (const void*)batched_lu_kernel<float, true> : (const void*)batched_lu_kernel<float, false>;
  allow_max_dynamic_smem(k);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kBatchThreads, kBatchSmem) != cudaSuccess) {
    cudaGetLastError();
    per_sm = 1;
  }
  return std::max(1, per_sm) * ctx->num_sms;
}

static int upload_meta(luhot_batch* p) {
  luhot_ctx* ctx = p->ctx;
  const size_t c = (size_t)p->count;
  const size_t bytes = c * (sizeof(int) + 2 * sizeof(int64_t) + sizeof(int)) + kBuckets * sizeof(int) + 256;
  if (!p->d_meta) {
    LUHOT_CUDA_TRY(ctx, cudaMalloc(&p->d_meta, bytes));
    LUHOT_CUDA_TRY(ctx, cudaMalloc(&p->d_counter, 256));
  }
  char* base = static_cast<char*>(p->d_meta);
  int64_t* aoff = reinterpret_cast<int64_t*>(base);
  int64_t* boff = aoff + c;
  int* sizes = reinterpret_cast<int*>(boff + c);
  int* order = sizes + c;
  int* tune = order + c;
  LUHOT_CUDA_TRY(ctx, cudaMemcpy(aoff, p->aoff.data(), c * sizeof(int64_t), cudaMemcpyHostToDevice));
  LUHOT_CUDA_TRY(ctx, cudaMemcpy(boff, p->boff.data(), c * sizeof(int64_t), cudaMemcpyHostToDevice));
  LUHOT_CUDA_TRY(ctx, cudaMemcpy(sizes, p->sizes.data(), c * sizeof(int), cudaMemcpyHostToDevice));
  LUHOT_CUDA_TRY(ctx, cudaMemcpy(order, p->order.data(), c * sizeof(int), cudaMemcpyHostToDevice));
  LUHOT_CUDA_TRY(ctx, cudaMemcpy(tune, p->tune, kBuckets * sizeof(int), cudaMemcpyHostToDevice));
  p->meta.sizes = sizes;
  p->meta.aoff = aoff;
  p->meta.boff = boff;
  p->meta.order = order;
  p->meta.tune = tune;
  p->meta.count = (int)p->count;
  p->meta.smem_n = p->smem_n;
  return LUHOT_OK;
}

static void drop_graph(luhot_batch* p) {
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  p->exec = nullptr;
  p->graph = nullptr;
  for (auto& q : p->g_ptrs) q = nullptr;
}

}  // namespace luhot

using namespace luhot;

extern "C" {

int luhot_batch_create(luhot_ctx* ctx, int64_t count, const int32_t* sizes, int dtype, int mode, luhot_batch** out) {
  LUHOT_NVTX_FN();
  if (!ctx || !out) return LUHOT_ERR_INVALID_ARG;
  CtxGuard g(ctx);
  *out = nullptr;
  if (count < 0 || count >= INT32_MAX || (count > 0 && !sizes) || (dtype != 0 && dtype != 1) ||
      (mode != LUHOT_MODE_FAST && mode != LUHOT_MODE_EXACT))
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "batch: invalid arguments");
  for (int64_t i = 0; i < count; ++i)
    if (sizes[i] < 1 || sizes[i] > kBatchMaxN)
      return set_error(ctx, LUHOT_ERR_UNSUPPORTED, "batch: system sizes must be in [1, 256]");
  luhot_batch* p = new (std::nothrow) luhot_batch();
  if (!p) return LUHOT_ERR_ALLOC;
  p->ctx = ctx;
  p->dtype = dtype;
  p->mode = mode;
  p->count = count;
  p->sizes.assign(sizes, sizes + count);
  p->aoff.resize(count);
  p->boff.resize(count);
  int64_t ao = 0, bo = 0;
  for (int64_t i = 0; i < count; ++i) {
    p->aoff[i] = ao;
    p->boff[i] = bo;
    ao += (int64_t)sizes[i] * sizes[i];
    bo += sizes[i];
  }
  p->a_elems = ao;
  p->b_elems = bo;
  p->order.resize(count);
  std::iota(p->order.begin(), p->order.end(), 0);
  std::stable_sort(p->order.begin(), p->order.end(), [&](int x, int y) { return p->sizes[x] > p->sizes[y]; });
  p->smem_n = smem_n_for(kBatchSmem, elem_size(dtype));
  // Untuned default: shared memory where it fits, else 32-wide panels.
  for (int bk = 0; bk < kBuckets; ++bk) {
    const int hi = bk == 0 ? 16 : bk == 1 ? 32 : bk == 2 ? 64 : 64 + 32 * (bk - 2);
    p->tune[bk] = hi <= p->smem_n ? 0 : 32;
  }
  p->grid = grid_for(ctx, dtype, mode);
  int rc = count > 0 ? upload_meta(p) : LUHOT_OK;
  if (rc) {
    luhot_batch_destroy(p);
    return rc;
  }
  *out = p;
  return LUHOT_OK;
}

void luhot_batch_destroy(luhot_batch* p) {
  if (!p) return;
  cudaSetDevice(p->ctx->device);
  drop_graph(p);
  if (p->d_meta) cudaFree(p->d_meta);
  if (p->d_counter) cudaFree(p->d_counter);
  delete p;
}

int luhot_batch_layout(const luhot_batch* p, int64_t* a_elems, int64_t* b_elems) {
  if (!p) return LUHOT_ERR_INVALID_ARG;
  if (a_elems) *a_elems = p->a_elems;
  if (b_elems) *b_elems = p->b_elems;
  return LUHOT_OK;
}

int luhot_batch_tuning(const luhot_batch* p, int32_t* nb_per_bucket, int32_t* smem_n) {
  if (!p) return LUHOT_ERR_INVALID_ARG;
  if (nb_per_bucket)
    for (int i = 0; i < kBuckets; ++i) nb_per_bucket[i] = p->tune[i];
  if (smem_n) *smem_n = p->smem_n;
  return LUHOT_OK;
}

int luhot_batch_solve(luhot_batch* p, void* d_a, void* d_b, int32_t* d_piv, int32_t* d_info) {
  LUHOT_NVTX_FN();
  if (!p) return LUHOT_ERR_INVALID_ARG;
  luhot_ctx* ctx = p->ctx;
  CtxGuard g(ctx);
  if (p->count == 0) return LUHOT_OK;
  if (!d_a || !d_b || !d_piv || !d_info) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "batch: null pointer");
  void* ptrs[4] = {d_a, d_b, d_piv, d_info};
  if (!p->exec || memcmp(ptrs, p->g_ptrs, sizeof(ptrs)) != 0) {
    drop_graph(p);
    // Capture [counter reset, persistent kernel] once for these buffers.
    LUHOT_CUDA_TRY(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = launch_plan(p, p->meta, p->grid, d_a, d_b, d_piv, d_info, p->d_counter, ctx->stream);
    cudaGraph_t graph = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &graph);
    if (e != cudaSuccess || e2 != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
      return set_error(ctx, LUHOT_ERR_CUDA, std::string("batch: graph capture failed: ") +
                                                cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    p->graph = graph;
    LUHOT_CUDA_TRY(ctx, cudaGraphInstantiate(&p->exec, p->graph, 0));
    memcpy(p->g_ptrs, ptrs, sizeof(ptrs));
  }
  prof_begin(ctx, kProfOther);
  LUHOT_CUDA_TRY(ctx, cudaGraphLaunch(p->exec, ctx->stream));
  double fl = 0.0;
  for (int n : p->sizes) fl += 2.0 / 3.0 * n * (double)n * n + 2.0 * n * (double)n;
  prof_end(ctx, kProfOther, fl, (double)(p->a_elems + p->b_elems) * 2 * elem_size(p->dtype));
  LUHOT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return LUHOT_OK;
}

// Time every candidate (shared-memory path where it fits, panels of 8, 16,
// 32) per size bucket on up to 48 sample systems of that bucket, copied from
// the caller's data into scratch before each run, and keep the fastest.
int luhot_batch_autotune(luhot_batch* p, const void* d_a, const void* d_b) {
  LUHOT_NVTX_FN();
  if (!p) return LUHOT_ERR_INVALID_ARG;
  luhot_ctx* ctx = p->ctx;
  CtxGuard g(ctx);
  if (p->count == 0) return LUHOT_OK;
  if (!d_a || !d_b) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "batch: null pointer");
  const size_t es = elem_size(p->dtype);
  std::vector<std::vector<int>> members(kBuckets);
  for (int64_t i = 0; i < p->count; ++i) {
    auto& v = members[batch_bucket(p->sizes[i])];
    if (v.size() < 48) v.push_back((int)i);
  }
  // Scratch: sample matrices + rhs, and a pristine copy to restore from.
  int64_t sa = 0, sb = 0;
  for (auto& v : members)
    for (int i : v) {
      sa += (int64_t)p->sizes[i] * p->sizes[i];
      sb += p->sizes[i];
    }
  const size_t scratch = (size_t)(2 * sa + 2 * sb) * es + (size_t)sb * sizeof(int) + (size_t)p->count * sizeof(int) +
                         8 * 256;
  int rc = ensure_buf(ctx, ctx->work[1], scratch);
  if (rc) return rc;
  char* base = static_cast<char*>(ctx->work[1].ptr);
  char* wa = base;
  char* wb = wa + sa * es;
  char* pa = wb + sb * es;
  char* pb = pa + sa * es;
  int* spiv = reinterpret_cast<int*>(pb + sb * es);
  int* sinfo = spiv + sb;
  // Per-bucket sample metadata in the plan's layout style.
  std::vector<int> s_sizes, s_order;
  std::vector<int64_t> s_aoff, s_boff;
  std::vector<int> bucket_first(kBuckets + 1, 0);
  int64_t ao = 0, bo = 0;
  for (int bk = 0; bk < kBuckets; ++bk) {
    bucket_first[bk] = (int)s_sizes.size();
    for (int i : members[bk]) {
      const int n = p->sizes[i];
      LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(pa + ao * es, static_cast<const char*>(d_a) + p->aoff[i] * es,
                                          (size_t)n * n * es, cudaMemcpyDeviceToDevice, ctx->stream));
      LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(pb + bo * es, static_cast<const char*>(d_b) + p->boff[i] * es, (size_t)n * es,
                                          cudaMemcpyDeviceToDevice, ctx->stream));
      s_sizes.push_back(n);
      s_aoff.push_back(ao);
      s_boff.push_back(bo);
      s_order.push_back((int)s_order.size());
      ao += (int64_t)n * n;
      bo += n;
    }
  }
  bucket_first[kBuckets] = (int)s_sizes.size();
  const int ns = (int)s_sizes.size();
  DevBuf meta_buf;
  rc = ensure_buf(ctx, meta_buf, (size_t)ns * (2 * sizeof(int64_t) + 2 * sizeof(int)) + kBuckets * sizeof(int) + 512);
  if (rc) return rc;
  int64_t* m_aoff = static_cast<int64_t*>(meta_buf.ptr);
  int64_t* m_boff = m_aoff + ns;
  int* m_sizes = reinterpret_cast<int*>(m_boff + ns);
  int* m_order = m_sizes + ns;
  int* m_tune = m_order + ns;
  int* m_counter = m_tune + kBuckets + 1;
  cudaMemcpy(m_aoff, s_aoff.data(), ns * sizeof(int64_t), cudaMemcpyHostToDevice);
  cudaMemcpy(m_boff, s_boff.data(), ns * sizeof(int64_t), cudaMemcpyHostToDevice);
  cudaMemcpy(m_sizes, s_sizes.data(), ns * sizeof(int), cudaMemcpyHostToDevice);
  cudaMemcpy(m_order, s_order.data(), ns * sizeof(int), cudaMemcpyHostToDevice);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int cands[4] = {0, 8, 16, 32};
  for (int bk = 0; bk < kBuckets; ++bk) {
    const int first = bucket_first[bk], cnt = bucket_first[bk + 1] - first;
    if (cnt == 0) continue;
    int maxn = 0;
    for (int q = first; q < first + cnt; ++q) maxn = std::max(maxn, s_sizes[q]);
    float best = 1e30f;
    int best_nb = p->tune[bk];
    for (int nb : cands) {
      if (nb == 0 && maxn > p->smem_n) continue;
      int tune_all[kBuckets];
      for (int q = 0; q < kBuckets; ++q) tune_all[q] = nb;
      cudaMemcpy(m_tune, tune_all, sizeof(tune_all), cudaMemcpyHostToDevice);
      BatchMeta m{m_sizes, m_aoff, m_boff, m_order + first, m_tune, cnt, p->smem_n};
      float ms = 0.f;
      for (int rep = 0; rep < 2; ++rep) {
        cudaMemcpyAsync(wa, pa, sa * es, cudaMemcpyDeviceToDevice, ctx->stream);
        cudaMemcpyAsync(wb, pb, sb * es, cudaMemcpyDeviceToDevice, ctx->stream);
        cudaEventRecord(e0, ctx->stream);
        cudaError_t e = launch_plan(p, m, p->grid, wa, wb, spiv, sinfo, m_counter, ctx->stream);
        cudaEventRecord(e1, ctx->stream);
        if (e != cudaSuccess) {
          cudaEventDestroy(e0);
          cudaEventDestroy(e1);
          cudaFree(meta_buf.ptr);
          return set_error(ctx, LUHOT_ERR_CUDA, std::string("batch autotune: ") + cudaGetErrorString(e));
        }
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
      }
      count_launch(ctx, 2);
      if (ms < best) {
        best = ms;
        best_nb = nb;
      }
    }
    p->tune[bk] = best_nb;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(meta_buf.ptr);
  drop_graph(p);
  return upload_meta(p);
}

// Host-buffer form: packed host arrays in the plan's layout, staged in and out.
int luhot_batch_solve_host(luhot_batch* p, void* a, void* b, int32_t* piv, int32_t* info) {
  LUHOT_NVTX_FN();
  if (!p) return LUHOT_ERR_INVALID_ARG;
  luhot_ctx* ctx = p->ctx;
  if (p->count == 0) return LUHOT_OK;
  if (!a || !b || !piv || !info) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "batch: null pointer");
  const size_t es = elem_size(p->dtype);
  void *d_a, *d_b;
  int *d_piv, *d_info;
  {
    CtxGuard g(ctx);
    int rc = ensure_buf(ctx, ctx->work[0], (size_t)p->a_elems * es);
    if (!rc) rc = ensure_buf(ctx, ctx->work[2], (size_t)p->b_elems * (es + sizeof(int)) + (size_t)p->count * sizeof(int) + 256);
    if (rc) return rc;
    d_a = ctx->work[0].ptr;
    d_b = ctx->work[2].ptr;
    d_piv = reinterpret_cast<int*>(static_cast<char*>(d_b) + (size_t)p->b_elems * es);
    d_info = d_piv + p->b_elems;
    LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(d_a, a, (size_t)p->a_elems * es, cudaMemcpyHostToDevice, ctx->stream));
    LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(d_b, b, (size_t)p->b_elems * es, cudaMemcpyHostToDevice, ctx->stream));
  }
  int rc = luhot_batch_solve(p, d_a, d_b, d_piv, d_info);
  if (rc) return rc;
  CtxGuard g(ctx);
  LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(a, d_a, (size_t)p->a_elems * es, cudaMemcpyDeviceToHost, ctx->stream));
  LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(b, d_b, (size_t)p->b_elems * es, cudaMemcpyDeviceToHost, ctx->stream));
  LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(piv, d_piv, (size_t)p->b_elems * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(info, d_info, (size_t)p->count * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  LUHOT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return LUHOT_OK;
}

}  // extern "C"
