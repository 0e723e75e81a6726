// Sync-free blocked triangular solve: one launch per sweep.
//
// op(A) x = b with op(A) triangular (lower/upper, unit/non-unit, A or A^T of
// a row-major LU factor), nrhs <= 16 columns of x (row-major, ldx), in place.
//
// The rows are cut into 64-row blocks.  CTAs take blocks by ticket (an atomic
// counter) in the order the sweep needs them (top-down for lower, bottom-up
// for upper).  The CTA of block I subtracts op(A)(I, J) x(J) for every
// earlier block J as soon as J's ready flag is set, then solves its
// diagonal block and sets its own flag.  A CTA only ever waits for blocks
// whose tickets were drawn before its own, i.e. for CTAs that are already
// running, so no co-residency is needed; each wait is bounded by the global
// timer (the context's wait limit) and reports LUHOT_ERR_TIMEOUT on expiry.
//
// Latency hiding: the next tile of op(A) is loaded into registers while the
// current one is used (A is read-only, so prefetching never waits on a
// flag); every thread carries up to four independent (row, rhs) chains.  In
// fast mode with fewer than four right-hand sides the 64 columns of a tile are
// also split among 256/(64*nrhs) threads per row and the partial sums are
// added once, before the diagonal block.
//
// Order: in exact mode (lower, unit; no k split) row i of x receives
// x[i] -= l[i][k] * x[k] for k increasing, multiply and subtract rounded
// apart, which is lair's forward substitution (src/lapack/getrs.rs:24-29),
// so the exact forward sweep is bit-identical.
#include <algorithm>

#include "common.cuh"
#include "luhot_internal.h"
#include "trsv.cuh"

namespace luhot {

constexpr int kBS = 64;         // block rows
constexpr int kMaxRhs = 16;     // right-hand sides per launch
constexpr int kThreads = 256;
constexpr int kLds = kBS + 1;   // odd stride: conflict-free row and column reads
constexpr int kPrefetch = kBS * kBS / kThreads;  // tile elements per thread (16)

template <bool kExact>
__device__ __forceinline__ double tsub(double c, double l, double u) {
  if (kExact) return __dsub_rn(c, __dmul_rn(l, u));
  return fma(-l, u, c);
}
template <bool kExact>
__device__ __forceinline__ float tsub(float c, float l, float u) {
  if (kExact) return __fsub_rn(c, __fmul_rn(l, u));
  return fmaf(-l, u, c);
}

// Element (i, k) of op(A), widened from the storage type TA to the
// arithmetic type T (FP32 factors can be applied in FP64 arithmetic).
template <typename T, typename TA, bool kTrans>
__device__ __forceinline__ T op_elem(const TA* a, int64_t lda, int i, int k) {
  return static_cast<T>(kTrans ? a[(int64_t)k * lda + i] : a[(int64_t)i * lda + k]);
}

// Element e of this thread's share of tile op(A)(i0.., k0..): (r, c) within
// the tile.  Consecutive threads walk the contiguous direction in memory.
template <bool kTrans>
__device__ __forceinline__ void tile_coord(int e, int& r, int& c) {
  const int idx = threadIdx.x + e * kThreads;
  if (kTrans) {
    c = idx / kBS;
    r = idx - c * kBS;
  } else {
    r = idx / kBS;
    c = idx - r * kBS;
  }
}

template <typename T, typename TA, bool kTrans>
__device__ __forceinline__ void tile_load(T (&reg)[kPrefetch], const TA* a, int64_t lda, int i0, int k0, int rows,
                                          int cols) {
#pragma unroll
  for (int e = 0; e < kPrefetch; ++e) {
    int r, c;
    tile_coord<kTrans>(e, r, c);
    reg[e] = (r < rows && c < cols) ? op_elem<T, TA, kTrans>(a, lda, i0 + r, k0 + c) : T(0);
  }
}

template <typename T, bool kTrans>
__device__ __forceinline__ void tile_store(T* tile, const T (&reg)[kPrefetch]) {
#pragma unroll
  for (int e = 0; e < kPrefetch; ++e) {
    int r, c;
    tile_coord<kTrans>(e, r, c);
    tile[r * kLds + c] = reg[e];
  }
}

__device__ __forceinline__ int ld_acquire_i32(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_i32(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Wait until flags[j] != 0; false if the wait (or an earlier one) gave up.
__device__ __forceinline__ bool wait_ready(const int* flags, int j, DeviceStatus* st) {
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    int ok = 1;
    if (ld_acquire_i32(flags + j) == 0) {
      const unsigned long long t0 = global_timer_ns();
      const unsigned long long limit = st->timeout_ns;
      unsigned int spins = 0;
      while (ld_acquire_i32(flags + j) == 0) {
        if ((++spins & 31u) == 0) {
          if (ld_relaxed_i32(&st->abort)) {
            ok = 0;
            break;
          }
          if (global_timer_ns() - t0 > limit) {
            atomicCAS(&st->error, kDevOk, kDevBarrierTimeout);
            atomicExch(&st->timeout_where, (unsigned long long)j);
            atomicExch(&st->abort, 1);
            ok = 0;
            break;
          }
        }
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// kNR: right-hand sides handled per launch (1, 2, 4 or 16; runtime nrhs <= kNR).
template <typename T, typename TA, bool kExact, bool kLower, bool kUnit, bool kTrans, int kNR>
__global__ void __launch_bounds__(kThreads) trsv_syncfree_kernel(const TA* __restrict__ a, int64_t lda, T* x,
                                                                 int64_t ldx, int n, int nrhs, int nchain,
                                                                 int* flags, int* ticket, DeviceStatus* st,
                                                                 const T* __restrict__ dinv) {
  // Threads per (row, rhs) pair: k split only in fast mode.
  constexpr int kKS = kExact ? 1 : (kNR >= 4 ? 1 : 4 / kNR);
  constexpr int kKLen = kBS / kKS;                      // k columns per thread and tile
  constexpr int kPairs = kBS * kNR;                      // (row, rhs) pairs
  constexpr int kPP = (kPairs * kKS + kThreads - 1) / kThreads;  // pair slots per thread (<= 4)
  static_assert(kPP >= 1 && kPP <= 4, "bad pair split");

  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* tile0 = reinterpret_cast<T*>(smem_raw);            // [64][65]
  T* tile1 = tile0 + kBS * kLds;                        // [64][65]
  T* xs = tile1 + kBS * kLds;                           // [64][kNR] x(J)
  T* xacc = xs + kBS * kNR;                             // [64][kNR]
  __shared__ int s_ticket;
  const int nblk = (n + kBS - 1) / kBS;
  if (threadIdx.x == 0) s_ticket = atomicAdd(ticket, 1);
  __syncthreads();
  // Ticket -> (chain, block): the chains (groups of kNR right-hand sides)
  // advance together, and a block of any chain only waits for blocks of its
  // own chain with smaller tickets.
  if (s_ticket >= nblk * nchain) return;
  const int chain = s_ticket % nchain, t = s_ticket / nchain;
  x += chain * kNR;
  nrhs = min(kNR, nrhs - chain * kNR);
  flags += (size_t)chain * nblk;
  const int I = kLower ? t : (nblk - 1 - t);
  const int i0 = I * kBS;
  const int rows = min(kBS, n - i0);

  // This thread's pair slots: slot q covers logical index L = tid + q*256;
  // pair = L / kKS (row = pair / kNR, rhs = pair % kNR), k part = L % kKS.
  int prow[kPP], pc[kPP], pk0[kPP];
  bool pon[kPP];
  T acc[kPP];
#pragma unroll
  for (int q = 0; q < kPP; ++q) {
    const int L = threadIdx.x + q * kThreads;
    const int pair = L / kKS;
    prow[q] = pair / kNR;
    pc[q] = pair % kNR;
    pk0[q] = (L % kKS) * kKLen;
    pon[q] = (pair < kPairs) && (pc[q] < nrhs) && (prow[q] < rows);
    // The k-part 0 slot carries the right-hand side; the others start at 0.
    acc[q] = (pon[q] && pk0[q] == 0) ? x[(int64_t)(i0 + prow[q]) * ldx + pc[q]] : T(0);
  }

  const int nupd = kLower ? I : (nblk - 1 - I);  // blocks before I in sweep order
  // Inverse of this block's diagonal tile (when given): fetched now, used last.
  T ireg[kPrefetch];
  // For op(A) = A^T the diagonal block of op(A) is the transpose of A's, and
  // so is its inverse: the tile is read transposed.
  if (!kExact && dinv != nullptr) tile_load<T, T, kTrans>(ireg, dinv + (int64_t)I * kBS * kBS, kBS, 0, 0, kBS, kBS);
  T reg[kPrefetch];
  if (nupd > 0) {
    const int J0 = kLower ? 0 : nblk - 1;
    tile_load<T, TA, kTrans>(reg, a, lda, i0, J0 * kBS, rows, min(kBS, n - J0 * kBS));
  }
  for (int s = 0; s < nupd; ++s) {
    const int J = kLower ? s : (nblk - 1 - s);
    const int j0 = J * kBS;
    const int cols = min(kBS, n - j0);
    T* tile = (s & 1) ? tile1 : tile0;
    tile_store<T, kTrans>(tile, reg);
    if (s + 1 < nupd) {  // prefetch the next tile while this one is used
      const int Jn = kLower ? s + 1 : (nblk - 2 - s);
      tile_load<T, TA, kTrans>(reg, a, lda, i0, Jn * kBS, rows, min(kBS, n - Jn * kBS));
    }
    if (!wait_ready(flags, J, st)) return;
    for (int idx = threadIdx.x; idx < kBS * kNR; idx += kThreads) {
      const int k = idx / kNR, c = idx - k * kNR;
      xs[idx] = (k < cols && c < nrhs) ? __ldcg(&x[(int64_t)(j0 + k) * ldx + c]) : T(0);
    }
    __syncthreads();
    if (kLower) {
#pragma unroll 4
      for (int kk = 0; kk < kKLen; ++kk) {
#pragma unroll
        for (int q = 0; q < kPP; ++q) {
          const int k = pk0[q] + kk;
          if (pon[q]) acc[q] = tsub<kExact>(acc[q], tile[prow[q] * kLds + k], xs[k * kNR + pc[q]]);
        }
      }
    } else {
#pragma unroll 4
      for (int kk = kKLen - 1; kk >= 0; --kk) {
#pragma unroll
        for (int q = 0; q < kPP; ++q) {
          const int k = pk0[q] + kk;
          if (pon[q]) acc[q] = tsub<kExact>(acc[q], tile[prow[q] * kLds + k], xs[k * kNR + pc[q]]);
        }
      }
    }
    __syncthreads();
  }

  if (!kExact && dinv != nullptr) {
    // Diagonal block by its precomputed inverse: x(I) = D^-1 xacc, a 64 x 64
    // matvec split like the updates (no sequential chain on the critical path).
    __syncthreads();
    tile_store<T, kTrans>(tile0, ireg);
#pragma unroll
    for (int q = 0; q < kPP; ++q) {
      T v = acc[q];
      if (kKS > 1) {
#pragma unroll
        for (int off = 1; off < kKS; off <<= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      }
      if (pon[q] && pk0[q] == 0) xacc[prow[q] * kNR + pc[q]] = v;
      if (!pon[q] && pk0[q] == 0 && (threadIdx.x + q * kThreads) / kKS < kPairs)
        xacc[prow[q] * kNR + pc[q]] = T(0);
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kPP; ++q) {
      T v = T(0);
      for (int kk = 0; kk < kKLen; ++kk) {
        const int k = pk0[q] + kk;
        v = fma(tile0[prow[q] * kLds + k], xacc[k * kNR + pc[q]], v);
      }
      if (kKS > 1) {
#pragma unroll
        for (int off = 1; off < kKS; off <<= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      }
      if (pon[q] && pk0[q] == 0) x[(int64_t)(i0 + prow[q]) * ldx + pc[q]] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      st_release_i32(flags + I, 1);
    }
    return;
  }

  // Sum the k parts of each pair into xacc.
  T* diag = tile0;
  {
    T dreg[kPrefetch];
    tile_load<T, TA, kTrans>(dreg, a, lda, i0, i0, rows, rows);
    for (int idx = threadIdx.x; idx < kBS * kNR; idx += kThreads) xacc[idx] = T(0);
    __syncthreads();
    tile_store<T, kTrans>(diag, dreg);
  }
#pragma unroll
  for (int q = 0; q < kPP; ++q) {
    T v = acc[q];
    if (kKS > 1) {
#pragma unroll
      for (int off = 1; off < kKS; off <<= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    }
    if (pon[q] && pk0[q] == 0) xacc[prow[q] * kNR + pc[q]] = v;
  }
  __syncthreads();

  // Diagonal block: column-oriented substitution, steps in sweep order.  For
  // at most four right-hand sides one warp does it with shuffles (no block
  // barriers); otherwise all threads, one barrier per step.
  if (kNR <= 4) {
    if (threadIdx.x < 32) {
      const int lane = threadIdx.x;
      T v[2][kNR];
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int c = 0; c < kNR; ++c) v[h][c] = xacc[(lane + 32 * h) * kNR + c];
      for (int step = 0; step < rows; ++step) {
        const int i = kLower ? step : (rows - 1 - step);
        const int hi = i >> 5, li = i & 31;
        const T dii = diag[i * kLds + i];
#pragma unroll
        for (int c = 0; c < kNR; ++c) {
          T xi = __shfl_sync(0xffffffffu, hi ? v[1][c] : v[0][c], li);
          if (!kUnit) xi = xi / dii;
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int r = lane + 32 * h;
            if (r == i) {
              v[h][c] = xi;
            } else if (kLower ? (r > i && r < rows) : (r < i)) {
              v[h][c] = tsub<kExact>(v[h][c], diag[r * kLds + i], xi);
            }
          }
        }
      }
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int c = 0; c < kNR; ++c) {
          const int r = lane + 32 * h;
          if (r < rows && c < nrhs) x[(int64_t)(i0 + r) * ldx + c] = v[h][c];
        }
    }
  } else {
    T* xout = xs;  // x(J) no longer needed
    for (int step = 0; step < rows; ++step) {
      const int i = kLower ? step : (rows - 1 - step);
      for (int p = threadIdx.x; p < kBS * kNR; p += kThreads) {
        const int r = p / kNR, c = p - r * kNR;
        T xi = xacc[i * kNR + c];
        if (!kUnit) xi = xi / diag[i * kLds + i];
        if (r == i) xout[r * kNR + c] = xi;
        else if (kLower ? (r > i && r < rows) : (r < i))
          xacc[r * kNR + c] = tsub<kExact>(xacc[r * kNR + c], diag[r * kLds + i], xi);
      }
      __syncthreads();
    }
    for (int p = threadIdx.x; p < rows * kNR; p += kThreads) {
      const int r = p / kNR, c = p - r * kNR;
      if (c < nrhs) x[(int64_t)(i0 + r) * ldx + c] = xout[r * kNR + c];
    }
  }
  // Every thread's x writes happen before thread 0's fence (CTA barrier); the
  // gpu-scope fence and release store then publish them together.
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    st_release_i32(flags + I, 1);
  }
}

size_t trsv_syncfree_smem(size_t elem) { return (2 * (size_t)kBS * kLds + 2 * (size_t)kBS * kMaxRhs) * elem; }
int trsv_syncfree_blocks(int n) { return (n + kBS - 1) / kBS; }

// Fast sweeps of more than four right-hand sides run as independent chains
// of four (one launch): each chain step (the last off-diagonal tile and the
// diagonal block of a 64-row block) is then a quarter of the FP64 work on
// the critical path of one chain of sixteen.
static int trsv_chains(bool exact, int nc) { return (!exact && nc > 4) ? (nc + 3) / 4 : 1; }

template <typename T, typename TA, bool EX, bool LO, bool UN, bool TR>
static cudaError_t launch_case(cudaStream_t stream, const TA* a, int64_t lda, T* x, int64_t ldx, int n, int nc,
                               int* flags, int* ticket, DeviceStatus* st, const T* dinv) {
  const int nblk = trsv_syncfree_blocks(n);
  const size_t smem = trsv_syncfree_smem(sizeof(T));
  const int nchain = trsv_chains(EX, nc);
  cudaError_t e;
#define LUHOT_TRSV_NR(NR)                                                                                \
  {                                                                                                      \
    auto k = trsv_syncfree_kernel<T, TA, EX, LO, UN, TR, NR>;                                            \
    e = allow_max_dynamic_smem(k);                                                                       \
    if (e != cudaSuccess) return e;                                                                      \
    k<<<nblk * nchain, kThreads, smem, stream>>>(a, lda, x, ldx, n, nc, nchain, flags, ticket, st, dinv); \
    return cudaGetLastError();                                                                           \
  }
  if (nc == 1) LUHOT_TRSV_NR(1)
  if (nc == 2) LUHOT_TRSV_NR(2)
  if (nc <= 4 || nchain > 1) LUHOT_TRSV_NR(4)
  LUHOT_TRSV_NR(16)
#undef LUHOT_TRSV_NR
}

template <typename T, typename TA>
cudaError_t launch_trsv_syncfree(cudaStream_t stream, const TA* a, int64_t lda, T* x, int64_t ldx, int n, int nrhs,
                                 bool lower, bool unit, bool trans, bool exact, int* flags, int* ticket,
                                 DeviceStatus* st, const T* dinv) {
  if (n <= 0 || nrhs <= 0) return cudaSuccess;
  const int nblk = trsv_syncfree_blocks(n);
  if (exact) dinv = nullptr;  // inverses serve the fast sweeps only
  for (int c0 = 0; c0 < nrhs; c0 += kMaxRhs) {
    const int nc = std::min(kMaxRhs, nrhs - c0);
    cudaError_t e = cudaMemsetAsync(flags, 0, (size_t)nblk * trsv_chains(exact, nc) * sizeof(int), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(ticket, 0, sizeof(int), stream);
    if (e != cudaSuccess) return e;
    T* xc = x + c0;
    if (exact && lower && unit && !trans)
      e = launch_case<T, TA, true, true, true, false>(stream, a, lda, xc, ldx, n, nc, flags, ticket, st, nullptr);
    else if (!exact && lower && unit && !trans)
      e = launch_case<T, TA, false, true, true, false>(stream, a, lda, xc, ldx, n, nc, flags, ticket, st, dinv);
    else if (!exact && !lower && !unit && !trans)
      e = launch_case<T, TA, false, false, false, false>(stream, a, lda, xc, ldx, n, nc, flags, ticket, st, dinv);
    else if (!exact && lower && !unit && trans)
      e = launch_case<T, TA, false, true, false, true>(stream, a, lda, xc, ldx, n, nc, flags, ticket, st, dinv);
    else if (!exact && !lower && unit && trans)
      e = launch_case<T, TA, false, false, true, true>(stream, a, lda, xc, ldx, n, nc, flags, ticket, st, dinv);
    else
      return cudaErrorNotSupported;
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Inverse of every 64 x 64 diagonal block of a triangular factor (lower unit
// or upper non-unit), row-major 64 x 64 per block, zero-padded past n.  One
// CTA per block, one thread per column of the inverse (substitution on the
// unit vector), all in shared memory.
template <typename T, typename TA, bool kLower, bool kUnit>
__global__ void __launch_bounds__(kBS) trsv_invert_diag_kernel(const TA* __restrict__ a, int64_t lda, int n, T* dinv) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* S = reinterpret_cast<T*>(smem_raw);  // [64][65] diagonal block
  T* Y = S + kBS * kLds;                   // [64][65] inverse, column c owned by thread c
  const int i0 = blockIdx.x * kBS;
  const int rows = min(kBS, n - i0);
  for (int idx = threadIdx.x; idx < kBS * kBS; idx += kBS) {
    const int r = idx / kBS, c = idx - r * kBS;
    S[r * kLds + c] = (r < rows && c < rows) ? static_cast<T>(a[(int64_t)(i0 + r) * lda + i0 + c]) : T(0);
  }
  __syncthreads();
  const int c = threadIdx.x;
  if (kLower) {
    for (int i = 0; i < kBS; ++i) {
      T v = T(0);
      if (c < rows && i < rows && i >= c) {
        v = (i == c) ? T(1) : T(0);
        for (int k = c; k < i; ++k) v = fma(-S[i * kLds + k], Y[k * kLds + c], v);
        if (!kUnit) v = v / S[i * kLds + i];
      }
      Y[i * kLds + c] = v;
    }
  } else {
    for (int i = kBS - 1; i >= 0; --i) {
      T v = T(0);
      if (c < rows && i < rows && i <= c) {
        v = (i == c) ? T(1) : T(0);
        for (int k = i + 1; k <= c; ++k) v = fma(-S[i * kLds + k], Y[k * kLds + c], v);
        if (!kUnit) v = v / S[i * kLds + i];
      }
      Y[i * kLds + c] = v;
    }
  }
  __syncthreads();
  T* out = dinv + (int64_t)blockIdx.x * kBS * kBS;
  for (int idx = threadIdx.x; idx < kBS * kBS; idx += kBS) out[idx] = Y[(idx / kBS) * kLds + idx % kBS];
}

size_t trsv_inverse_elems(int n) { return (size_t)trsv_syncfree_blocks(n) * kBS * kBS; }

template <typename T, typename TA>
cudaError_t launch_trsv_invert_diag(cudaStream_t stream, const TA* a, int64_t lda, int n, bool lower, T* dinv) {
  if (n <= 0) return cudaSuccess;
  const size_t smem = 2 * (size_t)kBS * kLds * sizeof(T);
  const int nblk = trsv_syncfree_blocks(n);
  auto k = lower ? trsv_invert_diag_kernel<T, TA, true, true> : trsv_invert_diag_kernel<T, TA, false, false>;
  cudaError_t e = allow_max_dynamic_smem(k);
  if (e != cudaSuccess) return e;
  k<<<nblk, kBS, smem, stream>>>(a, lda, n, dinv);
  return cudaGetLastError();
}

#define LUHOT_TRSV_INST(T, TA)                                                                                  \
  template cudaError_t launch_trsv_syncfree<T, TA>(cudaStream_t, const TA*, int64_t, T*, int64_t, int, int, bool, \
                                                   bool, bool, bool, int*, int*, DeviceStatus*, const T*);      \
  template cudaError_t launch_trsv_invert_diag<T, TA>(cudaStream_t, const TA*, int64_t, int, bool, T*);
LUHOT_TRSV_INST(double, double)
LUHOT_TRSV_INST(float, float)
LUHOT_TRSV_INST(double, float)
#undef LUHOT_TRSV_INST

}  // namespace luhot
