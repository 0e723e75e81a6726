// Blocked right-looking LU with partial pivoting on one GB300 (sm_103a).
//
// Matrix layout in HBM: row-major, leading dimension lda >= n (elements).
// Pivots: int32 on the device, LAPACK-style sequential interchanges
// (step i swapped row i with row piv[i]), the convention of lair's
// src/lapack/getrf.rs:12-27.
//
// One block step k0 (panel width w) runs four kernels:
//   1. panel_kernel   cooperative; factors rows [k0, m) x cols [k0, k0+w) held
//                     in shared memory across all CTAs; per column one
//                     exchange of step-tagged candidates through L2 (integer
//                     pivot keys, redux.sync reduce, deterministic order; the
//                     winner's row segment follows by cp.async off the
//                     critical path), row interchanges as id swaps, and the
//                     update of the previous step overlapping the exchange.
//   2. laswp_moves_kernel  applies the panel's interchanges to the columns
//                     left and right of it, as a gather of the (at most 2w)
//                     rows that moved.
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
#include "ozaki.cuh"
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
  unsigned long long* slots;  // [2][kMaxPanelCtas][kPanelSlotWords] exchange words
  int* moves;                 // (destination, source) rows of the panel's rows that moved
  int* move_count;            // zeroed before the launch
  DeviceStatus* st;
};

// Pivot search keys.  lair's iamax (src/blas/iamax.rs:6-21) takes the first
// index of the largest |x| with a strict `>`: larger value wins, equal values
// keep the smaller row, NaN never wins, and an all-zero/NaN column means a
// singular step.  For |x| >= 0 the IEEE bit pattern orders like the value,
// so the search compares integers (on the integer pipe; FP64 compares are
// slow on this part): key = bits of |x|, or 0 for NaN.  (key, row) ordered by
// key descending then row ascending is a total order, so any reduction tree
// gives the same answer; key 0 means "no positive entry".
template <typename T>
struct PivotKey;
template <>
struct PivotKey<float> {
  using K = unsigned int;
  __device__ static K of(float x) {
    const unsigned int b = __float_as_uint(x) & 0x7fffffffu;
    return b > 0x7f800000u ? 0u : b;
  }
  __device__ static K shfl(K k, int src) { return __shfl_sync(0xffffffffu, k, src); }
  __device__ static float value(K raw) { return __uint_as_float(raw); }
};
template <>
struct PivotKey<double> {
  using K = unsigned long long;
  __device__ static K of(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
    return b > 0x7ff0000000000000ull ? 0ull : b;
  }
  __device__ static K shfl(K k, int src) { return __shfl_sync(0xffffffffu, k, src); }
  __device__ static double value(K raw) { return __longlong_as_double((long long)raw); }
};

template <typename K>
__device__ __forceinline__ void key_combine(K& k, int& i, int& s, K k2, int i2, int s2) {
  if (k2 > k || (k2 == k && i2 < i)) {
    k = k2;
    i = i2;
    s = s2;
  }
}
// Warp-wide reduction of (key, id, slot) on the integer reduce unit
// (redux.sync): the largest key, then the smallest id among the lanes that
// hold it; the slot comes from that lane, whose index is returned.  The
// order is total, so this is the answer of any key_combine tree.
__device__ __forceinline__ int key_reduce_redux(unsigned int& k, int& i, int& s) {
  const unsigned int m = __reduce_max_sync(0xffffffffu, k);
  const int mi = __reduce_min_sync(0xffffffffu, k == m ? i : INT_MAX);
  const int src = __ffs(__ballot_sync(0xffffffffu, k == m && i == mi)) - 1;
  s = __shfl_sync(0xffffffffu, s, src);
  k = m;
  i = mi;
  return src;
}
__device__ __forceinline__ int key_reduce_redux(unsigned long long& k, int& i, int& s) {
  const unsigned int hi = (unsigned int)(k >> 32);
  const unsigned int mh = __reduce_max_sync(0xffffffffu, hi);
  const unsigned int ml = __reduce_max_sync(0xffffffffu, hi == mh ? (unsigned int)k : 0u);
  const unsigned long long m = ((unsigned long long)mh << 32) | ml;
  const int mi = __reduce_min_sync(0xffffffffu, k == m ? i : INT_MAX);
  const int src = __ffs(__ballot_sync(0xffffffffu, k == m && i == mi)) - 1;
  s = __shfl_sync(0xffffffffu, s, src);
  k = m;
  i = mi;
  return src;
}

// Exchange words: payload in the low 32 bits, the step tag in the high 32.
// A reader accepts a word only when its tag is the step it waits for, so no
// fence or counter orders the writers and readers: each 8-byte word is
// written and read whole.  Tags are step + 1 and the slots are zeroed before
// each factorization, so a stale word never carries a live tag.
// Reuse: the slots alternate by step parity, and a CTA rewrites its slot of
// parity j & 1 at step j + 2 only after it has seen every CTA's step j + 1
// header.  Each CTA publishes that header only after all its reads of step j
// have returned their values (the poll consumes them; the segment copy is
// waited for and its tags checked).  So no read of step j can observe a
// step j + 2 word; the order comes from the data dependencies, not from a
// fence.
__device__ __forceinline__ unsigned long long ld_word(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_word(unsigned long long* p, unsigned int bits, unsigned int tag) {
  const unsigned long long v = ((unsigned long long)tag << 32) | bits;
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ bool word_ok(unsigned long long v, unsigned int tag) {
  return (unsigned int)(v >> 32) == tag;
}
// Four words (one 32-byte L2 sector) in one load; each 8-byte element is
// read whole.  p 32-byte aligned.
__device__ __forceinline__ void ld_quad(const unsigned long long* p, unsigned long long* v) {
  asm volatile("ld.relaxed.gpu.global.v4.u64 {%0, %1, %2, %3}, [%4];"
               : "=l"(v[0]), "=l"(v[1]), "=l"(v[2]), "=l"(v[3])
               : "l"(p)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
// 16 bytes global -> shared through L2 (cp.async.cg), completed by
// cp_async_wait_all; no register holds the data in between.
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
  const unsigned int d = (unsigned int)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gmem_src) : "memory");
}

// Values and keys as one (FP32) or two (FP64) tagged words.  The header of
// a CTA's slot holds its candidate's key with the pivot's sign in the top
// bit (so the key word also gives the pivot value), the row id, and the
// candidate's column j+1 value: words [0, 4 * kHdrQuads), whole 32-byte
// sectors of the slot (slots are 32-byte aligned).
template <typename T>
struct Tagged;
template <>
struct Tagged<float> {
  using K = unsigned int;
  static constexpr int kWords = 1;
  static constexpr int kIdW = 1, kU1W = 2, kHdrQuads = 1;
  static constexpr K kSign = 0x80000000u;
  __device__ static void put(unsigned long long* p, float v, unsigned int tag) { st_word(p, __float_as_uint(v), tag); }
  __device__ static void put_key(unsigned long long* p, K k, unsigned int tag) { st_word(p, k, tag); }
  __device__ static K bits(const unsigned long long* w) { return (unsigned int)w[0]; }
  __device__ static float value(const unsigned long long* w) { return __uint_as_float((unsigned int)w[0]); }
  __device__ static bool ok(const unsigned long long* w, unsigned int tag) { return word_ok(w[0], tag); }
};
template <>
struct Tagged<double> {
  using K = unsigned long long;
  static constexpr int kWords = 2;
  static constexpr int kIdW = 2, kU1W = 3, kHdrQuads = 2;
  static constexpr K kSign = 0x8000000000000000ull;
  __device__ static void put_key(unsigned long long* p, K k, unsigned int tag) {
    st_word(p, (unsigned int)(k >> 32), tag);
    st_word(p + 1, (unsigned int)k, tag);
  }
  __device__ static void put(unsigned long long* p, double v, unsigned int tag) {
    put_key(p, (unsigned long long)__double_as_longlong(v), tag);
  }
  __device__ static K bits(const unsigned long long* w) {
    return ((unsigned long long)(unsigned int)w[0] << 32) | (unsigned int)w[1];
  }
  __device__ static double value(const unsigned long long* w) { return __longlong_as_double((long long)bits(w)); }
  __device__ static bool ok(const unsigned long long* w, unsigned int tag) {
    return word_ok(w[0], tag) && word_ok(w[1], tag);
  }
};

// Give up a wait: record the step, raise abort so every other wait of the
// launch returns at once.  Called by one lane.
__device__ __forceinline__ void panel_give_up(DeviceStatus* st, int step) {
  atomicCAS(&st->error, kDevOk, kDevBarrierTimeout);
  atomicExch(&st->timeout_where, (unsigned long long)step);
  atomicExch(&st->abort, 1);
}
// Warp-uniform test of the wait limit and of another CTA's abort.
__device__ __forceinline__ bool panel_wait_over(DeviceStatus* st, unsigned long long t0) {
  const int late = (global_timer_ns() - t0 > st->timeout_ns) ? 1 : 0;
  return __shfl_sync(0xffffffffu, late, 0) != 0 || __any_sync(0xffffffffu, ld_relaxed_i32(&st->abort) != 0);
}

// FP32 rows in 16-byte chunks: lane (sub, ch) of a warp takes columns
// [4ch, 4ch+4) of row sub of the warp's current row group (W/4 chunks a row,
// 32/(W/4) rows a warp instruction); two row groups per pass with all loads
// first.  Columns left of c0 in the first chunk keep their value (the same
// single update per element as the scalar form, so exact mode is unchanged);
// chunks at or beyond the padded width are not touched.  Needs rows and u
// 16-byte aligned (lds and the row base multiples of 4 floats).
template <int W, bool kExact>
__device__ __forceinline__ void panel_update_f32x4(float* S, int lds, int r0, int nloc, int skip, int jj, int c0,
                                                   int w, const float* u, int t, int nt) {
  constexpr int CH = W / 4, RPW = 32 / CH, kR = 2;
  const int lane = t & 31, wi = t >> 5, nw = nt >> 5;
  const int ch = lane % CH, sub = lane / CH;
  const int c = ch * 4;
  if (c + 4 <= c0 || c >= w || r0 >= nloc) return;
  const float4 uv = *reinterpret_cast<const float4*>(u + c);
  const int G = nw * RPW;
  for (int rb = r0 + wi * RPW + sub; rb < nloc; rb += kR * G) {
    float l[kR];
    float4 x[kR];
#pragma unroll
    for (int e = 0; e < kR; ++e) {
      const float* row = S + (rb + e * G < nloc ? rb + e * G : rb) * lds;
      l[e] = row[jj];
      x[e] = *reinterpret_cast<const float4*>(row + c);
    }
#pragma unroll
    for (int e = 0; e < kR; ++e) {
      const int r = rb + e * G;
      if (r < nloc && r != skip) {
        float4 y = x[e];
        if (c + 0 >= c0) y.x = upd<kExact>(y.x, l[e], uv.x);
        if (c + 1 >= c0) y.y = upd<kExact>(y.y, l[e], uv.y);
        if (c + 2 >= c0) y.z = upd<kExact>(y.z, l[e], uv.z);
        if (c + 3 >= c0) y.w = upd<kExact>(y.w, l[e], uv.w);
        *reinterpret_cast<float4*>(S + r * lds + c) = y;
      }
    }
  }
}
// A[r][c] -= A[r][jj] * u[c] for the rows [r0, nloc) other than `skip` and
// the columns [c0, w), by threads t of nt (a multiple of 32).  FP64 flattens
// (row, column) pairs so every lane is busy (the FP64 pipe bounds it); FP32
// gives each warp whole rows, lanes along the columns (no index arithmetic
// per element; shared-memory latency bounds it, hence the batched loads).
template <typename T, bool kExact>
__device__ __forceinline__ void panel_update(T* S, int lds, int r0, int nloc, int skip, int jj, int c0, int w,
                                             const T* u, int t, int nt) {
  const int wc = w - c0;
  if (wc <= 0 || r0 >= nloc) return;
  if constexpr (sizeof(T) == 8) {
    const int total = (nloc - r0) * wc;
    const int step_r = nt / wc, step_c = nt - step_r * wc;
    int r = r0 + t / wc, c = t - (t / wc) * wc;
    for (int idx = t; idx < total; idx += 2 * nt) {
      const int ra = r, ca = c;
      r += step_r;
      c += step_c;
      if (c >= wc) {
        c -= wc;
        ++r;
      }
      const int rb = r, cb = c;
      const bool on_b = idx + nt < total;
      r += step_r;
      c += step_c;
      if (c >= wc) {
        c -= wc;
        ++r;
      }
      T xa = T(0), la = T(0), ua = T(0), xb = T(0), lb = T(0), ub = T(0);
      const bool do_a = ra != skip, do_b = on_b && rb != skip;
      if (do_a) {
        xa = S[ra * lds + c0 + ca];
        la = S[ra * lds + jj];
        ua = u[c0 + ca];
      }
      if (do_b) {
        xb = S[rb * lds + c0 + cb];
        lb = S[rb * lds + jj];
        ub = u[c0 + cb];
      }
      if (do_a) S[ra * lds + c0 + ca] = upd<kExact>(xa, la, ua);
      if (do_b) S[rb * lds + c0 + cb] = upd<kExact>(xb, lb, ub);
    }
  } else {
    if (w <= 64)
      panel_update_f32x4<64, kExact>(S, lds, r0, nloc, skip, jj, c0, w, u, t, nt);
    else
      panel_update_f32x4<128, kExact>(S, lds, r0, nloc, skip, jj, c0, w, u, t, nt);
  }
}

// Cooperative panel factorization: rows [k0, m) x columns [k0, k0 + w) are
// spread over P CTAs (rows_per each) and held in shared memory for the whole
// panel.  Rows are never moved between CTAs during the panel: each CTA keeps
// the global row index (id) of every row it holds, and an interchange of rows
// ul and pr only swaps two ids.  The row that receives id ul is the pivot
// row; its CTA moves it into its block of retired rows [0, r0) (a local move).
// At the end every row is written to the global row its id names.
//
// Per column j (elimination step ul = k0 + j), with the update of step j-1
// to columns j+1.. still pending for all rows but this CTA's candidate row:
//   warp 0:     publish the candidate's header (key = |pivot| bits with the
//               pivot's sign on top, row id, column j+1 value after the
//               pending update) as tagged words; poll the P headers until all
//               carry this step's tag, folding them into the winner (the
//               pivot and its column j+1 value come with its header); start
//               the copy of the winner's segment into shared memory
//               (cp.async); relabel the ids of rows ul and pr.
//   warp 1:     meanwhile, the candidate row's pending update (columns
//               j+2..) and the publication of its segment j+2..;
//   warps 1-:   the pending update of step j-1 of the other rows (columns
//               j+1..), which thus overlaps the exchange.
//   barrier;    the pivot row's CTA retires it; warps 1- scale column j,
//               update column j+1 only and find its candidates while warp 0
//               checks the copied segment's tags and keeps it for the next
//               step's updates; barrier.
// The arithmetic and its order per element are those of lair's
// getrf_row_major (src/lapack/getrf.rs:56-89): 1/p rounded, l = a*(1/p)
// rounded, a - l*u (separately rounded in exact mode), steps in order.
template <typename T, bool kExact>
__global__ void __launch_bounds__(512, 1) panel_kernel(PanelArgs<T> p) {
  using K = typename PivotKey<T>::K;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* S = reinterpret_cast<T*>(smem_raw);                        // [rows_per][lds]
  T* segb = S + (size_t)p.rows_per * p.lds;                     // [2][kMaxPanelWidth] pivot rows
  int* ids = reinterpret_cast<int*>(segb + 2 * kMaxPanelWidth);  // [rows_per] global row of each slot
  int* orig = ids + p.rows_per;  // [rows_per] the row each slot's content started in
  __shared__ K red_k[16];
  __shared__ int red_i[16], red_s[16];
  __shared__ int ulslot[kMaxPanelWidth];  // slot holding row id k0 + jj in this CTA, or -1
  __shared__ __align__(16) unsigned long long stage[2 * kMaxPanelWidth];  // the winner's segment words
  __shared__ int s_ok, s_r0, s_pivoted, s_ret;
  __shared__ T s_recip, s_u1;

  constexpr unsigned kFull = 0xffffffffu;
  const int kWarps = blockDim.x >> 5;  // 8 or 16
  constexpr int kW = Tagged<T>::kWords;
  constexpr int kHdr = kPanelHeaderWords;
  const int P = gridDim.x;
  const int b = blockIdx.x;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int r_begin = p.k0 + b * p.rows_per;
  const int nloc = max(0, min(p.m, r_begin + p.rows_per) - r_begin);
  const int w = p.w;
  const int lds = p.lds;

  for (int idx = tid; idx < nloc * w; idx += blockDim.x) {
    const int r = idx / w, c = idx - r * w;
    S[r * lds + c] = p.a[(int64_t)(r_begin + r) * p.lda + p.k0 + c];
  }
  for (int r = tid; r < nloc; r += blockDim.x) ids[r] = orig[r] = r_begin + r;
  for (int jj = tid; jj < w; jj += blockDim.x) {
    const int s = p.k0 + jj - r_begin;
    ulslot[jj] = (s >= 0 && s < nloc) ? s : -1;
  }
  if (tid == 0) {
    s_r0 = 0;
    s_ok = 1;
  }
  __syncthreads();
  {
    // Column 0 candidates.
    K bk = 0;
    int bi = INT_MAX, bs = -1;
    for (int r = tid; r < nloc; r += blockDim.x) key_combine(bk, bi, bs, PivotKey<T>::of(S[r * lds]), ids[r], r);
    key_reduce_redux(bk, bi, bs);
    if (lane == 0) {
      red_k[warp] = bk;
      red_i[warp] = bi;
      red_s[warp] = bs;
    }
  }
  __syncthreads();

  const int nq = (P + 31) / 32;  // candidate CTAs per lane in the poll
  int dj = -1;                   // step whose update of columns dj+2.. is pending
  int dr0 = 0;                   // first active row of that step
  for (int j = 0; j < w; ++j) {
    const int ul = p.k0 + j;
    const unsigned int tag = (unsigned int)ul + 1u;
    unsigned long long* slots = p.slots + (size_t)(j & 1) * kMaxPanelCtas * kPanelSlotWords;
    T* seg = segb + (j & 1) * kMaxPanelWidth;
    // The CTA's candidate for column j (lanes below kWarps hold the warps').
    K ck = lane < kWarps ? red_k[lane] : K(0);
    int ci = lane < kWarps ? red_i[lane] : INT_MAX;
    int cs = lane < kWarps ? red_s[lane] : -1;
    key_reduce_redux(ck, ci, cs);
    bool seg_live = false;  // the winner's segment j+2.. is being copied into stage
    const unsigned long long* wseg = nullptr;
    unsigned long long t0 = 0;
    if (warp == 0) {
      unsigned long long* mine = slots + (size_t)b * kPanelSlotWords;
      const T* up = segb + (dj & 1) * kMaxPanelWidth;  // step dj's pivot row
      // The header only (warp 1 publishes the segment): the column j+1 value
      // after the pending update (kept in the row), the row id, then the key
      // with the pivot's sign.
      if (lane == 0) {
        K sgn = 0;
        if (cs >= 0) {
          if (j + 1 < w) {
            T u1 = S[cs * lds + j + 1];
            if (dj >= 0) {
              u1 = upd<kExact>(u1, S[cs * lds + dj], up[j + 1]);
              S[cs * lds + j + 1] = u1;
            }
            Tagged<T>::put(mine + Tagged<T>::kU1W, u1, tag);
          }
          if (signbit(S[cs * lds + j])) sgn = Tagged<T>::kSign;
        }
        st_word(mine + Tagged<T>::kIdW, (unsigned int)ci, tag);
        Tagged<T>::put_key(mine, ck | sgn, tag);
      }
      // Poll every CTA's header (32-byte loads); fold each one in as soon as
      // it is current.  A positive key comes with its column j+1 value.
      K k = 0, kraw = 0;
      int i = INT_MAX, win = -1;
      T u1b = T(0);
      unsigned pending = 0;
      for (int q = 0; q < nq; ++q)
        if (lane + 32 * q < P) pending |= 1u << q;
      t0 = global_timer_ns();
      unsigned int spins = 0;
      int ok = 1;
      while (true) {
        for (int q = 0; q < nq; ++q) {
          if (!(pending & (1u << q))) continue;
          const int cta = lane + 32 * q;
          const unsigned long long* h = slots + (size_t)cta * kPanelSlotWords;
          unsigned long long hw[4 * Tagged<T>::kHdrQuads];
#pragma unroll
          for (int v = 0; v < Tagged<T>::kHdrQuads; ++v) ld_quad(h + 4 * v, hw + 4 * v);
          const K hraw = Tagged<T>::bits(hw);
          const K hk = hraw & ~Tagged<T>::kSign;
          if (Tagged<T>::ok(hw, tag) && word_ok(hw[Tagged<T>::kIdW], tag) &&
              (hk == 0 || j + 1 >= w || Tagged<T>::ok(hw + Tagged<T>::kU1W, tag))) {
            const int hid = (int)(unsigned int)hw[Tagged<T>::kIdW];
            if (hk > k || (hk == k && hid < i)) {
              k = hk;
              i = hid;
              win = cta;
              kraw = hraw;
              u1b = Tagged<T>::value(hw + Tagged<T>::kU1W);
            }
            pending &= ~(1u << q);
          }
        }
        if (__all_sync(kFull, pending == 0)) break;
        if ((++spins & 15u) == 0 && panel_wait_over(p.st, t0)) {
          if (lane == 0 && !ld_relaxed_i32(&p.st->abort)) panel_give_up(p.st, ul);
          ok = 0;
          break;
        }
      }
      int ret = -1;
      if (ok) {
        const int src = key_reduce_redux(k, i, win);
        const K praw = PivotKey<T>::shfl(kraw, src);
        const T u1 = __shfl_sync(kFull, u1b, src);
        const int pr = (k > 0) ? i : ul;
        if (k > 0) {
          // Start the copy of the winner's segment j+2.. (whole 16-byte
          // pairs of its slot's words) into stage; it completes while the
          // step goes on.
          wseg = slots + (size_t)win * kPanelSlotWords + kHdr;
          const int o0 = ((j + 2) * kW) & ~1, o1 = (w * kW + 1) & ~1;
          seg_live = o1 > o0;
          for (int o = o0 + 2 * lane; o < o1; o += 64) cp_async16(stage + o, wseg + o);
          cp_async_commit();
          if (lane == 0) {
            s_recip = T(1) / PivotKey<T>::value(praw);
            s_u1 = u1;
          }
        } else if (b == 0 && lane == 0) {
          // lair: max == 0 -> the step is singular, no swap, no update
          // (src/lapack/getrf.rs:72-73).  The last such step wins.
          atomicMax(&p.st->singular, ul);
        }
        // Relabel: the row with id ul takes id pr and the row with id pr
        // takes id ul; the latter (the pivot row) retires after the barrier.
        // Row pr is the winning CTA's candidate (slot cs); row ul's slot
        // comes from the map of the panel's pending row ids.
        const int s_ul = ulslot[j];
        ret = s_ul;
        if (pr != ul) {
          const int s_pr = (win == b) ? cs : -1;
          if (lane == 0) {
            if (s_ul >= 0) ids[s_ul] = pr;
            if (s_pr >= 0) ids[s_pr] = ul;
            if (pr < p.k0 + w) ulslot[pr - p.k0] = s_ul;
          }
          ret = s_pr;
        }
        if (b == 0 && lane == 0) p.piv[ul] = pr;
        if (lane == 0) s_pivoted = k > 0 ? 1 : 0;
      }
      if (lane == 0) {
        s_ok = ok;
        s_ret = ret;
      }
    } else {
      if (warp == 1 && cs >= 0) {
        // The candidate row's pending update of columns j+2.. (warp 0 did
        // column j+1), then its segment j+2.., while warp 0 polls.
        unsigned long long* mine = slots + (size_t)b * kPanelSlotWords;
        if (dj >= 0) {
          const T* up = segb + (dj & 1) * kMaxPanelWidth;
          const T l = S[cs * lds + dj];
          for (int c = dj + 3 + lane; c < w; c += 32) S[cs * lds + c] = upd<kExact>(S[cs * lds + c], l, up[c]);
          __syncwarp();
        }
        for (int c = j + 2 + lane; c < w; c += 32) Tagged<T>::put(mine + kHdr + c * kW, S[cs * lds + c], tag);
      }
      if (dj >= 0)
        panel_update<T, kExact>(S, lds, dr0, nloc, cs, dj, dj + 2, w, segb + (dj & 1) * kMaxPanelWidth, tid - 32,
                                blockDim.x - 32);
    }
    __syncthreads();
    if (!s_ok) return;
    // Retire the pivot row into slot r0.
    int r0 = s_r0;
    const int ret = s_ret;
    if (ret >= 0) {
      if (warp == 0 && ret != r0) {
        for (int c = lane; c < w; c += 32) {
          const T x = S[ret * lds + c];
          S[ret * lds + c] = S[r0 * lds + c];
          S[r0 * lds + c] = x;
        }
        if (lane == 0) {
          const int t = ids[ret];
          const int moved = ids[r0];  // this row now lives in slot ret
          if (moved > ul && moved < p.k0 + w) ulslot[moved - p.k0] = ret;
          ids[ret] = moved;
          ids[r0] = t;
          const int o = orig[ret];
          orig[ret] = orig[r0];
          orig[r0] = o;
        }
      }
      ++r0;
      __syncthreads();
      if (tid == 0) s_r0 = r0;
    }

    // Warps 1-: scale column j, update column j+1 only, find its candidates.
    // Warp 0 meanwhile keeps the winner's segment for the next step.
    K bk = 0;
    int bi = INT_MAX, bs = -1;
    const int pivoted = s_pivoted;
    if (warp != 0) {
      const int t1 = tid - 32, n1 = blockDim.x - 32;
      if (pivoted) {
        const T recip = s_recip;
        for (int r = r0 + t1; r < nloc; r += n1) S[r * lds + j] = mul_rn(S[r * lds + j], recip);
        if (j + 1 < w) {
          const T u1 = s_u1;
          for (int r = r0 + t1; r < nloc; r += n1) {
            const T v = upd<kExact>(S[r * lds + j + 1], S[r * lds + j], u1);
            S[r * lds + j + 1] = v;
            key_combine(bk, bi, bs, PivotKey<T>::of(v), ids[r], r);
          }
        }
      } else if (j + 1 < w) {
        for (int r = r0 + t1; r < nloc; r += n1)
          key_combine(bk, bi, bs, PivotKey<T>::of(S[r * lds + j + 1]), ids[r], r);
      }
      key_reduce_redux(bk, bi, bs);
    } else if (seg_live) {
      // The winner's segment from stage into the pivot-row buffer; a word
      // whose tag is not yet this step's (relaxed stores land in any order)
      // is read again.
      cp_async_wait_all();
      __syncwarp();
      bool got = true;
      while (got) {
        for (int c = j + 2 + lane; c < w; c += 32) {
          unsigned long long* sw = stage + c * kW;
          if (Tagged<T>::ok(sw, tag)) {
            seg[c] = Tagged<T>::value(sw);
          } else {
#pragma unroll
            for (int e = 0; e < kW; ++e) sw[e] = ld_word(wseg + c * kW + e);
            got = false;
          }
        }
        if (__all_sync(kFull, got)) break;
        got = true;
        if (panel_wait_over(p.st, t0)) got = false;
      }
      if (!got && lane == 0) {
        if (!ld_relaxed_i32(&p.st->abort)) panel_give_up(p.st, ul);
        s_ok = 0;
      }
    }
    if (lane == 0) {
      red_k[warp] = bk;
      red_i[warp] = bi;
      red_s[warp] = bs;
    }
    dj = pivoted ? j : -1;
    dr0 = r0;
    __syncthreads();
    if (!s_ok) return;
  }
  for (int idx = tid; idx < nloc * w; idx += blockDim.x) {
    const int r = idx / w, c = idx - r * w;
    p.a[(int64_t)ids[r] * p.lda + p.k0 + c] = S[r * lds + c];
  }
  // The rows that changed place, for the interchanges outside the panel.
  for (int r = tid; r < nloc; r += blockDim.x) {
    if (ids[r] != orig[r]) {
      const int e = atomicAdd(p.move_count, 1);
      if (e < 2 * kMaxPanelWidth) {  // at most 2w rows move; the bound guards the list
        p.moves[2 * e] = ids[r];
        p.moves[2 * e + 1] = orig[r];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// 2. Row interchanges outside the panel, from the panel's list of moved rows
//    (the composition of its w interchanges: at most 2w rows, each row's
//    final content comes from one source row).  A CTA takes 32 columns: it
//    loads every moved row's source values into shared memory, then stores
//    them at the destinations -- all loads independent, 256-byte row
//    segments.  Pure data movement, so exact mode is unaffected.
template <typename T>
__global__ void __launch_bounds__(256) laswp_moves_kernel(T* a, int64_t lda, const int* moves,
                                                          const int* move_count, int capacity, int c_left_begin,
                                                          int c_left_end, int c_right_begin, int n) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* vals = reinterpret_cast<T*>(smem_raw);  // [capacity][32]
  __shared__ int mv[4 * kMaxPanelWidth];      // the (destination, source) pairs
  const int count = min(min(*move_count, capacity), 2 * kMaxPanelWidth);
  const int tid = threadIdx.y * 32 + threadIdx.x;
  for (int i = tid; i < 2 * count; i += blockDim.x * blockDim.y) mv[i] = moves[i];
  __syncthreads();
  const int nleft = max(0, c_left_end - c_left_begin);
  const int t = blockIdx.x * 32 + threadIdx.x;
  const int nright = max(0, n - c_right_begin);
  const bool on = t < nleft + nright;
  const int c = (t < nleft) ? (c_left_begin + t) : (c_right_begin + t - nleft);
  // Eight source rows per thread in flight before any is stored.
  constexpr int kB = 8;
  for (int e0 = threadIdx.y; e0 < count; e0 += blockDim.y * kB) {
    T v[kB];
#pragma unroll
    for (int q = 0; q < kB; ++q) {
      const int e = e0 + q * blockDim.y;
      v[q] = (on && e < count) ? a[(int64_t)mv[2 * e + 1] * lda + c] : T(0);
    }
#pragma unroll
    for (int q = 0; q < kB; ++q) {
      const int e = e0 + q * blockDim.y;
      if (on && e < count) vals[e * 32 + threadIdx.x] = v[q];
    }
  }
  __syncthreads();
  for (int e = threadIdx.y; e < count; e += blockDim.y)
    if (on) a[(int64_t)mv[2 * e] * lda + c] = vals[e * 32 + threadIdx.x];
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

// Fast-mode U12 solve, left-looking in blocks of 16 rows: one thread per
// column; for rows i0..i0+15 it accumulates x_i = b_i - sum_{k<i0} l_ik x_k
// in 16 registers (16 independent FMA chains per loaded x_k, the l_ik
// broadcast from shared memory with L11 stored transposed), then solves the
// 16 x 16 diagonal block.  x lives in shared memory (one column per thread,
// conflict-free).  W = 64 or 128 >= w; L11 is zero-padded to W x W.  The
// CTA's 256 threads stage L11 and the 64 columns of A12 together (the
// loads, not the solve, were most of the time with 64 threads); the first
// 64 then solve and all of them write the rows back.  The exact mode keeps
// trsm_kernel's order.
constexpr int kTrsmFastThreads = 256;

template <typename T, int W>
__global__ void __launch_bounds__(kTrsmFastThreads) trsm_fast_kernel(T* a, int64_t lda, int k0, int w, int c0,
                                                                      int n) {
  constexpr int RB = 16;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* Lt = reinterpret_cast<T*>(smem_raw);  // [W][W]: Lt[k][i] = L11[i][k] for i > k, else 0
  T* X = Lt + W * W;                       // [W][kTrsmCols]
  const int tid = threadIdx.x;
  const int cb = c0 + blockIdx.x * kTrsmCols;
  for (int idx = tid; idx < W * W; idx += blockDim.x) {
    const int k = idx / W, i = idx - k * W;
    Lt[idx] = (i > k && i < w && k < w) ? a[(int64_t)(k0 + i) * lda + k0 + k] : T(0);
  }
  for (int idx = tid; idx < W * kTrsmCols; idx += blockDim.x) {
    const int i = idx / kTrsmCols, cc = idx - i * kTrsmCols;
    X[idx] = (cb + cc < n && i < w) ? a[(int64_t)(k0 + i) * lda + cb + cc] : T(0);
  }
  __syncthreads();
  if (tid < kTrsmCols) {
    for (int i0 = 0; i0 < w; i0 += RB) {
      T acc[RB];
#pragma unroll
      for (int r = 0; r < RB; ++r) acc[r] = X[(i0 + r) * kTrsmCols + tid];
      for (int k = 0; k < i0; ++k) {
        const T xk = X[k * kTrsmCols + tid];
        const T* lk = Lt + k * W + i0;
#pragma unroll
        for (int r = 0; r < RB; ++r) acc[r] = fma(-lk[r], xk, acc[r]);
      }
#pragma unroll
      for (int kk = 0; kk < RB - 1; ++kk) {
        const T* lk = Lt + (i0 + kk) * W + i0;
#pragma unroll
        for (int r = 0; r < RB; ++r)
          if (r > kk) acc[r] = fma(-lk[r], acc[kk], acc[r]);
      }
#pragma unroll
      for (int r = 0; r < RB; ++r) X[(i0 + r) * kTrsmCols + tid] = acc[r];
    }
  }
  __syncthreads();
  for (int idx = kTrsmCols + tid; idx < w * kTrsmCols; idx += blockDim.x) {
    const int i = idx / kTrsmCols, cc = idx - i * kTrsmCols;
    if (cb + cc < n) a[(int64_t)(k0 + i) * lda + cb + cc] = X[idx];
  }
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

// Persistent form of the same update for aligned operands: one CTA per SM
// walks a contiguous range of 128 x 128 tiles in row-block order, so the
// L21 block (A) changes only when the range crosses a row block.  The next
// tile's U12 block (B) is copied into a second buffer by cp.async while the
// current tile runs on the FP64 pipe, and the C tile is prefetched into L2
// before its read-modify-write.  The FP64 pipe therefore stays busy across
// tile boundaries instead of idling through each tile's loads and stores.
// Needs 16-byte aligned rows and panel columns (even lda, kk0 and c0 and a
// 16-byte aligned base); the launcher falls back to gemm_dmma_kernel.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, int src_bytes) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes) : "memory");
}

__global__ void __launch_bounds__(256, 1) gemm_dmma_persistent_kernel(double* a, int64_t lda, int r0, int c0,
                                                                      int kk0, int K, int M, int N) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int Kpad = (K + 15) & ~15;
  const int Kp = Kpad + 4;
  const int ldb = kDmmaBN + 4;
  double* As = reinterpret_cast<double*>(smem_raw);  // [128][Kp]
  double* Bs0 = As + kDmmaBM * Kp;                   // [2][Kpad][ldb]
  const int tiles_n = (N + kDmmaBN - 1) / kDmmaBN;
  const int tiles = ((M + kDmmaBM - 1) / kDmmaBM) * tiles_n;
  const int G = gridDim.x;
  const int t_begin = (int)((int64_t)blockIdx.x * tiles / G);
  const int t_end = (int)((int64_t)(blockIdx.x + 1) * tiles / G);
  if (t_begin >= t_end) return;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int wr = (warp >> 1) * 32, wc = (warp & 1) * 64;
  const int g = lane >> 2, t4 = lane & 3;
  const int kchunks = Kpad / 2;  // 16-byte chunks per A row

  auto load_a = [&](int tm) {
    const int tile_r = r0 + tm * kDmmaBM;
    for (int idx = tid; idx < kDmmaBM * kchunks; idx += 256) {
      const int i = idx / kchunks, k = (idx - i * kchunks) * 2;
      const int r = tile_r + i;
      const int valid = (r < r0 + M) ? max(0, min(2, K - k)) : 0;
      const double* src = valid ? a + (int64_t)r * lda + kk0 + k : a;
      cp_async16(As + i * Kp + k, src, valid * 8);
    }
  };
  auto load_b = [&](int tn, double* Bs) {
    const int tile_c = c0 + tn * kDmmaBN;
    for (int idx = tid; idx < Kpad * (kDmmaBN / 2); idx += 256) {
      const int k = idx / (kDmmaBN / 2), j = (idx - k * (kDmmaBN / 2)) * 2;
      const int c = tile_c + j;
      const int valid = (k < K) ? max(0, min(2, c0 + N - c)) : 0;
      const double* src = valid ? a + (int64_t)(kk0 + k) * lda + c : a;
      cp_async16(Bs + k * ldb + j, src, valid * 8);
    }
  };

  int tm = t_begin / tiles_n, tn = t_begin - tm * tiles_n;
  load_a(tm);
  load_b(tn, Bs0);
  cp_async_commit();
  for (int t = t_begin; t < t_end; ++t) {
    double* Bs = Bs0 + (size_t)((t - t_begin) & 1) * Kpad * ldb;
    cp_async_wait_all();
    __syncthreads();
    const int tile_r = r0 + tm * kDmmaBM, tile_c = c0 + tn * kDmmaBN;
    // Next tile: its B block now (other buffer, last read two tiles ago).
    int tm_n = tm, tn_n = tn + 1;
    if (tn_n == tiles_n) {
      tn_n = 0;
      ++tm_n;
    }
    const bool more = t + 1 < t_end;
    if (more) {
      load_b(tn_n, Bs0 + (size_t)((t + 1 - t_begin) & 1) * Kpad * ldb);
      cp_async_commit();
    }
    // C tile into L2 ahead of its read-modify-write: 128 rows x 1 KB.
    for (int idx = tid; idx < kDmmaBM * 8; idx += 256) {
      const int i = idx >> 3, part = idx & 7;
      const int r = tile_r + i, c = tile_c + part * 16;
      if (r < r0 + M && c < c0 + N) asm volatile("prefetch.global.L2 [%0];" ::"l"(a + (int64_t)r * lda + c));
    }
    double acc[4][8][2];
#pragma unroll
    for (int mi = 0; mi < 4; ++mi)
#pragma unroll
      for (int ni = 0; ni < 8; ++ni) acc[mi][ni][0] = acc[mi][ni][1] = 0.0;
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
    if (more && tm_n != tm) {
      // The range crosses into the next row block: reload A once every warp
      // is done with it.
      __syncthreads();
      load_a(tm_n);
      cp_async_commit();
    }
#pragma unroll
    for (int mi = 0; mi < 4; ++mi) {
      const int r = tile_r + wr + mi * 8 + g;
      if (r >= r0 + M) continue;
#pragma unroll
      for (int ni = 0; ni < 8; ++ni) {
        const int c = tile_c + wc + ni * 8 + t4 * 2;
        double* dst = a + (int64_t)r * lda + c;
        if (c + 1 < c0 + N) {
          double2 v = *reinterpret_cast<double2*>(dst);
          v.x -= acc[mi][ni][0];
          v.y -= acc[mi][ni][1];
          *reinterpret_cast<double2*>(dst) = v;
        } else if (c < c0 + N) {
          dst[0] -= acc[mi][ni][0];
        }
      }
    }
    tm = tm_n;
    tn = tn_n;
  }
}

// ---------------------------------------------------------------------------
// Host driver.
// ---------------------------------------------------------------------------
// Shared-memory row stride of the panel: FP64 w + 1 (conflict-free column
// access); FP32 rows padded to a multiple of 4 floats plus 4, so every row
// starts on 16 bytes for the float4 look-ahead (column access then has
// 4-way bank conflicts, a small cost on two columns a step).
template <typename T>
static int panel_lds(int w) {
  return sizeof(T) == 4 ? ((w + 3) & ~3) + 4 : w + 1;
}
// Threads of a panel CTA: FP32 uses 16 warps so the look-ahead's shared-memory
// latency is hidden; FP64's look-ahead is bound by the FP64 pipe.
template <typename T>
static int panel_threads() {
  return sizeof(T) == 4 ? 512 : 256;
}
template <typename T>
static size_t panel_smem_bytes(int rows_per, int w) {
  return ((size_t)rows_per * panel_lds<T>(w) + 2 * kMaxPanelWidth) * sizeof(T) + 2 * (size_t)rows_per * sizeof(int);
}

template <typename T, bool kExact>
static int launch_panel(luhot_ctx* ctx, T* a, int64_t lda, int m, int k0, int w, int* piv,
                        cudaStream_t stream) {
  const int rows = m - k0;
  auto kern = panel_kernel<T, kExact>;
  cudaFuncAttributes fa;
  LUHOT_CUDA_TRY(ctx, cudaFuncGetAttributes(&fa, kern));
  const int max_smem = ctx->max_smem_optin - (int)fa.sharedSizeBytes;  // less the static exchange buffers
  // CTAs: FP32 panels (light update work) run fastest on 64 CTAs with >= 32
  // rows each; FP64 panels, whose look-ahead update needs FP64 pipes, on 96
  // CTAs with >= 64 rows each (measured at n = 16384 against 64 .. 152 CTAs:
  // fewer CTAs shorten the per-column exchange, more share the update).  The
  // count is raised, up to the SM count, when the rows of one CTA would not
  // fit in shared memory.
  const int pmax = std::min(ctx->num_sms, sizeof(T) == 4 ? 64 : 96);
  const int min_rows = sizeof(T) == 4 ? 32 : 64;
  int P = std::min(pmax, std::max(1, (rows + min_rows - 1) / min_rows));
  int rows_per = (rows + P - 1) / P;
  while (panel_smem_bytes<T>(rows_per, w) > (size_t)max_smem && P < ctx->num_sms) {
    P = std::min(ctx->num_sms, P * 2);
    rows_per = (rows + P - 1) / P;
  }
  if (panel_smem_bytes<T>(rows_per, w) > (size_t)max_smem)
    return set_error(ctx, LUHOT_ERR_UNSUPPORTED, "panel does not fit in shared memory");
  const size_t smem = panel_smem_bytes<T>(rows_per, w);
  LUHOT_CUDA_TRY(ctx, allow_max_dynamic_smem(kern));
  int per_sm = 0;
  LUHOT_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, panel_threads<T>(), smem));
  if (per_sm * ctx->num_sms < P)
    return set_error(ctx, LUHOT_ERR_UNSUPPORTED, "panel grid cannot be co-resident");
  PanelArgs<T> args;
  args.a = a;
  args.lda = lda;
  args.m = m;
  args.k0 = k0;
  args.w = w;
  args.rows_per = rows_per;
  args.lds = panel_lds<T>(w);
  args.piv = piv;
  args.slots = static_cast<unsigned long long*>(ctx->panel_scratch);
  args.moves = reinterpret_cast<int*>(static_cast<char*>(ctx->panel_scratch) + kPanelSlotBytes);
  args.move_count = args.moves + 4 * kMaxPanelWidth;
  args.st = ctx->d_status;
  LUHOT_CUDA_TRY(ctx, cudaMemsetAsync(args.move_count, 0, sizeof(int), stream));
  void* kargs[] = {&args};
  prof_begin(ctx, kProfPanel);
  LUHOT_CUDA_TRY(ctx, cudaLaunchCooperativeKernel((void*)kern, dim3(P), dim3(panel_threads<T>()), kargs, smem,
                                                  stream));
  // panel flops: sum over steps of (rows below) * (1 + 2 * cols right)
  double fl = 0.0;
  for (int j = 0; j < w; ++j) fl += (double)(rows - j - 1) * (1.0 + 2.0 * (w - j - 1));
  prof_end(ctx, kProfPanel, fl, 2.0 * rows * w * sizeof(T));
  return LUHOT_OK;
}

template <typename T, bool kExact>
static int launch_gemm(luhot_ctx* ctx, T* a, int64_t lda, int r0, int c0, int kk0, int K, int M,
                       int N, cudaStream_t stream) {
  if (M <= 0 || N <= 0 || K <= 0) return LUHOT_OK;
  if constexpr (std::is_same<T, double>::value && !kExact) {
    const int Kpad = (K + 15) & ~15;
    const size_t smem = ((size_t)kDmmaBM * (Kpad + 4) + (size_t)Kpad * (kDmmaBN + 4)) * sizeof(double);
    const size_t smem_p = smem + (size_t)Kpad * (kDmmaBN + 4) * sizeof(double);
    const int tiles = ((N + kDmmaBN - 1) / kDmmaBN) * ((M + kDmmaBM - 1) / kDmmaBM);
    const bool aligned = (lda % 2 == 0) && (kk0 % 2 == 0) && (c0 % 2 == 0) &&
                         (reinterpret_cast<uintptr_t>(a) % 16 == 0);
    if (aligned && smem_p <= (size_t)ctx->max_smem_optin) {
      LUHOT_CUDA_TRY(ctx, allow_max_dynamic_smem(gemm_dmma_persistent_kernel));
      prof_begin(ctx, kProfGemm);
      gemm_dmma_persistent_kernel<<<std::min(tiles, ctx->num_sms), 256, smem_p, stream>>>(a, lda, r0, c0, kk0, K,
                                                                                          M, N);
    } else {
      LUHOT_CUDA_TRY(ctx, allow_max_dynamic_smem(gemm_dmma_kernel));
      dim3 grid((N + kDmmaBN - 1) / kDmmaBN, (M + kDmmaBM - 1) / kDmmaBM);
      prof_begin(ctx, kProfGemm);
      gemm_dmma_kernel<<<grid, 256, smem, stream>>>(a, lda, r0, c0, kk0, K, M, N);
    }
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

// Row interchanges of a panel of width w, from the list of moved rows it
// reported (`moves`: kPanelMovesBytes, the layout of the panel scratch), on
// the columns [cl0, cl1) and [cr0, cr1).
template <typename T>
static int launch_laswp_cols(luhot_ctx* ctx, T* a, int64_t lda, const int* moves, int w, int cl0, int cl1, int cr0,
                             int cr1, cudaStream_t stream) {
  const int ncols_swap = std::max(0, cl1 - cl0) + std::max(0, cr1 - cr0);
  if (ncols_swap <= 0) return LUHOT_OK;
  prof_begin(ctx, kProfLaswp);
  const size_t lsm = (size_t)2 * w * 32 * sizeof(T);
  LUHOT_CUDA_TRY(ctx, allow_max_dynamic_smem(laswp_moves_kernel<T>));
  laswp_moves_kernel<T><<<(ncols_swap + 31) / 32, dim3(32, 8), lsm, stream>>>(
      a, lda, moves, moves + 4 * kMaxPanelWidth, 2 * w, cl0, std::max(cl0, cl1), cr0, std::max(cr0, cr1));
  prof_end(ctx, kProfLaswp, 0.0, 4.0 * w * ncols_swap * sizeof(T));
  LUHOT_CUDA_TRY(ctx, cudaGetLastError());
  return LUHOT_OK;
}

// Row interchanges of the panel [k0, k0 + w) (the moves it reported) on every
// column outside the panel: [0, k0) and [k0 + w, n).
template <typename T>
static int launch_laswp(luhot_ctx* ctx, T* a, int64_t lda, int k0, int w, int n, cudaStream_t stream) {
  const int* moves = reinterpret_cast<const int*>(static_cast<char*>(ctx->panel_scratch) + kPanelSlotBytes);
  return launch_laswp_cols<T>(ctx, a, lda, moves, w, 0, k0, k0 + w, n, stream);
}

// The tensor-core engine takes the U12 solve of fast-mode FP64 as well
// (ozaki_trsm: U12 = A12 - (I - L11^-1) A12) for at least 256 columns (128
// with LUHOT_UPDATE_OZAKI), when the trailing update runs on it.
static bool trsm_on_slices(const void* oz_ws, int engine, int ncols) {
  if (!oz_ws || engine == LUHOT_UPDATE_DMMA) return false;
  return ncols >= (engine == LUHOT_UPDATE_OZAKI ? 128 : 256);
}

// U12 = L11^-1 A12 for the panel [k0, k0 + w): rows [k0, k0 + w) of the
// columns [c_begin, c_end).
template <typename T, bool kExact>
static int launch_trsm(luhot_ctx* ctx, T* a, int64_t lda, int k0, int w, int c_begin, int c_end,
                       cudaStream_t stream, void* oz_ws = nullptr, int engine = LUHOT_UPDATE_DMMA) {
  if (c_begin >= c_end) return LUHOT_OK;
  const int tgrid = (c_end - c_begin + kTrsmCols - 1) / kTrsmCols;
  prof_begin(ctx, kProfTrsm);
  if constexpr (std::is_same<T, double>::value && !kExact) {
    if (w <= 64 && trsm_on_slices(oz_ws, engine, c_end - c_begin)) {
      const int rc = ozaki_trsm(ctx, a, lda, k0, w, c_begin, c_end, oz_ws, stream);
      prof_end(ctx, kProfTrsm, (double)w * (w - 1) * (c_end - c_begin),
               ((double)w * w + 2.0 * w * (c_end - c_begin)) * sizeof(T));
      return rc;
    }
  }
  if (!kExact && w <= 64) {
    const size_t smem = ((size_t)64 * 64 + (size_t)64 * kTrsmCols) * sizeof(T);
    LUHOT_CUDA_TRY(ctx, allow_max_dynamic_smem(trsm_fast_kernel<T, 64>));
    trsm_fast_kernel<T, 64><<<tgrid, kTrsmFastThreads, smem, stream>>>(a, lda, k0, w, c_begin, c_end);
  } else if (!kExact && std::is_same<T, float>::value && w <= 128) {
    if constexpr (std::is_same<T, float>::value) {
      const size_t smem = ((size_t)128 * 128 + (size_t)128 * kTrsmCols) * sizeof(T);
      LUHOT_CUDA_TRY(ctx, allow_max_dynamic_smem(trsm_fast_kernel<T, 128>));
      trsm_fast_kernel<T, 128><<<tgrid, kTrsmFastThreads, smem, stream>>>(a, lda, k0, w, c_begin, c_end);
    }
  } else {
    const size_t smem = ((size_t)w * w + (size_t)w * kTrsmCols) * sizeof(T);
    auto kern = trsm_kernel<T, kExact>;
    LUHOT_CUDA_TRY(ctx, allow_max_dynamic_smem(kern));
    kern<<<tgrid, kTrsmCols, smem, stream>>>(a, lda, k0, w, c_begin, c_end);
  }
  prof_end(ctx, kProfTrsm, (double)w * (w - 1) * (c_end - c_begin),
           ((double)w * w + 2.0 * w * (c_end - c_begin)) * sizeof(T));
  LUHOT_CUDA_TRY(ctx, cudaGetLastError());
  return LUHOT_OK;
}

// The trailing update of the panel [k0, k0 + w): a[r1.., r1..] -= L21 U12,
// r1 = k0 + w.  Fast-mode FP64 runs it on the FP16 tensor cores (ozaki.cu)
// when a workspace was given and the block is large enough for the engine
// setting, else on the FP64 tensor cores.
template <typename T, bool kExact>
static int schur_update(luhot_ctx* ctx, T* a, int64_t lda, int k0, int w, int m, int n, void* oz_ws, int engine,
                        cudaStream_t stream) {
  const int r1 = k0 + w;
  if constexpr (std::is_same<T, double>::value && !kExact) {
    const int M = m - r1, N = n - r1;
    const bool big = engine == LUHOT_UPDATE_OZAKI ? (M >= 128 && N >= 64) : (M >= 256 && N >= 256);
    if (oz_ws && engine != LUHOT_UPDATE_DMMA && big)
      return ozaki_update(ctx, a, lda, k0, w, r1, m, r1, n, oz_ws, stream);
  }
  return launch_gemm<T, kExact>(ctx, a, lda, r1, r1, k0, w, m - r1, n - r1, stream);
}

// Workspace of the tensor-core FP64 update for an m x n factorization
// (nullptr: the engine setting or the device rules it out).
static int ozaki_workspace(luhot_ctx* ctx, int m, int n, int engine, void** ws) {
  *ws = nullptr;
  if (engine == LUHOT_UPDATE_DMMA || !ozaki_available(ctx)) return LUHOT_OK;
  int rc = ensure_buf(ctx, ctx->oz_buf, ozaki_workspace_bytes(m, n));
  if (rc != LUHOT_OK) return rc;
  *ws = ctx->oz_buf.ptr;
  return LUHOT_OK;
}

int fp64_schur_update(luhot_ctx* ctx, double* a, int64_t lda, int k, int m, int n, int engine) {
  void* ws = nullptr;
  int rc = ozaki_workspace(ctx, m, n, engine, &ws);
  if (rc) return rc;
  return schur_update<double, false>(ctx, a, lda, 0, k, m, n, ws, engine, ctx->stream);
}

template <typename T, bool kExact>
static int getrf_impl(luhot_ctx* ctx, int m, int n, T* a, int64_t lda, int* piv, int nb, void* oz_ws,
                      cudaStream_t stream) {
  const int dim_min = std::min(m, n);
  // Exchange words carry step tags; clear them so no word of an earlier
  // factorization carries a live tag.
  LUHOT_CUDA_TRY(ctx, cudaMemsetAsync(ctx->panel_scratch, 0, kPanelScratchBytes, stream));
  for (int k0 = 0; k0 < dim_min; k0 += nb) {
    const int w = std::min(nb, dim_min - k0);
    int rc = launch_panel<T, kExact>(ctx, a, lda, m, k0, w, piv, stream);
    if (!rc) rc = launch_laswp<T>(ctx, a, lda, k0, w, n, stream);
    if (rc) return rc;
    const int c_right = k0 + w;
    if (c_right < n) {
      rc = launch_trsm<T, kExact>(ctx, a, lda, k0, w, c_right, n, stream, oz_ws, ctx->fp64_update);
      if (!rc) rc = schur_update<T, kExact>(ctx, a, lda, k0, w, m, n, oz_ws, ctx->fp64_update, stream);
      if (rc) return rc;
    }
  }
  return LUHOT_OK;
}

// The tensor-core factorization in slabs of two 128-column panels: the
// trailing matrix is updated once per slab (K = 256), which halves its reads
// and writes, the bound of that update.  The two K = 128 updates inside a
// slab (128 columns, or 128 rows) run as FP32 CUDA-core GEMMs: one launch
// each, at least as accurate as any of the tensor-core operand formats.
//
// Look-ahead: the trailing update of slab s is cut at the next slab's
// columns.  A high-priority stream (hs) factors slab s (panels A and B,
// their interchanges on the slab's own columns, the K = 128 step between
// them), then brings the next slab's columns up to date (interchanges, rows
// of U, update).  A low-priority stream (ls) then does the rest of slab s:
// its interchanges on the columns left of it and right of the next slab,
// the rows of U there and the update of those columns, on at most SM count
// - 64 CTAs, so that slab s + 1's panels (64 CTAs) run beside it.  hs waits
// for the rest of slab s - 2 before slab s's panels (it covered slab s's
// columns) and for the rest of slab s - 1 before the next slab's columns.
// Each panel's list of moved rows is saved per slab parity for ls.
static int* la_saved_moves(luhot_ctx* ctx, int parity, int half) {
  return reinterpret_cast<int*>(static_cast<char*>(ctx->la_moves.ptr) + (size_t)(2 * parity + half) * kPanelMovesBytes);
}

// Launches between its construction and destruction go to `s` (the
// profile's events are recorded on the context's stream).
struct OnStream {
  luhot_ctx* ctx;
  cudaStream_t old;
  OnStream(luhot_ctx* c, cudaStream_t s) : ctx(c), old(c->stream) { c->stream = s; }
  ~OnStream() { ctx->stream = old; }
};

static int la_setup(luhot_ctx* ctx) {
  if (!ctx->la_hi) {
    int least = 0, greatest = 0;
    LUHOT_CUDA_TRY(ctx, cudaDeviceGetStreamPriorityRange(&least, &greatest));
    LUHOT_CUDA_TRY(ctx, cudaStreamCreateWithPriority(&ctx->la_lo, cudaStreamNonBlocking, least));
    LUHOT_CUDA_TRY(ctx, cudaStreamCreateWithPriority(&ctx->la_hi, cudaStreamNonBlocking, greatest));
  }
  for (auto& e : ctx->la_ev)
    if (!e) LUHOT_CUDA_TRY(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  return ensure_buf(ctx, ctx->la_moves, 4 * kPanelMovesBytes);
}

// Rows [s0, s1) of U on the columns [c0, c1) (two trsm steps with the K =
// 128 update of panel B's rows between them), then the update of rows
// [s1, m) x columns [c0, c1) on the tensor cores (K = s1 - s0).
static int slab_columns(luhot_ctx* ctx, float* a, int64_t lda, int m, int s0, int h0, int h1, int c0, int c1,
                        int tc_kind, void* tc_a, void* tc_b, float* tc_scal, cudaStream_t st) {
  if (c0 >= c1) return LUHOT_OK;
  int rc = launch_trsm<float, false>(ctx, a, lda, s0, h0, c0, c1, st);
  if (!rc && h1 > 0) {
    rc = launch_gemm<float, false>(ctx, a, lda, s0 + h0, c0, s0, h0, h1, c1 - c0, st);
    if (!rc) rc = launch_trsm<float, false>(ctx, a, lda, s0 + h0, h1, c0, c1, st);
  }
  const int s1 = s0 + h0 + h1;
  if (!rc) rc = tc_gemm_update(ctx, tc_kind, a, lda, s0, h0 + h1, s1, m, c0, c1, tc_a, tc_b, tc_scal, st);
  return rc;
}

static int tc_slab_loop(luhot_ctx* ctx, int m, int n, float* a, int64_t lda, int* piv, int tc_kind, void* tc_a,
                        void* tc_b, float* tc_scal) {
  const int dim_min = std::min(m, n);
  cudaStream_t hs = ctx->la_hi, ls = ctx->la_lo;
  cudaEvent_t ev_ready = ctx->la_ev[1];
  const int* live_moves = reinterpret_cast<const int*>(static_cast<char*>(ctx->panel_scratch) + kPanelSlotBytes);
  constexpr int hw = kTcPanelWidth, sl = 2 * hw;
  const int cap_rest = std::max(1, ctx->num_sms - 64);
  int slab = 0;
  for (int s0 = 0; s0 < dim_min; s0 += sl, ++slab) {
    const int sw = std::min(sl, dim_min - s0);
    const int h0 = std::min(hw, sw), h1 = sw - h0;
    const int s1 = s0 + sw;
    const int e1 = std::min(n, s1 + sl);  // the next slab's columns: [s1, e1)
    const int par = slab & 1;
    int* mv_a = la_saved_moves(ctx, par, 0);
    int* mv_b = la_saved_moves(ctx, par, 1);
    {
      OnStream on(ctx, hs);
      if (slab >= 2) LUHOT_CUDA_TRY(ctx, cudaStreamWaitEvent(hs, ctx->la_ev[2 + par], 0));
      int rc = launch_panel<float, false>(ctx, a, lda, m, s0, h0, piv, hs);
      if (rc) return rc;
      LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(mv_a, live_moves, kPanelMovesBytes, cudaMemcpyDeviceToDevice, hs));
      rc = launch_laswp_cols<float>(ctx, a, lda, mv_a, h0, 0, 0, s0 + h0, s1, hs);
      if (!rc && h1 > 0) {
        rc = launch_trsm<float, false>(ctx, a, lda, s0, h0, s0 + h0, s1, hs);
        if (!rc) rc = launch_gemm<float, false>(ctx, a, lda, s0 + h0, s0 + h0, s0, h0, m - (s0 + h0), h1, hs);
        if (!rc) rc = launch_panel<float, false>(ctx, a, lda, m, s0 + h0, h1, piv, hs);
        if (rc) return rc;
        LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(mv_b, live_moves, kPanelMovesBytes, cudaMemcpyDeviceToDevice, hs));
        rc = launch_laswp_cols<float>(ctx, a, lda, mv_b, h1, s0, s0 + h0, 0, 0, hs);
      }
      if (!rc && s1 < e1) {
        if (slab >= 1) LUHOT_CUDA_TRY(ctx, cudaStreamWaitEvent(hs, ctx->la_ev[2 + (par ^ 1)], 0));
        rc = launch_laswp_cols<float>(ctx, a, lda, mv_a, h0, 0, 0, s1, e1, hs);
        if (!rc && h1 > 0) rc = launch_laswp_cols<float>(ctx, a, lda, mv_b, h1, 0, 0, s1, e1, hs);
        if (!rc) rc = slab_columns(ctx, a, lda, m, s0, h0, h1, s1, e1, tc_kind, tc_a, tc_b, tc_scal, hs);
      }
      if (rc) return rc;
      LUHOT_CUDA_TRY(ctx, cudaEventRecord(ev_ready, hs));
    }
    {
      OnStream on(ctx, ls);
      LUHOT_CUDA_TRY(ctx, cudaStreamWaitEvent(ls, ev_ready, 0));
      int rc = launch_laswp_cols<float>(ctx, a, lda, mv_a, h0, 0, s0, e1, n, ls);
      if (!rc && h1 > 0) rc = launch_laswp_cols<float>(ctx, a, lda, mv_b, h1, 0, s0, e1, n, ls);
      if (!rc && e1 < n) {
        ctx->tc_grid_cap = cap_rest;
        rc = slab_columns(ctx, a, lda, m, s0, h0, h1, e1, n, tc_kind, tc_a, tc_b, tc_scal, ls);
        ctx->tc_grid_cap = 0;
      }
      if (rc) return rc;
      LUHOT_CUDA_TRY(ctx, cudaEventRecord(ctx->la_ev[2 + par], ls));
    }
  }
  return LUHOT_OK;
}

static int getrf_tc_slabs(luhot_ctx* ctx, int m, int n, float* a, int64_t lda, int* piv, int tc_kind, void* tc_a,
                          void* tc_b, float* tc_scal, cudaStream_t stream) {
  LUHOT_CUDA_TRY(ctx, cudaMemsetAsync(ctx->panel_scratch, 0, kPanelScratchBytes, stream));
  int rc = la_setup(ctx);
  if (rc) return rc;
  LUHOT_CUDA_TRY(ctx, cudaEventRecord(ctx->la_ev[0], stream));
  LUHOT_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->la_hi, ctx->la_ev[0], 0));
  LUHOT_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->la_lo, ctx->la_ev[0], 0));
  rc = tc_slab_loop(ctx, m, n, a, lda, piv, tc_kind, tc_a, tc_b, tc_scal);
  ctx->tc_grid_cap = 0;
  // The caller's stream waits for both streams, also after an error.
  cudaError_t e = cudaEventRecord(ctx->la_ev[0], ctx->la_hi);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, ctx->la_ev[0], 0);
  if (e == cudaSuccess) e = cudaEventRecord(ctx->la_ev[1], ctx->la_lo);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, ctx->la_ev[1], 0);
  if (rc) return rc;
  if (e != cudaSuccess) return set_error(ctx, LUHOT_ERR_CUDA, std::string("look-ahead join: ") + cudaGetErrorString(e));
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
  void* oz_ws = nullptr;
  if (std::is_same<T, double>::value && mode != LUHOT_MODE_EXACT) {
    rc = ozaki_workspace(ctx, m, n, ctx->fp64_update, &oz_ws);
    if (rc != LUHOT_OK) return rc;
  }
  if (mode == LUHOT_MODE_EXACT)
    rc = getrf_impl<T, true>(ctx, m, n, a, lda, piv, nb, nullptr, stream);
  else
    rc = getrf_impl<T, false>(ctx, m, n, a, lda, piv, nb, oz_ws, stream);
  if (rc != LUHOT_OK) return rc;
  return finish_status(ctx, singular);
}

template int getrf_device<double>(luhot_ctx*, int, int, double*, int64_t, int*, int, int64_t*);
template int getrf_device<float>(luhot_ctx*, int, int, float*, int64_t, int*, int, int64_t*);

int getrf_device_tc(luhot_ctx* ctx, int m, int n, float* a, int64_t lda, int* piv, int tc_kind, int64_t* singular) {
  if (m < 0 || n < 0 || lda < std::max(1, n)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrf: bad shape or lda");
  if (singular) *singular = -1;
  if (m == 0 || n == 0) return LUHOT_OK;
  const int nb = 2 * kTcPanelWidth;  // a slab's K
  const size_t bytes = tc_operand_bytes(tc_kind, m, nb) + tc_operand_bytes(tc_kind, n, nb) + 4096;
  int rc = ensure_buf(ctx, ctx->tc_buf, bytes);
  if (rc) return rc;
  char* base = static_cast<char*>(ctx->tc_buf.ptr);
  void* tc_a = base;
  void* tc_b = base + (tc_operand_bytes(tc_kind, m, nb) + 1023) / 1024 * 1024;
  float* tc_scal = reinterpret_cast<float*>(base + bytes - 1024);
  rc = reset_status(ctx);
  if (rc != LUHOT_OK) return rc;
  rc = getrf_tc_slabs(ctx, m, n, a, lda, piv, tc_kind, tc_a, tc_b, tc_scal, ctx->stream);
  if (rc != LUHOT_OK) return rc;
  return finish_status(ctx, singular);
}

}  // namespace luhot
