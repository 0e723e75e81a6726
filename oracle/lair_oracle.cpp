// CPU restatement of lair 0.8.0's LU path.  Test infrastructure only: the
// GPU library never links or calls this file; the tests, the smoke check and
// the benchmark's CPU-baseline leg use it as the checker.
//
// Build with -ffp-contract=off (see oracle/Makefile): every `x -= p * q` in
// lair rounds the product and the difference separately, and so must this.
// Each routine cites the lair function it restates (paths inside lair's tree).
#include "lair_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <functional>
#include <thread>
#include <limits>
#include <vector>

namespace {

template <typename T>
inline T& at(T* a, int64_t i, int64_t j, int64_t rs, int64_t cs) {
  return a[i * rs + j * cs];
}

// src/blas/iamax.rs:6-21: first index of the largest |x| (strict `>`, so a
// NaN never wins and an all-zero column yields (0, 0)).
template <typename T>
int64_t iamax(int64_t n, const T* x, int64_t incx, T* max_val_out) {
  T max_val = T(0);
  int64_t max_idx = 0;
  for (int64_t i = 0; i < n; ++i) {
    T v = x[incx * i];
    // re().abs() + im().abs(); for real types im() is 0, and |v| + 0 == |v|.
    T val = std::fabs(v) + T(0);
    if (val > max_val) {
      max_val = val;
      max_idx = i;
    }
  }
  if (max_val_out) *max_val_out = max_val;
  return max_idx;
}

// src/lapack/getrf.rs:324-333
template <typename T>
void swap_rows(int64_t n, T* row1, T* row2, int64_t stride) {
  for (int64_t k = 0; k < n; ++k) std::swap(row1[k * stride], row2[k * stride]);
}

// src/lapack/laswp.rs:11-40: sequential swaps of rows i <-> piv[i], i >= begin.
template <typename T>
void laswp(int64_t ncols, T* a, int64_t rs, int64_t cs, int64_t begin, const uint64_t* piv,
           int64_t npiv) {
  for (int64_t i = begin; i < npiv; ++i) {
    int64_t p = (int64_t)piv[i];
    if (i == p) continue;
    // lair's loop body runs at least once even for ncols == 0; callers never
    // pass 0, and the restatement treats it as "nothing to swap".
    for (int64_t k = 0; k < ncols; ++k) std::swap(a[i * rs + k * cs], a[p * rs + k * cs]);
  }
}

// src/lapack/getrf.rs:46-120: unblocked right-looking elimination.  The three
// stride branches of the original perform the same arithmetic in the same
// order, so one strided loop restates all of them.
template <typename T>
int64_t getrf_row_major_range(int64_t m, int64_t n, T* a, int64_t rs, int64_t cs, uint64_t* piv,
                              int64_t step_begin, int64_t step_end) {
  int64_t singular = -1;
  for (int64_t ul = step_begin; ul < step_end; ++ul) {
    T max_val;
    int64_t max_idx = iamax<T>(m - ul, a + rs * ul + cs * ul, rs, &max_val);
    if (max_idx != 0) {
      int64_t max_row = max_idx + ul;
      piv[ul] = (uint64_t)max_row;
      swap_rows<T>(n, a + ul * rs, a + max_row * rs, cs);
    }
    if (max_val == T(0)) {
      singular = max_idx + ul;
    } else {
      const T pivot_recip = T(1) / at(a, ul, ul, rs, cs);
      const T* urow = a + ul * rs;
      for (int64_t j = ul + 1; j < m; ++j) {
        T* row = a + j * rs;
        row[ul * cs] *= pivot_recip;
        const T ratio = row[ul * cs];
        for (int64_t c = ul + 1; c < n; ++c) {
          const T elem = ratio * urow[c * cs];
          row[c * cs] -= elem;
        }
      }
    }
  }
  return singular;
}

template <typename T>
int64_t getrf_row_major(int64_t m, int64_t n, T* a, int64_t rs, int64_t cs, uint64_t* piv,
                        int64_t max_steps) {
  const int64_t dim_min = std::min(m, n);
  const int64_t steps = (max_steps < 0) ? dim_min : std::min(dim_min, max_steps);
  return getrf_row_major_range<T>(m, n, a, rs, cs, piv, 0, steps);
}

// The same elimination as getrf_row_major_range for a C-order array (row
// stride lda, column stride 1), reordered across elements but never within
// one, so that large fixtures can be made in minutes: every element receives
// lair's updates a[i][c] -= l[i][t] * u[t][c] in increasing t, each product
// and difference rounded apart, with the same multipliers (scaled by the
// same reciprocal) and the same pivot searches, interchanges and singular
// steps, so the result is bit-identical to the unblocked order.  Steps run
// in blocks of w: the block's columns are eliminated step by step (with the
// full-row interchanges lair makes, applied to the other columns once the
// block's steps are known, since nothing reads those columns meanwhile);
// then the block's rows of the columns to the right receive their updates in
// step order (each row t is final before rows below use it), and the rows
// below receive the block's w updates per element, split over threads.
// Optionally records, per step, the largest candidate |a| and the gap to the
// second largest (the margin by which the pivot won).
template <typename T>
int64_t getrf_row_major_blocked(int64_t m, int64_t n, T* a, int64_t lda, uint64_t* piv, int64_t w,
                                int nthreads, double* colmax, double* gap) {
  const int64_t dim_min = std::min(m, n);
  if (w < 1) w = 64;
  if (nthreads < 1) nthreads = 1;
  int64_t singular = -1;
  std::vector<char> skip((size_t)std::max<int64_t>(dim_min, 1), 0);
  auto run_threads = [&](int64_t count, const std::function<void(int64_t, int64_t)>& fn) {
    const int64_t nt = std::min<int64_t>(nthreads, std::max<int64_t>(count, 1));
    if (nt <= 1) {
      fn(0, count);
      return;
    }
    std::vector<std::thread> th;
    for (int64_t t = 0; t < nt; ++t) {
      const int64_t lo = count * t / nt, hi = count * (t + 1) / nt;
      th.emplace_back([&fn, lo, hi] { fn(lo, hi); });
    }
    for (auto& x : th) x.join();
  };
  for (int64_t k0 = 0; k0 < dim_min; k0 += w) {
    const int64_t kend = std::min(k0 + w, dim_min);
    const int64_t pend = std::min(k0 + w, n);
    // Block columns [k0, pend), every row, step by step.
    for (int64_t ul = k0; ul < kend; ++ul) {
      T max_val = T(0), second = T(0);
      int64_t max_idx = 0;
      for (int64_t i = 0; i < m - ul; ++i) {  // iamax, strict `>`; NaN never wins
        const T val = std::fabs(a[(ul + i) * lda + ul]) + T(0);
        if (val > max_val) {
          second = max_val;
          max_val = val;
          max_idx = i;
        } else if (val > second) {
          second = val;
        }
      }
      if (colmax) colmax[ul] = (double)max_val;
      if (gap) gap[ul] = (double)(max_val - second);
      piv[ul] = (uint64_t)ul;
      if (max_idx != 0) {
        const int64_t r = max_idx + ul;
        piv[ul] = (uint64_t)r;
        for (int64_t c = k0; c < pend; ++c) std::swap(a[ul * lda + c], a[r * lda + c]);
      }
      if (max_val == T(0)) {
        singular = max_idx + ul;
        skip[(size_t)ul] = 1;
        continue;
      }
      const T pivot_recip = T(1) / a[ul * lda + ul];
      const T* urow = a + ul * lda;
      for (int64_t j = ul + 1; j < m; ++j) {
        T* row = a + j * lda;
        row[ul] *= pivot_recip;
        const T ratio = row[ul];
        for (int64_t c = ul + 1; c < pend; ++c) {
          const T elem = ratio * urow[c];
          row[c] -= elem;
        }
      }
    }
    // The block's interchanges, on the columns outside the block, in order.
    for (int64_t ul = k0; ul < kend; ++ul) {
      const int64_t r = (int64_t)piv[ul];
      if (r == ul) continue;
      for (int64_t c = 0; c < k0; ++c) std::swap(a[ul * lda + c], a[r * lda + c]);
      for (int64_t c = pend; c < n; ++c) std::swap(a[ul * lda + c], a[r * lda + c]);
    }
    if (pend >= n) continue;
    constexpr int64_t kTile = 256;
    const int64_t ncols = n - pend, ntiles = (ncols + kTile - 1) / kTile;
    // The block's own rows, columns to the right: row t is final before the
    // rows below it use it.
    run_threads(ntiles, [&](int64_t lo, int64_t hi) {
      for (int64_t tile = lo; tile < hi; ++tile) {
        const int64_t c0 = pend + tile * kTile, c1 = std::min(n, c0 + kTile);
        for (int64_t t = k0; t < kend; ++t) {
          if (skip[(size_t)t]) continue;
          const T* urow = a + t * lda;
          for (int64_t i = t + 1; i < kend; ++i) {
            T* row = a + i * lda;
            const T ratio = row[t];
            for (int64_t c = c0; c < c1; ++c) {
              const T elem = ratio * urow[c];
              row[c] -= elem;
            }
          }
        }
      }
    });
    // The rows below the block: the block's updates in step order.
    const int64_t rows = m - kend;
    run_threads(rows, [&](int64_t lo, int64_t hi) {
      for (int64_t c0 = pend; c0 < n; c0 += kTile) {
        const int64_t c1 = std::min(n, c0 + kTile);
        for (int64_t i = kend + lo; i < kend + hi; ++i) {
          T* row = a + i * lda;
          for (int64_t t = k0; t < kend; ++t) {
            if (skip[(size_t)t]) continue;
            const T ratio = row[t];
            const T* urow = a + t * lda;
            for (int64_t c = c0; c < c1; ++c) {
              const T elem = ratio * urow[c];
              row[c] -= elem;
            }
          }
        }
      }
    });
  }
  return singular;
}

// src/blas/dot.rs:39-133: four partial sums over blocks of four, combined as
// ((s0 + s1) + s2) + s3, then up to three tail terms added in order.  The
// contiguous and strided branches of the original are arithmetically equal.
template <typename T>
T dot(int64_t n, const T* x, int64_t incx, const T* y, int64_t incy) {
  int64_t remaining = n;
  T sum;
  if (remaining >= 4) {
    T s0 = T(0), s1 = T(0), s2 = T(0), s3 = T(0);
    for (;;) {
      s0 += x[0] * y[0];
      s1 += x[incx] * y[incy];
      s2 += x[2 * incx] * y[2 * incy];
      s3 += x[3 * incx] * y[3 * incy];
      x += 4 * incx;
      y += 4 * incy;
      remaining -= 4;
      if (remaining < 4) break;
    }
    sum = s0 + s1 + s2 + s3;
  } else {
    sum = T(0);
  }
  if (remaining > 0) {
    sum += x[0] * y[0];
    x += incx;
    y += incy;
  }
  if (remaining > 1) {
    sum += x[0] * y[0];
    x += incx;
    y += incy;
  }
  if (remaining > 2) sum += x[0] * y[0];
  return sum;
}

// src/blas/gemv.rs:6-47 (notrans): y = beta*y, then for each column j in
// order, y += (alpha * x[j]) * a[:, j].
template <typename T>
void gemv_notrans(int64_t m, int64_t n, T alpha, const T* a, int64_t rs, int64_t cs, const T* x,
                  int64_t incx, T beta, T* y, int64_t incy) {
  if (beta == T(0)) {
    for (int64_t r = 0; r < m; ++r) y[r * incy] = T(0);
  } else if (beta != T(1)) {
    for (int64_t r = 0; r < m; ++r) y[r * incy] *= beta;
  }
  if (alpha == T(0)) return;
  for (int64_t j = 0; j < n; ++j) {
    const T alpha_x = alpha * x[j * incx];
    for (int64_t r = 0; r < m; ++r) y[r * incy] += alpha_x * a[r * rs + j * cs];
  }
}

// src/lapack/getrf.rs:128-213: left-looking (Crout) elimination used for
// every non-standard layout.
template <typename T>
int64_t getrf_col_major(int64_t nrows, int64_t ncols, T* a, int64_t rs, int64_t cs,
                        uint64_t* piv) {
  int64_t singular = -1;
  for (int64_t ul = 0; ul < ncols; ++ul) {
    T* col = a + ul * cs;  // column ul, element r at col[r * rs]
    const int64_t n_upper_rows = std::min(ul, nrows);
    for (int64_t i = 0; i < n_upper_rows; ++i) {
      int64_t ip = (int64_t)piv[i];
      if (ip != i) std::swap(col[i * rs], col[ip * rs]);
    }
    // left.row(i) holds a[i][0..ul]; only its first i entries enter the dot.
    for (int64_t i = 1; i < n_upper_rows; ++i) {
      const T sum = dot<T>(i, a + i * rs, cs, col, rs);
      col[i * rs] -= sum;
    }
    if (ul < nrows) {
      // gemv::notrans(-1, a[ul.., ..ul], col[..ul], 1, col[ul..])
      gemv_notrans<T>(nrows - ul, ul, T(-1), a + ul * rs, rs, cs, col, rs, T(1), col + ul * rs,
                      rs);
      const int64_t max_row = iamax<T>(nrows - ul, col + ul * rs, rs, nullptr);
      const int64_t pivot_row = ul + max_row;
      piv[ul] = (uint64_t)pivot_row;
      const T pivot = col[pivot_row * rs];
      if (pivot == T(0)) {
        singular = ul;
      } else {
        const T pivot_recip = T(1) / pivot;
        if (pivot_row != ul) swap_rows<T>(ul + 1, a + ul * rs, a + pivot_row * rs, cs);
        for (int64_t row = ul + 1; row < nrows; ++row) col[row * rs] *= pivot_recip;
      }
    }
  }
  return singular;
}

// ndarray 0.17 ArrayBase::is_standard_layout for two axes: empty arrays are
// standard; otherwise every axis of length != 1 must have the C-order stride.
bool is_standard_layout(int64_t m, int64_t n, int64_t rs, int64_t cs) {
  if (m == 0 || n == 0) return true;
  int64_t contig = 1;
  if (n != 1) {
    if (cs != contig) return false;
    contig *= n;
  }
  if (m != 1) {
    if (rs != contig) return false;
  }
  return true;
}

template <typename T>
int64_t getrf(int64_t m, int64_t n, T* a, int64_t rs, int64_t cs, uint64_t* piv) {
  // src/lapack/getrf.rs:12-27: pivots start as the identity 0..min(m, n).
  const int64_t dim_min = std::min(m, n);
  for (int64_t i = 0; i < dim_min; ++i) piv[i] = (uint64_t)i;
  if (is_standard_layout(m, n, rs, cs)) return getrf_row_major<T>(m, n, a, rs, cs, piv, -1);
  return getrf_col_major<T>(m, n, a, rs, cs, piv);
}

// src/blas/trsm.rs:6-22: B <- L^-1 B with unit-lower L read through `a`,
// column by column, skipping zero right-hand entries.
template <typename T>
void trsm(const T* a, int64_t rs, int64_t cs, T* b, int64_t bm, int64_t bn, int64_t brs,
          int64_t bcs) {
  for (int64_t j = 0; j < bn; ++j) {
    for (int64_t k = 0; k < bm; ++k) {
      const T bkj = b[k * brs + j * bcs];
      if (bkj == T(0)) continue;
      for (int64_t i = k + 1; i < bm; ++i) {
        const T prod = b[k * brs + j * bcs] * a[rs * i + cs * k];
        b[i * brs + j * bcs] -= prod;
      }
    }
  }
}

// src/blas/gemm.rs:6-32: C += alpha * (A B) with a left-to-right fold per entry.
template <typename T>
void gemm(T alpha, const T* a, int64_t am, int64_t ak, int64_t ars, int64_t acs, const T* b,
          int64_t bn, int64_t brs, int64_t bcs, T* c, int64_t crs, int64_t ccs) {
  for (int64_t i = 0; i < am; ++i) {
    for (int64_t j = 0; j < bn; ++j) {
      T s = T(0);
      for (int64_t k = 0; k < ak; ++k) s = s + a[i * ars + k * acs] * b[k * brs + j * bcs];
      c[i * crs + j * ccs] += alpha * s;
    }
  }
}

// src/lapack/getrf.rs:215-322 (recursive_inner).  Returns the Singular row or
// 0 for Ok, exactly like the original's use of 0 as "no singular row".
template <typename T>
int64_t recursive_inner(int64_t m, int64_t n, T* a, int64_t rs, int64_t cs, uint64_t* piv,
                        bool* err) {
  *err = false;
  if (m == 0 || n == 0) return 0;
  if (m == 1) {
    piv[0] = 0;
    if (a[0] == T(0)) {
      *err = true;
      return 0;
    }
    return 0;
  }
  if (n == 1) {
    T max_val;
    const int64_t max_idx = iamax<T>(m, a, rs, &max_val);
    piv[0] = (uint64_t)max_idx;
    if (max_val == T(0)) {
      *err = true;
      return 0;
    }
    if (max_idx != 0) std::swap(a[0], a[max_idx * rs]);
    if (max_val >= std::numeric_limits<T>::min()) {
      const T s = T(1) / a[0];
      for (int64_t r = 1; r < m; ++r) a[r * rs] *= s;
    } else {
      const T pivot = a[0];
      for (int64_t r = 1; r < m; ++r) a[r * rs] /= pivot;
    }
    return 0;
  }
  const int64_t left_cols = std::min(m, n) / 2;
  const int64_t right_cols = n - left_cols;
  bool e = false;
  int64_t singular_row = recursive_inner<T>(m, left_cols, a, rs, cs, piv, &e);
  if (!e) singular_row = 0;
  laswp<T>(right_cols, a + cs * left_cols, rs, cs, 0, piv, left_cols);
  trsm<T>(a, rs, cs, a + cs * left_cols, left_cols, right_cols, rs, cs);
  const int64_t min_dim = std::min(m, n);
  gemm<T>(T(-1), a + left_cols * rs, m - left_cols, left_cols, rs, cs, a + left_cols * cs,
          right_cols, rs, cs, a + left_cols * rs + left_cols * cs, rs, cs);
  bool e2 = false;
  const int64_t row2 = recursive_inner<T>(m - left_cols, n - left_cols,
                                          a + left_cols * rs + left_cols * cs, rs, cs,
                                          piv + left_cols, &e2);
  if (e2 && singular_row == 0) singular_row = left_cols + row2;
  for (int64_t i = left_cols; i < min_dim; ++i) piv[i] += (uint64_t)left_cols;
  laswp<T>(left_cols, a, rs, cs, left_cols, piv, min_dim);
  *err = singular_row != 0;
  return singular_row;
}

// src/lapack/getrs.rs:12-38
template <typename T>
void getrs(int64_t m, int64_t ncols, const T* lu, int64_t rs, int64_t cs, const uint64_t* piv,
           const T* b, int64_t incb, T* x) {
  (void)ncols;
  for (int64_t i = 0; i < m; ++i) x[i] = b[i * incb];
  laswp<T>(1, x, 1, 1, 0, piv, m);
  for (int64_t i = 0; i < m; ++i) {
    for (int64_t k = 0; k < i; ++k) {
      const T prod = lu[i * rs + k * cs] * x[k];
      x[i] -= prod;
    }
  }
  for (int64_t i = m - 1; i >= 0; --i) {
    for (int64_t k = i + 1; k < m; ++k) {
      const T prod = lu[i * rs + k * cs] * x[k];
      x[i] -= prod;
    }
    x[i] /= lu[i * rs + i * cs];
  }
}

}  // namespace


// ---------------------------------------------------------------------------
// QR: lair's unblocked Householder geqrf and its helpers (real element types).
// ---------------------------------------------------------------------------

// src/scalar.rs:393-402: eps = epsilon / 2, sfmin = smallest positive normal.
template <typename T>
T lair_eps() {
  return std::numeric_limits<T>::epsilon() / (T(1) + T(1));
}
template <typename T>
T lair_sfmin() {
  return std::numeric_limits<T>::min();
}

// Rust's powi (LLVM's powi by repeated squaring, compiler-rt __powidf2 order).
template <typename T>
T powi(T a, int b) {
  const bool recip = b < 0;
  T r = T(1);
  for (;;) {
    if (b & 1) r *= a;
    b /= 2;
    if (b == 0) break;
    a *= a;
  }
  return recip ? T(1) / r : r;
}

// src/blas/nrm2.rs:6-15: sqrt of the sequential sum of v*v (+ im*im = 0).
template <typename T>
T nrm2(int64_t n, const T* x, int64_t inc) {
  T sum = -T(0);  // Rust's float Sum folds from -0.0
  for (int64_t i = 0; i < n; ++i) {
    const T v = x[i * inc];
    sum = sum + (v * v + T(0) * T(0));
  }
  return std::sqrt(sum);
}

// src/lapack.rs:63-65
template <typename T>
T lapy3(T x, T y, T z) {
  return std::sqrt(x * x + y * y + z * z);
}

// src/lapack/larfg.rs:9-43 (real alpha): scales x in place, returns beta and tau.
template <typename T>
void larfg(T alpha, int64_t n, T* x, int64_t inc, T* beta_out, T* tau_out) {
  T x_norm = nrm2<T>(n, x, inc);
  if (x_norm == T(0)) {  // alpha.im() == 0 for real types
    *beta_out = alpha;
    *tau_out = T(0);
    return;
  }
  T beta = -std::copysign(lapy3<T>(alpha, T(0), x_norm), alpha);
  const T safe_min = lair_sfmin<T>() / lair_eps<T>();
  int knt = 0;
  if (std::fabs(beta) < safe_min) {
    const T safe_min_recip = T(1) / safe_min;
    for (;;) {
      ++knt;
      for (int64_t i = 0; i < n; ++i) x[i * inc] *= safe_min_recip;
      beta *= safe_min_recip;
      alpha *= safe_min_recip;
      if (std::fabs(beta) >= safe_min || knt >= 20) break;
    }
    x_norm = nrm2<T>(n, x, inc);
    beta = -std::copysign(alpha * alpha + x_norm * x_norm, alpha);
  }
  const T tau = (beta - alpha) / beta;
  alpha = T(1) / (alpha - beta);
  for (int64_t i = 0; i < n; ++i) x[i * inc] *= alpha;
  beta *= powi<T>(safe_min, knt);
  *beta_out = beta;
  *tau_out = tau;
}

// src/lapack/ilal.rs:6-22: last column with a non-zero entry, or -1.
template <typename T>
int64_t ilalc(int64_t rows, int64_t cols, const T* c, int64_t rs, int64_t cs) {
  if (rows == 0 || cols == 0) return -1;
  if (c[(rows - 1) * rs + (cols - 1) * cs] != T(0)) return cols - 1;
  for (int64_t j = cols - 1; j >= 0; --j)
    for (int64_t i = 0; i < rows; ++i)
      if (c[i * rs + j * cs] != T(0)) return j;
  return -1;
}

// src/lapack/larf.rs:10-52: C <- (I - tau v v^T) C via w = C^T v
// (gemv::conjtrans, src/blas/gemv.rs:58-86) and C += (-tau v) w^T
// (gerc, src/blas/gerc.rs).  v has m entries (C is m x n).
template <typename T>
void larf_left(int64_t m, int64_t n, const T* v, int64_t incv, T tau, T* c, int64_t rs, int64_t cs) {
  if (tau == T(0)) return;
  int64_t last_v = m - 1;
  while (last_v >= 0 && v[last_v * incv] == T(0)) --last_v;  // lair unwraps: v has a non-zero
  const int64_t last_c = ilalc<T>(last_v + 1, n, c, rs, cs);
  if (last_c < 0) return;
  std::vector<T> w((size_t)last_c + 1);
  for (int64_t j = 0; j <= last_c; ++j) {
    T sum = T(0);
    for (int64_t i = 0; i <= last_v; ++i) sum = sum + c[i * rs + j * cs] * v[i * incv];
    w[(size_t)j] = T(0) + T(1) * sum;
  }
  for (int64_t i = 0; i <= last_v; ++i) {
    const T factor = -tau * v[i * incv];
    for (int64_t j = 0; j <= last_c; ++j) c[i * rs + j * cs] += factor * w[(size_t)j];
  }
}

// src/lapack/geqrf.rs:9-27
template <typename T>
void geqrf(int64_t m, int64_t n, T* a, int64_t rs, int64_t cs, T* tau) {
  const int64_t k = std::min(m, n);
  for (int64_t i = 0; i < k; ++i) {
    T beta, t;
    larfg<T>(a[i * rs + i * cs], m - i - 1, a + (i + 1) * rs + i * cs, rs, &beta, &t);
    tau[i] = t;
    a[i * rs + i * cs] = T(1);
    std::vector<T> v((size_t)(m - i));
    for (int64_t r = i; r < m; ++r) v[(size_t)(r - i)] = a[r * rs + i * cs];
    larf_left<T>(m - i, n - i - 1, v.data(), 1, t, a + i * rs + (i + 1) * cs, rs, cs);
    a[i * rs + i * cs] = beta;
  }
}

// src/decomposition/qr.rs:26-60: Q (m x m, row-major) from the factored array and tau.
template <typename T>
void qr_q(int64_t m, int64_t n, const T* qr, int64_t rs, int64_t cs, const T* tau, int64_t ntau, T* q) {
  for (int64_t i = 0; i < m * m; ++i) q[i] = T(0);
  for (int64_t j = 0; j < ntau; ++j)
    for (int64_t i = 0; i < m; ++i) q[i * m + j] = qr[i * rs + j * cs];
  for (int64_t j = ntau; j < m; ++j) {
    for (int64_t l = 0; l < m; ++l) q[l * m + j] = T(0);
    q[j * m + j] = T(1);
  }
  for (int64_t i = ntau - 1; i >= 0; --i) {
    if (i < m - 1) {
      q[i * m + i] = T(1);
      std::vector<T> v((size_t)(m - i));
      for (int64_t r = i; r < m; ++r) v[(size_t)(r - i)] = q[r * m + i];
      larf_left<T>(m - i, m - i - 1, v.data(), 1, tau[i], q + i * m + i + 1, m, 1);
    }
    if (i < m - 1)
      for (int64_t r = i + 1; r < m; ++r) q[r * m + i] *= -tau[i];
    q[i * m + i] = T(1) - tau[i];
    for (int64_t l = 0; l < i; ++l) q[l * m + i] = T(0);
  }
  (void)n;
}

extern "C" {

int oracle_is_standard_layout(int64_t m, int64_t n, int64_t rs, int64_t cs) {
  return is_standard_layout(m, n, rs, cs) ? 1 : 0;
}

int64_t oracle_diamax(int64_t n, const double* x, int64_t incx, double* max_val) {
  return iamax<double>(n, x, incx, max_val);
}
int64_t oracle_siamax(int64_t n, const float* x, int64_t incx, float* max_val) {
  return iamax<float>(n, x, incx, max_val);
}

void oracle_dlaswp(int64_t ncols, double* a, int64_t rs, int64_t cs, int64_t begin,
                   const uint64_t* piv, int64_t npiv) {
  laswp<double>(ncols, a, rs, cs, begin, piv, npiv);
}
void oracle_slaswp(int64_t ncols, float* a, int64_t rs, int64_t cs, int64_t begin,
                   const uint64_t* piv, int64_t npiv) {
  laswp<float>(ncols, a, rs, cs, begin, piv, npiv);
}

int64_t oracle_dgetrf_row_major(int64_t m, int64_t n, double* a, int64_t rs, int64_t cs,
                                uint64_t* piv, int64_t max_steps) {
  return getrf_row_major<double>(m, n, a, rs, cs, piv, max_steps);
}
int64_t oracle_sgetrf_row_major(int64_t m, int64_t n, float* a, int64_t rs, int64_t cs,
                                uint64_t* piv, int64_t max_steps) {
  return getrf_row_major<float>(m, n, a, rs, cs, piv, max_steps);
}

int64_t oracle_dgetrf_row_major_range(int64_t m, int64_t n, double* a, int64_t rs, int64_t cs,
                                      uint64_t* piv, int64_t step_begin, int64_t step_end) {
  const int64_t dim_min = std::min(m, n);
  return getrf_row_major_range<double>(m, n, a, rs, cs, piv, std::max<int64_t>(0, step_begin),
                                       std::min(dim_min, step_end));
}

int64_t oracle_dgetrf_row_major_blocked(int64_t m, int64_t n, double* a, int64_t lda, uint64_t* piv,
                                        int64_t w, int nthreads, double* colmax, double* gap) {
  return getrf_row_major_blocked<double>(m, n, a, lda, piv, w, nthreads, colmax, gap);
}

int64_t oracle_dgetrf_col_major(int64_t m, int64_t n, double* a, int64_t rs, int64_t cs,
                                uint64_t* piv) {
  return getrf_col_major<double>(m, n, a, rs, cs, piv);
}
int64_t oracle_sgetrf_col_major(int64_t m, int64_t n, float* a, int64_t rs, int64_t cs,
                                uint64_t* piv) {
  return getrf_col_major<float>(m, n, a, rs, cs, piv);
}

int64_t oracle_dgetrf(int64_t m, int64_t n, double* a, int64_t rs, int64_t cs, uint64_t* piv) {
  return getrf<double>(m, n, a, rs, cs, piv);
}
int64_t oracle_sgetrf(int64_t m, int64_t n, float* a, int64_t rs, int64_t cs, uint64_t* piv) {
  return getrf<float>(m, n, a, rs, cs, piv);
}

int oracle_dgetrf_recursive(int64_t m, int64_t n, double* a, int64_t rs, int64_t cs,
                            uint64_t* piv, int64_t* singular_row) {
  // src/lapack/getrf.rs:29-40: pivots start as vec![0; nrows].
  for (int64_t i = 0; i < m; ++i) piv[i] = 0;
  bool err = false;
  const int64_t row = recursive_inner<double>(m, n, a, rs, cs, piv, &err);
  if (singular_row) *singular_row = err ? row : -1;
  return err ? 1 : 0;
}

void oracle_dgetrs(int64_t m, int64_t ncols, const double* lu, int64_t rs, int64_t cs,
                   const uint64_t* piv, const double* b, int64_t incb, double* x) {
  getrs<double>(m, ncols, lu, rs, cs, piv, b, incb, x);
}
void oracle_sgetrs(int64_t m, int64_t ncols, const float* lu, int64_t rs, int64_t cs,
                   const uint64_t* piv, const float* b, int64_t incb, float* x) {
  getrs<float>(m, ncols, lu, rs, cs, piv, b, incb, x);
}

double oracle_ddot(int64_t n, const double* x, int64_t incx, const double* y, int64_t incy) {
  return dot<double>(n, x, incx, y, incy);
}
void oracle_dgemv_notrans(int64_t m, int64_t n, double alpha, const double* a, int64_t rs,
                          int64_t cs, const double* x, int64_t incx, double beta, double* y,
                          int64_t incy) {
  gemv_notrans<double>(m, n, alpha, a, rs, cs, x, incx, beta, y, incy);
}

void oracle_dgeqrf(int64_t m, int64_t n, double* a, int64_t rs, int64_t cs, double* tau) {
  geqrf<double>(m, n, a, rs, cs, tau);
}
void oracle_sgeqrf(int64_t m, int64_t n, float* a, int64_t rs, int64_t cs, float* tau) {
  geqrf<float>(m, n, a, rs, cs, tau);
}
void oracle_dqr_q(int64_t m, int64_t n, const double* qr, int64_t rs, int64_t cs, const double* tau,
                  int64_t ntau, double* q) {
  qr_q<double>(m, n, qr, rs, cs, tau, ntau, q);
}
void oracle_sqr_q(int64_t m, int64_t n, const float* qr, int64_t rs, int64_t cs, const float* tau,
                  int64_t ntau, float* q) {
  qr_q<float>(m, n, qr, rs, cs, tau, ntau, q);
}
void oracle_dlarfg(double alpha, int64_t n, double* x, int64_t inc, double* beta, double* tau) {
  larfg<double>(alpha, n, x, inc, beta, tau);
}
void oracle_dlarf_left(int64_t m, int64_t n, const double* v, int64_t incv, double tau, double* c, int64_t rs,
                       int64_t cs) {
  larf_left<double>(m, n, v, incv, tau, c, rs, cs);
}
double oracle_dnrm2(int64_t n, const double* x, int64_t inc) { return nrm2<double>(n, x, inc); }

}  // extern "C"
