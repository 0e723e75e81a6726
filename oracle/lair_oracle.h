/*
 * CPU restatement of lair's LU path (test infrastructure only).
 *
 * This is the oracle the GPU library is checked against.  It is NOT part of
 * the product: only the test suite, the smoke check and the benchmark's CPU
 * baseline leg may load it.  Every routine follows one function of lair 0.8.0
 * (paths below are relative to the lair source tree) and keeps its exact
 * operation order.  It must be compiled with -ffp-contract=off: Rust never
 * fuses `a -= l * b` into an FMA, so every multiply and every subtract rounds
 * on its own, and this file reproduces that rounding sequence bit for bit.
 *
 * Strides are in elements and may be negative, as in ndarray views.
 * Pivots are 0-based LAPACK-style sequential interchanges: at step i row i
 * was swapped with row piv[i] (piv[i] >= i).
 * "singular" follows lair's Option<usize>: -1 means None.
 */
#ifndef LAIR_ORACLE_H
#define LAIR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ndarray's ArrayBase::is_standard_layout for a 2-D array (C-contiguous,
 * length-1 axes ignored, any empty array counts as standard). */
int oracle_is_standard_layout(int64_t m, int64_t n, int64_t rs, int64_t cs);

/* src/blas/iamax.rs:6-21 */
int64_t oracle_diamax(int64_t n, const double* x, int64_t incx, double* max_val);
int64_t oracle_siamax(int64_t n, const float* x, int64_t incx, float* max_val);

/* src/lapack/laswp.rs:11-40 (element type only moves, so one routine per width) */
void oracle_dlaswp(int64_t ncols, double* a, int64_t rs, int64_t cs, int64_t begin,
                   const uint64_t* piv, int64_t npiv);
void oracle_slaswp(int64_t ncols, float* a, int64_t rs, int64_t cs, int64_t begin,
                   const uint64_t* piv, int64_t npiv);

/* src/lapack/getrf.rs:46-120 (getrf_row_major).  Runs elimination steps
 * [0, min(max_steps, min(m,n))); max_steps < 0 means all.  Returns singular. */
int64_t oracle_dgetrf_row_major(int64_t m, int64_t n, double* a, int64_t rs, int64_t cs,
                                uint64_t* piv, int64_t max_steps);
int64_t oracle_sgetrf_row_major(int64_t m, int64_t n, float* a, int64_t rs, int64_t cs,
                                uint64_t* piv, int64_t max_steps);
/* The same elimination, steps [step_begin, step_end) only (piv must already
 * hold the identity for those steps).  Used to time a bounded slice of a
 * large factorization. */
int64_t oracle_dgetrf_row_major_range(int64_t m, int64_t n, double* a, int64_t rs, int64_t cs,
                                      uint64_t* piv, int64_t step_begin, int64_t step_end);

/* getrf_row_major's arithmetic, bit for bit, for a C-order array with row
 * stride lda, in blocks of w steps with the updates of the rows below a
 * block split over nthreads threads (for fixtures at large n).  piv is
 * written in full.  colmax / gap (may be NULL) receive, per step, the largest
 * candidate |a| and its margin over the second largest. */
int64_t oracle_dgetrf_row_major_blocked(int64_t m, int64_t n, double* a, int64_t lda, uint64_t* piv,
                                        int64_t w, int nthreads, double* colmax, double* gap);

/* src/lapack/getrf.rs:128-213 (getrf_col_major, left-looking Crout). */
int64_t oracle_dgetrf_col_major(int64_t m, int64_t n, double* a, int64_t rs, int64_t cs,
                                uint64_t* piv);
int64_t oracle_sgetrf_col_major(int64_t m, int64_t n, float* a, int64_t rs, int64_t cs,
                                uint64_t* piv);

/* src/lapack/getrf.rs:12-27 (layout dispatcher).  piv has min(m,n) entries. */
int64_t oracle_dgetrf(int64_t m, int64_t n, double* a, int64_t rs, int64_t cs, uint64_t* piv);
int64_t oracle_sgetrf(int64_t m, int64_t n, float* a, int64_t rs, int64_t cs, uint64_t* piv);

/* src/lapack/getrf.rs:29-40,215-322 (getrf_recursive, unused by lair's API).
 * piv has m entries.  Returns 0 for Ok, else 1 and *singular_row = Singular(row). */
int oracle_dgetrf_recursive(int64_t m, int64_t n, double* a, int64_t rs, int64_t cs,
                            uint64_t* piv, int64_t* singular_row);

/* src/lapack/getrs.rs:12-38.  lu is m x ncols with m == npiv, b has m entries,
 * x receives the solution (b is not modified). */
void oracle_dgetrs(int64_t m, int64_t ncols, const double* lu, int64_t rs, int64_t cs,
                   const uint64_t* piv, const double* b, int64_t incb, double* x);
void oracle_sgetrs(int64_t m, int64_t ncols, const float* lu, int64_t rs, int64_t cs,
                   const uint64_t* piv, const float* b, int64_t incb, float* x);

/* src/blas/dot.rs:39-133 (4-accumulator dot) and src/blas/gemv.rs:6-47 (notrans). */
double oracle_ddot(int64_t n, const double* x, int64_t incx, const double* y, int64_t incy);
void oracle_dgemv_notrans(int64_t m, int64_t n, double alpha, const double* a, int64_t rs,
                          int64_t cs, const double* x, int64_t incx, double beta, double* y,
                          int64_t incy);

#ifdef __cplusplus
}
#endif
#endif
