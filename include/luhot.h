/*
 * luhot: GB300-native (sm_103a) LU hot path of lair, behind a C ABI.
 *
 * These entry points are what lair's Rust shim would bind (through an
 * `extern "C"` crate) from inside `lapack::getrf` / `lapack::getrs` for f64
 * and f32, selected by `TypeId::of::<A>()`; every other element type keeps
 * lair's own code.  Citations name the lair 0.8.0 function each entry point
 * replaces (paths inside lair's source tree).
 *
 * Conventions shared by every call:
 *  - Every function returns an int status (LUHOT_OK == 0).  A failed call
 *    leaves a message in luhot_last_error(ctx).  No call aborts the process.
 *  - Host matrices are described by a pointer to element (0, 0) and signed
 *    element strides (rs = row stride, cs = column stride).  Negative strides
 *    and any layout an ndarray view can have are accepted.  Caller memory is
 *    never freed or retained after the call returns.
 *  - Pivots are 0-based LAPACK-style sequential interchanges, as lair returns
 *    them: at step i, row i was swapped with row piv[i] (piv[i] >= i).
 *  - `singular` mirrors lair's Option<usize>: -1 is None, otherwise the LAST
 *    elimination step whose pivot column was all zero.
 *  - mode LUHOT_MODE_EXACT reproduces lair's operation order bit for bit
 *    (row-major getrf order, src/lapack/getrf.rs:46-120, and getrs order,
 *    src/lapack/getrs.rs:12-38); LUHOT_MODE_FAST uses the FP64 tensor cores
 *    and FMA, with identical pivots wherever the pivot candidates are
 *    distinct and a backward error of the same order.  For a host array
 *    that is not in ndarray's standard layout (F order, negative strides,
 *    padded row views) lair uses its column-major order
 *    (src/lapack/getrf.rs:20-26, 128-213); exact mode follows that order for
 *    at most 4096 rows and returns LUHOT_ERR_UNSUPPORTED beyond, never a
 *    different order.
 *  - A context is safe to share between threads: calls on one context are
 *    serialised by a mutex.  Use one context per thread for concurrency.
 */
#ifndef LUHOT_H
#define LUHOT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define LUHOT_OK 0
#define LUHOT_ERR_INVALID_ARG 1   /* shape / stride / null-pointer error */
#define LUHOT_ERR_CUDA 2          /* a CUDA runtime call failed */
#define LUHOT_ERR_ALLOC 3         /* device or pinned allocation failed */
#define LUHOT_ERR_TIMEOUT 4       /* a device-side bounded wait gave up */
#define LUHOT_ERR_NOT_CONVERGED 5 /* iterative refinement did not reach tol */
#define LUHOT_ERR_SINGULAR 6      /* a solve met an exactly singular factor */
#define LUHOT_ERR_UNSUPPORTED 7   /* size or option outside what is built */

/* Arithmetic modes. */
#define LUHOT_MODE_FAST 0
#define LUHOT_MODE_EXACT 1

typedef struct luhot_ctx luhot_ctx;

/* Library version string, e.g. "0.1.0". */
const char* luhot_version(void);
/* Human-readable name of a status code. */
const char* luhot_status_string(int status);

/* Create a context on `device` (its own CUDA stream and workspace). */
int luhot_create(luhot_ctx** out, int device);
/* Release a context and its device memory.  NULL is accepted. */
void luhot_destroy(luhot_ctx* ctx);
/* Message of the last failed call on this context ("" if none). */
const char* luhot_last_error(const luhot_ctx* ctx);
/* Run subsequent calls on a caller-owned cudaStream_t (NULL: own stream). */
int luhot_set_stream(luhot_ctx* ctx, void* cuda_stream);
/* Panel width override (0 = default 64); for tuning and tests. */
int luhot_set_block(luhot_ctx* ctx, int nb);
/* Schur-update engine of fast-mode FP64 getrf (no lair counterpart).
 * LUHOT_UPDATE_AUTO (default): trailing blocks of at least 256 x 256 are
 * updated on the FP16 tensor cores by an exact integer-slice product (Ozaki
 * scheme: seven 8-bit slices per operand, 28 slice products, FP32 sums that
 * are exact, one FP64 rounding; error at or below an FP64 GEMM's), smaller
 * ones on the FP64 tensor cores (DMMA); the U12 solves of at least 256
 * columns run as the same product, U12 = A12 - (I - L11^-1) A12.
 * LUHOT_UPDATE_DMMA: DMMA updates and FMA substitutions only.
 * LUHOT_UPDATE_OZAKI: the tensor-core product on every block of at least
 * 128 x 64 (U12 solves from 128 columns).  Exact mode and FP32 ignore the
 * setting. */
#define LUHOT_UPDATE_AUTO 0
#define LUHOT_UPDATE_DMMA 1
#define LUHOT_UPDATE_OZAKI 2
int luhot_set_fp64_update(luhot_ctx* ctx, int engine);
/* One trailing update of fast-mode FP64 getrf on its own (no lair
 * counterpart): for the row-major m x n FP64 device matrix d_a (lda),
 *   d_a[k.., k..] -= d_a[k.., 0..k) d_a[0..k), k..],   1 <= k <= 64,
 * with the given LUHOT_UPDATE_* engine (AUTO chooses by size as getrf does).
 * For callers that block their own factorizations, and for tests. */
int luhot_dschur_update_dev(luhot_ctx* ctx, int64_t m, int64_t n, int64_t k, double* d_a, int64_t lda, int engine);
/* Kernel launches issued by this context since creation. */
int64_t luhot_launch_count(const luhot_ctx* ctx);
/* Self-test of the device-side wait limit: launches two CTAs that wait on a
 * grid barrier nothing completes, with the given limit (1..10000 ms).
 * Returns LUHOT_ERR_TIMEOUT and leaves the context usable.  No lair
 * counterpart (lair has no device waits). */
int luhot_selftest_wait_timeout(luhot_ctx* ctx, int64_t timeout_ms);

/* Per-kernel-class CUDA-event profile (no lair counterpart).  Classes:
 * 0 panel, 1 laswp, 2 trsm, 3 Schur GEMM, 4 triangular solve (getrs),
 * 5 permutation, 6 refinement (residual / update), 7 other (in getrf: the
 * operand splits of the tensor-core FP64 update).  flops and bytes are the
 * algorithmic work of the timed launches. */
typedef struct luhot_profile {
  double ms[8];
  double flops[8];
  double bytes[8];
  int64_t launches[8];
} luhot_profile;
/* Enable (1) or disable (0) event bracketing; clears what was recorded. */
int luhot_profile_enable(luhot_ctx* ctx, int on);
/* Synchronise, sum the recorded launches per class into *out, and clear. */
int luhot_profile_read(luhot_ctx* ctx, luhot_profile* out);
/* Measured FP64 tensor-core (DMMA, mma.sync m8n8k4) throughput of this GPU
 * in TFLOP/s, from a register-resident kernel with no memory traffic; the
 * denominator of the FP64 roofline fraction. */
int luhot_measure_dmma_peak(luhot_ctx* ctx, double* tflops);

/* ---- Host-buffer (drop-in) entry points ------------------------------- */

/* LU with partial pivoting of an m x n matrix, in place (the caller's array
 * becomes L\U, in its own layout).  piv receives min(m, n) entries.
 * Replaces lapack::getrf, src/lapack/getrf.rs:12-27 (and through it
 * getrf_row_major :46-120 / getrf_col_major :128-213). */
int luhot_dgetrf(luhot_ctx* ctx, int64_t m, int64_t n, double* a, int64_t rs, int64_t cs,
                 uint64_t* piv, int64_t* singular, int mode);
int luhot_sgetrf(luhot_ctx* ctx, int64_t m, int64_t n, float* a, int64_t rs, int64_t cs,
                 uint64_t* piv, int64_t* singular, int mode);

/* Solve A X = B (trans = 0) or A^T X = B (trans = 1) for nrhs right-hand
 * sides with the factors of luhot_?getrf: lu is n x ncols (only its first n
 * columns are read), piv has n entries, B and X are n x nrhs (X may alias B).
 * Replaces lapack::getrs, src/lapack/getrs.rs:12-38 (one column of B is
 * lair's single right-hand side; trans = 1 has no lair counterpart and
 * serves the adjoint). */
int luhot_dgetrs(luhot_ctx* ctx, int64_t n, int64_t nrhs, const double* lu, int64_t lu_rs,
                 int64_t lu_cs, const uint64_t* piv, const double* b, int64_t b_rs, int64_t b_cs,
                 double* x, int64_t x_rs, int64_t x_cs, int trans, int mode);
int luhot_sgetrs(luhot_ctx* ctx, int64_t n, int64_t nrhs, const float* lu, int64_t lu_rs,
                 int64_t lu_cs, const uint64_t* piv, const float* b, int64_t b_rs, int64_t b_cs,
                 float* x, int64_t x_rs, int64_t x_cs, int trans, int mode);

/* One-shot solve of a square system: the work of equation::solve
 * (src/equation.rs:32-59): factor a copy of A, report singularity
 * (LUHOT_ERR_SINGULAR, A untouched), else solve for nrhs columns. */
int luhot_dgesv(luhot_ctx* ctx, int64_t n, int64_t nrhs, const double* a, int64_t rs,
                int64_t cs, const double* b, int64_t b_rs, int64_t b_cs, double* x, int64_t x_rs,
                int64_t x_cs, int mode);

/* ---- Mixed-precision LU with iterative refinement ---------------------
 * No lair counterpart: an alternative to luhot_dgesv for square FP64
 * systems.  A is factored in a low precision; FP64 is used only for the
 * residual r = b - A x, the update x += d and the stopping test on the
 * normwise backward error ||r||_inf / (||A||_inf ||x||_inf + ||b||_inf) <= tol
 * (tol <= 0 selects n * 2^-53, lair's Real::eps for f64 times n).
 * LUHOT_REFINE_IR: d = (LU)^-1 r in the low precision (converges for
 * kappa * u_low < 1); LUHOT_REFINE_GMRES: d from FP64 GMRES preconditioned
 * by the low-precision LU (Carson & Higham), for larger kappa * u_low. */
/* Factorization precisions.  FP32: FP32 LU on the CUDA cores.  BF16 / FP16:
 * FP32 storage and panels, Schur updates on the tensor cores (tcgen05) with
 * BF16 / FP16 operands scaled per panel by a power of two and FP32
 * accumulation.  TF32: the same with FP32 operands read as TF32.  BF16X3:
 * FP32-accurate Schur updates on the BF16 tensor cores, each FP32 operand
 * split into three BF16 pieces and six piece products accumulated in FP32. */
#define LUHOT_PREC_FP32 0
#define LUHOT_PREC_BF16 1
#define LUHOT_PREC_FP16 2
#define LUHOT_PREC_TF32 3
#define LUHOT_PREC_BF16X3 4
#define LUHOT_REFINE_IR 0
#define LUHOT_REFINE_GMRES 1

typedef struct luhot_ir_info {
  int iterations;         /* refinement steps (max over right-hand sides) */
  int inner_iterations;   /* GMRES iterations, summed (0 for plain IR) */
  int converged;          /* 1 when every column reached tol */
  int precision;          /* LUHOT_PREC_* used for the factorization */
  int solver;             /* LUHOT_REFINE_* */
  double backward_error;  /* final normwise backward error (max over columns) */
  double factor_ms;       /* conversion + low-precision LU (CUDA events) */
  double refine_ms;       /* everything after the factorization */
  int64_t singular;       /* singular step of the low-precision LU, -1 none */
} luhot_ir_info;

/* Device-resident: A (n x n, lda) and B (n x nrhs, ldb) row-major FP64 in HBM
 * are not modified; X (n x nrhs, ldx) receives the solution.  Returns
 * LUHOT_ERR_NOT_CONVERGED (X holds the last iterate) when tol is not reached
 * within max_iter steps or the iteration stops contracting, and
 * LUHOT_ERR_SINGULAR when the low-precision factor is singular. */
int luhot_dgesv_ir_dev(luhot_ctx* ctx, int64_t n, int64_t nrhs, const double* d_a, int64_t lda,
                       const double* d_b, int64_t ldb, double* d_x, int64_t ldx, int precision,
                       int solver, double tol, int max_iter, luhot_ir_info* info);
/* The low-precision factorization of the solves above, on its own: LU with
 * partial pivoting of an m x n row-major FP32 device matrix (lda, in place;
 * int32 pivots), FP32 panels and triangular solves, Schur updates in the
 * given LUHOT_PREC_* (BF16 / FP16 operands scaled per panel by powers of two,
 * TF32 operands rounded to nearest, FP32 accumulation).  For callers that
 * keep the preconditioner themselves, and for measuring its quality.  No
 * lair counterpart. */
int luhot_sgetrf_mixed_dev(luhot_ctx* ctx, int64_t m, int64_t n, float* d_a, int64_t lda, int32_t* d_piv,
                           int precision, int64_t* singular);
/* Host-buffer form of luhot_dgesv_ir_dev (any strides). */
int luhot_dgesv_ir(luhot_ctx* ctx, int64_t n, int64_t nrhs, const double* a, int64_t rs, int64_t cs,
                   const double* b, int64_t b_rs, int64_t b_cs, double* x, int64_t x_rs, int64_t x_cs,
                   int precision, int solver, double tol, int max_iter, luhot_ir_info* info);

/* ---- Adjoint of the solve ----------------------------------------------
 * No lair counterpart (lair has no differentiation).  For X = A^-1 B and a
 * scalar loss with upstream gradient W = dL/dX (n x nrhs):
 *   lambda = A^-T W  (transposed getrs on the stored factors and pivots),
 *   dB = lambda,  dA = -lambda X^T  (skipped when dA is NULL). */
int luhot_dgesv_backward(luhot_ctx* ctx, int64_t n, int64_t nrhs, const double* lu, int64_t lu_rs,
                         int64_t lu_cs, const uint64_t* piv, const double* x, int64_t x_rs, int64_t x_cs,
                         const double* w, int64_t w_rs, int64_t w_cs, double* db, int64_t db_rs,
                         int64_t db_cs, double* da, int64_t da_rs, int64_t da_cs, int mode);
/* Device-resident form: factors (lda) and int32 pivots from luhot_dgetrf_dev. */
int luhot_dgesv_backward_dev(luhot_ctx* ctx, int64_t n, int64_t nrhs, const double* d_lu, int64_t lda,
                             const int32_t* d_piv, const double* d_x, int64_t ldx, const double* d_w,
                             int64_t ldw, double* d_db, int64_t lddb, double* d_da, int64_t ldda, int mode);
/* Mixed-precision form: lambda by refinement on A^T (low-precision factors,
 * FP64 residual; same options and statuses as luhot_dgesv_ir_dev), dA in FP64. */
int luhot_dgesv_backward_ir_dev(luhot_ctx* ctx, int64_t n, int64_t nrhs, const double* d_a, int64_t lda,
                                const double* d_x, int64_t ldx, const double* d_w, int64_t ldw,
                                double* d_db, int64_t lddb, double* d_da, int64_t ldda, int precision,
                                int solver, double tol, int max_iter, luhot_ir_info* info);

/* ---- Batched uneven solves ----------------------------------------------
 * No lair counterpart: lair factors one matrix per call; these factor and
 * solve `count` independent systems A_i x_i = b_i (1 <= n_i <= 256) in one
 * persistent kernel launch replayed from a CUDA graph, with lair's per-system
 * semantics (pivots, last-zero-pivot singular step; LUHOT_MODE_EXACT gives
 * lair's bits for every system).  Packed layout: A_i row-major at element
 * offset sum_{j<i} n_j^2, b_i (overwritten by x_i) and int32 pivots at
 * sum_{j<i} n_j, info[i] = singular step or -1.  dtype 0 = f64, 1 = f32. */
typedef struct luhot_batch luhot_batch;
int luhot_batch_create(luhot_ctx* ctx, int64_t count, const int32_t* sizes, int dtype, int mode,
                       luhot_batch** out);
void luhot_batch_destroy(luhot_batch* plan);
/* Total elements of the packed A and b arrays. */
int luhot_batch_layout(const luhot_batch* plan, int64_t* a_elems, int64_t* b_elems);
/* Choose, per size bucket, the shared-memory path or a panel width (8, 16,
 * 32) by timing each on sample systems copied from d_a / d_b (not modified). */
int luhot_batch_autotune(luhot_batch* plan, const void* d_a, const void* d_b);
/* Chosen per-bucket settings (9 buckets: 0 = shared memory, else the panel
 * width) and the largest n of the shared-memory path. */
int luhot_batch_tuning(const luhot_batch* plan, int32_t* nb_per_bucket, int32_t* smem_n);
/* Factor and solve every system in place on the device (one graph launch). */
int luhot_batch_solve(luhot_batch* plan, void* d_a, void* d_b, int32_t* d_piv, int32_t* d_info);
/* Same with packed host arrays (copied in and out). */
int luhot_batch_solve_host(luhot_batch* plan, void* a, void* b, int32_t* piv, int32_t* info);

/* ---- Device-resident entry points ------------------------------------ */
/* Matrices are row-major on the device with leading dimension ld (elements);
 * pivots are int32 on the device.  The call is asynchronous on the context's
 * stream except where a host output (singular) forces a synchronisation. */

/* In-place LU of a device matrix.  Replaces the same lair code as luhot_dgetrf. */
int luhot_dgetrf_dev(luhot_ctx* ctx, int64_t m, int64_t n, double* d_a, int64_t lda, int32_t* d_piv,
                     int64_t* singular, int mode);
int luhot_sgetrf_dev(luhot_ctx* ctx, int64_t m, int64_t n, float* d_a, int64_t lda, int32_t* d_piv,
                     int64_t* singular, int mode);
/* Solve with device factors; B (n x nrhs, ldb) is overwritten by X. */
int luhot_dgetrs_dev(luhot_ctx* ctx, int64_t n, int64_t nrhs, const double* d_lu, int64_t lda,
                     const int32_t* d_piv, double* d_b, int64_t ldb, int trans, int mode);
int luhot_sgetrs_dev(luhot_ctx* ctx, int64_t n, int64_t nrhs, const float* d_lu, int64_t lda,
                     const int32_t* d_piv, float* d_b, int64_t ldb, int trans, int mode);

/* ---- Device-resident factors ------------------------------------------
 * Replaces lair's lu::Factorized (src/decomposition/lu.rs:12-20, 156-171) and
 * Factorized::solve (lu.rs:87-98) for callers that solve repeatedly: the
 * factored array stays on the GPU with its pivots, the row permutation
 * composed from them and (fast mode) the inverses of the 64 x 64 diagonal
 * blocks, so each solve moves only b and x.  The pivots and the singular step
 * (-1 = None) are returned at creation, as Factorized::from fills its fields;
 * the factored array reaches the host only through luhot_factor_read (what
 * lair's p()/l()/u(), lu.rs:28-72, read).  A factor belongs to the context
 * that made it: destroy it before the context; its calls serialise on the
 * context's lock and run on the context's stream.  Solves need m <= n (lair's
 * getrs asserts a.nrows() == p.len(), src/lapack/getrs.rs:18). */
typedef struct luhot_factor luhot_factor;
int luhot_dfactor_create(luhot_ctx* ctx, int64_t m, int64_t n, const double* a, int64_t rs, int64_t cs, int mode,
                         uint64_t* piv, int64_t* singular, luhot_factor** out);
int luhot_sfactor_create(luhot_ctx* ctx, int64_t m, int64_t n, const float* a, int64_t rs, int64_t cs, int mode,
                         uint64_t* piv, int64_t* singular, luhot_factor** out);
/* Same from a row-major device matrix (not modified). */
int luhot_dfactor_create_dev(luhot_ctx* ctx, int64_t m, int64_t n, const double* d_a, int64_t lda, int mode,
                             uint64_t* piv, int64_t* singular, luhot_factor** out);
/* X = A^-1 B (trans: A^-T B), host B and X with element strides (they may
 * be the same array). */
int luhot_dfactor_solve(luhot_factor* f, int64_t nrhs, const double* b, int64_t b_rs, int64_t b_cs, double* x,
                        int64_t x_rs, int64_t x_cs, int trans);
int luhot_sfactor_solve(luhot_factor* f, int64_t nrhs, const float* b, int64_t b_rs, int64_t b_cs, float* x,
                        int64_t x_rs, int64_t x_cs, int trans);
/* Device B (m x nrhs row-major, ldb), overwritten by X. */
int luhot_dfactor_solve_dev(luhot_factor* f, int64_t nrhs, double* d_b, int64_t ldb, int trans);
/* Copy the factored array (L\U, m x n) to a host array with element strides. */
int luhot_factor_read(luhot_factor* f, void* a, int64_t rs, int64_t cs);
/* The factor's device storage (row-major, lda) and int32 pivots. */
int luhot_factor_device(const luhot_factor* f, const void** d_lu, int64_t* lda, const int32_t** d_piv);
void luhot_factor_destroy(luhot_factor* f);

/* ---- Householder QR ----------------------------------------------------
 * Replaces lair's lapack::geqrf (src/lapack/geqrf.rs:9-27), reached through
 * qr::Factorized::from (src/decomposition/qr.rs:75-86): a (m x n, element
 * strides) is overwritten by R on and above the diagonal and the reflectors
 * below it; tau receives min(m, n) scalars.  LUHOT_MODE_EXACT reproduces
 * lair's arithmetic (larfg's sequential nrm2, larf's increasing-row dots,
 * separately rounded products and sums) bit for bit. */
int luhot_dgeqrf(luhot_ctx* ctx, int64_t m, int64_t n, double* a, int64_t rs, int64_t cs, double* tau, int mode);
int luhot_sgeqrf(luhot_ctx* ctx, int64_t m, int64_t n, float* a, int64_t rs, int64_t cs, float* tau, int mode);
/* Same on a row-major device matrix (leading dimension lda) and device tau. */
int luhot_dgeqrf_dev(luhot_ctx* ctx, int64_t m, int64_t n, double* d_a, int64_t lda, double* d_tau, int mode);
/* Q (m x m, written with element strides q_rs, q_cs) from a factored array
 * and tau: lair's qr::Factorized::q (src/decomposition/qr.rs:26-60). */
int luhot_dqr_q(luhot_ctx* ctx, int64_t m, int64_t n, const double* qr, int64_t rs, int64_t cs, const double* tau,
                double* q, int64_t q_rs, int64_t q_cs, int mode);
int luhot_sqr_q(luhot_ctx* ctx, int64_t m, int64_t n, const float* qr, int64_t rs, int64_t cs, const float* tau,
                float* q, int64_t q_rs, int64_t q_cs, int mode);

/* Scratch held by luhot_dgetrs_dev_noalloc in a static device array. */
#define LUHOT_NOALLOC_SCRATCH_BYTES (4u << 20)

/* luhot_dgetrs_dev without any allocation: for callers that cannot call
 * cudaMalloc, such as programs whose device memory is owned by their own pool
 * or caching allocator, and solve loops that cannot take the device-wide
 * synchronisation cudaMalloc/cudaFree may cause.  It needs no context (a
 * context allocates): its scratch is a static device array of
 * LUHOT_NOALLOC_SCRATCH_BYTES (4 MiB) that every GPU loading this library
 * keeps until exit.  The caller passes factors, pivots and B (overwritten by
 * X) in device memory and the stream to run on (NULL = legacy default).
 * Limit: 4*n rounded up to 256 bytes plus 8*n*nrhs bytes must fit in the
 * scratch, else LUHOT_ERR_UNSUPPORTED (e.g. n = 1024 takes up to 511
 * right-hand sides); nothing else limits nrhs.  The first call on each device
 * looks up the array's device address (cudaGetSymbolAddress), so make that
 * first call before any stream capture; the lookup runs again after the
 * device's context changes (after a cudaDeviceReset), so make the first call
 * after a reset outside any capture too.  All calls share the array: calls
 * that overlap on the GPU race on it.  Exact mode without trans gives the
 * bits of luhot_dgetrs_dev (lair's order); fast mode and trans agree with it
 * to fast-mode rounding (the sweeps group the sums differently).  No
 * counterpart in lair (lair's getrs allocates its result on the host). */
int luhot_dgetrs_dev_noalloc(int64_t n, int64_t nrhs, const double* d_lu, int64_t lda,
                             const int32_t* d_piv, double* d_b, int64_t ldb, int trans, int mode,
                             void* cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* LUHOT_H */
