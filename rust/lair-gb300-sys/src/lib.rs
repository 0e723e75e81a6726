//! Raw FFI bindings of `include/luhot.h`, the C ABI of `liblair_gb300.so`.
//!
//! lair's `lapack::getrf` / `lapack::getrs` (and through them
//! `equation::solve` and `lu::Factorized`) call these from its `gb300`
//! feature for `f64` and `f32` (see `rust/lair-shim/gpu.rs`); every other
//! element type keeps lair's own code.  The meaning of each argument, the
//! status codes and the threading rules are those of the header.
//!
//! Unbuilt in this repository: no machine of this project has cargo.  The
//! declarations are checked against the header by
//! `tests/test_rust_bindings.py` (names, argument counts, constants).
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_void};

pub const LUHOT_OK: c_int = 0;
pub const LUHOT_ERR_INVALID_ARG: c_int = 1;
pub const LUHOT_ERR_CUDA: c_int = 2;
pub const LUHOT_ERR_ALLOC: c_int = 3;
pub const LUHOT_ERR_TIMEOUT: c_int = 4;
pub const LUHOT_ERR_NOT_CONVERGED: c_int = 5;
pub const LUHOT_ERR_SINGULAR: c_int = 6;
pub const LUHOT_ERR_UNSUPPORTED: c_int = 7;

pub const LUHOT_MODE_FAST: c_int = 0;
pub const LUHOT_MODE_EXACT: c_int = 1;

pub const LUHOT_UPDATE_AUTO: c_int = 0;
pub const LUHOT_UPDATE_DMMA: c_int = 1;
pub const LUHOT_UPDATE_OZAKI: c_int = 2;

pub const LUHOT_PREC_FP32: c_int = 0;
pub const LUHOT_PREC_BF16: c_int = 1;
pub const LUHOT_PREC_FP16: c_int = 2;
pub const LUHOT_PREC_TF32: c_int = 3;
pub const LUHOT_PREC_BF16X3: c_int = 4;
pub const LUHOT_REFINE_IR: c_int = 0;
pub const LUHOT_REFINE_GMRES: c_int = 1;

pub const LUHOT_NOALLOC_SCRATCH_BYTES: usize = 4 << 20;

#[repr(C)]
pub struct luhot_ctx {
    _private: [u8; 0],
}
#[repr(C)]
pub struct luhot_factor {
    _private: [u8; 0],
}
#[repr(C)]
pub struct luhot_batch {
    _private: [u8; 0],
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct luhot_profile {
    pub ms: [f64; 8],
    pub flops: [f64; 8],
    pub bytes: [f64; 8],
    pub launches: [i64; 8],
}

#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct luhot_ir_info {
    pub iterations: c_int,
    pub inner_iterations: c_int,
    pub converged: c_int,
    pub precision: c_int,
    pub solver: c_int,
    pub backward_error: f64,
    pub factor_ms: f64,
    pub refine_ms: f64,
    pub singular: i64,
}

extern "C" {
    pub fn luhot_version() -> *const c_char;
    pub fn luhot_status_string(status: c_int) -> *const c_char;

    pub fn luhot_create(out: *mut *mut luhot_ctx, device: c_int) -> c_int;
    pub fn luhot_destroy(ctx: *mut luhot_ctx);
    pub fn luhot_last_error(ctx: *const luhot_ctx) -> *const c_char;
    pub fn luhot_set_stream(ctx: *mut luhot_ctx, cuda_stream: *mut c_void) -> c_int;
    pub fn luhot_set_block(ctx: *mut luhot_ctx, nb: c_int) -> c_int;
    pub fn luhot_set_fp64_update(ctx: *mut luhot_ctx, engine: c_int) -> c_int;
    pub fn luhot_dschur_update_dev(ctx: *mut luhot_ctx, m: i64, n: i64, k: i64, d_a: *mut f64, lda: i64,
                                   engine: c_int) -> c_int;
    pub fn luhot_launch_count(ctx: *const luhot_ctx) -> i64;
    pub fn luhot_selftest_wait_timeout(ctx: *mut luhot_ctx, timeout_ms: i64) -> c_int;
    pub fn luhot_profile_enable(ctx: *mut luhot_ctx, on: c_int) -> c_int;
    pub fn luhot_profile_read(ctx: *mut luhot_ctx, out: *mut luhot_profile) -> c_int;
    pub fn luhot_measure_dmma_peak(ctx: *mut luhot_ctx, tflops: *mut f64) -> c_int;

    // lapack::getrf (src/lapack/getrf.rs:12-27) and lapack::getrs (src/lapack/getrs.rs:12-38)
    pub fn luhot_dgetrf(ctx: *mut luhot_ctx, m: i64, n: i64, a: *mut f64, rs: i64, cs: i64, piv: *mut u64,
                        singular: *mut i64, mode: c_int) -> c_int;
    pub fn luhot_sgetrf(ctx: *mut luhot_ctx, m: i64, n: i64, a: *mut f32, rs: i64, cs: i64, piv: *mut u64,
                        singular: *mut i64, mode: c_int) -> c_int;
    pub fn luhot_dgetrs(ctx: *mut luhot_ctx, n: i64, nrhs: i64, lu: *const f64, lu_rs: i64, lu_cs: i64,
                        piv: *const u64, b: *const f64, b_rs: i64, b_cs: i64, x: *mut f64, x_rs: i64, x_cs: i64,
                        trans: c_int, mode: c_int) -> c_int;
    pub fn luhot_sgetrs(ctx: *mut luhot_ctx, n: i64, nrhs: i64, lu: *const f32, lu_rs: i64, lu_cs: i64,
                        piv: *const u64, b: *const f32, b_rs: i64, b_cs: i64, x: *mut f32, x_rs: i64, x_cs: i64,
                        trans: c_int, mode: c_int) -> c_int;
    // equation::solve (src/equation.rs:32-59)
    pub fn luhot_dgesv(ctx: *mut luhot_ctx, n: i64, nrhs: i64, a: *const f64, rs: i64, cs: i64, b: *const f64,
                       b_rs: i64, b_cs: i64, x: *mut f64, x_rs: i64, x_cs: i64, mode: c_int) -> c_int;

    // Mixed precision with FP64 refinement (no lair counterpart)
    pub fn luhot_dgesv_ir_dev(ctx: *mut luhot_ctx, n: i64, nrhs: i64, d_a: *const f64, lda: i64, d_b: *const f64,
                              ldb: i64, d_x: *mut f64, ldx: i64, precision: c_int, solver: c_int, tol: f64,
                              max_iter: c_int, info: *mut luhot_ir_info) -> c_int;
    pub fn luhot_sgetrf_mixed_dev(ctx: *mut luhot_ctx, m: i64, n: i64, d_a: *mut f32, lda: i64, d_piv: *mut i32,
                                  precision: c_int, singular: *mut i64) -> c_int;
    pub fn luhot_dgesv_ir(ctx: *mut luhot_ctx, n: i64, nrhs: i64, a: *const f64, rs: i64, cs: i64, b: *const f64,
                          b_rs: i64, b_cs: i64, x: *mut f64, x_rs: i64, x_cs: i64, precision: c_int,
                          solver: c_int, tol: f64, max_iter: c_int, info: *mut luhot_ir_info) -> c_int;

    // Adjoint of the solve (no lair counterpart)
    pub fn luhot_dgesv_backward(ctx: *mut luhot_ctx, n: i64, nrhs: i64, lu: *const f64, lu_rs: i64, lu_cs: i64,
                                piv: *const u64, x: *const f64, x_rs: i64, x_cs: i64, w: *const f64, w_rs: i64,
                                w_cs: i64, db: *mut f64, db_rs: i64, db_cs: i64, da: *mut f64, da_rs: i64,
                                da_cs: i64, mode: c_int) -> c_int;
    pub fn luhot_dgesv_backward_dev(ctx: *mut luhot_ctx, n: i64, nrhs: i64, d_lu: *const f64, lda: i64,
                                    d_piv: *const i32, d_x: *const f64, ldx: i64, d_w: *const f64, ldw: i64,
                                    d_db: *mut f64, lddb: i64, d_da: *mut f64, ldda: i64, mode: c_int) -> c_int;
    pub fn luhot_dgesv_backward_ir_dev(ctx: *mut luhot_ctx, n: i64, nrhs: i64, d_a: *const f64, lda: i64,
                                       d_x: *const f64, ldx: i64, d_w: *const f64, ldw: i64, d_db: *mut f64,
                                       lddb: i64, d_da: *mut f64, ldda: i64, precision: c_int, solver: c_int,
                                       tol: f64, max_iter: c_int, info: *mut luhot_ir_info) -> c_int;

    // Batched uneven solves (no lair counterpart)
    pub fn luhot_batch_create(ctx: *mut luhot_ctx, count: i64, sizes: *const i32, dtype: c_int, mode: c_int,
                              out: *mut *mut luhot_batch) -> c_int;
    pub fn luhot_batch_destroy(plan: *mut luhot_batch);
    pub fn luhot_batch_layout(plan: *const luhot_batch, a_elems: *mut i64, b_elems: *mut i64) -> c_int;
    pub fn luhot_batch_autotune(plan: *mut luhot_batch, d_a: *const c_void, d_b: *const c_void) -> c_int;
    pub fn luhot_batch_tuning(plan: *const luhot_batch, nb_per_bucket: *mut i32, smem_n: *mut i32) -> c_int;
    pub fn luhot_batch_solve(plan: *mut luhot_batch, d_a: *mut c_void, d_b: *mut c_void, d_piv: *mut i32,
                             d_info: *mut i32) -> c_int;
    pub fn luhot_batch_solve_host(plan: *mut luhot_batch, a: *mut c_void, b: *mut c_void, piv: *mut i32,
                                  info: *mut i32) -> c_int;

    // Device-resident entry points
    pub fn luhot_dgetrf_dev(ctx: *mut luhot_ctx, m: i64, n: i64, d_a: *mut f64, lda: i64, d_piv: *mut i32,
                            singular: *mut i64, mode: c_int) -> c_int;
    pub fn luhot_sgetrf_dev(ctx: *mut luhot_ctx, m: i64, n: i64, d_a: *mut f32, lda: i64, d_piv: *mut i32,
                            singular: *mut i64, mode: c_int) -> c_int;
    pub fn luhot_dgetrs_dev(ctx: *mut luhot_ctx, n: i64, nrhs: i64, d_lu: *const f64, lda: i64, d_piv: *const i32,
                            d_b: *mut f64, ldb: i64, trans: c_int, mode: c_int) -> c_int;
    pub fn luhot_sgetrs_dev(ctx: *mut luhot_ctx, n: i64, nrhs: i64, d_lu: *const f32, lda: i64, d_piv: *const i32,
                            d_b: *mut f32, ldb: i64, trans: c_int, mode: c_int) -> c_int;

    // lu::Factorized with device-resident factors (src/decomposition/lu.rs:12-20, 87-98, 156-171)
    pub fn luhot_dfactor_create(ctx: *mut luhot_ctx, m: i64, n: i64, a: *const f64, rs: i64, cs: i64, mode: c_int,
                                piv: *mut u64, singular: *mut i64, out: *mut *mut luhot_factor) -> c_int;
    pub fn luhot_sfactor_create(ctx: *mut luhot_ctx, m: i64, n: i64, a: *const f32, rs: i64, cs: i64, mode: c_int,
                                piv: *mut u64, singular: *mut i64, out: *mut *mut luhot_factor) -> c_int;
    pub fn luhot_dfactor_create_dev(ctx: *mut luhot_ctx, m: i64, n: i64, d_a: *const f64, lda: i64, mode: c_int,
                                    piv: *mut u64, singular: *mut i64, out: *mut *mut luhot_factor) -> c_int;
    pub fn luhot_dfactor_solve(f: *mut luhot_factor, nrhs: i64, b: *const f64, b_rs: i64, b_cs: i64, x: *mut f64,
                               x_rs: i64, x_cs: i64, trans: c_int) -> c_int;
    pub fn luhot_sfactor_solve(f: *mut luhot_factor, nrhs: i64, b: *const f32, b_rs: i64, b_cs: i64, x: *mut f32,
                               x_rs: i64, x_cs: i64, trans: c_int) -> c_int;
    pub fn luhot_dfactor_solve_dev(f: *mut luhot_factor, nrhs: i64, d_b: *mut f64, ldb: i64, trans: c_int) -> c_int;
    pub fn luhot_factor_read(f: *mut luhot_factor, a: *mut c_void, rs: i64, cs: i64) -> c_int;
    pub fn luhot_factor_device(f: *const luhot_factor, d_lu: *mut *const c_void, lda: *mut i64,
                               d_piv: *mut *const i32) -> c_int;
    pub fn luhot_factor_destroy(f: *mut luhot_factor);

    // lapack::geqrf (src/lapack/geqrf.rs:9-27) and qr::Factorized::q (src/decomposition/qr.rs:26-60)
    pub fn luhot_dgeqrf(ctx: *mut luhot_ctx, m: i64, n: i64, a: *mut f64, rs: i64, cs: i64, tau: *mut f64,
                        mode: c_int) -> c_int;
    pub fn luhot_sgeqrf(ctx: *mut luhot_ctx, m: i64, n: i64, a: *mut f32, rs: i64, cs: i64, tau: *mut f32,
                        mode: c_int) -> c_int;
    pub fn luhot_dgeqrf_dev(ctx: *mut luhot_ctx, m: i64, n: i64, d_a: *mut f64, lda: i64, d_tau: *mut f64,
                            mode: c_int) -> c_int;
    pub fn luhot_dqr_q(ctx: *mut luhot_ctx, m: i64, n: i64, qr: *const f64, rs: i64, cs: i64, tau: *const f64,
                       q: *mut f64, q_rs: i64, q_cs: i64, mode: c_int) -> c_int;
    pub fn luhot_sqr_q(ctx: *mut luhot_ctx, m: i64, n: i64, qr: *const f32, rs: i64, cs: i64, tau: *const f32,
                       q: *mut f32, q_rs: i64, q_cs: i64, mode: c_int) -> c_int;

    // Allocation-free getrs (no context; static device scratch; see the header)
    pub fn luhot_dgetrs_dev_noalloc(n: i64, nrhs: i64, d_lu: *const f64, lda: i64, d_piv: *const i32,
                                    d_b: *mut f64, ldb: i64, trans: c_int, mode: c_int,
                                    cuda_stream: *mut c_void) -> c_int;
}
