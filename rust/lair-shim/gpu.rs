//! GB300 path of lair's LU, for `src/lapack/gpu.rs` inside lair 0.8.0.
//!
//! Unbuilt in this repository (no machine of this project has cargo); it is
//! the code a lair maintainer adds behind a `gb300` feature, with these hooks
//! in lair's own files (no public signature changes):
//!
//! ```text
//! // src/lapack/mod.rs
//! #[cfg(feature = "gb300")] pub(crate) mod gpu;
//!
//! // src/lapack/getrf.rs, first lines of `getrf` (getrf.rs:12)
//! #[cfg(feature = "gb300")]
//! if let Some(r) = crate::lapack::gpu::try_getrf(&mut a) { return r; }
//!
//! // src/lapack/getrs.rs, after the three assert!s of `getrs` (getrs.rs:18-20)
//! #[cfg(feature = "gb300")]
//! if let Some(x) = crate::lapack::gpu::try_getrs(a, p, b) { return x; }
//! ```
//!
//! and, in Cargo.toml, `lair-gb300-sys = { path = "…/rust/lair-gb300-sys", optional = true }`
//! with `gb300 = ["lair-gb300-sys"]`.  f64 and f32 go to the GPU (chosen by
//! `TypeId`, legal because `Scalar: 'static`, src/scalar.rs:344); complex
//! element types return `None` and keep lair's code.  A CUDA failure panics
//! with the library's message: it is never turned into a silent CPU result.
//! `LAIR_GB300_EXACT=1` selects the exact mode (lair's rounding bit for bit).

use std::any::TypeId;
use std::ffi::CStr;
use std::ptr;

use lair_gb300_sys as sys;
use ndarray::{Array1, ArrayBase, ArrayViewMut2, Axis, Data, Ix1, Ix2};

use crate::Scalar;

/// One luhot context per thread: calls on different threads run concurrently
/// (the library is thread-safe across contexts).
struct Ctx(*mut sys::luhot_ctx);

impl Ctx {
    fn new() -> Ctx {
        let mut c = ptr::null_mut();
        let rc = unsafe { sys::luhot_create(&mut c, 0) };
        assert_eq!(rc, sys::LUHOT_OK, "luhot_create failed (status {rc}): a CUDA GPU is required");
        Ctx(c)
    }
    fn error(&self) -> String {
        unsafe { CStr::from_ptr(sys::luhot_last_error(self.0)) }.to_string_lossy().into_owned()
    }
}

impl Drop for Ctx {
    fn drop(&mut self) {
        unsafe { sys::luhot_destroy(self.0) }
    }
}

thread_local!(static CTX: Ctx = Ctx::new());

fn mode() -> i32 {
    match std::env::var("LAIR_GB300_EXACT") {
        Ok(v) if v == "1" => sys::LUHOT_MODE_EXACT,
        _ => sys::LUHOT_MODE_FAST,
    }
}

/// `lapack::getrf` for f64 / f32 on the GPU; `None` for other element types.
pub(crate) fn try_getrf<A: Scalar>(a: &mut ArrayViewMut2<A>) -> Option<(Vec<usize>, Option<usize>)> {
    let (m, n) = (a.nrows() as i64, a.ncols() as i64);
    let (rs, cs) = (a.stride_of(Axis(0)) as i64, a.stride_of(Axis(1)) as i64);
    let mut piv = vec![0u64; m.min(n) as usize];
    let mut singular = -1i64;
    let f64_ = TypeId::of::<A>() == TypeId::of::<f64>();
    if !f64_ && TypeId::of::<A>() != TypeId::of::<f32>() {
        return None;
    }
    CTX.with(|c| {
        let rc = unsafe {
            if f64_ {
                sys::luhot_dgetrf(c.0, m, n, a.as_mut_ptr() as *mut f64, rs, cs, piv.as_mut_ptr(), &mut singular,
                                  mode())
            } else {
                sys::luhot_sgetrf(c.0, m, n, a.as_mut_ptr() as *mut f32, rs, cs, piv.as_mut_ptr(), &mut singular,
                                  mode())
            }
        };
        assert_eq!(rc, sys::LUHOT_OK, "luhot getrf failed: {}", c.error());
    });
    Some((piv.into_iter().map(|p| p as usize).collect(), (singular >= 0).then(|| singular as usize)))
}

/// `lapack::getrs` for f64 / f32 on the GPU (lair's asserts already ran).
pub(crate) fn try_getrs<A, SA, SB>(a: &ArrayBase<SA, Ix2>, p: &[usize], b: &ArrayBase<SB, Ix1>) -> Option<Array1<A>>
where
    A: Scalar,
    SA: Data<Elem = A>,
    SB: Data<Elem = A>,
{
    let f64_ = TypeId::of::<A>() == TypeId::of::<f64>();
    if !f64_ && TypeId::of::<A>() != TypeId::of::<f32>() {
        return None;
    }
    let n = a.nrows() as i64;
    let piv: Vec<u64> = p.iter().map(|&v| v as u64).collect();
    let mut x = Array1::<A>::zeros(a.nrows());
    let (ars, acs) = (a.stride_of(Axis(0)) as i64, a.stride_of(Axis(1)) as i64);
    let brs = b.stride_of(Axis(0)) as i64;
    CTX.with(|c| {
        let rc = unsafe {
            if f64_ {
                sys::luhot_dgetrs(c.0, n, 1, a.as_ptr() as *const f64, ars, acs, piv.as_ptr(),
                                  b.as_ptr() as *const f64, brs, 1, x.as_mut_ptr() as *mut f64, 1, 1, 0, mode())
            } else {
                sys::luhot_sgetrs(c.0, n, 1, a.as_ptr() as *const f32, ars, acs, piv.as_ptr(),
                                  b.as_ptr() as *const f32, brs, 1, x.as_mut_ptr() as *mut f32, 1, 1, 0, mode())
            }
        };
        assert_eq!(rc, sys::LUHOT_OK, "luhot getrs failed: {}", c.error());
    });
    Some(x)
}

/// Factors kept on the device for `lu::Factorized` (one more private field
/// there, behind the feature): `From` fills `pivots` / `singular` from
/// `new`, `solve` calls `solve`, and `p()` / `l()` / `u()` / `into_pl()` call
/// `sync_into` once before lair's host code reads `lu`.
pub(crate) struct Resident {
    f: *mut sys::luhot_factor,
    f64_: bool,
}

impl Resident {
    pub(crate) fn new<A: Scalar, S: Data<Elem = A>>(a: &ArrayBase<S, Ix2>)
                                                    -> Option<(Resident, Vec<usize>, Option<usize>)> {
        let f64_ = TypeId::of::<A>() == TypeId::of::<f64>();
        if !f64_ && TypeId::of::<A>() != TypeId::of::<f32>() {
            return None;
        }
        let (m, n) = (a.nrows() as i64, a.ncols() as i64);
        let (rs, cs) = (a.stride_of(Axis(0)) as i64, a.stride_of(Axis(1)) as i64);
        let mut piv = vec![0u64; m.min(n) as usize];
        let mut singular = -1i64;
        let mut f = ptr::null_mut();
        CTX.with(|c| {
            let rc = unsafe {
                if f64_ {
                    sys::luhot_dfactor_create(c.0, m, n, a.as_ptr() as *const f64, rs, cs, mode(), piv.as_mut_ptr(),
                                              &mut singular, &mut f)
                } else {
                    sys::luhot_sfactor_create(c.0, m, n, a.as_ptr() as *const f32, rs, cs, mode(), piv.as_mut_ptr(),
                                              &mut singular, &mut f)
                }
            };
            assert_eq!(rc, sys::LUHOT_OK, "luhot factor failed: {}", c.error());
        });
        Some((Resident { f, f64_ }, piv.into_iter().map(|p| p as usize).collect(),
              (singular >= 0).then(|| singular as usize)))
    }

    pub(crate) fn solve<A: Scalar, SB: Data<Elem = A>>(&self, b: &ArrayBase<SB, Ix1>) -> Array1<A> {
        let mut x = Array1::<A>::zeros(b.len());
        let brs = b.stride_of(Axis(0)) as i64;
        let rc = unsafe {
            if self.f64_ {
                sys::luhot_dfactor_solve(self.f, 1, b.as_ptr() as *const f64, brs, 1, x.as_mut_ptr() as *mut f64, 1,
                                         1, 0)
            } else {
                sys::luhot_sfactor_solve(self.f, 1, b.as_ptr() as *const f32, brs, 1, x.as_mut_ptr() as *mut f32, 1,
                                         1, 0)
            }
        };
        assert_eq!(rc, sys::LUHOT_OK, "luhot factor solve failed (status {rc})");
        x
    }

    /// Writes L\U into lair's host array (the layout it already has).
    pub(crate) fn sync_into<A: Scalar>(&self, lu: &mut ArrayViewMut2<A>) {
        let (rs, cs) = (lu.stride_of(Axis(0)) as i64, lu.stride_of(Axis(1)) as i64);
        let rc = unsafe { sys::luhot_factor_read(self.f, lu.as_mut_ptr() as *mut std::os::raw::c_void, rs, cs) };
        assert_eq!(rc, sys::LUHOT_OK, "luhot factor read failed (status {rc})");
    }
}

impl Drop for Resident {
    fn drop(&mut self) {
        unsafe { sys::luhot_factor_destroy(self.f) }
    }
}
