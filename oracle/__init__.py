"""CPU oracle for lair's LU path (test infrastructure only).

This package wraps ``liblair_oracle.so``, a C++ restatement of lair 0.8.0's
``getrf``/``getrs``/``laswp``/``iamax`` (``src/lapack/getrf.rs``,
``src/lapack/getrs.rs``, ``src/lapack/laswp.rs``, ``src/blas/iamax.rs``) that
keeps lair's operation order and rounding.  Only the tests, the smoke check
and the benchmark's CPU-baseline leg may import it; the GPU library never
calls it.

Arrays are numpy views with any strides (C order, F order, negative), which
map one to one onto ndarray views.  Functions mutate their input exactly as
the lair function does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liblair_oracle.so")
_lib = None

_i64 = ctypes.c_int64
_vp = ctypes.c_void_p


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH)
        < max(os.path.getmtime(os.path.join(_HERE, f)) for f in ("lair_oracle.cpp", "lair_oracle.h"))
    ):
        subprocess.run(["make", "-s"] + (["-B"] if force else []) + ["-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        for name in ("oracle_dgetrf_row_major", "oracle_sgetrf_row_major"):
            getattr(L, name).argtypes = [_i64, _i64, _vp, _i64, _i64, _vp, _i64]
            getattr(L, name).restype = _i64
        for name in ("oracle_dgetrf_col_major", "oracle_sgetrf_col_major", "oracle_dgetrf", "oracle_sgetrf"):
            getattr(L, name).argtypes = [_i64, _i64, _vp, _i64, _i64, _vp]
            getattr(L, name).restype = _i64
        L.oracle_dgetrf_row_major_range.argtypes = [_i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64]
        L.oracle_dgetrf_row_major_range.restype = _i64
        L.oracle_dgetrf_row_major_blocked.argtypes = [_i64, _i64, _vp, _i64, _vp, _i64, ctypes.c_int, _vp, _vp]
        L.oracle_dgetrf_row_major_blocked.restype = _i64
        L.oracle_dgetrf_recursive.argtypes = [_i64, _i64, _vp, _i64, _i64, _vp, _vp]
        L.oracle_dgetrf_recursive.restype = ctypes.c_int
        for name in ("oracle_dgetrs", "oracle_sgetrs"):
            getattr(L, name).argtypes = [_i64, _i64, _vp, _i64, _i64, _vp, _vp, _i64, _vp]
            getattr(L, name).restype = None
        for name in ("oracle_dlaswp", "oracle_slaswp"):
            getattr(L, name).argtypes = [_i64, _vp, _i64, _i64, _i64, _vp, _i64]
            getattr(L, name).restype = None
        for name in ("oracle_diamax", "oracle_siamax"):
            getattr(L, name).argtypes = [_i64, _vp, _i64, _vp]
            getattr(L, name).restype = _i64
        L.oracle_is_standard_layout.argtypes = [_i64, _i64, _i64, _i64]
        L.oracle_is_standard_layout.restype = ctypes.c_int
        L.oracle_ddot.argtypes = [_i64, _vp, _i64, _vp, _i64]
        L.oracle_ddot.restype = ctypes.c_double
        L.oracle_dgemv_notrans.argtypes = [_i64, _i64, ctypes.c_double, _vp, _i64, _i64, _vp, _i64,
                                           ctypes.c_double, _vp, _i64]
        L.oracle_dgemv_notrans.restype = None
        for name in ("oracle_dgeqrf", "oracle_sgeqrf"):
            getattr(L, name).argtypes = [_i64, _i64, _vp, _i64, _i64, _vp]
            getattr(L, name).restype = None
        for name in ("oracle_dqr_q", "oracle_sqr_q"):
            getattr(L, name).argtypes = [_i64, _i64, _vp, _i64, _i64, _vp, _i64, _vp]
            getattr(L, name).restype = None
        L.oracle_dlarfg.argtypes = [ctypes.c_double, _i64, _vp, _i64, _vp, _vp]
        L.oracle_dlarfg.restype = None
        L.oracle_dlarf_left.argtypes = [_i64, _i64, _vp, _i64, ctypes.c_double, _vp, _i64, _i64]
        L.oracle_dlarf_left.restype = None
        L.oracle_dnrm2.argtypes = [_i64, _vp, _i64]
        L.oracle_dnrm2.restype = ctypes.c_double
        _lib = L
    return _lib


def _prefix(a: np.ndarray) -> str:
    if a.dtype == np.float64:
        return "d"
    if a.dtype == np.float32:
        return "s"
    raise TypeError(f"oracle supports float64/float32, got {a.dtype}")


def _estrides(a: np.ndarray):
    return tuple(s // a.itemsize for s in a.strides)


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _singular(v: int):
    return None if v < 0 else int(v)


def is_standard_layout(a: np.ndarray) -> bool:
    m, n = a.shape
    rs, cs = _estrides(a)
    return bool(lib().oracle_is_standard_layout(m, n, rs, cs))


def iamax(x: np.ndarray):
    """src/blas/iamax.rs:6-21 -> (index, max |x|)."""
    p = _prefix(x)
    mv = np.zeros(1, dtype=x.dtype)
    idx = getattr(lib(), f"oracle_{p}iamax")(x.shape[0], _ptr(x), _estrides(x)[0], _ptr(mv))
    return int(idx), mv[0].item()


def laswp(a: np.ndarray, begin: int, piv) -> None:
    """src/lapack/laswp.rs:11-40, on every column of a 2-D view (in place)."""
    p = _prefix(a)
    pv = np.ascontiguousarray(np.asarray(piv, dtype=np.uint64))
    rs, cs = _estrides(a)
    getattr(lib(), f"oracle_{p}laswp")(a.shape[1], _ptr(a), rs, cs, begin, _ptr(pv), pv.shape[0])


def getrf(a: np.ndarray):
    """src/lapack/getrf.rs:12-27: factor ``a`` in place; returns (pivots, singular)."""
    p = _prefix(a)
    m, n = a.shape
    rs, cs = _estrides(a)
    piv = np.zeros(min(m, n), dtype=np.uint64)
    s = getattr(lib(), f"oracle_{p}getrf")(m, n, _ptr(a), rs, cs, _ptr(piv))
    return [int(v) for v in piv], _singular(s)


def getrf_row_major(a: np.ndarray, max_steps: int = -1):
    """src/lapack/getrf.rs:46-120 regardless of layout; optional step limit."""
    p = _prefix(a)
    m, n = a.shape
    rs, cs = _estrides(a)
    piv = np.arange(min(m, n), dtype=np.uint64)
    s = getattr(lib(), f"oracle_{p}getrf_row_major")(m, n, _ptr(a), rs, cs, _ptr(piv), max_steps)
    return [int(v) for v in piv], _singular(s)


def getrf_row_major_range(a: np.ndarray, piv: np.ndarray, step_begin: int, step_end: int):
    """Elimination steps [step_begin, step_end) of getrf_row_major on a float64 view.

    ``piv`` is a uint64 array of min(m, n) entries carried between calls.
    """
    m, n = a.shape
    rs, cs = _estrides(a)
    s = lib().oracle_dgetrf_row_major_range(m, n, _ptr(a), rs, cs, _ptr(piv), step_begin, step_end)
    return _singular(s)


def getrf_row_major_blocked(a: np.ndarray, block: int = 64, threads: int = 0, margins: bool = False):
    """getrf_row_major (src/lapack/getrf.rs:46-120) on a C-order float64 array,
    bit-identical, in blocks of ``block`` steps on ``threads`` threads (0: all
    cores), for large fixtures.  Returns (pivots, singular) or, with
    ``margins``, (pivots, singular, colmax, gap): per step the largest pivot
    candidate |a| and its margin over the second largest."""
    if a.dtype != np.float64 or not a.flags.c_contiguous and a.strides[1] != a.itemsize:
        raise TypeError("blocked oracle: float64 with unit column stride")
    m, n = a.shape
    lda = a.strides[0] // a.itemsize if m > 1 else n
    k = min(m, n)
    piv = np.arange(k, dtype=np.uint64)
    colmax = np.zeros(max(k, 1)) if margins else None
    gap = np.zeros(max(k, 1)) if margins else None
    threads = threads or (os.cpu_count() or 1)
    s = lib().oracle_dgetrf_row_major_blocked(m, n, _ptr(a), lda, _ptr(piv), block, threads,
                                              _ptr(colmax) if margins else None, _ptr(gap) if margins else None)
    if margins:
        return piv, _singular(s), colmax[:k], gap[:k]
    return piv, _singular(s)


def getrf_col_major(a: np.ndarray):
    """src/lapack/getrf.rs:128-213 regardless of layout."""
    p = _prefix(a)
    m, n = a.shape
    rs, cs = _estrides(a)
    piv = np.arange(min(m, n), dtype=np.uint64)
    s = getattr(lib(), f"oracle_{p}getrf_col_major")(m, n, _ptr(a), rs, cs, _ptr(piv))
    return [int(v) for v in piv], _singular(s)


def getrf_recursive(a: np.ndarray):
    """src/lapack/getrf.rs:29-40 -> (ok, pivots, singular_row)."""
    if a.dtype != np.float64:
        raise TypeError("recursive oracle is float64 only")
    m, n = a.shape
    rs, cs = _estrides(a)
    piv = np.zeros(m, dtype=np.uint64)
    row = np.zeros(1, dtype=np.int64)
    err = lib().oracle_dgetrf_recursive(m, n, _ptr(a), rs, cs, _ptr(piv), _ptr(row))
    return err == 0, [int(v) for v in piv], (None if err == 0 else int(row[0]))


def getrs(lu: np.ndarray, piv, b: np.ndarray) -> np.ndarray:
    """src/lapack/getrs.rs:12-38 for one right-hand side; returns a new array."""
    p = _prefix(lu)
    m, ncols = lu.shape
    pv = np.ascontiguousarray(np.asarray(piv, dtype=np.uint64))
    if not (m == pv.shape[0] == b.shape[0] and ncols >= pv.shape[0]):
        raise AssertionError("getrs: nrows == p.len() == b.len() and ncols >= p.len() required")
    rs, cs = _estrides(lu)
    x = np.empty(m, dtype=lu.dtype)
    getattr(lib(), f"oracle_{p}getrs")(m, ncols, _ptr(lu), rs, cs, _ptr(pv), _ptr(b), _estrides(b)[0], _ptr(x))
    return x


def getrs_multi(lu: np.ndarray, piv, B: np.ndarray) -> np.ndarray:
    """lair's single-RHS getrs applied column by column to an n x nrhs block."""
    return np.stack([getrs(lu, piv, np.ascontiguousarray(B[:, j])) for j in range(B.shape[1])], axis=1)


def dot(x: np.ndarray, y: np.ndarray, n: int) -> float:
    return lib().oracle_ddot(n, _ptr(x), _estrides(x)[0], _ptr(y), _estrides(y)[0])


# ------------------------------------------------------------------- QR
def geqrf(a: np.ndarray) -> np.ndarray:
    """src/lapack/geqrf.rs:9-27: Householder QR of ``a`` in place; returns tau."""
    p = _prefix(a)
    m, n = a.shape
    rs, cs = _estrides(a)
    tau = np.zeros(min(m, n), dtype=a.dtype)
    getattr(lib(), f"oracle_{p}geqrf")(m, n, _ptr(a), rs, cs, _ptr(tau))
    return tau


def qr_q(qr: np.ndarray, tau: np.ndarray) -> np.ndarray:
    """src/decomposition/qr.rs:26-60: Q (m x m) from the factored array and tau."""
    p = _prefix(qr)
    m, n = qr.shape
    rs, cs = _estrides(qr)
    t = np.ascontiguousarray(tau, dtype=qr.dtype)
    q = np.zeros((m, m), dtype=qr.dtype)
    getattr(lib(), f"oracle_{p}qr_q")(m, n, _ptr(qr), rs, cs, _ptr(t), t.shape[0], _ptr(q))
    return q


def qr_r(qr: np.ndarray) -> np.ndarray:
    """src/decomposition/qr.rs:63-72: the array with its strictly lower part zeroed."""
    r = qr.copy()
    for i in range(1, r.shape[0]):
        r[i, : min(i, r.shape[1])] = 0
    return r


def larfg(alpha: float, x: np.ndarray):
    """src/lapack/larfg.rs:9-43 (float64): scales x in place; returns (beta, tau)."""
    beta = np.zeros(1)
    tau = np.zeros(1)
    lib().oracle_dlarfg(alpha, x.shape[0], _ptr(x), _estrides(x)[0] if x.size else 1, _ptr(beta), _ptr(tau))
    return float(beta[0]), float(tau[0])


def larf_left(v: np.ndarray, tau: float, c: np.ndarray) -> None:
    """src/lapack/larf.rs:10-52 (float64): c <- (I - tau v v^T) c in place."""
    rs, cs = _estrides(c)
    lib().oracle_dlarf_left(c.shape[0], c.shape[1], _ptr(v), _estrides(v)[0], tau, _ptr(c), rs, cs)


def nrm2(x: np.ndarray) -> float:
    """src/blas/nrm2.rs:6-15 (float64)."""
    return float(lib().oracle_dnrm2(x.shape[0], _ptr(x), _estrides(x)[0] if x.size else 1))
