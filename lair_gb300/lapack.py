"""GPU drop-ins for lair's ``lapack::getrf`` and ``lapack::getrs``.

Arrays are numpy views playing the part of ndarray views: any strides
(C order, F order, negative) are accepted and written back in place, as lair
does.  Only float64 and float32 run on the GPU; lair's other element types
(complex) are outside this hot path and are rejected here.
"""
from __future__ import annotations

import ctypes
from typing import List, Optional, Tuple

import numpy as np

from . import _lib


def _estrides(a: np.ndarray):
    return tuple(s // a.itemsize for s in a.strides)


def _prefix(dtype) -> str:
    if dtype == np.float64:
        return "d"
    if dtype == np.float32:
        return "s"
    raise TypeError(f"the GPU LU path supports float64 and float32, got {dtype}")


def getrf(a: np.ndarray, mode: str = "fast") -> Tuple[List[int], Optional[int]]:
    """LU-factorize ``a`` in place with partial pivoting.

    Mirrors ``lapack::getrf`` (lair src/lapack/getrf.rs:12-27): returns the
    pivots (length min(m, n); row i was swapped with row pivots[i] at step i)
    and ``singular`` (None, or the last step whose pivot column was all zero).
    ``mode="exact"`` reproduces lair's row-major operation order bit for bit.
    """
    if a.ndim != 2:
        raise ValueError("getrf expects a 2-D array")
    if not a.flags.writeable:
        raise ValueError("getrf factors in place: the array must be writeable")
    p = _prefix(a.dtype)
    lib = _lib.load()
    ctx = _lib.context()
    m, n = a.shape
    rs, cs = _estrides(a)
    k = min(m, n)
    piv = np.zeros(max(k, 1), dtype=np.uint64)
    sing = ctypes.c_int64(-1)
    rc = getattr(lib, f"luhot_{p}getrf")(ctx, m, n, a.ctypes.data if a.size else None, rs, cs,
                                          piv.ctypes.data, ctypes.byref(sing), _lib.mode_id(mode))
    _lib.check(rc, ctx)
    return [int(v) for v in piv[:k]], (None if sing.value < 0 else int(sing.value))


def getrs(a: np.ndarray, p, b: np.ndarray, mode: str = "fast", trans: bool = False) -> np.ndarray:
    """Solve ``a x = b`` with factors from :func:`getrf`; returns a new array.

    Mirrors ``lapack::getrs`` (lair src/lapack/getrs.rs:12-38), including its
    panics (AssertionError here) when ``a.nrows() != p.len()``,
    ``p.len() != b.len()`` or ``a.ncols() < p.len()``.  ``b`` may also be 2-D
    (n x nrhs), which solves every column; ``trans=True`` solves a^T x = b.
    """
    if a.ndim != 2:
        raise ValueError("getrs expects a 2-D factor array")
    piv = np.ascontiguousarray(np.asarray(p, dtype=np.uint64))
    n = a.shape[0]
    assert n == piv.shape[0], "assertion `left == right` failed: a.nrows() == p.len()"
    assert piv.shape[0] == b.shape[0], "assertion `left == right` failed: p.len() == b.len()"
    assert a.shape[1] >= piv.shape[0], "assertion failed: a.ncols() >= p.len()"
    if b.dtype != a.dtype:
        raise TypeError("a and b must have the same element type")
    pfx = _prefix(a.dtype)
    one_d = b.ndim == 1
    B = b.reshape(n, 1) if one_d else b
    nrhs = B.shape[1]
    x = np.empty((n, nrhs), dtype=a.dtype)
    if n == 0 or nrhs == 0:
        return x.reshape(n) if one_d else x
    lib = _lib.load()
    ctx = _lib.context()
    ars, acs = _estrides(a)
    brs, bcs = _estrides(B)
    xrs, xcs = _estrides(x)
    rc = getattr(lib, f"luhot_{pfx}getrs")(ctx, n, nrhs, a.ctypes.data, ars, acs, piv.ctypes.data,
                                           B.ctypes.data, brs, bcs, x.ctypes.data, xrs, xcs,
                                           1 if trans else 0, _lib.mode_id(mode))
    _lib.check(rc, ctx)
    return x.reshape(n) if one_d else x
