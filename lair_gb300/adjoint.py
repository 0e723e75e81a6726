"""Adjoint (backward) of the linear solve X = A^-1 B (no lair counterpart).

For a scalar loss L(X) with upstream gradient W = dL/dX:

    lambda = A^-T W          (transposed getrs on the stored LU factors)
    dL/dB  = lambda
    dL/dA  = -lambda X^T

``solve_backward`` reuses a ``lu.Factorized`` (or raw factors + pivots);
``solve_backward_ir`` obtains lambda by mixed-precision refinement on A^T.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def _es(a: np.ndarray):
    return tuple(s // a.itemsize for s in a.strides)


def solve_backward(lu_factors, pivots, x: np.ndarray, w: np.ndarray, mode: str = "fast", with_da: bool = True):
    """Return (dA, dB) for X = A^-1 B given the factors of A (from ``lapack.getrf``)."""
    lu = np.asarray(lu_factors)
    n = lu.shape[0]
    W = w.reshape(n, 1) if w.ndim == 1 else w
    X = x.reshape(n, 1) if x.ndim == 1 else x
    nrhs = W.shape[1]
    piv = np.ascontiguousarray(np.asarray(pivots, dtype=np.uint64))
    db = np.empty((n, nrhs))
    da = np.empty((n, n)) if with_da else None
    lib, ctx = _lib.load(), _lib.context()
    rc = lib.luhot_dgesv_backward(
        ctx, n, nrhs, lu.ctypes.data, *_es(lu), piv.ctypes.data, X.ctypes.data, *_es(X), W.ctypes.data, *_es(W),
        db.ctypes.data, *_es(db), da.ctypes.data if with_da else None, *(_es(da) if with_da else (0, 0)),
        _lib.mode_id(mode))
    _lib.check(rc, ctx)
    return da, (db.reshape(n) if w.ndim == 1 else db)


def solve_backward_ir_dev(a_dev_ptr: int, lda: int, n: int, nrhs: int, x_ptr: int, w_ptr: int, db_ptr: int,
                          da_ptr, precision: str = "fp32", solver: str = "ir", tol: float = 0.0, max_iter: int = 30):
    """Device-pointer form of the mixed-precision backward; returns the refinement info."""
    info = _lib.IrInfo()
    lib, ctx = _lib.load(), _lib.context()
    rc = lib.luhot_dgesv_backward_ir_dev(ctx, n, nrhs, a_dev_ptr, lda, x_ptr, nrhs, w_ptr, nrhs, db_ptr, nrhs,
                                         da_ptr, n, _lib.PRECISIONS[precision], _lib.SOLVERS[solver], float(tol),
                                         int(max_iter), ctypes.byref(info))
    _lib.check(rc, ctx)
    return info.as_dict()
