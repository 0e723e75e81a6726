"""Mixed-precision LU with iterative refinement (no lair counterpart).

``gesv_ir(a, b)`` solves a square FP64 system with the LU factorization done
in a low precision on the GPU and FP64 only for the residual, the update and
the backward-error test ||b - Ax||_inf / (||A||_inf ||x||_inf + ||b||_inf) <= tol
(default n * 2^-53).  ``solver="ir"`` is classical refinement;
``solver="gmres"`` is GMRES-IR (FP64 GMRES preconditioned by the low-precision
LU), for matrices whose condition number is too large for plain IR.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .errors import InvalidInput


def gesv_ir(a: np.ndarray, b: np.ndarray, precision: str = "fp32", solver: str = "ir", tol: float = 0.0,
            max_iter: int = 30, raise_on_failure: bool = True):
    """Return (x, info).  ``a``: n x n float64 (any strides), ``b``: n or n x nrhs.

    Raises ``InvalidInput.Shape`` for non-square ``a`` or mismatched ``b`` and
    ``InvalidInput.Value`` when the low-precision factor is singular; when the
    refinement does not reach ``tol`` it raises ``LuhotError`` (status 5)
    unless ``raise_on_failure`` is False, in which case ``info["converged"]``
    is 0 and x is the last iterate.
    """
    if a.ndim != 2 or a.shape[0] != a.shape[1]:
        raise InvalidInput.Shape("input matrix is not square")
    if a.dtype != np.float64 or b.dtype != np.float64:
        raise TypeError("gesv_ir works on float64 systems")
    n = a.shape[0]
    if b.shape[0] != n:
        raise InvalidInput.Shape(f"b must have {n} rows")
    one_d = b.ndim == 1
    B = b.reshape(n, 1) if one_d else b
    nrhs = B.shape[1]
    x = np.empty((n, nrhs), dtype=np.float64)
    info = _lib.IrInfo()
    lib, ctx = _lib.load(), _lib.context()
    it = a.itemsize
    rc = lib.luhot_dgesv_ir(ctx, n, nrhs, a.ctypes.data, a.strides[0] // it, a.strides[1] // it, B.ctypes.data,
                            B.strides[0] // it, B.strides[1] // it, x.ctypes.data, x.strides[0] // it,
                            x.strides[1] // it, _lib.PRECISIONS[precision], _lib.SOLVERS[solver], float(tol),
                            int(max_iter), ctypes.byref(info))
    if rc == _lib.LUHOT_ERR_SINGULAR:
        raise InvalidInput.Value("the low-precision factor of `a` is singular")
    if rc != _lib.LUHOT_OK and not (rc == _lib.LUHOT_ERR_NOT_CONVERGED and not raise_on_failure):
        _lib.check(rc, ctx)
    out = x.reshape(n) if one_d else x
    return out, info.as_dict()
