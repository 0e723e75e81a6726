"""``decomposition::qr::Factorized`` and ``lapack::geqrf`` on the GPU.

Mirrors lair src/decomposition/qr.rs and src/lapack/geqrf.rs: ``Factorized(a)``
factors the array in place (R on and above the diagonal, the Householder
reflectors below it) and keeps tau; ``q()`` accumulates Q (m x m) on the GPU
in lair's backward order; ``r()`` is the host-side read of the upper
trapezoid.  ``mode="exact"`` reproduces lair's arithmetic bit for bit.
"""
from __future__ import annotations

import numpy as np

from . import _lib, lapack


def geqrf(a: np.ndarray, mode: str = "fast") -> np.ndarray:
    """QR-factorize ``a`` in place (any strides); returns tau (src/lapack/geqrf.rs:9-27)."""
    if a.ndim != 2:
        raise ValueError("geqrf expects a 2-D array")
    if not a.flags.writeable:
        raise ValueError("geqrf factors in place: the array must be writeable")
    p = lapack._prefix(a.dtype)
    m, n = a.shape
    tau = np.zeros(min(m, n), dtype=a.dtype)
    if tau.size:
        lib, ctx = _lib.load(), _lib.context()
        rs, cs = lapack._estrides(a)
        rc = getattr(lib, f"luhot_{p}geqrf")(ctx, m, n, a.ctypes.data, rs, cs, tau.ctypes.data, _lib.mode_id(mode))
        _lib.check(rc, ctx)
    return tau


class Factorized:
    """QR factors of a matrix (lair's ``qr::Factorized``, src/decomposition/qr.rs:12-20)."""

    def __init__(self, a: np.ndarray, mode: str = "fast"):
        self.tau = geqrf(a, mode=mode)
        self.qr = a
        self.mode = mode

    @classmethod
    def from_array(cls, a: np.ndarray, mode: str = "fast") -> "Factorized":
        return cls(a, mode=mode)

    def q(self) -> np.ndarray:
        """qr.rs:26-60: Q (m x m) from the reflectors."""
        m, n = self.qr.shape
        q = np.empty((m, m), dtype=self.qr.dtype)
        if m:
            lib, ctx = _lib.load(), _lib.context()
            p = lapack._prefix(self.qr.dtype)
            rs, cs = lapack._estrides(self.qr)
            tau = np.ascontiguousarray(self.tau)
            rc = getattr(lib, f"luhot_{p}qr_q")(ctx, m, n, self.qr.ctypes.data if self.qr.size else None, rs, cs,
                                               tau.ctypes.data, q.ctypes.data, m, 1, _lib.mode_id(self.mode))
            _lib.check(rc, ctx)
        return q

    def r(self) -> np.ndarray:
        """qr.rs:63-72: the factored array with its strictly lower part zeroed."""
        r = np.array(self.qr, copy=True)
        for i in range(1, r.shape[0]):
            r[i, : min(i, r.shape[1])] = 0
        return r
