"""``decomposition::lu::Factorized`` over the GPU getrf/getrs.

Mirrors lair src/decomposition/lu.rs: the factorization owns the L\\U array
(the caller's array, factored in place), the pivots and the singular flag;
``p()``, ``l()``, ``u()`` and ``into_pl()`` are host-side reads of that array
exactly as in lair, and ``solve`` runs getrs on the GPU.

``Factorized(a, device_resident=True)`` keeps the factors in GPU memory
between solves (with the composed row permutation and, in fast mode, the
inverses of the diagonal blocks); the caller's array receives L\\U only when
``lu``, ``p()``, ``l()``, ``u()`` or ``into_pl()`` first reads it.
"""
from __future__ import annotations

import ctypes
from typing import List, Optional

import numpy as np

from . import _lib, lapack
from .errors import InvalidInput


def permutation(nrows: int, pivots) -> List[int]:
    """Row order of P (lair src/decomposition/lu.rs:28-33): laswp on 0..nrows."""
    perm = list(range(nrows))
    for i, p in enumerate(pivots):
        if i != p:
            perm[i], perm[p] = perm[p], perm[i]
    return perm


def p_matrix(nrows: int, pivots, dtype=np.float64) -> np.ndarray:
    """lu.rs:28-39: P with P[perm[i], i] = 1."""
    p = np.zeros((nrows, nrows), dtype=dtype)
    for i, piv in enumerate(permutation(nrows, pivots)):
        p[piv, i] = 1
    return p


def l_matrix(lu: np.ndarray) -> np.ndarray:
    """lu.rs:42-57: unit lower-trapezoidal L (m x min(m, n))."""
    m, n = lu.shape
    rank = min(m, n)
    l = np.zeros((m, rank), dtype=lu.dtype)
    for i in range(m):
        for j in range(min(i, rank)):
            l[i, j] = lu[i, j]
        if i < rank:
            l[i, i] = 1
    return l


def u_matrix(lu: np.ndarray) -> np.ndarray:
    """lu.rs:60-72: upper-trapezoidal U (min(m, n) x n)."""
    m, n = lu.shape
    rank = min(m, n)
    u = np.zeros((rank, n), dtype=lu.dtype)
    for i in range(rank):
        u[i, i:] = lu[i, i:]
    return u


def into_pl(lu: np.ndarray, pivots) -> np.ndarray:
    """lu.rs:107-153: overwrite the first min(m, n) columns of ``lu`` with P*L.

    Follows lair's cycle walk: pivots are first turned into the inverse
    permutation in place, then each cycle moves rows of L to their permuted
    positions, writing the unit diagonal and the zeros above it.
    """
    piv = list(pivots)
    nrows, ncols = lu.shape
    if len(piv) < nrows:
        piv.extend(range(len(piv), nrows))
    for i in range(len(piv) - 1, -1, -1):
        target = piv[i]
        if i == target:
            continue
        piv[i] = piv[target]
        piv[target] = i
    kcols = min(nrows, ncols)
    pl = lu[:, :kcols]
    end = len(piv)
    dst = 0
    i = dst
    while True:
        src = piv[dst]
        for k in range(min(src, kcols)):
            pl[dst, k] = pl[src, k]
        if src < kcols:
            pl[dst, src] = 1
        for k in range(src + 1, kcols):
            pl[dst, k] = 0
        piv[dst] = end
        if piv[src] == end:
            dst = i + 1
            while dst < end and piv[dst] == end:
                dst += 1
            if dst == end:
                break
            i = dst
        else:
            dst = src
    return lu


class DeviceFactor:
    """LU factors held in GPU memory (``luhot_[ds]factor_*``).

    Factors ``a`` (any strides; not modified) on creation; ``solve`` moves
    only the right-hand sides; ``read_into`` writes L\\U to a host array.
    """

    def __init__(self, a: np.ndarray, mode: str = "fast"):
        if a.ndim != 2:
            raise ValueError("a factor needs a 2-D array")
        self._pfx = lapack._prefix(a.dtype)
        self.dtype = a.dtype
        self.shape = a.shape
        self._handle = None
        lib, ctx = _lib.load(), _lib.context()
        m, n = a.shape
        k = min(m, n)
        rs, cs = lapack._estrides(a)
        piv = np.zeros(max(k, 1), dtype=np.uint64)
        sing = ctypes.c_int64(-1)
        h = ctypes.c_void_p()
        rc = getattr(lib, f"luhot_{self._pfx}factor_create")(
            ctx, m, n, a.ctypes.data if a.size else None, rs, cs, _lib.mode_id(mode), piv.ctypes.data,
            ctypes.byref(sing), ctypes.byref(h))
        _lib.check(rc, ctx)
        self._handle = h
        self.pivots: List[int] = [int(v) for v in piv[:k]]
        self.singular: Optional[int] = None if sing.value < 0 else int(sing.value)

    def solve(self, b: np.ndarray, trans: bool = False) -> np.ndarray:
        """A x = b (or A^T x = b) for b of length n or shape (n, nrhs); new array."""
        if b.dtype != self.dtype:
            raise TypeError("b must have the factor's element type")
        n = self.shape[0]
        one_d = b.ndim == 1
        B = b.reshape(n, 1) if one_d else b
        nrhs = B.shape[1]
        x = np.empty((n, nrhs), dtype=self.dtype)
        if n and nrhs:
            lib, ctx = _lib.load(), _lib.context()
            brs, bcs = lapack._estrides(B)
            rc = getattr(lib, f"luhot_{self._pfx}factor_solve")(
                self._handle, nrhs, B.ctypes.data, brs, bcs, x.ctypes.data, nrhs, 1, 1 if trans else 0)
            _lib.check(rc, ctx)
        return x.reshape(n) if one_d else x

    def read_into(self, a: np.ndarray) -> None:
        if a.shape != self.shape or a.dtype != self.dtype:
            raise ValueError("read_into needs an array of the factor's shape and type")
        if a.size:
            rs, cs = lapack._estrides(a)
            _lib.check(_lib.load().luhot_factor_read(self._handle, a.ctypes.data, rs, cs), _lib.context())

    def close(self) -> None:
        if self._handle is not None:
            lib = _lib.load()
            lib.luhot_factor_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # interpreter shutdown
            pass


class Factorized:
    """LU factors of a matrix (lair's ``lu::Factorized``).

    ``Factorized(a)`` is lair's ``Factorized::from(a)`` (lu.rs:156-171): it
    takes the array and factors it in place on the GPU.  With
    ``device_resident=True`` the factors stay on the GPU for repeated solves
    and ``a`` is overwritten with L\\U on the first read of it.
    """

    def __init__(self, a: np.ndarray, mode: str = "fast", device_resident: bool = False):
        self.mode = mode
        self._array = a
        self._device: Optional[DeviceFactor] = None
        if device_resident:
            if not a.flags.writeable:
                raise ValueError("Factorized owns the array: it must be writeable")
            self._device = DeviceFactor(a, mode=mode)
            self._stale = True
            pivots, singular = self._device.pivots, self._device.singular
        else:
            pivots, singular = lapack.getrf(a, mode=mode)
            self._stale = False
        self.pivots: List[int] = pivots
        self.singular: Optional[int] = singular

    @classmethod
    def from_array(cls, a: np.ndarray, mode: str = "fast", device_resident: bool = False) -> "Factorized":
        return cls(a, mode=mode, device_resident=device_resident)

    @property
    def lu(self) -> np.ndarray:
        """The factored array (L below the diagonal, U on and above)."""
        if self._stale:
            self._device.read_into(self._array)
            self._stale = False
        return self._array

    def p(self) -> np.ndarray:
        return p_matrix(self.lu.shape[0], self.pivots, self.lu.dtype)

    def l(self) -> np.ndarray:  # noqa: E743 - lair's method name
        return l_matrix(self.lu)

    def u(self) -> np.ndarray:
        return u_matrix(self.lu)

    def is_singular(self) -> bool:
        """lu.rs:75-77"""
        return self.singular is not None

    def solve(self, b: np.ndarray) -> np.ndarray:
        """lu.rs:87-98: Shape error when len(b) != nrows, else getrs."""
        if b.ndim != 1:
            raise InvalidInput.Shape("b must be one-dimensional (solve_matrix takes several columns)")
        return self._solve(b)

    def solve_matrix(self, b: np.ndarray) -> np.ndarray:
        """Every column of the n x nrhs array ``b`` (additive multi-RHS form of solve)."""
        if b.ndim != 2:
            raise InvalidInput.Shape("b must be two-dimensional")
        return self._solve(b)

    def _solve(self, b: np.ndarray) -> np.ndarray:
        nrows = self._array.shape[0]
        if b.shape[0] != nrows:
            raise InvalidInput.Shape(f"b must have {nrows} elements")
        if self._device is not None:
            k = len(self.pivots)
            assert nrows == k, "assertion `left == right` failed: a.nrows() == p.len()"
            return self._device.solve(b)
        return lapack.getrs(self.lu, self.pivots, b, mode=self.mode)

    def into_pl(self) -> np.ndarray:
        return into_pl(self.lu, self.pivots)
