"""``decomposition::lu::Factorized`` over the GPU getrf/getrs.

Mirrors lair src/decomposition/lu.rs: the factorization owns the L\\U array
(the caller's array, factored in place), the pivots and the singular flag;
``p()``, ``l()``, ``u()`` and ``into_pl()`` are host-side reads of that array
exactly as in lair, and ``solve`` runs getrs on the GPU.
"""
from __future__ import annotations

from typing import List, Optional

import numpy as np

from . import lapack
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


class Factorized:
    """LU factors of a matrix (lair's ``lu::Factorized``).

    ``Factorized(a)`` is lair's ``Factorized::from(a)`` (lu.rs:156-171): it
    takes the array and factors it in place on the GPU.
    """

    def __init__(self, a: np.ndarray, mode: str = "fast"):
        pivots, singular = lapack.getrf(a, mode=mode)
        self.lu = a
        self.pivots: List[int] = pivots
        self.singular: Optional[int] = singular
        self.mode = mode

    @classmethod
    def from_array(cls, a: np.ndarray, mode: str = "fast") -> "Factorized":
        return cls(a, mode=mode)

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
        if b.shape[0] != self.lu.shape[0]:
            raise InvalidInput.Shape(f"b must have {self.lu.shape[0]} elements")
        return lapack.getrs(self.lu, self.pivots, b, mode=self.mode)

    def into_pl(self) -> np.ndarray:
        return into_pl(self.lu, self.pivots)
