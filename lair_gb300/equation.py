"""``equation::solve`` (lair src/equation.rs:32-59) on the GPU LU path."""
from __future__ import annotations

import numpy as np

from .errors import InvalidInput
from .lu import Factorized


def solve(a: np.ndarray, b: np.ndarray, mode: str = "fast") -> np.ndarray:
    """Solve ``a x = b`` for square ``a``.

    Errors, as in lair: ``InvalidInput.Shape`` if ``a`` is not square or
    ``len(b) != a.nrows()``; ``InvalidInput.Value`` if ``a`` is singular.
    ``a`` itself is not modified (lair factors ``a.to_owned()``; the copy keeps
    ``a``'s memory order, which this copy does too).
    """
    if a.ndim != 2 or a.shape[0] != a.shape[1]:
        raise InvalidInput.Shape("input matrix is not square")
    if b.shape[0] != a.shape[0]:
        raise InvalidInput.Shape(
            f"The number of elements in `b`, {b.shape[0]}, must be the same as the number of rows in `a`, {a.shape[0]}")
    if b.ndim != 1:
        raise InvalidInput.Shape("b must be one-dimensional (solve_matrix takes several columns)")
    return _factor_checked(a, mode).solve(b)


def solve_matrix(a: np.ndarray, b: np.ndarray, mode: str = "fast") -> np.ndarray:
    """``a X = B`` for every column of the n x nrhs array ``b``: the additive
    multi-right-hand-side form of :func:`solve`, with the same errors."""
    if a.ndim != 2 or a.shape[0] != a.shape[1]:
        raise InvalidInput.Shape("input matrix is not square")
    if b.ndim != 2 or b.shape[0] != a.shape[0]:
        raise InvalidInput.Shape(
            f"`b` must be two-dimensional with as many rows as `a`, {a.shape[0]}")
    return _factor_checked(a, mode).solve_matrix(b)


def _factor_checked(a: np.ndarray, mode: str) -> Factorized:
    owned = np.array(a, order="F" if (a.flags.f_contiguous and not a.flags.c_contiguous) else "C", copy=True)
    factorized = Factorized(owned, mode=mode)
    if factorized.is_singular():
        raise InvalidInput.Value("`a` is a singular matrix")
    return factorized
