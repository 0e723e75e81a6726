"""``equation::solve`` (lair src/equation.rs:32-59) on the GPU LU path."""
from __future__ import annotations

import numpy as np

from .errors import InvalidInput
from .lu import Factorized


def solve(a: np.ndarray, b: np.ndarray, mode: str = "fast") -> np.ndarray:
    """Solve ``a x = b`` for square ``a``.

    Errors, as in lair: ``InvalidInput.Shape`` if ``a`` is not square or
    ``len(b) != a.nrows()``; ``InvalidInput.Value`` if ``a`` is singular.
    ``a`` itself is not modified (lair factors ``a.to_owned()``, which keeps the
    strides of a contiguous array, so F-order and reversed arrays are factored
    in lair's column-major order; this copy does the same).
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


def _to_owned(a: np.ndarray) -> np.ndarray:
    """ndarray's ``to_owned``: a copy with the same strides when the elements
    fill one block of memory (C or F order, either sign), else a C-order copy."""
    neg = tuple(ax for ax in range(a.ndim) if a.strides[ax] < 0 and a.shape[ax] > 1)
    v = np.flip(a, axis=neg) if neg else a
    if v.flags.c_contiguous or v.flags.f_contiguous:
        owned = v.copy(order="F" if (v.flags.f_contiguous and not v.flags.c_contiguous) else "C")
        return np.flip(owned, axis=neg) if neg else owned
    return np.array(a, order="C", copy=True)


def _factor_checked(a: np.ndarray, mode: str) -> Factorized:
    factorized = Factorized(_to_owned(a), mode=mode)
    if factorized.is_singular():
        raise InvalidInput.Value("`a` is a singular matrix")
    return factorized
