"""Host-side argument checks of the Python mirror, on the CPU.

lair reports shape mismatches before any arithmetic: ``equation::solve``
returns ``InvalidInput::Shape`` (src/equation.rs:42-53) and raw ``getrs``
panics on mismatched lengths (src/lapack/getrs.rs:18-20).  The mirror makes
the same checks before it touches the device, so these run without a GPU;
empty systems need no device either (src/lapack/getrf.rs:349-355).
"""
import numpy as np
import pytest

from lair_gb300 import equation, lapack, refine
from lair_gb300.errors import InvalidInput


def test_error_kinds_display_like_lair():
    e = InvalidInput.Shape("input matrix is not square")
    assert isinstance(e, InvalidInput) and str(e) == "shape error: input matrix is not square"
    v = InvalidInput.Value("`a` is a singular matrix")
    assert isinstance(v, InvalidInput) and str(v) == "value error: `a` is a singular matrix"
    assert not isinstance(v, InvalidInput.Shape)


def test_equation_solve_shape_errors():
    with pytest.raises(InvalidInput.Shape, match="not square"):
        equation.solve(np.zeros((3, 4)), np.zeros(3))
    with pytest.raises(InvalidInput.Shape, match=r"The number of elements in `b`, 2, must be the same as the "
                                                 r"number of rows in `a`, 3"):
        equation.solve(np.eye(3), np.zeros(2))
    with pytest.raises(InvalidInput.Shape):
        equation.solve(np.eye(3), np.zeros((3, 2)))  # several columns go through solve_matrix
    with pytest.raises(InvalidInput.Shape):
        equation.solve_matrix(np.eye(3), np.zeros(3))
    with pytest.raises(InvalidInput.Shape):
        equation.solve_matrix(np.zeros((2, 3)), np.zeros((2, 1)))


def test_getrs_panics_like_lair():
    a = np.eye(3)
    with pytest.raises(AssertionError, match=r"a.nrows\(\) == p.len\(\)"):
        lapack.getrs(a, [0, 1], np.zeros(3))
    with pytest.raises(AssertionError, match=r"p.len\(\) == b.len\(\)"):
        lapack.getrs(a, [0, 1, 2], np.zeros(2))
    with pytest.raises(AssertionError, match=r"a.ncols\(\) >= p.len\(\)"):
        lapack.getrs(np.zeros((3, 2)), [0, 1, 2], np.zeros(3))
    with pytest.raises(TypeError):
        lapack.getrs(a, [0, 1, 2], np.zeros(3, dtype=np.float32))


def test_empty_getrs_needs_no_device():
    x = lapack.getrs(np.zeros((0, 0)), [], np.zeros(0))
    assert x.shape == (0,)
    x2 = lapack.getrs(np.eye(2), [0, 1], np.zeros((2, 0)))
    assert x2.shape == (2, 0)


def test_refinement_argument_errors():
    with pytest.raises(InvalidInput.Shape):
        refine.gesv_ir(np.zeros((3, 4)), np.zeros(3))
    with pytest.raises(InvalidInput.Shape):
        refine.gesv_ir(np.eye(4), np.zeros(3))
    with pytest.raises(TypeError):
        refine.gesv_ir(np.eye(4, dtype=np.float32), np.zeros(4, dtype=np.float32))
