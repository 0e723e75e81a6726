"""Exact mode on non-standard layouts: lair's getrf_col_major order, bit for bit.

lair's getrf dispatcher (src/lapack/getrf.rs:12-27) factors every array that
is not in ndarray's standard layout (F order, sliced views with padded rows,
negative strides) with its left-looking Crout variant (getrf.rs:128-213).
The GPU's exact mode follows that order for up to 4096 rows, so LU, pivots
and the singular step equal the oracle's exactly.
"""
import numpy as np
import pytest

import oracle
from lair_gb300 import lapack

pytestmark = pytest.mark.gpu


def rand(seed, m, n, dtype=np.float64):
    return np.random.default_rng(seed).uniform(-1, 1, (m, n)).astype(dtype)


def check(view_fn, m, n, seed, dtype=np.float64, fill=None):
    a0 = rand(seed, m, n, dtype)
    if fill is not None:
        fill(a0)
    gpu = view_fn(a0.copy())
    ref = view_fn(a0.copy())
    piv, sing = lapack.getrf(gpu, mode="exact")
    piv_r, sing_r = oracle.getrf(ref)
    assert piv == piv_r
    assert sing == sing_r
    assert np.array_equal(gpu, ref, equal_nan=True)
    return gpu, piv


SHAPES = [(2, 2), (5, 5), (17, 17), (31, 31), (32, 32), (33, 33), (64, 64), (100, 100), (130, 130),
          (300, 300), (70, 200), (200, 70), (3, 40), (40, 3)]


@pytest.mark.parametrize("m,n", SHAPES)
def test_fortran_order_bitwise(m, n):
    check(np.asfortranarray, m, n, m * 7 + n)


@pytest.mark.parametrize("m,n", [(9, 9), (65, 65), (120, 50), (50, 120)])
def test_negative_strides_bitwise(m, n):
    check(lambda a: a[::-1, :], m, n, m + 3 * n)
    check(lambda a: a[:, ::-1], m, n, m + 5 * n)
    check(lambda a: np.asfortranarray(a)[::-1, ::-1], m, n, m + 11 * n)


def test_sliced_view_with_padded_rows_bitwise():
    # C order but the row stride exceeds the row length: not standard layout in ndarray.
    big = rand(77, 150, 180)
    gpu, ref = big.copy(), big.copy()
    piv, sing = lapack.getrf(gpu[:, :150], mode="exact")
    piv_r, sing_r = oracle.getrf(ref[:, :150])
    assert piv == piv_r and sing == sing_r
    assert np.array_equal(gpu, ref)


def test_float32_fortran_bitwise():
    check(np.asfortranarray, 257, 257, 3, dtype=np.float32)


def test_large_fortran_bitwise():
    check(np.asfortranarray, 1024, 1024, 5)


def test_singular_and_nan_columns_follow_col_major_rules():
    # A zero column is singular; a NaN column is not singular in the Crout
    # variant (its pivot *value* is NaN, not zero) -- unlike the row-major
    # order, which tests the pivot's magnitude.
    def zero_col(a):
        a[:, 4] = 0.0

    def nan_col(a):
        a[:, 6] = np.nan

    _, _ = check(np.asfortranarray, 12, 12, 21, fill=zero_col)
    _, _ = check(np.asfortranarray, 12, 12, 22, fill=nan_col)


def test_solve_with_fortran_factors_is_lairs():
    n = 200
    a0 = np.asfortranarray(rand(31, n, n))
    b = rand(32, n, 1)[:, 0]
    gpu, ref = a0.copy(order="F"), a0.copy(order="F")
    piv, _ = lapack.getrf(gpu, mode="exact")
    piv_r, _ = oracle.getrf(ref)
    x = lapack.getrs(gpu, piv, b, mode="exact")
    assert np.array_equal(x, oracle.getrs(ref, piv_r, b))


def test_exact_nonstandard_beyond_4096_rows_is_unsupported():
    """Exact mode never switches order: past 4096 rows a non-standard layout
    is refused (LUHOT_ERR_UNSUPPORTED) on both the one-shot and the
    device-resident paths."""
    from lair_gb300 import _lib, lu

    a = np.asfortranarray(rand(40, 4097, 6))
    with pytest.raises(_lib.LuhotError) as e:
        lapack.getrf(a.copy(order="F"), mode="exact")
    assert e.value.status == _lib.LUHOT_ERR_UNSUPPORTED
    with pytest.raises(_lib.LuhotError) as e:
        lu.Factorized(a.copy(order="F"), mode="exact", device_resident=True)
    assert e.value.status == _lib.LUHOT_ERR_UNSUPPORTED
    piv, _ = lapack.getrf(a.copy(order="F"), mode="fast")  # fast mode takes it
    assert len(piv) == 6


@pytest.mark.parametrize("view", ["fortran", "reversed"])
def test_resident_exact_nonstandard_is_lairs_bits(view):
    from lair_gb300 import lu

    n = 300
    a0 = rand(41, n, n)
    make = (lambda x: np.asfortranarray(x)) if view == "fortran" else (lambda x: x[::-1, ::-1])
    ref = make(a0.copy())
    piv_r, sing_r = oracle.getrf(ref)
    f = lu.Factorized(make(a0.copy()), mode="exact", device_resident=True)
    assert f.pivots == piv_r and f.singular == sing_r
    assert np.array_equal(f.lu, ref)
    b = rand(42, n, 1)[:, 0]
    assert np.array_equal(f.solve(b), oracle.getrs(ref, piv_r, b))


@pytest.mark.parametrize("view", ["fortran", "reversed", "padded_rows", "c_order"])
def test_gesv_exact_follows_lairs_copy_layout(view):
    """luhot_dgesv is equation::solve: lair factors a.to_owned(), which keeps
    the strides of a contiguous array (F order, reversed) and makes any other
    array standard; exact mode then gives the bits of lair's getrf on that
    copy and its getrs (src/equation.rs:54-58)."""
    from lair_gb300 import _lib
    from lair_gb300.equation import _to_owned

    n, nrhs = 150, 3
    big = rand(43, n, n + 7)
    views = {"fortran": lambda: np.asfortranarray(big[:, :n]), "reversed": lambda: big[:, :n].copy()[::-1, ::-1],
             "padded_rows": lambda: big[:, :n], "c_order": lambda: big[:, :n].copy()}
    a = views[view]()
    b = rand(44, n, nrhs)
    owned = _to_owned(a)
    assert (view in ("fortran", "reversed")) == (not oracle.is_standard_layout(owned))
    ref = owned.copy() if oracle.is_standard_layout(owned) else owned
    piv_r, _ = oracle.getrf(ref)
    x_ref = oracle.getrs_multi(ref, piv_r, b)
    lib, ctx = _lib.load(), _lib.context()
    x = np.empty((n, nrhs))
    es = lambda v: tuple(s // v.itemsize for s in v.strides)  # noqa: E731
    _lib.check(lib.luhot_dgesv(ctx, n, nrhs, a.ctypes.data, *es(a), b.ctypes.data, *es(b), x.ctypes.data, *es(x),
                               _lib.MODE_EXACT), ctx)
    assert np.array_equal(x, x_ref)
