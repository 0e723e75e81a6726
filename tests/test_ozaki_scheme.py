"""CPU checks of the integer-slice (Ozaki) FP64 Schur update's arithmetic,
on its numpy restatement (tests/ozaki_emulation.py): the exactness bound of
the FP32 group sums, the digit split, and the accuracy of the whole update
against exact arithmetic and against a plain FP64 GEMM.  The GPU kernel is
compared with the same restatement bit for bit in test_gpu_ozaki.py."""
import numpy as np
import pytest

import ozaki_emulation as oz


def exact_update(c, l, u):
    """C - L U in extended precision (longdouble: 64-bit or more significand)."""
    ld = np.longdouble
    return c.astype(ld) - l.astype(ld) @ u.astype(ld)


def test_group_sums_exact_in_fp32():
    # every partial sum of every group is an integer below 2^24 for K <= 64
    assert oz.group_bound(64) < 2 ** 24
    assert oz.group_bound(64) == 9 * 2 ** 20


@pytest.mark.parametrize("scale", [1.0, 2.0 ** 300, 2.0 ** -300, 2.0 ** -1060])
def test_digits_reconstruct(scale):
    rng = np.random.default_rng(1)
    x = rng.standard_normal((64, 64)) * np.exp(rng.uniform(-20, 20, (64, 64))) * scale
    x[3] = 0.0
    x[5, :7] = 0.0
    e = oz.exponents(x, 1)
    d = oz.digits(x, e[:, None])
    assert np.abs(d[0]).max() <= 256
    assert all(np.abs(v).max() <= 128 for v in d[1:])
    rec = sum(np.ldexp(v.astype(np.float64), -8 * (p + 1)) for p, v in enumerate(d))
    rec = np.ldexp(rec, e[:, None].astype(np.int32))
    # each element is represented to within 2^(e - 57) of its row's scale
    tol = np.ldexp(1.0, (e - 57).astype(np.int32))[:, None]
    if scale < 2.0 ** -1000:
        tol = np.maximum(tol, np.ldexp(1.0, -1074))  # the reconstruction itself rounds in the subnormals
    assert np.all(np.abs(rec - x) <= tol)
    assert np.all(rec[3] == 0.0)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_update_accuracy_matches_fp64_gemm(seed):
    rng = np.random.default_rng(seed)
    m, n, k = 200, 150, 64
    l = rng.uniform(-1, 1, (m, k))  # a pivoted L21: |l| <= 1
    u = rng.standard_normal((k, n)) * np.exp(rng.uniform(-3, 3, (1, n)))
    c = rng.standard_normal((m, n)) * 4.0
    ref = exact_update(c, l, u)
    scale = np.abs(c) + np.abs(l) @ np.abs(u)
    err_oz = float(np.max(np.abs(oz.schur_update(c, l, u) - ref) / scale))
    err_64 = float(np.max(np.abs((c - l @ u) - ref) / scale))
    # the final subtraction rounds once in both; the product part is below FP64's
    assert err_oz <= max(err_64, 2.0 ** -52)
    assert err_oz <= 2.0 ** -51


def test_update_wide_dynamic_range():
    rng = np.random.default_rng(7)
    m, n, k = 96, 80, 64
    l = rng.uniform(-1, 1, (m, k)) * np.exp2(rng.integers(-200, 200, (m, 1)))
    u = rng.standard_normal((k, n)) * np.exp2(rng.integers(-200, 200, (1, n)))
    c = l[:, :1] * u[:1, :]
    ref = exact_update(c, l, u)
    scale = np.abs(c) + np.abs(l) @ np.abs(u)
    err = float(np.max(np.abs(oz.schur_update(c, l, u) - ref) / scale))
    assert err <= 2.0 ** -51


def test_update_zeros_and_nonfinite():
    rng = np.random.default_rng(3)
    m, n, k = 40, 30, 20
    l = rng.standard_normal((m, k))
    u = rng.standard_normal((k, n))
    l[4] = 0.0            # zero row: C row unchanged
    u[:, 6] = 0.0         # zero column: C column unchanged
    l[9, 2] = np.inf      # row 9 -> NaN
    u[3, 11] = np.nan     # column 11 -> NaN
    c = rng.standard_normal((m, n))
    out = oz.schur_update(c, l, u)
    cols = np.arange(n) != 11  # 0 * NaN is NaN: column 11 is NaN in every row
    assert np.array_equal(out[4][cols], c[4][cols])
    assert np.array_equal(out[:, 6][np.arange(m) != 9], c[:, 6][np.arange(m) != 9])
    assert np.all(np.isnan(out[9])) and np.all(np.isnan(out[:, 11]))
    fin = np.ones((m, n), bool)
    fin[9] = False
    fin[:, 11] = False
    assert np.all(np.isfinite(out[fin]))


def test_ragged_k():
    rng = np.random.default_rng(4)
    for k in (1, 7, 33, 64):
        l = rng.standard_normal((50, k))
        u = rng.standard_normal((k, 45))
        c = rng.standard_normal((50, 45))
        ref = exact_update(c, l, u)
        scale = np.abs(c) + np.abs(l) @ np.abs(u)
        assert float(np.max(np.abs(oz.schur_update(c, l, u) - ref) / scale)) <= 2.0 ** -51


@pytest.mark.parametrize("seed", [0, 1, 4])
def test_triangular_solve_as_slice_product(seed):
    """The U12 solve of fast-mode FP64 getrf on the tensor cores:
    U12 = A12 - N A12 with N = I - L11^-1 (strictly lower), the product taken
    as the slice product.  The digits of a row of N are relative to the row's
    largest entry, and the rows of an inverse span a wider range than a
    pivoted L21's, so the error against exact arithmetic is a few times that
    of an FP64 product: measured 3-13 eps of |L11^-1| |A12| on pivoted random
    panels (FP64 GEMM 1.5-2.5 eps); the bound here is 32 eps, against exact
    arithmetic and against LAPACK's substitution."""
    rng = np.random.default_rng(seed)
    w, ncols = 64, 300
    # L11 from partial pivoting of a random panel: unit lower, |l| <= 1
    panel = rng.standard_normal((512, w))
    lu = panel.copy()
    for j in range(w):
        p = j + int(np.argmax(np.abs(lu[j:, j])))
        lu[[j, p]] = lu[[p, j]]
        lu[j + 1:, j] /= lu[j, j]
        lu[j + 1:, j + 1:] -= np.outer(lu[j + 1:, j], lu[j, j + 1:])
    l11 = np.tril(lu[:w], -1) + np.eye(w)
    a12 = rng.standard_normal((w, ncols))
    inv = np.linalg.inv(l11)
    nmat = np.eye(w) - inv
    u12 = oz.schur_update(a12, nmat, a12)
    ld = np.longdouble
    exact = np.linalg.solve(l11, a12)  # LAPACK's substitution in FP64
    # exact arithmetic for the product part: A12 - N A12 with N as computed
    ref = a12.astype(ld) - nmat.astype(ld) @ a12.astype(ld)
    scale = np.abs(inv) @ np.abs(a12)
    assert float(np.max(np.abs(u12 - ref) / scale)) <= 32 * 2.0 ** -52
    assert float(np.max(np.abs(u12 - exact) / scale)) <= 32 * 2.0 ** -52
