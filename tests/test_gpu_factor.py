"""Device-resident factors (``luhot_[ds]factor_*``, lu.Factorized(device_resident=True)).

The factor kept in HBM must give what the one-shot path gives on the same
input: the same pivots, singular step and L\\U bits (the same getrf kernels),
the same solutions bit for bit (the same sweeps with the same diagonal-block
inverses; one FP64 right-hand side in fast mode takes the block-scaled sweeps
instead and agrees to fast-mode rounding), and in exact mode lair's bits (the
oracle).  The host array must stay untouched until the factored array is
first read.
"""
import ctypes

import numpy as np
import pytest

import oracle
from lair_gb300 import _lib, equation, lapack, lu
from lair_gb300.errors import InvalidInput

pytestmark = pytest.mark.gpu

EPS64 = 2.0 ** -53


def rand(seed, m, n, dtype=np.float64):
    return np.random.default_rng(seed).uniform(-1, 1, (m, n)).astype(dtype)


@pytest.mark.parametrize("n", [1, 63, 64, 65, 300, 1000])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_resident_matches_one_shot_path_bitwise(n, dtype):
    a0 = rand(n + 7, n, n, dtype)
    b = rand(n + 8, n, 3, dtype)
    ref = a0.copy()
    piv_r, sing_r = lapack.getrf(ref)
    x_r = lapack.getrs(ref, piv_r, b)

    a = a0.copy()
    f = lu.Factorized(a, device_resident=True)
    assert f.pivots == piv_r and f.singular == sing_r
    assert np.array_equal(a, a0)  # nothing written back yet
    x = f.solve_matrix(b)
    assert np.array_equal(x, x_r)
    x1, x1_r = f.solve(b[:, 1]), lapack.getrs(ref, piv_r, b[:, 1])
    if dtype == np.float64:
        # one FP64 right-hand side takes the block-scaled sweeps: same
        # solution to fast-mode rounding
        np.testing.assert_allclose(x1, x1_r, rtol=0, atol=1e-9 * np.abs(x1_r).max())
    else:
        assert np.array_equal(x1, x1_r)
    assert np.array_equal(f.lu, ref)  # first read writes L\U into the caller's array
    assert f.lu is a


def test_resident_exact_mode_is_lairs_bits():
    n = 200
    a0 = rand(5, n, n)
    b = rand(6, n, 1)[:, 0]
    ref = a0.copy()
    piv_r, sing_r = oracle.getrf(ref)
    x_r = oracle.getrs(ref, piv_r, b)
    f = lu.Factorized(a0.copy(), mode="exact", device_resident=True)
    assert f.pivots == piv_r and f.singular == sing_r
    assert np.array_equal(f.solve(b), x_r)
    assert np.array_equal(f.lu, ref)


def test_resident_many_rhs_strides_and_repeat():
    n = 700
    a0 = rand(11, n, n) + n ** 0.5 * np.eye(n)
    f = lu.Factorized(a0.copy(), device_resident=True)
    b = np.asfortranarray(rand(12, n, 37))  # F order, three launches of <= 16 columns
    x = f.solve_matrix(b)
    for c in (0, 16, 36):
        r = b[:, c] - a0 @ x[:, c]
        assert np.abs(r).max() / (np.abs(a0).sum(1).max() * np.abs(x[:, c]).max()) <= n * EPS64
    for _ in range(3):
        assert np.array_equal(f.solve_matrix(b), x)
    b_neg = np.flipud(np.flipud(b).copy())  # same values, negative row stride
    assert b_neg.strides[0] < 0
    assert np.array_equal(f.solve_matrix(b_neg), x)


def test_resident_transposed_solve():
    n = 513
    a0 = rand(21, n, n) + n ** 0.5 * np.eye(n)
    d = lu.DeviceFactor(a0)
    b = rand(22, n, 2)
    x = d.solve(b, trans=True)
    ref = np.linalg.solve(a0.T, b)
    assert np.abs(x - ref).max() <= 1e-12 * np.abs(ref).max()
    d.close()
    d.close()  # idempotent


def test_resident_p_l_u_and_into_pl():
    n = 130
    a0 = rand(31, n, n)
    f = lu.Factorized(a0.copy(), device_resident=True)
    pa = f.p().T @ a0
    assert np.abs(pa - f.l() @ f.u()).max() <= 10 * n * EPS64 * np.abs(a0).max()
    g = lu.Factorized(a0.copy())
    assert np.array_equal(f.into_pl(), g.into_pl())


def test_resident_rectangular_and_singular():
    wide = rand(41, 70, 200)
    f = lu.Factorized(wide.copy(), device_resident=True)
    ref = wide.copy()
    piv_r, _ = lapack.getrf(ref)
    assert f.pivots == piv_r
    b = rand(42, 70, 1)[:, 0]
    assert np.array_equal(f.solve(b), lapack.getrs(ref, piv_r, b))
    tall = lu.Factorized(rand(43, 200, 70), device_resident=True)
    with pytest.raises(AssertionError):
        tall.solve(np.zeros(200))
    s = lu.Factorized(np.ones((4, 4)), device_resident=True)
    assert s.is_singular() and s.singular == lapack.getrf(np.ones((4, 4)))[1]
    with pytest.raises(InvalidInput.Shape):
        lu.Factorized(np.eye(3), device_resident=True).solve(np.zeros(4))


def test_solve_matrix_api():
    n = 90
    a = rand(51, n, n) + n * np.eye(n)
    b = rand(52, n, 5)
    x = equation.solve_matrix(a, b)
    xe = equation.solve_matrix(a, b, mode="exact")
    for c in range(5):
        # fast mode splits the sums differently for one and for several
        # right-hand sides; exact mode runs lair's order for each column
        x1 = equation.solve(a, b[:, c])
        assert np.abs(x[:, c] - x1).max() <= 4 * n * EPS64 * np.abs(x1).max()
        assert np.array_equal(xe[:, c], equation.solve(a, b[:, c], mode="exact"))
    with pytest.raises(InvalidInput.Shape):
        equation.solve_matrix(a, b[:, 0])
    with pytest.raises(InvalidInput.Shape):
        equation.solve(a, b)


def test_resident_device_solve_and_status():
    torch = pytest.importorskip("torch")
    lib, ctx = _lib.load(), _lib.context()
    n = 400
    a0 = rand(61, n, n) + n ** 0.5 * np.eye(n)
    d_a = torch.from_numpy(a0).cuda()
    torch.cuda.synchronize()
    piv = np.zeros(n, dtype=np.uint64)
    sing = ctypes.c_int64(0)
    h = ctypes.c_void_p()
    _lib.check(lib.luhot_dfactor_create_dev(ctx, n, n, d_a.data_ptr(), n, 0, piv.ctypes.data, ctypes.byref(sing),
                                            ctypes.byref(h)), ctx)
    assert sing.value == -1
    assert torch.equal(d_a.cpu(), torch.from_numpy(a0))  # input not modified
    b = rand(62, n, 4)
    d_b = torch.from_numpy(b).cuda()
    torch.cuda.synchronize()
    _lib.check(lib.luhot_dfactor_solve_dev(h, 4, d_b.data_ptr(), 4, 0), ctx)
    x_host = np.empty_like(b)
    _lib.check(lib.luhot_dfactor_solve(h, 4, b.ctypes.data, 4, 1, x_host.ctypes.data, 4, 1, 0), ctx)
    assert np.array_equal(d_b.cpu().numpy(), x_host)
    # wrong element type and bad arguments come back as statuses
    xf = np.empty((n, 1), dtype=np.float32)
    assert lib.luhot_sfactor_solve(h, 1, xf.ctypes.data, 1, 1, xf.ctypes.data, 1, 1, 0) == _lib.LUHOT_ERR_INVALID_ARG
    assert lib.luhot_dfactor_solve(h, -1, b.ctypes.data, 1, 1, b.ctypes.data, 1, 1, 0) == _lib.LUHOT_ERR_INVALID_ARG
    lda = ctypes.c_int64(0)
    ptr = ctypes.c_void_p()
    _lib.check(lib.luhot_factor_device(h, ctypes.byref(ptr), ctypes.byref(lda), None), ctx)
    assert lda.value >= n and ptr.value
    lib.luhot_factor_destroy(h)


@pytest.mark.parametrize("n", [1, 2, 63, 64, 65, 127, 129, 300, 1000, 2500])
def test_resident_single_rhs_scaled_sweeps(n):
    """One FP64 right-hand side (lair's Factorized::solve) runs the
    block-scaled sweeps: W = D^-1 T formed at the first solve, then 64-row
    blocks split over four CTAs.  Solutions must agree with the multi-RHS
    sweeps to fast-mode rounding, meet the backward-error bound, and stay the
    same on repeated solves (W is formed once)."""
    a0 = np.random.default_rng(n + 90).standard_normal((n, n))
    f = lu.Factorized(a0.copy(), device_resident=True)
    rng = np.random.default_rng(n + 91)
    for rep in range(3):
        b = rng.standard_normal(n)
        x = f.solve(b)
        x2 = f.solve_matrix(np.stack([b, b], axis=1))[:, 0]  # the 64-row sync-free sweeps
        np.testing.assert_allclose(x, x2, rtol=0, atol=1e-9 * np.abs(x2).max())
        berr = np.abs(b - a0 @ x).max() / (np.abs(a0).sum(1).max() * np.abs(x).max() + np.abs(b).max())
        assert berr <= max(n, 1) * EPS64, (rep, berr)
        assert np.array_equal(f.solve(b), x)  # deterministic
