"""GPU parity of getrf / getrs against the lair oracle, through the C ABI.

exact mode: bit-identical LU, pivots, singular flag and solutions.
fast mode (DMMA Schur update): identical pivots where candidates are
distinct, ||PA - LU||_max / (n eps ||A||_max) <= 10 (eps = 2^-53, lair's
Real::eps for f64), normwise backward error of the solve <= n eps.
"""
import ctypes
import json
import os

import numpy as np
import pytest

import oracle
from lair_gb300 import _lib, equation, lapack, lu
from lair_gb300.errors import InvalidInput

pytestmark = pytest.mark.gpu

EPS64 = 2.0 ** -53
KATS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "lair_kats.json")))["tests"]


def rand(seed, m, n, dtype=np.float64):
    return np.random.default_rng(seed).uniform(-1, 1, (m, n)).astype(dtype)


def pa_minus_lu(a0, lu_, piv):
    """max |P^T A - L U| / (n eps max|A|) for square or rectangular factors."""
    m, n = a0.shape
    k = min(m, n)
    pa = a0.copy()
    oracle.laswp(pa, 0, piv)
    L = lu.l_matrix(lu_)
    U = lu.u_matrix(lu_)
    r = np.abs(pa - L @ U).max()
    return r / (max(m, n) * EPS64 * np.abs(a0).max())


def berr(a, x, b):
    r = b - a @ x
    return np.abs(r).max() / (np.abs(a).sum(1).max() * np.abs(x).max() + np.abs(b).max())


# ---------------------------------------------------------------- exact mode
SHAPES = [(1, 1), (2, 2), (5, 5), (17, 17), (63, 63), (64, 64), (65, 65), (127, 127), (128, 128),
          (129, 129), (256, 256), (300, 300), (70, 200), (200, 70), (1, 5), (5, 1), (64, 130), (130, 64)]


@pytest.mark.parametrize("m,n", SHAPES)
def test_exact_getrf_bitwise(m, n):
    a0 = rand(m * 1000 + n, m, n)
    a = a0.copy()
    piv, sing = lapack.getrf(a, mode="exact")
    ref = a0.copy()
    piv_r, sing_r = oracle.getrf(ref)
    assert piv == piv_r
    assert sing == sing_r
    assert np.array_equal(a, ref)


@pytest.mark.parametrize("nb", [8, 16, 32, 64])
def test_exact_getrf_bitwise_any_panel_width(nb):
    load = _lib.load()
    ctx = _lib.context()
    _lib.check(load.luhot_set_block(ctx, nb), ctx)
    try:
        a0 = rand(nb, 211, 211)
        a = a0.copy()
        piv, _ = lapack.getrf(a, mode="exact")
        ref = a0.copy()
        piv_r, _ = oracle.getrf(ref)
        assert piv == piv_r and np.array_equal(a, ref)
    finally:
        load.luhot_set_block(ctx, 0)


def test_exact_getrf_bitwise_1024():
    a0 = rand(3, 1024, 1024)
    a = a0.copy()
    piv, _ = lapack.getrf(a, mode="exact")
    ref = a0.copy()
    piv_r, _ = oracle.getrf(ref)
    assert piv == piv_r and np.array_equal(a, ref)


def test_exact_float32_bitwise():
    a0 = rand(5, 150, 150, np.float32)
    a = a0.copy()
    piv, _ = lapack.getrf(a, mode="exact")
    ref = a0.copy()
    piv_r, _ = oracle.getrf_row_major(ref)
    assert piv == piv_r and np.array_equal(a, ref)


@pytest.mark.parametrize("n,nrhs", [(1, 1), (5, 1), (64, 2), (256, 3), (333, 1)])
def test_exact_getrs_bitwise(n, nrhs):
    a0 = rand(n, n, n)
    b = rand(n + 1, n, nrhs)
    ref = a0.copy()
    piv, _ = oracle.getrf(ref)
    x = lapack.getrs(ref, piv, b, mode="exact")
    x_ref = oracle.getrs_multi(ref, piv, b)
    assert np.array_equal(x, x_ref)


def test_exact_getrs_one_dimensional_rhs():
    a0 = rand(9, 40, 40)
    b = rand(10, 40, 1)[:, 0].copy()
    ref = a0.copy()
    piv, _ = oracle.getrf(ref)
    x = lapack.getrs(ref, piv, b, mode="exact")
    assert x.shape == (40,)
    assert np.array_equal(x, oracle.getrs(ref, piv, b))


# ------------------------------------------------------------ lair KATs (GPU)
@pytest.mark.parametrize("name", ["getrf::square_row_major", "getrf::square_col_major",
                                  "getrf::square_negative_strides", "getrf::tall", "getrf::wide"])
@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_kats_on_gpu(name, mode):
    t = KATS[name]
    a = np.array(t["arrays"][0]["value"], dtype=np.float64)
    for tr in t["transforms"]:
        a = {"swap_axes(0, 1)": lambda v: v.T, "invert_axis(Axis(0))": lambda v: v[::-1, :],
             "invert_axis(Axis(1))": lambda v: v[:, ::-1]}[tr](a)
    piv, sing = lapack.getrf(a, mode=mode)
    assert piv == t["vecs"][0] and sing is None
    expect = np.array(t["arrays"][1]["value"])
    np.testing.assert_allclose(a, expect, rtol=0, atol=t["epsilon"][0] if t["epsilon"] else 1e-15)


def test_kat_singular_and_small():
    a = np.array(KATS["getrf::singular"]["arrays"][0]["value"])
    _, sing = lapack.getrf(a, mode="exact")
    assert sing == 1
    a = np.array([[3.0]])
    assert lapack.getrf(a) == ([0], None) and a[0, 0] == 3.0
    assert lapack.getrf(np.zeros((0, 0))) == ([], None)
    assert lapack.getrf(np.zeros((0, 4))) == ([], None)


def test_kat_getrs_on_gpu():
    t = KATS["getrs::square_5x5"]
    a = np.array(t["arrays"][0]["value"])
    piv, _ = lapack.getrf(a, mode="exact")
    x = lapack.getrs(a, piv, np.array(t["arrays"][1]["value"]), mode="exact")
    assert np.all(np.abs(x - 1.0) <= np.finfo(np.float64).eps)


def test_equation_doctest_exact_on_gpu():
    x = equation.solve(np.array([[3.0, 1.0], [1.0, 2.0]]), np.array([9.0, 8.0]), mode="exact")
    assert np.array_equal(x, np.array([2.0, 3.0]))


@pytest.mark.parametrize("name", ["lu::square", "lu::wide", "lu::tall"])
def test_lu_kats_on_gpu(name):
    t = KATS[name]
    a = np.array(t["arrays"][0]["value"], dtype=np.float32)
    f = lu.Factorized(a, mode="exact")
    mats = {"p": f.p(), "l": f.l(), "u": f.u()}
    for s in t["indexed"]:
        got = mats[s["var"]][s["i"], s["j"]]
        if s["macro"] == "eq":
            assert got == s["value"]
        else:
            np.testing.assert_allclose(got, s["value"], rtol=t["max_relative"][0])


@pytest.mark.parametrize("name", ["lu::lu_pl_singular", "lu::lu_pl_square", "lu::lu_pl_tall_l",
                                  "lu::lu_pl_wide_u"])
def test_into_pl_kats_on_gpu(name):
    t = KATS[name]
    m = np.array(t["arrays"][0]["value"], dtype=np.float32)
    k = min(m.shape)
    pl = lu.Factorized(m, mode="exact").into_pl()
    np.testing.assert_array_equal(pl[:, :k], np.array(t["arrays"][1]["value"], dtype=np.float32))


# ------------------------------------------------------------ singular input
def test_singular_last_zero_pivot_wins():
    a0 = rand(1, 50, 50)
    a0[:, 7] = 0.0
    a0[:, 31] = 0.0
    for mode in ("exact", "fast"):
        a = a0.copy()
        piv, sing = lapack.getrf(a, mode=mode)
        ref = a0.copy()
        piv_r, sing_r = oracle.getrf(ref)
        assert sing == sing_r
        assert piv == piv_r
    zero = np.zeros((6, 6))
    _, sing = lapack.getrf(zero)
    assert sing == 5


def test_nan_never_wins_pivot_search():
    a0 = rand(2, 20, 20)
    a0[0, 0] = np.nan
    a = a0.copy()
    piv, _ = lapack.getrf(a, mode="exact")
    ref = a0.copy()
    piv_r, _ = oracle.getrf(ref)
    assert piv == piv_r
    np.testing.assert_array_equal(np.isnan(a), np.isnan(ref))
    np.testing.assert_array_equal(np.nan_to_num(a), np.nan_to_num(ref))


def test_ties_pick_first_row():
    a = np.array([[1.0, 2.0, 0.0], [-3.0, 1.0, 1.0], [3.0, 5.0, 2.0]])
    piv, _ = lapack.getrf(a.copy(), mode="fast")
    piv_r, _ = oracle.getrf(a.copy())
    assert piv == piv_r and piv[0] == 1


# ------------------------------------------------------------------ fast mode
@pytest.mark.parametrize("n", [256, 1000, 2048])
def test_fast_getrf_pivots_and_residual(n):
    rng = np.random.default_rng(n)
    a0 = rng.standard_normal((n, n))
    a = a0.copy()
    piv, sing = lapack.getrf(a, mode="fast")
    assert sing is None
    ref = a0.copy()
    piv_r, _ = oracle.getrf(ref) if n <= 1000 else (None, None)
    if piv_r is not None:
        assert piv == piv_r
        np.testing.assert_allclose(a, ref, rtol=0, atol=1e-9 * np.abs(ref).max())
    else:
        scipy_lapack = pytest.importorskip("scipy.linalg.lapack")
        _, piv_sp, _ = scipy_lapack.dgetrf(a0)
        assert piv == [int(p) for p in piv_sp]
    assert pa_minus_lu(a0, a, piv) <= 10.0


@pytest.mark.parametrize("n,nrhs", [(256, 1), (1000, 16), (2048, 16)])
def test_fast_solve_backward_error(n, nrhs):
    rng = np.random.default_rng(n + nrhs)
    a0 = rng.standard_normal((n, n))
    b = rng.standard_normal((n, nrhs))
    a = a0.copy()
    piv, _ = lapack.getrf(a, mode="fast")
    x = lapack.getrs(a, piv, b, mode="fast")
    assert berr(a0, x, b) <= n * EPS64
    # relative error against lair's own FP64 solution (oracle), stated
    if n <= 1000:
        ref = a0.copy()
        piv_r, _ = oracle.getrf(ref)
        x_ref = oracle.getrs_multi(ref, piv_r, b)
        rel = np.abs(x - x_ref).max() / np.abs(x_ref).max()
        assert rel <= 1e-8


def test_transposed_solve():
    rng = np.random.default_rng(4)
    n = 300
    a0 = rng.standard_normal((n, n))
    b = rng.standard_normal((n, 4))
    a = a0.copy()
    piv, _ = lapack.getrf(a, mode="fast")
    x = lapack.getrs(a, piv, b, mode="fast", trans=True)
    assert berr(a0.T, x, b) <= n * EPS64


def test_gesv_matches_factor_then_solve():
    rng = np.random.default_rng(5)
    n = 500
    a0 = rng.standard_normal((n, n))
    b = rng.standard_normal((n, 3))
    x = np.empty_like(b)
    lib, ctx = _lib.load(), _lib.context()
    rc = lib.luhot_dgesv(ctx, n, 3, a0.ctypes.data, n, 1, b.ctypes.data, 3, 1, x.ctypes.data, 3, 1, 0)
    _lib.check(rc, ctx)
    a = a0.copy()
    piv, _ = lapack.getrf(a)
    np.testing.assert_array_equal(x, lapack.getrs(a, piv, b))


@pytest.mark.parametrize("n,order", [(1024, "C"), (1536, "C"), (1024, "F")])
def test_gesv_large_host_inputs(n, order):
    """Host inputs of 8 MiB or more: a contiguous row-major A (n a multiple of
    32) is read by the GPU straight from pageable memory where the device
    reaches it (else page-locked for the call); other layouts take the staged
    copy.  The solution equals the one from the device-resident factor and
    solve bit for bit, and the caller's A is left untouched."""
    rng = np.random.default_rng(n)
    a0 = np.asarray(rng.standard_normal((n, n)), order=order)
    keep = a0.copy(order="K")
    b = rng.standard_normal((n, 16))
    x = np.empty_like(b)
    lib, ctx = _lib.load(), _lib.context()
    rc = lib.luhot_dgesv(ctx, n, 16, a0.ctypes.data, a0.strides[0] // 8, a0.strides[1] // 8, b.ctypes.data, 16, 1,
                         x.ctypes.data, 16, 1, 0)
    _lib.check(rc, ctx)
    assert np.array_equal(a0, keep)
    a = np.ascontiguousarray(keep)
    piv, _ = lapack.getrf(a)
    np.testing.assert_array_equal(x, lapack.getrs(a, piv, b))


def test_gesv_singular_status():
    lib, ctx = _lib.load(), _lib.context()
    a = np.ones((4, 4))
    b = np.ones((4, 1))
    x = np.empty_like(b)
    rc = lib.luhot_dgesv(ctx, 4, 1, a.ctypes.data, 4, 1, b.ctypes.data, 1, 1, x.ctypes.data, 1, 1, 0)
    assert rc == _lib.LUHOT_ERR_SINGULAR


# ------------------------------------------------------------- API behaviour
def test_equation_solve_errors():
    with pytest.raises(InvalidInput.Shape):
        equation.solve(np.zeros((2, 3)), np.zeros(2))
    with pytest.raises(InvalidInput.Shape):
        equation.solve(np.eye(3), np.zeros(2))
    with pytest.raises(InvalidInput.Value):
        equation.solve(np.ones((3, 3)), np.ones(3))
    a = np.array([[3.0, 1.0], [1.0, 2.0]])
    equation.solve(a, np.array([9.0, 8.0]))
    assert np.array_equal(a, np.array([[3.0, 1.0], [1.0, 2.0]]))  # input untouched


def test_factorized_solve_shape_error_and_getrs_panics():
    f = lu.Factorized(np.eye(3))
    with pytest.raises(InvalidInput.Shape):
        f.solve(np.zeros(4))
    with pytest.raises(AssertionError):
        lapack.getrs(np.eye(3), [0, 1], np.zeros(3))
    with pytest.raises(AssertionError):
        lapack.getrs(np.eye(3), [0, 1, 2], np.zeros(2))


def test_invalid_arguments_return_status_not_crash():
    lib, ctx = _lib.load(), _lib.context()
    assert lib.luhot_dgetrf(ctx, -1, 2, None, 1, 1, None, None, 0) == _lib.LUHOT_ERR_INVALID_ARG
    a = np.eye(2)
    piv = np.zeros(2, dtype=np.uint64)
    assert lib.luhot_dgetrf(ctx, 2, 2, a.ctypes.data, 2, 1, None, None, 0) == _lib.LUHOT_ERR_INVALID_ARG
    assert lib.luhot_dgetrf(ctx, 2, 2, a.ctypes.data, 2, 1, piv.ctypes.data, None, 7) == _lib.LUHOT_ERR_INVALID_ARG
    bad_piv = np.array([5, 1], dtype=np.uint64)
    b = np.ones((2, 1))
    x = np.empty_like(b)
    rc = lib.luhot_dgetrs(ctx, 2, 1, a.ctypes.data, 2, 1, bad_piv.ctypes.data, b.ctypes.data, 1, 1,
                          x.ctypes.data, 1, 1, 0, 0)
    assert rc == _lib.LUHOT_ERR_INVALID_ARG
    assert b"pivot" in lib.luhot_last_error(ctx)


def test_wait_timeout_is_reported_and_context_survives():
    lib, ctx = _lib.load(), _lib.context()
    rc = lib.luhot_selftest_wait_timeout(ctx, 50)
    assert rc == _lib.LUHOT_ERR_TIMEOUT
    assert b"timed out" in lib.luhot_last_error(ctx)
    a0 = rand(8, 100, 100)
    a = a0.copy()
    piv, _ = lapack.getrf(a, mode="exact")
    ref = a0.copy()
    assert oracle.getrf(ref)[0] == piv and np.array_equal(a, ref)


def test_device_entry_points_with_torch_buffers():
    torch = pytest.importorskip("torch")
    n, nrhs = 384, 2
    a0 = rand(21, n, n)
    b0 = rand(22, n, nrhs)
    lda = n + 16
    d_a = torch.zeros((n, lda), dtype=torch.float64, device="cuda")
    d_a[:, :n] = torch.from_numpy(a0).cuda()
    d_piv = torch.zeros(n, dtype=torch.int32, device="cuda")
    d_b = torch.from_numpy(b0).cuda().contiguous()
    torch.cuda.synchronize()
    lib, ctx = _lib.load(), _lib.context()
    sing = ctypes.c_int64(0)
    _lib.check(lib.luhot_dgetrf_dev(ctx, n, n, d_a.data_ptr(), lda, d_piv.data_ptr(), ctypes.byref(sing), 1), ctx)
    _lib.check(lib.luhot_dgetrs_dev(ctx, n, nrhs, d_a.data_ptr(), lda, d_piv.data_ptr(), d_b.data_ptr(), nrhs, 0, 1), ctx)
    ref = a0.copy()
    piv_r, _ = oracle.getrf(ref)
    assert sing.value == -1
    assert d_piv.cpu().tolist() == piv_r
    assert np.array_equal(d_a[:, :n].cpu().numpy(), ref)
    assert np.array_equal(d_b.cpu().numpy(), oracle.getrs_multi(ref, piv_r, b0))


def test_profile_and_launch_count():
    _lib.profile_enable(True)
    n0 = _lib.launch_count()
    a = rand(30, 512, 512)
    lapack.getrf(a, mode="fast")
    prof = _lib.profile_read()
    _lib.profile_enable(False)
    assert _lib.launch_count() > n0
    assert prof["gemm"]["launches"] > 0 and prof["panel"]["launches"] == 8
    total_flops = sum(v["flops"] for v in prof.values())
    assert abs(total_flops - 2 / 3 * 512 ** 3) / (2 / 3 * 512 ** 3) < 0.05
