"""Pin the CPU oracle to lair's own known-answer tests (no GPU).

tests/golden/lair_kats.json holds the literal inputs and expected outputs of
lair's unit tests for the LU path (extracted by tests/golden/make_lair_kats.py
from src/lapack/getrf.rs, src/lapack/getrs.rs, src/decomposition/lu.rs,
src/blas/iamax.rs and the equation::solve doc-test).  Each test below replays
one of them through the oracle, with lair's own tolerance.  The host-side
Factorized helpers (p/l/u/into_pl) are checked on the oracle's factors too.
"""
import json
import os

import numpy as np
import pytest

import oracle
from lair_gb300 import lu as host_lu

KATS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "lair_kats.json")))
T = KATS["tests"]


def arr(v, dtype=np.float64):
    return np.array(v, dtype=dtype)


def test_kat_file_covers_lu_path():
    expected = {"getrf::singular", "getrf::empty", "getrf::smallest", "getrf::recursive_square",
                "getrf::square_row_major", "getrf::square_col_major", "getrf::square_negative_strides",
                "getrf::wide", "getrf::tall", "getrs::square_2x2", "getrs::square_5x5", "iamax::iamax",
                "lu::square", "lu::wide", "lu::tall", "lu::lu_pl_identity_l", "lu::lu_pl_singular",
                "lu::lu_pl_square", "lu::lu_pl_tall_l", "lu::lu_pl_wide_u", "getrf::recursive_empty",
                "getrf::recursive_smallest", "getrf::square_complex"}
    assert expected <= set(T)


def test_getrf_singular():
    t = T["getrf::singular"]
    a = arr(t["arrays"][0]["value"])
    _, singular = oracle.getrf(a)
    assert singular == t["somes"][0] == 1


def test_getrf_empty():
    a = np.zeros((0, 0), dtype=np.float32)
    piv, singular = oracle.getrf(a)
    assert piv == [] and singular is None
    ok, piv, _ = oracle.getrf_recursive(np.zeros((0, 0)))
    assert ok and piv == []


@pytest.mark.parametrize("name", ["getrf::smallest", "getrf::recursive_smallest"])
def test_getrf_smallest(name):
    t = T[name]
    a = arr(t["arrays"][0]["value"])
    if "recursive" in name:
        ok, piv, _ = oracle.getrf_recursive(a)
        assert ok
    else:
        piv, singular = oracle.getrf(a)
        assert singular is None
    assert piv == t["vecs"][0]
    np.testing.assert_array_equal(a, arr(t["arrays"][1]["value"]))


def _view(t, a):
    for tr in t["transforms"]:
        if tr == "swap_axes(0, 1)":
            a = a.T
        elif tr == "invert_axis(Axis(0))":
            a = a[::-1, :]
        elif tr == "invert_axis(Axis(1))":
            a = a[:, ::-1]
    return a


@pytest.mark.parametrize("name", ["getrf::square_row_major", "getrf::square_col_major",
                                  "getrf::square_negative_strides", "getrf::tall", "getrf::wide"])
def test_getrf_square_layouts(name):
    t = T[name]
    a = _view(t, arr(t["arrays"][0]["value"]))
    piv, singular = oracle.getrf(a)
    assert piv == t["vecs"][0]
    assert singular is None
    expect = arr(t["arrays"][1]["value"])
    if t["epsilon"]:
        np.testing.assert_allclose(a, expect, rtol=0, atol=t["epsilon"][0])
    else:  # lair asserts exact equality (wide)
        np.testing.assert_array_equal(a, expect)


def test_layout_dispatch_matches_lair():
    """F-order and negative-stride views must take the col-major path."""
    base = np.arange(25, dtype=np.float64).reshape(5, 5)
    assert oracle.is_standard_layout(base)
    assert not oracle.is_standard_layout(base.T)
    assert not oracle.is_standard_layout(base[::-1, ::-1])
    assert oracle.is_standard_layout(base[:1, :])  # length-1 axes are ignored
    assert oracle.is_standard_layout(np.zeros((0, 3)))


def test_getrf_recursive_square():
    t = T["getrf::recursive_square"]
    a = arr(t["arrays"][0]["value"])
    ok, piv, _ = oracle.getrf_recursive(a)
    assert ok and piv == t["vecs"][0]
    np.testing.assert_allclose(a, arr(t["arrays"][1]["value"]), rtol=0, atol=t["epsilon"][0])


def test_getrs_2x2():
    t = T["getrs::square_2x2"]
    a = arr(t["arrays"][0]["value"])
    piv, _ = oracle.getrf(a)
    assert piv == t["vecs"][0]
    x = oracle.getrs(a, piv, arr(t["arrays"][1]["value"]))
    for s in t["scalar"]:
        np.testing.assert_allclose(x[s["i"]], s["value"], rtol=t["max_relative"][0])


def test_getrs_5x5_within_machine_epsilon():
    t = T["getrs::square_5x5"]
    a = arr(t["arrays"][0]["value"])
    piv, _ = oracle.getrf(a)
    x = oracle.getrs(a, piv, arr(t["arrays"][1]["value"]))
    # assert_abs_diff_eq! with the default epsilon, f64::EPSILON
    for s in t["scalar"]:
        assert abs(x[s["i"]] - s["value"]) <= np.finfo(np.float64).eps


def test_iamax():
    t = T["iamax::iamax"]
    idx, mx = oracle.iamax(arr(t["arrays"][0]["value"]))
    want = {s["var"]: s["value"] for s in t["scalar"]}
    assert idx == want["idx"] and mx == want["max"]


def test_iamax_edge_semantics():
    # first index wins ties; NaN never wins; all-zero gives (0, 0)
    assert oracle.iamax(np.array([1.0, -3.0, 3.0]))[0] == 1
    assert oracle.iamax(np.array([np.nan, 2.0, np.nan]))[0] == 1
    assert oracle.iamax(np.array([0.0, -0.0, 0.0])) == (0, 0.0)


def test_equation_doctest_exact():
    t = KATS["doctest_equation_solve"]
    a = arr(t["a"])
    piv, singular = oracle.getrf(a)
    assert singular is None
    x = oracle.getrs(a, piv, arr(t["b"]))
    np.testing.assert_array_equal(x, arr(t["x"]))


@pytest.mark.parametrize("name", ["lu::square", "lu::wide", "lu::tall"])
def test_lu_plu_extraction(name):
    t = T[name]
    a = arr(t["arrays"][0]["value"], np.float32)
    piv, _ = oracle.getrf(a)
    mats = {"p": host_lu.p_matrix(a.shape[0], piv, np.float32), "l": host_lu.l_matrix(a),
            "u": host_lu.u_matrix(a)}
    shape_order = ["p", "l", "u"]
    for var, shp in zip(shape_order, t["shapes"]):
        assert list(mats[var].shape) == shp
    for s in t["indexed"]:
        got = mats[s["var"]][s["i"], s["j"]]
        if s["macro"] == "eq":
            assert got == s["value"]
        else:
            np.testing.assert_allclose(got, s["value"], rtol=t["max_relative"][0])


@pytest.mark.parametrize("name", ["lu::lu_pl_identity_l", "lu::lu_pl_singular", "lu::lu_pl_square",
                                  "lu::lu_pl_tall_l", "lu::lu_pl_wide_u"])
def test_lu_into_pl(name):
    t = T[name]
    m = arr(t["arrays"][0]["value"], np.float32)
    expect = m.copy() if name == "lu::lu_pl_identity_l" else arr(t["arrays"][1]["value"], np.float32)
    k = min(m.shape)
    piv, _ = oracle.getrf(m)
    pl = host_lu.into_pl(m, piv)
    np.testing.assert_array_equal(pl[:, :k], expect)


def test_complex_kat_is_out_of_scope():
    # lair's square_complex KAT exercises Complex64, which stays on lair's own
    # code path (the GPU path covers f64/f32 only).
    assert T["getrf::square_complex"]["indexed"]


# ---------------------------------------------------------------------------
# Beyond lair's KATs: the three getrf variants and scipy agree on pivots for
# random inputs with distinct candidates; the row-major oracle is exactly the
# unblocked right-looking algorithm.
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("seed,m,n", [(0, 37, 37), (1, 64, 40), (2, 40, 64), (3, 100, 100)])
def test_variants_agree_on_pivots(seed, m, n):
    rng = np.random.default_rng(seed)
    a0 = rng.uniform(-1, 1, (m, n))
    a_row = a0.copy()
    piv_row, s_row = oracle.getrf(a_row)
    a_col = np.asfortranarray(a0)
    piv_col, s_col = oracle.getrf(a_col)
    assert piv_row == piv_col and s_row is None and s_col is None
    np.testing.assert_allclose(a_row, a_col, rtol=0, atol=1e-11)
    if m >= n:  # lair's recursive variant is only meant for tall/square
        a_rec = a0.copy()
        ok, piv_rec, _ = oracle.getrf_recursive(a_rec)
        assert ok and piv_rec[:min(m, n)] == piv_row
        np.testing.assert_allclose(a_rec, a_row, rtol=0, atol=1e-11)


def test_oracle_matches_scipy_getrf_pivots():
    scipy_lapack = pytest.importorskip("scipy.linalg.lapack")
    rng = np.random.default_rng(7)
    a0 = rng.uniform(-1, 1, (256, 256))
    a = a0.copy()
    piv, singular = oracle.getrf(a)
    lu_sp, piv_sp, info = scipy_lapack.dgetrf(a0)
    assert info == 0 and singular is None
    assert piv == [int(p) for p in piv_sp]
    np.testing.assert_allclose(a, lu_sp, rtol=0, atol=1e-10)


def test_oracle_row_major_is_plain_unblocked_elimination():
    """A direct numpy restatement of src/lapack/getrf.rs:55-89 gives the same bits."""
    rng = np.random.default_rng(11)
    a0 = rng.uniform(-1, 1, (24, 24))
    a = a0.copy()
    oracle.getrf(a)
    b = a0.copy()
    n = b.shape[0]
    for ul in range(n):
        col = np.abs(b[ul:, ul])
        idx = int(np.argmax(col))
        if idx:
            b[[ul, ul + idx]] = b[[ul + idx, ul]]
        r = 1.0 / b[ul, ul]
        for j in range(ul + 1, n):
            b[j, ul] *= r
            b[j, ul + 1:] -= b[j, ul] * b[ul, ul + 1:]
    np.testing.assert_array_equal(a, b)
