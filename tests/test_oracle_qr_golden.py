"""Pin the oracle's QR restatement to lair's own known-answer tests (no GPU).

The entries come from lair's test modules for geqrf (src/lapack/geqrf.rs),
qr::Factorized (src/decomposition/qr.rs), larfg (src/lapack/larfg.rs),
larf::left (src/lapack/larf.rs) and nrm2 (src/blas/nrm2.rs), extracted as
text by tests/golden/make_lair_kats.py.  Each test replays one of them
through the oracle with lair's own tolerance; complex-valued tests are out of
scope (the GPU path covers f64 and f32).
"""
import json
import os

import numpy as np
import pytest

import oracle

KATS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "lair_kats.json")))
T = KATS["tests"]


def arr(v, dtype=np.float64):
    return np.array(v, dtype=dtype)


def test_kat_file_covers_qr():
    expected = {"geqrf::square_real_smallest", "geqrf::square_real", "geqrf::tall", "geqrf::wide",
                "qr::square", "qr::tall", "qr::wide", "larfg::larfg_empty", "larfg::larfg_real",
                "larf::left_real", "nrm2::real"}
    assert expected <= set(T)


@pytest.mark.parametrize("name,dtype", [("geqrf::square_real_smallest", np.float64),
                                        ("geqrf::square_real", np.float64), ("geqrf::tall", np.float64),
                                        ("geqrf::wide", np.float32)])
def test_geqrf(name, dtype):
    t = T[name]
    a = arr(t["arrays"][0]["value"], dtype)
    tau = oracle.geqrf(a)
    eps = t["epsilon"][0]
    np.testing.assert_allclose(a, arr(t["arrays"][1]["value"]), rtol=0, atol=eps)
    np.testing.assert_allclose(tau, arr(t["arrays"][2]["value"]), rtol=0, atol=eps)


def test_qr_square_q_and_r():
    t = T["qr::square"]
    a = arr(t["arrays"][0]["value"])
    tau = oracle.geqrf(a)
    np.testing.assert_allclose(a, arr(t["arrays"][1]["value"]), atol=1e-6)
    np.testing.assert_allclose(tau, arr(t["arrays"][2]["value"]), atol=1e-6)
    np.testing.assert_allclose(oracle.qr_q(a, tau), arr(t["arrays"][3]["value"]), atol=1e-6)
    np.testing.assert_allclose(oracle.qr_r(a), arr(t["arrays"][4]["value"]), atol=1e-6)


@pytest.mark.parametrize("name,dtype", [("qr::tall", np.float64), ("qr::wide", np.float32)])
def test_qr_q_and_r(name, dtype):
    t = T[name]
    a0 = arr(t["arrays"][0]["value"], dtype)
    a = a0.copy()
    tau = oracle.geqrf(a)
    q, r = oracle.qr_q(a, tau), oracle.qr_r(a)
    np.testing.assert_allclose(q, arr(t["arrays"][1]["value"]), atol=1e-6)
    np.testing.assert_allclose(r, arr(t["arrays"][2]["value"]), atol=1e-6)
    np.testing.assert_allclose(q @ r, a0, atol=1e-5)


def test_larfg():
    t = T["larfg::larfg_real"]
    x = arr(t["arrays"][0]["value"])
    beta, tau = oracle.larfg(t["call_args"][0][0], x)
    got = {"beta": beta, "tau": tau}
    for s in t["scalar"]:
        assert abs(got[s["var"]] - s["value"]) <= 1e-6
    np.testing.assert_allclose(x, arr(t["arrays"][1]["value"]), atol=1e-6)
    t = T["larfg::larfg_empty"]
    beta, tau = oracle.larfg(t["call_args"][0][0], np.zeros(0))
    assert (beta, tau) == (2.0, 0.0)


def test_larf_left():
    t = T["larf::left_real"]
    v = arr(t["arrays"][0]["value"])
    c = arr(t["arrays"][1]["value"])
    oracle.larf_left(v, t["call_args"][0][0], c)
    np.testing.assert_allclose(c, arr(t["arrays"][2]["value"]), atol=1e-8)


def test_nrm2():
    t = T["nrm2::real"]
    assert oracle.nrm2(arr(t["arrays"][0]["value"])) == t["scalar"][0]["value"]


def test_geqrf_matches_numpy_householder_up_to_signs():
    # An independent check at a larger size: R agrees with LAPACK's up to the
    # sign of each row, and Q R reproduces A.
    rng = np.random.default_rng(3)
    a0 = rng.standard_normal((40, 30))
    a = a0.copy()
    tau = oracle.geqrf(a)
    r = oracle.qr_r(a)[:30]
    r_np = np.linalg.qr(a0, mode="r")
    np.testing.assert_allclose(np.abs(r), np.abs(r_np), atol=1e-12)
    q = oracle.qr_q(a, tau)
    np.testing.assert_allclose(q[:, :30] @ r, a0, atol=1e-12)
    np.testing.assert_allclose(q.T @ q, np.eye(40), atol=1e-13)
