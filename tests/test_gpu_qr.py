"""GPU Householder QR (luhot_[ds]geqrf, luhot_[ds]qr_q) against the oracle.

exact mode: the factored array, tau and Q equal the oracle's (lair's geqrf and
qr::Factorized::q restated) bit for bit, for square, tall, wide, f32, strided
inputs, zero columns (tau = 0) and columns small enough for larfg's rescaling.
fast mode: ||A - QR|| and ||Q^T Q - I|| within a small multiple of n * eps.
"""
import numpy as np
import pytest

import oracle
from lair_gb300 import _lib, qr

pytestmark = pytest.mark.gpu


def rand(seed, m, n, dtype=np.float64):
    return np.random.default_rng(seed).uniform(-1, 1, (m, n)).astype(dtype)


def exact_pair(a0):
    gpu, ref = a0.copy(), a0.copy()
    f = qr.Factorized(gpu, mode="exact")
    tau_r = oracle.geqrf(ref)
    return f, ref, tau_r


@pytest.mark.parametrize("m,n", [(1, 1), (3, 3), (4, 3), (3, 4), (17, 17), (64, 40), (40, 64), (130, 130),
                                 (300, 200), (200, 300)])
def test_exact_geqrf_and_q_bitwise(m, n):
    a0 = rand(m * 13 + n, m, n)
    f, ref, tau_r = exact_pair(a0)
    assert np.array_equal(f.qr, ref)
    assert np.array_equal(f.tau, tau_r)
    assert np.array_equal(f.q(), oracle.qr_q(ref, tau_r))
    assert np.array_equal(f.r(), oracle.qr_r(ref))


def test_exact_float32_and_strided_inputs():
    a0 = rand(5, 90, 70, np.float32)
    f, ref, tau_r = exact_pair(a0)
    assert np.array_equal(f.qr, ref) and np.array_equal(f.tau, tau_r)
    big = rand(6, 120, 100)
    view_g, view_r = np.asfortranarray(big)[::-1, :80], np.asfortranarray(big)[::-1, :80]
    tau_g = qr.geqrf(view_g, mode="exact")
    tau_o = oracle.geqrf(view_r)
    assert np.array_equal(view_g, view_r) and np.array_equal(tau_g, tau_o)


def test_exact_zero_and_tiny_columns():
    a0 = rand(7, 50, 30)
    a0[:, 3] = 0.0             # tau = 0, column untouched
    a0[10:, 5] = 0.0           # x = 0 below the diagonal
    a0[:, 8] *= 1e-300         # larfg's rescaling loop (|beta| < sfmin / eps)
    f, ref, tau_r = exact_pair(a0)
    assert np.array_equal(f.qr, ref)
    assert np.array_equal(f.tau, tau_r)
    assert f.tau[3] == 0.0
    assert np.array_equal(f.q(), oracle.qr_q(ref, tau_r))


@pytest.mark.parametrize("m,n", [(512, 512), (1000, 600), (600, 1000)])
def test_fast_qr_accuracy(m, n):
    a0 = rand(m + n, m, n)
    f = qr.Factorized(a0.copy())
    q, r = f.q(), f.r()
    eps = 2.0 ** -53
    k = max(m, n)
    assert np.abs(q @ r - a0).max() <= 20 * k * eps * np.abs(a0).max()
    assert np.abs(q.T @ q - np.eye(m)).max() <= 20 * k * eps
    _, ref, tau_r = exact_pair(a0)
    np.testing.assert_allclose(f.tau, tau_r, rtol=0, atol=1e-10)


def test_qr_kats_on_gpu():
    import json
    import os
    kats = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "lair_kats.json")))["tests"]
    t = kats["qr::square"]
    a = np.array(t["arrays"][0]["value"])
    f = qr.Factorized(a, mode="exact")
    np.testing.assert_allclose(f.qr, np.array(t["arrays"][1]["value"]), atol=1e-6)
    np.testing.assert_allclose(f.tau, np.array(t["arrays"][2]["value"]), atol=1e-6)
    np.testing.assert_allclose(f.q(), np.array(t["arrays"][3]["value"]), atol=1e-6)
    np.testing.assert_allclose(f.r(), np.array(t["arrays"][4]["value"]), atol=1e-6)
    t = kats["geqrf::wide"]
    a = np.array(t["arrays"][0]["value"], dtype=np.float32)
    tau = qr.geqrf(a, mode="exact")
    np.testing.assert_allclose(a, np.array(t["arrays"][1]["value"]), atol=1e-6)
    np.testing.assert_allclose(tau, np.array(t["arrays"][2]["value"]), atol=1e-6)


def test_qr_device_entry_and_errors():
    torch = pytest.importorskip("torch")
    lib, ctx = _lib.load(), _lib.context()
    a0 = rand(9, 256, 200)
    d = torch.from_numpy(a0).cuda()
    tau = torch.zeros(200, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    _lib.check(lib.luhot_dgeqrf_dev(ctx, 256, 200, d.data_ptr(), 200, tau.data_ptr(), 1), ctx)
    torch.cuda.synchronize()  # the device entry is asynchronous on the context's stream
    ref = a0.copy()
    tau_r = oracle.geqrf(ref)
    assert np.array_equal(d.cpu().numpy(), ref) and np.array_equal(tau.cpu().numpy(), tau_r)
    assert lib.luhot_dgeqrf(ctx, -1, 2, None, 1, 1, None, 0) == _lib.LUHOT_ERR_INVALID_ARG
    x = np.zeros((2, 2))
    t = np.zeros(2)
    assert lib.luhot_dgeqrf(ctx, 2, 2, x.ctypes.data, 2, 1, t.ctypes.data, 9) == _lib.LUHOT_ERR_INVALID_ARG
