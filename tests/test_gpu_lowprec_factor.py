"""The low-precision factorization behind the mixed-precision solves, against
its CPU emulation (tests/lowprec_emulation.py; no lair counterpart exists).

On A = Q1 diag(sigma) Q2^T (sigma geometric 1 -> 1/kappa) the quality of a
factor M = P^T L U as a preconditioner is what decides whether refinement
converges: ||I - M^-1 A||_2 and the number of singular values of M^-1 A far
from 1.  The GPU's factors (``luhot_sgetrf_mixed_dev``: FP32 panels,
tensor-core Schur updates with scaled BF16 / FP16 or rounded TF32 operands)
must be as good as the emulation of the same algorithm: within a factor 2
of its ||I - M^-1 A||_2 where that norm is below 100 (beyond, it is set by a
few nearly singular directions and is rounding noise), and with the number
of far singular values within a factor 1.5 (+-8).  The figures are printed
(``pytest -s``).  With 11-bit factors at kappa = 1e4 GMRES-IR must converge,
in at most twice the iterations the emulated unrestarted GMRES-IR needs.
"""
import ctypes

import numpy as np
import pytest

import lowprec_emulation as emu
from lair_gb300 import _lib

pytestmark = pytest.mark.gpu


def gpu_factor(torch, a, kind):
    lib, ctx = _lib.load(), _lib.context()
    n = a.shape[0]
    d = torch.from_numpy(a.astype(np.float32)).cuda()
    piv = torch.zeros(n, dtype=torch.int32, device="cuda")
    sing = ctypes.c_int64(0)
    torch.cuda.synchronize()
    _lib.check(lib.luhot_sgetrf_mixed_dev(ctx, n, n, d.data_ptr(), n, piv.data_ptr(), _lib.PRECISIONS[kind],
                                          ctypes.byref(sing)), ctx)
    assert sing.value == -1
    return d.cpu().numpy(), emu.perm_from_pivots(piv.cpu().numpy())


@pytest.mark.parametrize("kind,kappa", [("fp32", 1e6), ("tf32", 1e2), ("tf32", 1e4), ("fp16", 1e4), ("bf16", 1e2),
                                        ("bf16", 1e4)])
def test_gpu_factor_as_good_as_emulation(kind, kappa):
    torch = pytest.importorskip("torch")
    n = 1024
    a, _ = emu.conditioned(n, kappa, seed=3)
    lu_g, perm_g = gpu_factor(torch, a, kind)
    lu_e, perm_e = emu.factor(a, kind)
    qg, qe = emu.quality(a, lu_g, perm_g), emu.quality(a, lu_e, perm_e)
    print(f"\nn={n} kappa={kappa:g} {kind}: gpu {qg}\n  emulation {qe}")
    if qe["norm_I_minus_MinvA"] < 100:
        assert qg["norm_I_minus_MinvA"] <= 2.0 * qe["norm_I_minus_MinvA"] + 1e-3
    else:
        # A factor that poor has a few nearly singular directions whose size
        # is rounding noise; how many directions are bad is what compares.
        assert qg["norm_I_minus_MinvA"] > 10
    assert qg["sv_far_from_1"] <= 1.5 * qe["sv_far_from_1"] + 8
    assert qg["sv_far_from_1"] >= qe["sv_far_from_1"] / 1.5 - 8
    assert qg["growth"] <= 2.0 * qe["growth"]


@pytest.mark.parametrize("kind", ["tf32", "fp16"])
def test_gmres_ir_with_11_bit_factors_converges_at_kappa_1e4(kind):
    torch = pytest.importorskip("torch")
    n = 2048
    a, b = emu.conditioned(n, 1e4, seed=3)
    lib, ctx = _lib.load(), _lib.context()
    d_a = torch.from_numpy(a).cuda()
    d_b = torch.from_numpy(b).cuda()
    d_x = torch.empty_like(d_b)
    info = _lib.IrInfo()
    torch.cuda.synchronize()
    rc = lib.luhot_dgesv_ir_dev(ctx, n, 1, d_a.data_ptr(), n, d_b.data_ptr(), 1, d_x.data_ptr(), 1,
                                _lib.PRECISIONS[kind], _lib.REFINE_GMRES, 0.0, 50, ctypes.byref(info))
    x = d_x.cpu().numpy()
    berr = np.abs(b - a @ x).max() / (np.abs(a).sum(1).max() * np.abs(x).max() + np.abs(b).max())
    lu_e, perm_e = emu.factor(a, kind)
    _, inner_e, _ = emu.gmres_ir(a, b, lu_e, perm_e, restart=1000, max_inner=1000)
    print(f"\nn={n} kappa=1e4 {kind} GMRES-IR: gpu outer {info.iterations} inner {info.inner_iterations} "
          f"berr {berr:.2e}; emulated unrestarted inner {inner_e}")
    assert rc == _lib.LUHOT_OK and info.converged
    assert berr <= n * 2.0 ** -53
    assert info.inner_iterations <= 2 * inner_e + 10


@pytest.mark.parametrize("kind", ["bf16x3", "tf32"])
@pytest.mark.parametrize("m,n", [(1000, 1000), (1300, 700), (700, 1300), (257, 257), (129, 900), (900, 129)])
def test_tensor_core_factor_shapes(kind, m, n):
    """The tensor-core factorization runs in slabs of 256 columns with a
    look-ahead (the next slab's columns on one stream, the rest of each
    trailing update on another).  On square, tall and wide shapes whose sizes
    are not multiples of the slab, the factor reproduces P A = L U to the
    accuracy of its operand format: max |PA - LU| / max |A| at most 64 n 2^-24
    for the FP32-accurate BF16x3 products and 16 sqrt(n) 2^-11 for TF32 (a
    missed or repeated update would leave O(1) entries)."""
    torch = pytest.importorskip("torch")
    lib, ctx = _lib.load(), _lib.context()
    a = np.random.default_rng(m * 7 + n).standard_normal((m, n)).astype(np.float32)
    d = torch.from_numpy(a).cuda()
    k = min(m, n)
    piv = torch.zeros(k, dtype=torch.int32, device="cuda")
    sing = ctypes.c_int64(0)
    torch.cuda.synchronize()
    _lib.check(lib.luhot_sgetrf_mixed_dev(ctx, m, n, d.data_ptr(), n, piv.data_ptr(), _lib.PRECISIONS[kind],
                                          ctypes.byref(sing)), ctx)
    assert sing.value == -1
    lu = d.cpu().numpy().astype(np.float64)
    lo = np.tril(lu, -1)[:, :k] + np.eye(m, k)
    up = np.triu(lu)[:k, :]
    pa = a.astype(np.float64)
    for i, p in enumerate(piv.cpu().numpy()):
        pa[[i, p]] = pa[[p, i]]
    bound = 64 * max(m, n) * 2.0 ** -24 if kind == "bf16x3" else 16 * np.sqrt(max(m, n)) * 2.0 ** -11
    err = np.abs(pa - lo @ up).max() / np.abs(a).max()
    assert err <= bound, err
    assert np.abs(np.tril(lu, -1)).max() <= 1.0 + 1e-6  # partial pivoting: |L| <= 1
