"""Mixed-precision LU + iterative refinement against the FP64 oracle.

Matrices follow the benchmark's construction at test sizes:
A = Q1 diag(sigma) Q2^T with Q1, Q2 from Householder QR of seeded N(0,1)
matrices and sigma geometric from 1 to 1/kappa.  Every result must reach the
normwise backward error n * 2^-53; the forward error against lair's FP64
solution (the oracle) is bounded by kappa * n * 2^-53 up to a small factor.
"""
import numpy as np
import pytest

import oracle
from lair_gb300 import _lib, refine
from lair_gb300.errors import InvalidInput

pytestmark = pytest.mark.gpu
EPS64 = 2.0 ** -53


def conditioned(n, kappa, seed):
    rng = np.random.default_rng(seed)
    q1, _ = np.linalg.qr(rng.standard_normal((n, n)))
    q2, _ = np.linalg.qr(rng.standard_normal((n, n)))
    sigma = np.geomspace(1.0, 1.0 / kappa, n)
    return (q1 * sigma) @ q2.T


def berr(a, x, b):
    r = b - a @ x
    return np.abs(r).max() / (np.abs(a).sum(1).max() * np.abs(x).max() + np.abs(b).max())


@pytest.mark.parametrize("kappa", [1e2, 1e4, 1e6])
@pytest.mark.parametrize("solver", ["ir", "gmres"])
def test_fp32_refinement_reaches_fp64_backward_error(kappa, solver):
    n = 1024
    a = conditioned(n, kappa, 1)
    b = np.random.default_rng(2).standard_normal(n)
    x, info = refine.gesv_ir(a, b, precision="fp32", solver=solver)
    assert info["converged"] == 1
    assert berr(a, x, b) <= n * EPS64
    assert info["backward_error"] <= n * EPS64
    ref = a.copy()
    piv, _ = oracle.getrf(ref)
    x_ref = oracle.getrs(ref, piv, b)
    rel = np.abs(x - x_ref).max() / np.abs(x_ref).max()
    assert rel <= 50 * kappa * n * EPS64
    if solver == "gmres":
        assert info["inner_iterations"] >= info["iterations"]


@pytest.mark.parametrize("precision", ["tf32", "bf16", "fp16"])
def test_tensor_core_factor_is_a_valid_preconditioner(precision):
    """One low-precision solve (no refinement) already has the backward error
    of the operand precision (tf32/fp16 ~ 2^-11, bf16 ~ 2^-8); a broken
    tcgen05 Schur update would give O(1)."""
    n = 1000  # not a multiple of the 128-wide panels or tiles
    a = conditioned(n, 1e2, 11)
    b = np.random.default_rng(12).standard_normal(n)
    x, info = refine.gesv_ir(a, b, precision=precision, solver="ir", max_iter=0, raise_on_failure=False)
    assert berr(a, x, b) <= {"tf32": 5e-3, "fp16": 5e-3, "bf16": 5e-2}[precision]


@pytest.mark.parametrize("precision,kappa", [("tf32", 1e4), ("fp16", 1e4), ("bf16", 1e2)])
def test_tensor_core_gmres_ir_reaches_fp64_backward_error(precision, kappa):
    # With 11-bit (tf32, fp16) or 8-bit (bf16) factors, kappa * u_low must stay
    # well below ~1e3 for restarted GMRES to contract; kappa = 1e6 is left to
    # the FP32-accurate factorizations.
    n = 2048
    a = conditioned(n, kappa, 13)
    b = np.random.default_rng(14).standard_normal(n)
    x, info = refine.gesv_ir(a, b, precision=precision, solver="gmres", max_iter=30)
    assert info["converged"] == 1
    assert berr(a, x, b) <= n * EPS64


@pytest.mark.parametrize("kappa", [1e2, 1e4, 1e6])
def test_bf16x3_tensor_core_factor_with_plain_ir(kappa):
    """The three-piece BF16 Schur update is FP32-accurate, so plain IR
    converges where the FP32 LU does (kappa up to ~1e6)."""
    n = 2048
    a = conditioned(n, kappa, 17)
    b = np.random.default_rng(18).standard_normal(n)
    x, info = refine.gesv_ir(a, b, precision="bf16x3", solver="ir")
    assert info["converged"] == 1 and berr(a, x, b) <= n * EPS64
    x1, _ = refine.gesv_ir(a, b, precision="bf16x3", solver="ir", max_iter=0, raise_on_failure=False)
    x2, _ = refine.gesv_ir(a, b, precision="fp32", solver="ir", max_iter=0, raise_on_failure=False)
    # one solve with the tensor-core factors is as good as with the FFMA FP32 factors
    assert berr(a, x1, b) <= 4 * berr(a, x2, b) + 1e-12


def test_bf16x3_split_accumulators_keep_refinement_short():
    """The BF16x3 update keeps its leading piece product apart from the five
    small ones (separate TMEM accumulators), which makes the factor more
    accurate as an FFMA FP32 one: plain IR at kappa = 1e6 needs about as many
    corrections as with the FP32 factor (measured 4 and 4 here; 5 against 9
    at n = 16384, where one accumulator took 14)."""
    n = 2048
    a = conditioned(n, 1e6, 21)
    b = np.random.default_rng(22).standard_normal(n)
    _, info3 = refine.gesv_ir(a, b, precision="bf16x3", solver="ir")
    _, info32 = refine.gesv_ir(a, b, precision="fp32", solver="ir")
    print(f"\nbf16x3: {info3['iterations']} corrections, fp32: {info32['iterations']}")
    assert info3["converged"] == 1 and info32["converged"] == 1
    assert info3["iterations"] <= info32["iterations"] + 1


def test_tensor_core_plain_ir_small_kappa():
    n = 1536
    a = conditioned(n, 1e2, 15)
    b = np.random.default_rng(16).standard_normal(n)
    x, info = refine.gesv_ir(a, b, precision="tf32", solver="ir")
    assert info["converged"] == 1 and berr(a, x, b) <= n * EPS64


def test_refinement_multiple_rhs_and_strides():
    n = 600
    a = conditioned(n, 1e3, 3)
    b = np.random.default_rng(4).standard_normal((n, 3))
    x, info = refine.gesv_ir(np.asfortranarray(a), b)
    for c in range(3):
        assert berr(a, x[:, c], b[:, c]) <= n * EPS64
    assert info["converged"] == 1


def test_refinement_reports_non_convergence_for_hopeless_kappa():
    n = 512
    a = conditioned(n, 1e14, 5)
    b = np.random.default_rng(6).standard_normal(n)
    x, info = refine.gesv_ir(a, b, solver="ir", max_iter=5, raise_on_failure=False)
    assert info["converged"] == 0
    with pytest.raises(_lib.LuhotError):
        refine.gesv_ir(a, b, solver="ir", max_iter=5)


def test_refinement_errors():
    with pytest.raises(InvalidInput.Shape):
        refine.gesv_ir(np.zeros((3, 4)), np.zeros(3))
    with pytest.raises(InvalidInput.Value):
        refine.gesv_ir(np.zeros((4, 4)), np.ones(4))
