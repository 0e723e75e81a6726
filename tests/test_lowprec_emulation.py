"""The CPU emulation of the mixed-precision LU (the checker of the GPU's
low-precision factors, tests/lowprec_emulation.py) on small cases.

Its factors must satisfy P A = L U to the accuracy of their format, its
operand rounding must be round-to-nearest in the stated format, and its
GMRES-IR restatement must converge where theory says it does (kappa * u
well below 1) and report failure where the preconditioner is too poor.
"""
import numpy as np
import pytest

import lowprec_emulation as emu

U = {"fp32": 2.0 ** -24, "tf32": 2.0 ** -11, "fp16": 2.0 ** -11, "bf16": 2.0 ** -8}


@pytest.mark.parametrize("kind", ["fp32", "tf32", "fp16", "bf16"])
def test_factor_reproduces_the_matrix_to_its_format(kind):
    n = 300
    a = np.random.default_rng(4).standard_normal((n, n))
    lu, perm = emu.factor(a, kind)
    L = np.tril(lu.astype(np.float64), -1) + np.eye(n)
    Uu = np.triu(lu.astype(np.float64))
    err = np.abs(a[perm] - L @ Uu).max() / np.abs(a).max()
    assert err <= 50 * n ** 0.5 * max(U[kind], 2.0 ** -24)
    assert err >= (U[kind] / 50 if kind != "fp32" else 0.0)  # the rounding really happens


def test_operand_rounding_is_to_nearest():
    assert emu._bf16(np.float32([1.0 + 2.0 ** -9]))[0] == np.float32(1.0)  # below half an ulp (2^-7): down
    assert emu._bf16(np.float32([1.0 + 3 * 2.0 ** -9]))[0] == np.float32(1.0 + 2.0 ** -7)  # above half: up
    assert emu._bf16(np.float32([-(1.0 + 3 * 2.0 ** -9)]))[0] == np.float32(-(1.0 + 2.0 ** -7))
    assert emu._bf16(np.float32([1.0 + 2.0 ** -8]))[0] == np.float32(1.0)  # tie to even: down
    assert emu._tf32(np.float32([1.0 + 2.0 ** -11]))[0] == np.float32(1.0 + 2.0 ** -10)  # tie away from zero
    assert emu._tf32(np.float32([1.0 + 2.0 ** -12]))[0] == np.float32(1.0)
    assert emu._scale(np.array([3.0])) == 2.0 ** 12  # 3 * 2^12 lies in [2^13, 2^14)


def test_gmres_ir_converges_when_the_factor_is_good_and_not_otherwise():
    n = 256
    a, b = emu.conditioned(n, 1e2, seed=1)
    lu, perm = emu.factor(a, "tf32")
    q = emu.quality(a, lu, perm)
    assert q["norm_I_minus_MinvA"] < 0.5
    _, inner, berr = emu.gmres_ir(a, b, lu, perm)
    assert berr <= n * 2.0 ** -53 and inner < 20
    a, b = emu.conditioned(n, 1e6, seed=1)
    lu, perm = emu.factor(a, "bf16")
    q = emu.quality(a, lu, perm)
    assert q["norm_I_minus_MinvA"] > 10 and q["sv_far_from_1"] > 10
    _, inner, berr = emu.gmres_ir(a, b, lu, perm, restart=40, max_inner=120)
    assert berr > n * 2.0 ** -53
