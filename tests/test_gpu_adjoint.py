"""Adjoint of the solve, against central finite differences and an FP64 CPU gradient.

Workload of the adjoint benchmark configuration: n = 2048, nrhs = 8,
A = N(0,1)/sqrt(n) + I, B and W iid N(0,1), loss = sum(W * X) with X = A^-1 B.
Finite differences perturb 64 random entries of A (h = 1e-6, central);
the CPU reference gradient uses lair's FP64 getrf/getrs (the oracle) on A^T.
"""
import numpy as np
import pytest

import oracle
from lair_gb300 import adjoint, lapack

pytestmark = pytest.mark.gpu


def problem(n, nrhs, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((n, n)) / np.sqrt(n) + np.eye(n)
    b = rng.standard_normal((n, nrhs))
    w = rng.standard_normal((n, nrhs))
    return a, b, w


def solve(a, b):
    f = a.copy()
    piv, _ = lapack.getrf(f)
    return lapack.getrs(f, piv, b), f, piv


def test_adjoint_matches_finite_differences_n2048():
    n, nrhs = 2048, 8
    a, b, w = problem(n, nrhs, 0)
    x, f, piv = solve(a, b)
    da, db = adjoint.solve_backward(f, piv, x, w)
    rng = np.random.default_rng(1)
    h = 1e-6
    # A central difference with h = 1e-6 in FP64 carries about
    # kappa(A) * eps / h of relative noise (each solve is accurate to
    # kappa * eps); kappa of I + N(0,1)/sqrt(n) is ~1e3 here, so entries are
    # compared to 2e-4 relative and the median to 2e-5.  The exact comparison
    # of the gradient is against the FP64 CPU reference below.
    idx = rng.integers(0, n, size=(64, 2))
    rel = []
    for i, j in idx:
        ap = a.copy()
        ap[i, j] += h
        am = a.copy()
        am[i, j] -= h
        lp = np.sum(w * solve(ap, b)[0])
        lm = np.sum(w * solve(am, b)[0])
        fd = (lp - lm) / (2 * h)
        rel.append(abs(fd - da[i, j]) / max(1.0, abs(fd)))
        assert rel[-1] <= 2e-4, (i, j, fd, da[i, j])
    assert np.median(rel) <= 2e-5
    # dB by finite differences on 16 entries
    for i, c in rng.integers(0, [n, nrhs], size=(16, 2)):
        bp = b.copy()
        bp[i, c] += h
        bm = b.copy()
        bm[i, c] -= h
        fd = (np.sum(w * solve(a, bp)[0]) - np.sum(w * solve(a, bm)[0])) / (2 * h)
        assert abs(fd - db[i, c]) <= 2e-4 * max(1.0, abs(fd))


def test_adjoint_matches_fp64_cpu_reference_gradient():
    n, nrhs = 512, 8
    a, b, w = problem(n, nrhs, 2)
    x, f, piv = solve(a, b)
    da, db = adjoint.solve_backward(f, piv, x, w)
    at = np.ascontiguousarray(a.T)
    piv_t, _ = oracle.getrf(at)
    lam = oracle.getrs_multi(at, piv_t, w)
    np.testing.assert_allclose(db, lam, rtol=0, atol=1e-12 * np.abs(lam).max())
    np.testing.assert_allclose(da, -lam @ x.T, rtol=0, atol=1e-12 * np.abs(lam @ x.T).max())


def test_adjoint_mixed_precision_form():
    torch = pytest.importorskip("torch")
    n, nrhs = 2048, 8
    a, b, w = problem(n, nrhs, 3)
    x, f, piv = solve(a, b)
    da64, db64 = adjoint.solve_backward(f, piv, x, w)
    d_a = torch.from_numpy(a).cuda().contiguous()
    d_x = torch.from_numpy(x).cuda().contiguous()
    d_w = torch.from_numpy(w).cuda().contiguous()
    d_db = torch.empty_like(d_w)
    d_da = torch.empty_like(d_a)
    torch.cuda.synchronize()
    info = adjoint.solve_backward_ir_dev(d_a.data_ptr(), n, n, nrhs, d_x.data_ptr(), d_w.data_ptr(), d_db.data_ptr(),
                                         d_da.data_ptr(), precision="fp32", solver="ir")
    assert info["converged"] == 1 and info["backward_error"] <= n * 2.0 ** -53
    db = d_db.cpu().numpy()
    np.testing.assert_allclose(db, db64, rtol=0, atol=1e-10 * np.abs(db64).max())
    np.testing.assert_allclose(d_da.cpu().numpy(), da64, rtol=0, atol=1e-10 * np.abs(da64).max())


def test_adjoint_without_da_and_one_dimensional():
    n = 300
    a, b, w = problem(n, 1, 4)
    x, f, piv = solve(a, b[:, 0])
    da, db = adjoint.solve_backward(f, piv, x, w[:, 0], with_da=False)
    assert da is None and db.shape == (n,)
    np.testing.assert_allclose(a.T @ db, w[:, 0], rtol=0, atol=1e-10)
