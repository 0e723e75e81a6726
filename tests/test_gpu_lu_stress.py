"""Wider GPU coverage of the LU path: sizes around every blocking boundary.

The panel kernel spreads rows over a number of CTAs that depends on the
height (>= 32 rows each; at most 64 CTAs for FP32, the SM count for FP64),
the Schur update switches between the persistent and the one-tile kernels on
alignment, and the triangular sweeps work in 64-row blocks.  These tests walk
sizes across those boundaries (square, tall, wide) and check exact mode
bit for bit against the oracle and fast mode against the parity bounds.
"""
import numpy as np
import pytest

import oracle
from lair_gb300 import lapack, lu

pytestmark = pytest.mark.gpu

EPS = {np.float64: 2.0 ** -53, np.float32: 2.0 ** -24}


def rand(seed, m, n, dtype=np.float64):
    return np.random.default_rng(seed).standard_normal((m, n)).astype(dtype)


def pa_minus_lu(a0, f, piv, dtype):
    m, n = a0.shape
    pa = a0.astype(np.float64)
    oracle.laswp(pa, 0, piv)
    L = lu.l_matrix(f.astype(np.float64))
    U = lu.u_matrix(f.astype(np.float64))
    return np.abs(pa - L @ U).max() / (max(m, n) * EPS[dtype] * np.abs(a0).max())


@pytest.mark.parametrize("m,n", [(1500, 1500), (2049, 700), (700, 2049), (1025, 1025)])
def test_exact_bitwise_larger(m, n):
    a0 = rand(m + 2 * n, m, n)
    a, ref = a0.copy(), a0.copy()
    piv, sing = lapack.getrf(a, mode="exact")
    piv_r, sing_r = oracle.getrf(ref)
    assert piv == piv_r and sing == sing_r
    assert np.array_equal(a, ref)


SIZES = [(31, 31), (33, 33), (95, 95), (127, 127), (129, 129), (255, 257), (1023, 1023), (1025, 1031),
         (2047, 2047), (2048, 1000), (1000, 2048), (3001, 3001), (4097, 4097), (6000, 2000)]


@pytest.mark.parametrize("m,n", SIZES)
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_fast_factor_bound(m, n, dtype):
    a0 = rand(7 * m + n, m, n, dtype)
    a = a0.copy()
    piv, sing = lapack.getrf(a)
    assert sing is None
    assert pa_minus_lu(a0, a, piv, dtype) <= 10
    if dtype == np.float64 and max(m, n) <= 2048:
        # distinct candidates (continuous random data): the pivots are lair's
        ref = a0.copy()
        piv_r, _ = oracle.getrf(ref)
        assert piv == piv_r


@pytest.mark.parametrize("n,nrhs", [(4097, 1), (4097, 17), (3001, 33)])
def test_fast_solve_sizes(n, nrhs):
    a0 = rand(n, n, n)
    b = rand(n + 1, n, nrhs)
    a = a0.copy()
    piv, _ = lapack.getrf(a)
    x = lapack.getrs(a, piv, b)
    r = b - a0 @ x
    berr = np.abs(r).max() / (np.abs(a0).sum(1).max() * np.abs(x).max() + np.abs(b).max())
    assert berr <= n * EPS[np.float64]
    xt = lapack.getrs(a, piv, b, trans=True)
    rt = b - a0.T @ xt
    assert np.abs(rt).max() / (np.abs(a0).sum(0).max() * np.abs(xt).max() + np.abs(b).max()) <= n * EPS[np.float64]
