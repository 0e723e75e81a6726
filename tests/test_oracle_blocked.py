"""The blocked, threaded restatement of lair's row-major getrf that makes the
large parity fixtures, and the portable input generator they depend on.

``oracle.getrf_row_major_blocked`` must give the bits of
``oracle.getrf_row_major`` (lair's src/lapack/getrf.rs:46-120) for every
shape, block width and thread count, including singular steps (zero columns,
where lair skips the update) and NaN columns (which never win a pivot
search).  The generator must give the same values for any thread count, and
the committed n = 4096 fixture must be what the oracle computes today.
"""
import os

import numpy as np
import pytest

import oracle
from lair_gb300 import synthetic

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("m,n,w,threads", [(300, 300, 64, 4), (700, 513, 64, 3), (513, 700, 32, 8),
                                           (129, 129, 16, 2), (1000, 1000, 64, 8), (257, 65, 64, 5),
                                           (65, 257, 7, 1), (1, 1, 64, 1), (2, 3, 64, 2)])
def test_blocked_equals_unblocked(m, n, w, threads):
    a0 = np.random.default_rng(m * 1000 + n).standard_normal((m, n))
    a1, a2 = a0.copy(), a0.copy()
    p1, s1 = oracle.getrf_row_major(a1)
    p2, s2 = oracle.getrf_row_major_blocked(a2, block=w, threads=threads)
    assert p1 == [int(v) for v in p2] and s1 == s2
    assert np.array_equal(a1, a2)


def test_blocked_singular_and_nan_columns():
    rng = np.random.default_rng(5)
    for col in ((3,), (70,), (3, 64, 65)):
        a0 = rng.standard_normal((200, 200))
        a0[:, list(col)] = 0.0
        a1, a2 = a0.copy(), a0.copy()
        p1, s1 = oracle.getrf_row_major(a1)
        p2, s2 = oracle.getrf_row_major_blocked(a2, block=64, threads=4)
        assert p1 == [int(v) for v in p2] and s1 == s2
        assert np.array_equal(a1, a2)
    a0 = rng.standard_normal((150, 150))
    a0[40:, 10] = np.nan
    a1, a2 = a0.copy(), a0.copy()
    p1, s1 = oracle.getrf_row_major(a1)
    p2, s2 = oracle.getrf_row_major_blocked(a2, block=32, threads=4)
    assert p1 == [int(v) for v in p2] and s1 == s2
    assert np.array_equal(a1, a2, equal_nan=True)


def test_blocked_margins():
    a = np.random.default_rng(9).standard_normal((100, 100))
    ref = a.copy()
    _, _, colmax, gap = oracle.getrf_row_major_blocked(a, margins=True)
    for step in (0, 1):  # the first two steps' candidates, checked directly
        col = np.abs(ref[step:, step])
        top = np.sort(col)[::-1]
        assert colmax[step] == top[0] and gap[step] == top[0] - top[1]
        oracle.getrf_row_major_range(ref, np.arange(100, dtype=np.uint64), step, step + 1)


def test_generator_independent_of_threads():
    a = synthetic.normal(3, 3 * synthetic.BLOCK + 12345, threads=1)
    b = synthetic.normal(3, 3 * synthetic.BLOCK + 12345, threads=8)
    assert np.array_equal(a, b)
    assert abs(a.mean()) < 3e-3 and abs(a.std() - 1) < 3e-3
    # the prefix of a longer draw is the shorter draw (blocks are independent)
    assert np.array_equal(synthetic.normal(3, 1000), a[:1000])


def test_committed_fixture_n4096_matches_oracle():
    fx = np.load(os.path.join(HERE, "golden", "getrf_normal_n4096.npz"))
    n = int(fx["n"])
    a = synthetic.normal_matrix(int(fx["seed_a"]), n, n)
    assert synthetic.digest(a) == str(fx["a_digest"])
    piv, sing = oracle.getrf_row_major_blocked(a)
    assert np.array_equal(piv.astype(np.uint16), fx["piv"]) and (sing is None) == (int(fx["singular"]) < 0)
    assert synthetic.digest(a) == str(fx["lu_digest"])
    assert np.array_equal(a[fx["lu_rows"], fx["lu_cols"]], fx["lu_vals"])
