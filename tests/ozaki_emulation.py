"""CPU restatement of the tensor-core FP64 Schur update (integer-slice
product, Ozaki scheme) of fast-mode FP64 getrf.

The update C -= L U (K <= 64) has no lair counterpart beyond its result (lair
computes the trailing update in FP64 inside getrf_row_major,
src/lapack/getrf.rs:46-120); this module restates the GPU kernel's arithmetic
step for step so that a GPU test can compare the kernel with it bit for bit:

* per row of L and per column of U the exponent e of frexp(max |x|);
* each element rounded to N = round(|x| 2^(56-e)) (ties up) and split into
  seven balanced base-256 digits, signed like x;
* T_G = sum_{p+q=G} A_p B_q^T for G = 0..6 (integers, exact in float64 and,
  being below 2^24, in the kernel's FP32 accumulators);
* R = T_6 2^38, then R = T_G 2^38 + floor(R / 2^8) for G = 5..0 (int64);
* C - float64(R) 2^(ea+eb-54), NaN where a row or column held Inf or NaN.

It is test infrastructure (numpy, vectorised), not a product path.
"""
from __future__ import annotations

import numpy as np

SLICES = 7
GROUPS = 7
FRAC = 38
NONFINITE = 1 << 20
ZERO = -(1 << 20)


def _fields(x: np.ndarray):
    bits = np.ascontiguousarray(x, dtype=np.float64).view(np.uint64)
    E = ((bits >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    m = (bits & np.uint64((1 << 52) - 1)).astype(np.int64)
    neg = (bits >> np.uint64(63)).astype(bool)
    return E, m, neg


def exponents(x: np.ndarray, axis: int) -> np.ndarray:
    """frexp exponent of the largest |x| along `axis` (0 for all-zero,
    NONFINITE where Inf or NaN is present), int64."""
    E, m, _ = _fields(x)
    sub_len = np.frexp(m.astype(np.float64))[1].astype(np.int64)  # bit length of m (m < 2^52: exact)
    e = np.where(E == 0x7FF, NONFINITE,
                 np.where(E != 0, E - 1022, np.where(m == 0, ZERO, sub_len - 1074)))
    e = e.max(axis=axis)
    return np.where(e == ZERO, 0, e)


def digits(x: np.ndarray, e: np.ndarray) -> list[np.ndarray]:
    """Seven balanced base-256 digits (int64 arrays, most significant first) of
    round(|x| 2^(56-e)), signed like x; e broadcasts against x."""
    E, m, neg = _fields(x)
    ex = np.where(E != 0, E - 1075, -1074)
    m = np.where(E != 0, m | (1 << 52), m)
    sh = ex - e + 56
    ok = (m != 0) & (sh > -64) & (np.broadcast_to(e, x.shape) < NONFINITE) & (E != 0x7FF)
    up = ok & (sh >= 0)
    down = ok & (sh < 0)
    mu = m.astype(np.uint64)
    s_up = np.where(up, sh, 0).astype(np.uint64)
    s_dn = np.where(down, -sh, 1).astype(np.uint64)
    n_up = mu << s_up
    n_dn = (mu + (np.uint64(1) << (s_dn - np.uint64(1)))) >> s_dn
    N = np.where(up, n_up, np.where(down, n_dn, np.uint64(0))).astype(np.uint64)
    d = [None] * SLICES
    carry = np.zeros(x.shape, dtype=np.int64)
    for p in range(SLICES - 1, 0, -1):
        v = (N & np.uint64(255)).astype(np.int64) + carry
        N = N >> np.uint64(8)
        carry = (v >= 128).astype(np.int64)
        d[p] = v - (carry << 8)
    d[0] = N.astype(np.int64) + carry
    return [np.where(neg, -v, v) for v in d]


def schur_update(c: np.ndarray, l: np.ndarray, u: np.ndarray) -> np.ndarray:
    """C - L U (L: M x K, U: K x N, K <= 64) exactly as the GPU computes it."""
    assert l.shape[1] == u.shape[0] <= 64
    ea = exponents(l, 1)
    eb = exponents(u, 0)
    A = [v.astype(np.float64) for v in digits(l, ea[:, None])]
    B = [v.astype(np.float64) for v in digits(u, eb[None, :])]
    R = None
    for G in range(GROUPS - 1, -1, -1):
        T = np.zeros((l.shape[0], u.shape[1]))
        for p in range(max(0, G - SLICES + 1), min(G, SLICES - 1) + 1):
            T += A[p] @ B[G - p]
        assert np.abs(T).max(initial=0) < 2 ** 24
        t = T.astype(np.int64) << FRAC
        R = t if R is None else t + (R >> 8)
    s = ea[:, None] + eb[None, :] - (FRAC + 16)
    s = np.clip(s, -4000, 4000).astype(np.int32)
    with np.errstate(over="ignore", invalid="ignore"):
        out = c - np.ldexp(R.astype(np.float64), s)
    bad = (ea[:, None] >= NONFINITE) | (eb[None, :] >= NONFINITE)
    return np.where(bad, np.nan, out)


def group_bound(k: int) -> int:
    """Largest |partial sum| any T_G can reach for K = k (digit bounds 256 and 128)."""
    worst = 0
    for G in range(GROUPS):
        s = 0
        for p in range(max(0, G - SLICES + 1), min(G, SLICES - 1) + 1):
            s += (256 if p == 0 else 128) * (256 if G - p == 0 else 128)
        worst = max(worst, s * k)
    return worst
