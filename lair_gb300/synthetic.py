"""Seeded synthetic inputs that come out bit for bit the same on every machine.

The parity fixtures for the plain FP64 solve (A and B iid N(0,1) at n = 4096,
8192 and 16384) are computed once on one machine with the CPU oracle and
checked on another (an aarch64 GPU host), so the inputs must be reproduced
exactly there.  numpy's ``Generator.standard_normal`` may change between numpy
versions and goes through the platform's libm, so this module builds normals
from parts whose results are fixed by IEEE 754 alone:

* uniform words from the PCG64 bit generator (integer arithmetic), one
  generator per block of 2**20 values seeded by ``SeedSequence([seed, block])``
  (so blocks can be made in parallel and in any order);
* u = (word >> 11) * 2**-53 in [0, 1);
* Marsaglia's polar method: v1, v2 = 2u - 1, s = v1^2 + v2^2, keep 0 < s < 1,
  z = v * sqrt(-2 ln(s) / s), using only +, -, *, /, sqrt (correctly rounded
  everywhere) and a logarithm written here from its series:
  ln s = e ln 2 + 2 atanh(f), s = m 2^e with m in [1/sqrt2, sqrt2) (frexp is
  exact), f = (m - 1)/(m + 1), atanh(f) = f (1 + f^2/3 + f^4/5 + ...) summed to
  f^26 by Horner's rule (|f| <= 0.172, so the truncation is below 1e-20).

The logarithm is within a few ulps of the true value: the samples are
N(0,1) to that accuracy and identical wherever numpy runs.
"""
from __future__ import annotations

import concurrent.futures as cf
import os

import numpy as np

BLOCK = 1 << 20
_LN2 = 0.6931471805599453  # nearest double to ln 2
_SQRT_HALF = 0.7071067811865476


def _log(s: np.ndarray) -> np.ndarray:
    m, e = np.frexp(s)
    small = m < _SQRT_HALF
    m = np.where(small, m * 2.0, m)
    e = (e - small).astype(np.float64)
    f = (m - 1.0) / (m + 1.0)
    f2 = f * f
    p = np.full_like(f, 1.0 / 27.0)
    for k in range(12, -1, -1):
        p = p * f2 + 1.0 / (2 * k + 1)
    return e * _LN2 + 2.0 * f * p


def _normal_block(seed: int, block: int, count: int, out: np.ndarray) -> None:
    bg = np.random.PCG64(np.random.SeedSequence([seed, block]))
    got = 0
    while got < count:
        pairs = int((count - got) * 0.66) + 1024
        u = (bg.random_raw(2 * pairs) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
        v1 = 2.0 * u[0::2] - 1.0
        v2 = 2.0 * u[1::2] - 1.0
        s = v1 * v1 + v2 * v2
        keep = (s < 1.0) & (s > 0.0)
        v1, v2, s = v1[keep], v2[keep], s[keep]
        r = np.sqrt(-2.0 * _log(s) / s)
        z = np.empty(2 * s.size)
        z[0::2] = v1 * r
        z[1::2] = v2 * r
        take = min(count - got, z.size)
        out[got:got + take] = z[:take]
        got += take


def normal(seed: int, count: int, threads: int = 0) -> np.ndarray:
    """``count`` iid N(0,1) doubles, identical on every machine for a given seed."""
    out = np.empty(count)
    nblocks = (count + BLOCK - 1) // BLOCK
    work = [(b, min(BLOCK, count - b * BLOCK)) for b in range(nblocks)]
    threads = threads or min(16, os.cpu_count() or 1)
    if threads <= 1 or nblocks <= 1:
        for b, c in work:
            _normal_block(seed, b, c, out[b * BLOCK:b * BLOCK + c])
    else:
        with cf.ThreadPoolExecutor(threads) as ex:
            list(ex.map(lambda bc: _normal_block(seed, bc[0], bc[1], out[bc[0] * BLOCK:bc[0] * BLOCK + bc[1]]), work))
    return out


def normal_matrix(seed: int, rows: int, cols: int, threads: int = 0) -> np.ndarray:
    """rows x cols C-order matrix of iid N(0,1), row by row."""
    return normal(seed, rows * cols, threads).reshape(rows, cols)


def digest(a: np.ndarray) -> str:
    """SHA-256 of an array's bytes in C order (checks that inputs were reproduced)."""
    import hashlib

    h = hashlib.sha256()
    flat = np.ascontiguousarray(a).reshape(-1).view(np.uint8)
    step = 1 << 26
    for i in range(0, flat.size, step):
        h.update(flat[i:i + step].data)
    return h.hexdigest()
