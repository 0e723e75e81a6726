"""Write the plain-FP64 parity fixtures at n = 4096, 8192 and 16384.

Workload: A (n x n) and B (n x 16) iid N(0,1) from ``lair_gb300.synthetic``
(bit-identical on every machine), A from seed 10*n + 1, B from 10*n + 2.
For each size this runs lair's elimination order (the oracle's
``getrf_row_major_blocked``, bit-identical to ``getrf_row_major``,
src/lapack/getrf.rs:46-120) and lair's single-right-hand-side ``getrs``
(src/lapack/getrs.rs:12-38) on columns 0 and 1 of B, and stores, compressed,
in ``getrf_normal_n{n}.npz``:

* ``a_digest``, ``b_digest``: SHA-256 of A and B (the GPU test regenerates
  the inputs and checks these first);
* ``piv`` (uint16), ``singular`` (-1 = None): lair's pivots and singular step;
* ``colmax``, ``gap`` (float32): per step, the largest pivot candidate |a| and
  its margin over the second largest, so a test that meets a different pivot
  can report by how little the candidates differed;
* ``lu_rows``, ``lu_cols``, ``lu_vals``: 2048 entries of lair's L\\U at seeded
  positions, and ``lu_digest`` of the whole factor;
* ``x01``: lair's solutions for columns 0 and 1 of B (n x 2, float64).

Run from the repository root: ``python tests/golden/make_getrf_normal_fixtures.py [sizes...]``
(about 10 minutes on 8 cores, most of it at n = 16384).
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from lair_gb300 import synthetic  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
SIZES = (4096, 8192, 16384)
NRHS = 16
SAMPLES = 2048


def seeds(n: int):
    return 10 * n + 1, 10 * n + 2


def path(n: int) -> str:
    return os.path.join(HERE, f"getrf_normal_n{n}.npz")


def make(n: int) -> None:
    t0 = time.time()
    sa, sb = seeds(n)
    a = synthetic.normal_matrix(sa, n, n)
    b = synthetic.normal_matrix(sb, n, NRHS)
    a_digest, b_digest = synthetic.digest(a), synthetic.digest(b)
    lu = a.copy()
    piv, singular, colmax, gap = oracle.getrf_row_major_blocked(lu, margins=True)
    t1 = time.time()
    x01 = np.stack([oracle.getrs(lu, piv, np.ascontiguousarray(b[:, j])) for j in range(2)], axis=1)
    rng = np.random.default_rng(n)
    rows = rng.integers(0, n, SAMPLES).astype(np.int32)
    cols = rng.integers(0, n, SAMPLES).astype(np.int32)
    np.savez_compressed(
        path(n), n=n, nrhs=NRHS, seed_a=sa, seed_b=sb, a_digest=a_digest, b_digest=b_digest,
        piv=piv.astype(np.uint16), singular=-1 if singular is None else singular,
        colmax=colmax.astype(np.float32), gap=gap.astype(np.float32), lu_rows=rows, lu_cols=cols,
        lu_vals=lu[rows, cols], lu_digest=synthetic.digest(lu), x01=x01)
    print(f"n={n}: getrf {t1 - t0:.1f} s, total {time.time() - t0:.1f} s, "
          f"min relative pivot margin {np.min(gap / colmax):.3e}")


if __name__ == "__main__":
    for n in (int(v) for v in sys.argv[1:]) if len(sys.argv) > 1 else SIZES:
        make(n)
