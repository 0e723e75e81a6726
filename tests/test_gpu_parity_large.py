"""Plain FP64 parity with lair at the benchmark's sizes: n = 4096, 8192, 16384.

Workload: A (n x n) and B (n x 16) iid N(0,1), regenerated bit for bit from
the seeds in ``tests/golden/getrf_normal_n{n}.npz`` (``lair_gb300.synthetic``),
whose reference data come from lair's own order run by the oracle
(``make_getrf_normal_fixtures.py``: getrf_row_major, src/lapack/getrf.rs:46-120,
and getrs, src/lapack/getrs.rs:12-38).  The GPU factors in fast mode (FP64
tensor-core Schur updates, FMA elsewhere) through the C ABI, and the test
asserts:

* pivots: identical to lair's; if a step differs, the candidates at the
  first differing step must have been within 64 n eps max|column| of each
  other (a tie to within the rounding of the two orders), and the step and
  margin are reported;
* ||PA - LU||_max / (n eps ||A||_max) <= 10, computed on the GPU in FP64;
* the solution's relative error against lair's FP64 solution (columns 0 and
  1 of B), max|x - x_lair| / max|x_lair| <= 1e-8, and the backward error of
  all 16 columns <= n eps (eps = 2^-53, lair's Real::eps, src/scalar.rs:393-395);
* 2048 sampled entries of L\\U agree with lair's to 1e-9 of max|L\\U|.

The measured figures are printed (``pytest -s``) and reported by the
benchmark's ``parity`` key at n = 16384.
"""
import ctypes
import os

import numpy as np
import pytest

from lair_gb300 import _lib, synthetic

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
EPS = 2.0 ** -53


def load_fixture(n):
    return np.load(os.path.join(HERE, "golden", f"getrf_normal_n{n}.npz"))


def compose_perm(piv):
    perm = np.arange(len(piv))
    for i, p in enumerate(piv):
        if p != i:
            perm[i], perm[p] = perm[p], perm[i]
    return perm


def parity_report(torch, n, fx, d_a0, d_lu, piv_gpu, d_x, b):
    """Parity figures of a GPU factorization and solve against lair's (fixture)."""
    piv_ref = fx["piv"].astype(np.int64)
    diff = np.nonzero(piv_gpu != piv_ref)[0]
    first = int(diff[0]) if diff.size else -1
    perm = torch.from_numpy(compose_perm(piv_gpu)).cuda()
    L = torch.tril(d_lu, -1)
    L.diagonal().fill_(1.0)
    U = torch.triu(d_lu)
    err = (d_a0[perm] - L @ U).abs().max().item()
    del L, U
    ratio = err / (n * EPS * d_a0.abs().max().item())
    x = d_x.cpu().numpy()
    x_ref = fx["x01"]
    sol = float(np.abs(x[:, :2] - x_ref).max() / np.abs(x_ref).max())
    d_b = torch.from_numpy(b).cuda()
    r = (d_b - d_a0 @ d_x).abs().max(dim=0).values
    berr = (r / (d_a0.abs().sum(1).max() * d_x.abs().max(dim=0).values + d_b.abs().max(dim=0).values)).max().item()
    rows = torch.from_numpy(fx["lu_rows"].astype(np.int64)).cuda()
    cols = torch.from_numpy(fx["lu_cols"].astype(np.int64)).cuda()
    lu_s = d_lu[rows, cols].cpu().numpy()
    lu_diff = float(np.abs(lu_s - fx["lu_vals"]).max() / max(np.abs(fx["lu_vals"]).max(), 1e-300))
    rep = {"n": n, "pivots_identical": first < 0, "first_divergent_step": first,
           "pa_minus_lu_over_n_eps_a": ratio, "solution_rel_err_vs_lair": sol, "backward_error": berr,
           "lu_sample_rel_diff": lu_diff}
    if first >= 0:
        rep["margin_at_divergence"] = float(fx["gap"][first])
        rep["allowed_margin"] = float(64 * n * EPS * fx["colmax"][first])
    return rep


@pytest.mark.parametrize("n", [4096, 8192, 16384])
def test_fast_mode_parity_with_lair_at_benchmark_sizes(n):
    torch = pytest.importorskip("torch")
    fx = load_fixture(n)
    nrhs = int(fx["nrhs"])
    a0 = synthetic.normal_matrix(int(fx["seed_a"]), n, n)
    b = synthetic.normal_matrix(int(fx["seed_b"]), n, nrhs)
    assert synthetic.digest(a0) == str(fx["a_digest"]), "A was not reproduced bit for bit"
    assert synthetic.digest(b) == str(fx["b_digest"]), "B was not reproduced bit for bit"
    lib, ctx = _lib.load(), _lib.context()
    d_a0 = torch.from_numpy(a0).cuda()
    d_lu = d_a0.clone()
    d_piv = torch.zeros(n, dtype=torch.int32, device="cuda")
    d_x = torch.from_numpy(b).cuda()
    torch.cuda.synchronize()
    sing = ctypes.c_int64(0)
    _lib.check(lib.luhot_dgetrf_dev(ctx, n, n, d_lu.data_ptr(), n, d_piv.data_ptr(), ctypes.byref(sing),
                                    _lib.MODE_FAST), ctx)
    assert sing.value == int(fx["singular"]) == -1
    _lib.check(lib.luhot_dgetrs_dev(ctx, n, nrhs, d_lu.data_ptr(), n, d_piv.data_ptr(), d_x.data_ptr(), nrhs, 0,
                                    _lib.MODE_FAST), ctx)
    torch.cuda.synchronize()
    piv_gpu = d_piv.cpu().numpy().astype(np.int64)
    rep = parity_report(torch, n, fx, d_a0, d_lu, piv_gpu, d_x, b)
    print(rep)
    if not rep["pivots_identical"]:
        assert rep["margin_at_divergence"] <= rep["allowed_margin"], rep
    assert rep["pa_minus_lu_over_n_eps_a"] <= 10, rep
    assert rep["solution_rel_err_vs_lair"] <= 1e-8, rep
    assert rep["backward_error"] <= n * EPS, rep
    assert rep["lu_sample_rel_diff"] <= 1e-9, rep
