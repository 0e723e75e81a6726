"""The tensor-core FP64 Schur update (integer digit slices on the FP16 tensor
cores, lair_gb300/csrc/ozaki.cu) against its CPU restatement
(tests/ozaki_emulation.py), bit for bit, and fast-mode FP64 getrf with it
against the FP64-tensor-core (DMMA) engine.

The update has no lair counterpart beyond its result (lair's trailing update
is FP64 inside getrf_row_major, src/lapack/getrf.rs:46-120); its accuracy
against exact arithmetic is checked on the restatement in
test_ozaki_scheme.py, and the factorization's parity with lair (pivots, PA -
LU, solutions at n = 4096 ... 16384) in test_gpu_parity_large.py, which runs
with the default engine (this update on every block of at least 256 x 256).
"""
import numpy as np
import pytest

import ozaki_emulation as oz
from lair_gb300 import _lib, lapack

pytestmark = pytest.mark.gpu


def gpu_update(torch, full, k, engine="ozaki"):
    lib, ctx = _lib.load(), _lib.context()
    m, n = full.shape
    d = torch.from_numpy(np.ascontiguousarray(full)).cuda()
    torch.cuda.synchronize()
    _lib.check(lib.luhot_dschur_update_dev(ctx, m, n, k, d.data_ptr(), n, _lib.FP64_UPDATES[engine]), ctx)
    return d.cpu().numpy()


def emulated(full, k):
    out = full.copy()
    out[k:, k:] = oz.schur_update(full[k:, k:], full[k:, :k], full[:k, k:])
    return out


# (m, n, k): whole tiles, ragged edges in both directions, K < 64, K = 1,
# and more tiles than SMs (several row blocks per CTA).
SHAPES = [(64 + 128, 64 + 64, 64), (64 + 129, 64 + 65, 64), (37 + 300, 37 + 130, 37), (1 + 200, 1 + 100, 1),
          (64 + 1000, 64 + 700, 64), (64 + 2304, 64 + 1600, 64)]


@pytest.mark.parametrize("m,n,k", SHAPES)
def test_update_bit_exact(m, n, k):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(m * 7919 + n * 31 + k)
    full = rng.standard_normal((m, n))
    full[:, :k] *= np.exp2(rng.integers(-30, 30, (m, 1)))  # row scales of L21
    full[:k, :] *= np.exp2(rng.integers(-30, 30, (1, n)))  # column scales of U12
    got = gpu_update(torch, full, k)
    want = emulated(full, k)
    assert np.array_equal(got, want)


def test_update_edge_values():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    m, n, k = 64 + 256, 64 + 192, 64
    full = rng.standard_normal((m, n))
    full[k + 5, :k] = 0.0                  # zero row of L21: C row unchanged
    full[:k, k + 7] = 0.0                  # zero column of U12
    full[k + 10, :k] *= 2.0 ** 600         # huge row
    full[:k, k + 20] *= 2.0 ** -600        # tiny column
    full[k + 11, :k] *= 2.0 ** -1030       # subnormal row
    full[:k, k + 21] *= 2.0 ** 1000        # huge column: overflows against the huge row
    full[k + 12, 3] = np.inf               # Inf in L21: row -> NaN
    full[5, k + 30] = np.nan               # NaN in U12: column -> NaN
    got = gpu_update(torch, full, k)
    want = emulated(full, k)
    assert np.array_equal(got, want, equal_nan=True)
    assert np.all(np.isnan(got[k + 12, k:])) and np.all(np.isnan(got[k:, k + 30]))
    assert np.isinf(got[k + 10, k + 21])


def test_update_engines_agree():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    m, n, k = 64 + 700, 64 + 500, 64
    full = rng.standard_normal((m, n))
    full[k:, :k] = rng.uniform(-1, 1, (m - k, k))
    oz_out = gpu_update(torch, full, k, "ozaki")
    dmma = gpu_update(torch, full, k, "dmma")
    auto = gpu_update(torch, full, k, "auto")
    assert np.array_equal(auto, oz_out)  # a 700 x 500 block takes the tensor-core engine
    ref = full[k:, k:].astype(np.longdouble) - full[k:, :k].astype(np.longdouble) @ full[:k, k:].astype(np.longdouble)
    scale = np.abs(full[k:, k:]) + np.abs(full[k:, :k]) @ np.abs(full[:k, k:])
    e_oz = float(np.max(np.abs(oz_out[k:, k:] - ref) / scale))
    e_dm = float(np.max(np.abs(dmma[k:, k:] - ref) / scale))
    print(f"\nrelative error vs exact: tensor-core slices {e_oz:.2e}, DMMA {e_dm:.2e}")
    assert e_oz <= max(e_dm, 2.0 ** -52)


@pytest.mark.parametrize("n", [700, 2048])
def test_getrf_ozaki_matches_dmma(n):
    rng = np.random.default_rng(n)
    a0 = rng.standard_normal((n, n))
    try:
        _lib.set_fp64_update("dmma")
        a_d = a0.copy()
        piv_d, sing_d = lapack.getrf(a_d, mode="fast")
        _lib.set_fp64_update("ozaki")
        a_o = a0.copy()
        piv_o, sing_o = lapack.getrf(a_o, mode="fast")
    finally:
        _lib.set_fp64_update("auto")
    assert piv_o == piv_d and sing_o == sing_d
    assert np.abs(a_o - a_d).max() <= 1e-11 * np.abs(a_d).max()
    lo = np.tril(a_o, -1) + np.eye(n)
    up = np.triu(a_o)
    pa = a0.copy()
    for i, p in enumerate(piv_o):
        pa[[i, p]] = pa[[p, i]]
    berr = np.abs(pa - lo @ up).max() / (n * np.finfo(float).eps * np.abs(a0).max())
    print(f"\nn={n}: max|PA - LU| / (n eps max|A|) = {berr:.3f}")
    assert berr < 1.0


@pytest.mark.parametrize("m,n", [(300, 2000), (1000, 1000), (2000, 300)])
def test_getrf_triangular_solves_on_slices(m, n):
    """With the tensor-core engine the U12 solves of fast-mode FP64 getrf run
    as U12 = A12 - (I - L11^-1) A12 on the FP16 slice products (from 128
    columns with LUHOT_UPDATE_OZAKI, 256 with the default engine).  Wide,
    square and tall shapes: the pivots equal the DMMA engine's (whose solves
    are FMA substitutions), the factors agree to 1e-11 of max |LU| and
    max |PA - LU| stays below n eps max |A|."""
    rng = np.random.default_rng(m * 13 + n)
    a0 = rng.standard_normal((m, n))
    outs = {}
    try:
        for engine in ("dmma", "ozaki", "auto"):
            _lib.set_fp64_update(engine)
            a = a0.copy()
            piv, sing = lapack.getrf(a, mode="fast")
            outs[engine] = (a, piv, sing)
    finally:
        _lib.set_fp64_update("auto")
    a_d, piv_d, sing_d = outs["dmma"]
    k = min(m, n)
    for engine in ("ozaki", "auto"):
        a_o, piv_o, sing_o = outs[engine]
        assert piv_o == piv_d and sing_o == sing_d
        assert np.abs(a_o - a_d).max() <= 1e-11 * np.abs(a_d).max()
        lo = np.tril(a_o, -1)[:, :k] + np.eye(m, k)
        up = np.triu(a_o)[:k, :]
        pa = a0.copy()
        for i, p in enumerate(piv_o):
            pa[[i, p]] = pa[[p, i]]
        err = np.abs(pa - lo @ up).max() / (max(m, n) * np.finfo(float).eps * np.abs(a0).max())
        assert err < 1.0, (engine, err)
