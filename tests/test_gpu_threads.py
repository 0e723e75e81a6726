"""Concurrent calls from several host threads, one luhot context each.

lair is reentrant (it keeps no globals), so the Rust shim may call the C
library from several threads at once: each thread owns a context, and calls
on different contexts overlap on the host and the GPU.  Kernel attributes and
page-locked host ranges are process-wide, so these tests run, at the same
time, calls that launch the same kernels with different shared-memory sizes
(FP64 and FP32 LU, exact and fast mode, the column-major exact order, the
tensor-core refinement) plus an allocation-free solve on its own stream, and
two threads that solve from the same large host array (it is page-locked by
whichever call comes first and must stay locked while the other copies).
Every threaded result must equal, bit for bit, what the same call gives when
run alone (the kernels are deterministic), and exact-mode factors must equal
the oracle's (lair's getrf order, src/lapack/getrf.rs:46-120 and :128-213).
"""
import ctypes
import threading

import numpy as np
import pytest

import oracle
from lair_gb300 import _lib

pytestmark = pytest.mark.gpu

ROUNDS = 3


def _new_ctx(lib):
    h = ctypes.c_void_p()
    assert lib.luhot_create(ctypes.byref(h), 0) == _lib.LUHOT_OK
    return h


def _es(a):
    return tuple(s // a.itemsize for s in a.strides)


def _gesv(lib, ctx, a, b):
    n, nrhs = b.shape
    x = np.empty_like(b)
    rc = lib.luhot_dgesv(ctx, n, nrhs, a.ctypes.data, *_es(a), b.ctypes.data, *_es(b), x.ctypes.data, *_es(x),
                         _lib.MODE_FAST)
    _lib.check(rc, ctx)
    return x


def _getrf(lib, ctx, a, mode):
    m, n = a.shape
    piv = np.zeros(min(m, n), dtype=np.uint64)
    sing = ctypes.c_int64(0)
    fn = lib.luhot_dgetrf if a.dtype == np.float64 else lib.luhot_sgetrf
    _lib.check(fn(ctx, m, n, a.ctypes.data, *_es(a), piv.ctypes.data, ctypes.byref(sing), mode), ctx)
    return piv, sing.value


def _getrs(lib, ctx, lu, piv, b, mode):
    n, nrhs = b.shape
    x = np.empty_like(b)
    fn = lib.luhot_dgetrs if lu.dtype == np.float64 else lib.luhot_sgetrs
    _lib.check(fn(ctx, n, nrhs, lu.ctypes.data, *_es(lu), piv.ctypes.data, b.ctypes.data, *_es(b), x.ctypes.data,
                  *_es(x), 0, mode), ctx)
    return x


def _ir(lib, ctx, a, b):
    n, nrhs = b.shape
    x = np.empty_like(b)
    info = _lib.IrInfo()
    rc = lib.luhot_dgesv_ir(ctx, n, nrhs, a.ctypes.data, *_es(a), b.ctypes.data, *_es(b), x.ctypes.data, *_es(x),
                            _lib.PREC_BF16X3, _lib.REFINE_IR, 0.0, 50, ctypes.byref(info))
    _lib.check(rc, ctx)
    return x, info.iterations


def _workloads(torch, lib):
    """(name, run(ctx) -> result) pairs; each run is self-contained."""
    rng = np.random.default_rng(77)
    n_big = 1200  # 11.5 MB: the host-buffer calls page-lock it
    a_shared = rng.standard_normal((n_big, n_big))
    b_shared = rng.standard_normal((n_big, 4))
    a_exact = rng.uniform(-1, 1, (600, 600))
    a_f = np.asfortranarray(rng.uniform(-1, 1, (500, 500)))
    a_s = rng.standard_normal((1500, 1500)).astype(np.float32)
    b_s = rng.standard_normal((1500, 3)).astype(np.float32)
    q1, _ = np.linalg.qr(rng.standard_normal((1024, 1024)))
    q2, _ = np.linalg.qr(rng.standard_normal((1024, 1024)))
    a_ir = (q1 * np.geomspace(1, 1e-4, 1024)) @ q2.T
    b_ir = rng.standard_normal((1024, 1))

    def gesv_shared(ctx):
        return _gesv(lib, ctx, a_shared, b_shared)

    def exact_rowmajor(ctx):
        a = a_exact.copy()
        piv, sing = _getrf(lib, ctx, a, _lib.MODE_EXACT)
        x = _getrs(lib, ctx, a, piv, b_shared[:600].copy(), _lib.MODE_EXACT)
        return a, piv, sing, x

    def exact_colmajor(ctx):
        a = a_f.copy(order="F")
        piv, sing = _getrf(lib, ctx, a, _lib.MODE_EXACT)
        return a, piv, sing

    def fp32_fast(ctx):
        a = a_s.copy()
        piv, sing = _getrf(lib, ctx, a, _lib.MODE_FAST)
        return a, piv, _getrs(lib, ctx, a, piv, b_s, _lib.MODE_FAST)

    def refine(ctx):
        return _ir(lib, ctx, a_ir, b_ir)

    # allocation-free solve on its own stream, with factors made beforehand
    n_na, nrhs_na = 900, 6
    fctx = _lib.context()
    d_lu = torch.from_numpy(rng.standard_normal((n_na, n_na))).cuda()
    d_piv = torch.zeros(n_na, dtype=torch.int32, device="cuda")
    sing = ctypes.c_int64(0)
    torch.cuda.synchronize()
    _lib.check(lib.luhot_dgetrf_dev(fctx, n_na, n_na, d_lu.data_ptr(), n_na, d_piv.data_ptr(), ctypes.byref(sing),
                                    _lib.MODE_FAST), fctx)
    b_na = rng.standard_normal((n_na, nrhs_na))
    stream = torch.cuda.Stream()

    def noalloc(_ctx):
        d_b = torch.from_numpy(b_na).to("cuda")
        torch.cuda.synchronize()
        rc = lib.luhot_dgetrs_dev_noalloc(n_na, nrhs_na, d_lu.data_ptr(), n_na, d_piv.data_ptr(), d_b.data_ptr(),
                                          nrhs_na, 0, _lib.MODE_FAST, ctypes.c_void_p(stream.cuda_stream))
        assert rc == _lib.LUHOT_OK
        stream.synchronize()
        return d_b.cpu().numpy()

    return {
        "gesv_shared_a": gesv_shared,
        "gesv_shared_b": gesv_shared,
        "exact_rowmajor": exact_rowmajor,
        "exact_colmajor": exact_colmajor,
        "fp32_fast": fp32_fast,
        "refine": refine,
        "noalloc": noalloc,
    }, (a_exact, a_f)


def _same(x, y):
    if isinstance(x, tuple):
        return all(_same(p, q) for p, q in zip(x, y))
    if isinstance(x, np.ndarray):
        return x.shape == y.shape and np.array_equal(x, y)
    return x == y


def test_threads_with_own_contexts_match_serial_results():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    work, (a_exact, a_f) = _workloads(torch, lib)
    ctxs = {name: _new_ctx(lib) for name in work}
    try:
        # each workload alone, one after another: the expected results
        expected = {name: fn(ctxs[name]) for name, fn in work.items()}

        # exact-mode factors are lair's bits
        a_ref = a_exact.copy()
        piv_ref, sing_ref = oracle.getrf(a_ref)
        a_gpu, piv_gpu, sing_gpu, _ = expected["exact_rowmajor"]
        assert list(piv_gpu) == piv_ref and (None if sing_gpu < 0 else sing_gpu) == sing_ref
        assert np.array_equal(a_gpu, a_ref)
        f_ref = a_f.copy(order="F")
        fpiv_ref, _ = oracle.getrf(f_ref)
        assert list(expected["exact_colmajor"][1]) == fpiv_ref
        assert np.array_equal(expected["exact_colmajor"][0], f_ref)

        # all of them at once, ROUNDS times each
        results = {name: [] for name in work}
        errors = []
        start = threading.Barrier(len(work))

        def runner(name):
            try:
                start.wait(timeout=60)
                for _ in range(ROUNDS):
                    results[name].append(work[name](ctxs[name]))
            except BaseException as e:  # noqa: BLE001 - reported below
                errors.append((name, repr(e)))

        threads = [threading.Thread(target=runner, args=(name,)) for name in work]
        for t in threads:
            t.start()
        for t in threads:
            t.join(timeout=600)
        assert not any(t.is_alive() for t in threads), "a thread did not finish"
        assert not errors, errors
        for name in work:
            assert len(results[name]) == ROUNDS
            for r in results[name]:
                assert _same(r, expected[name]), f"{name}: threaded result differs from the serial one"
    finally:
        for h in ctxs.values():
            lib.luhot_destroy(h)
