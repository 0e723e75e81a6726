"""The allocation-free solve entry point, luhot_dgetrs_dev_noalloc.

It serves callers that cannot call cudaMalloc (their device memory belongs to
their own pool or caching allocator, or their solve loop cannot take the
synchronisation an allocation may cause): it takes device buffers, uses no
luhot context and keeps its scratch in a static device array.  These tests
call it through the C ABI twice in a row, with different systems, and
compare each result with luhot_dgetrs_dev's on the same factors.  The exact
forward/backward order is lair's in both, so exact-mode results agree bit for
bit; fast-mode sweeps may group the FMAs differently, so there the suite's
fast-mode tolerance applies (relative 1e-8 of max |x|).  The file is named to
be collected last; it passes alone in a fresh process as well.
"""
import ctypes

import numpy as np
import pytest

from lair_gb300 import _lib

pytestmark = pytest.mark.gpu


def _factor(torch, lib, ctx, n, seed):
    rng = np.random.default_rng(seed)
    a0 = rng.standard_normal((n, n))
    d_a = torch.from_numpy(a0).cuda().contiguous()
    d_piv = torch.zeros(n, dtype=torch.int32, device="cuda")
    sing = ctypes.c_int64(0)
    _lib.check(lib.luhot_dgetrf_dev(ctx, n, n, d_a.data_ptr(), n, d_piv.data_ptr(), ctypes.byref(sing), 0), ctx)
    assert sing.value == -1
    return a0, d_a, d_piv


@pytest.mark.parametrize("mode", [_lib.MODE_FAST, _lib.MODE_EXACT])
@pytest.mark.parametrize("trans", [0, 1])
def test_noalloc_matches_existing_entry_point_twice(mode, trans):
    torch = pytest.importorskip("torch")
    lib, ctx = _lib.load(), _lib.context()
    stream = torch.cuda.Stream()
    _lib.check(lib.luhot_set_stream(ctx, ctypes.c_void_p(stream.cuda_stream)), ctx)
    try:
        for call, (n, nrhs) in enumerate([(777, 5), (1536, 16)]):
            _, d_a, d_piv = _factor(torch, lib, ctx, n, 100 + call)
            b = np.random.default_rng(200 + call).standard_normal((n, nrhs))
            d_ref = torch.from_numpy(b).cuda().contiguous()
            d_new = torch.from_numpy(b).cuda().contiguous()
            torch.cuda.synchronize()
            _lib.check(lib.luhot_dgetrs_dev(ctx, n, nrhs, d_a.data_ptr(), n, d_piv.data_ptr(), d_ref.data_ptr(),
                                            nrhs, trans, mode), ctx)
            rc = lib.luhot_dgetrs_dev_noalloc(n, nrhs, d_a.data_ptr(), n, d_piv.data_ptr(), d_new.data_ptr(),
                                              nrhs, trans, mode, ctypes.c_void_p(stream.cuda_stream))
            assert rc == _lib.LUHOT_OK
            torch.cuda.synchronize()
            ref = d_ref.cpu().numpy()
            new = d_new.cpu().numpy()
            bitwise = mode == _lib.MODE_EXACT and trans == 0
            np.testing.assert_allclose(new, ref, rtol=0, atol=0 if bitwise else 1e-8 * np.abs(ref).max())
            assert np.isfinite(new).all()
    finally:
        lib.luhot_set_stream(ctx, None)


@pytest.mark.parametrize("mode", [_lib.MODE_FAST, _lib.MODE_EXACT])
def test_noalloc_many_right_hand_sides(mode):
    """400 right-hand sides of order 64 fit the scratch; the block updates
    take them 256 at a time, so shared memory sets no smaller limit."""
    torch = pytest.importorskip("torch")
    lib, ctx = _lib.load(), _lib.context()
    n, nrhs = 64, 400
    _, d_a, d_piv = _factor(torch, lib, ctx, n, 300)
    b = np.random.default_rng(301).standard_normal((n, nrhs))
    d_ref = torch.from_numpy(b).cuda().contiguous()
    d_new = torch.from_numpy(b).cuda().contiguous()
    torch.cuda.synchronize()
    _lib.check(lib.luhot_dgetrs_dev(ctx, n, nrhs, d_a.data_ptr(), n, d_piv.data_ptr(), d_ref.data_ptr(), nrhs, 0,
                                    mode), ctx)
    torch.cuda.synchronize()
    for _ in range(2):
        d_new.copy_(torch.from_numpy(b).cuda())
        torch.cuda.synchronize()
        rc = lib.luhot_dgetrs_dev_noalloc(n, nrhs, d_a.data_ptr(), n, d_piv.data_ptr(), d_new.data_ptr(), nrhs, 0,
                                          mode, None)
        assert rc == _lib.LUHOT_OK
        torch.cuda.synchronize()
        ref, new = d_ref.cpu().numpy(), d_new.cpu().numpy()
        atol = 0 if mode == _lib.MODE_EXACT else 1e-8 * np.abs(ref).max()
        np.testing.assert_allclose(new, ref, rtol=0, atol=atol)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    n = 1024
    nrhs = _lib_limit_nrhs(n) + 1
    d_lu = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    d_piv = torch.arange(n, dtype=torch.int32, device="cuda")
    d_b = torch.zeros((n, nrhs), dtype=torch.float64, device="cuda")
    rc = lib.luhot_dgetrs_dev_noalloc(n, nrhs, d_lu.data_ptr(), n, d_piv.data_ptr(), d_b.data_ptr(), nrhs, 0, 0,
                                      None)
    assert rc == _lib.LUHOT_ERR_UNSUPPORTED
    assert lib.luhot_dgetrs_dev_noalloc(-1, 1, None, 1, None, None, 1, 0, 0, None) == _lib.LUHOT_ERR_INVALID_ARG


def _lib_limit_nrhs(n):
    scratch = 4 << 20
    perm = (4 * n + 255) // 256 * 256
    return (scratch - perm) // (8 * n)
