"""Batched uneven solves against lair's per-system algorithm (the oracle)."""
import numpy as np
import pytest

import oracle
from lair_gb300 import batched

pytestmark = pytest.mark.gpu
EPS = {np.float64: 2.0 ** -53, np.float32: 2.0 ** -24}


def reference(sizes, a, b):
    out = []
    ao = bo = 0
    for n in sizes:
        m = a[ao:ao + n * n].reshape(n, n).copy()
        piv, sing = oracle.getrf(m)
        x = oracle.getrs(m, piv, b[bo:bo + n].copy())
        out.append((m, piv, sing, x))
        ao += n * n
        bo += n
    return out


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_batched_exact_is_bitwise_lair(dtype):
    sizes = [1, 2, 5, 8, 16, 17, 31, 32, 33, 63, 64, 65, 96, 97, 120, 128, 129, 150, 160, 161, 200, 224, 250, 256]
    rng = np.random.default_rng(0)
    mats = [rng.uniform(-1, 1, (n, n)) + (n if i % 2 else 0) * np.eye(n) for i, n in enumerate(sizes)]
    rhs = [rng.uniform(-1, 1, n) for n in sizes]
    a, b = batched.pack(mats, rhs, dtype)
    ref = reference(sizes, a, b)
    solver = batched.BatchSolver(sizes, dtype=dtype, mode="exact")
    piv, info = solver.solve(a, b)
    for (lu, x, pv), (m_ref, piv_ref, sing_ref, x_ref), s in zip(batched.unpack(sizes, a, b, piv), ref, info):
        assert list(pv) == piv_ref
        assert (s if s >= 0 else None) == sing_ref
        assert np.array_equal(lu, m_ref)
        assert np.array_equal(x, x_ref)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_batched_fast_backward_error_and_autotune(dtype):
    torch = pytest.importorskip("torch")
    sizes, a0, b0 = batched.synthetic_batch(600, seed=1, dtype=dtype)
    solver = batched.BatchSolver(sizes, dtype=dtype, mode="fast")
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    d_a = torch.from_numpy(a0).cuda()
    d_b = torch.from_numpy(b0).cuda()
    solver.autotune(d_a.data_ptr(), d_b.data_ptr())
    t = solver.tuning()
    assert len(t["buckets"]) == 9 and t["smem_max_n"] >= 64
    d_piv = torch.zeros(int(sizes.sum()), dtype=torch.int32, device="cuda")
    d_info = torch.zeros(len(sizes), dtype=torch.int32, device="cuda")
    for rep in range(2):  # the second call replays the captured graph
        d_a.copy_(torch.from_numpy(a0))
        d_b.copy_(torch.from_numpy(b0))
        torch.cuda.synchronize()
        solver.solve_device(d_a.data_ptr(), d_b.data_ptr(), d_piv.data_ptr(), d_info.data_ptr())
        x_all = d_b.cpu().numpy()
        if rep == 0:
            first = x_all.copy()
        else:
            assert np.array_equal(first, x_all)
    assert d_a.dtype == tdt
    ao = bo = 0
    for n in sizes:
        A = a0[ao:ao + n * n].reshape(n, n).astype(np.float64)
        x = x_all[bo:bo + n].astype(np.float64)
        bb = b0[bo:bo + n].astype(np.float64)
        berr = np.abs(bb - A @ x).max() / (np.abs(A).sum(1).max() * np.abs(x).max() + np.abs(bb).max())
        assert berr <= 4 * n * EPS[dtype], (n, berr)
        ao += n * n
        bo += n
    assert (d_info.cpu().numpy() == -1).all()


def test_batched_singular_systems_reported():
    sizes = [3, 40, 130]
    mats = [np.ones((3, 3)), np.zeros((40, 40)), np.random.default_rng(2).uniform(-1, 1, (130, 130))]
    mats[2][:, 77] = 0.0
    rhs = [np.ones(n) for n in sizes]
    a, b = batched.pack(mats, rhs)
    ref = reference(sizes, a.copy(), b.copy())
    piv, info = batched.BatchSolver(sizes, mode="exact").solve(a, b)
    assert [(s if s >= 0 else None) for s in info] == [r[2] for r in ref]


def test_batched_rejects_oversized_systems():
    from lair_gb300 import _lib
    with pytest.raises(_lib.LuhotError):
        batched.BatchSolver([10, 257])
