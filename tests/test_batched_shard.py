"""Data-parallel sharding of a batch (host logic, CPU): contiguous slices
balanced by sum n^3, agreed by every rank without communication; checked
with two gloo ranks that each solve their slice with the oracle and gather
the per-system singular flags."""
import os
import socket

import numpy as np
import pytest

from lair_gb300 import batched


def test_shards_cover_the_batch_and_balance_work():
    sizes, _, _ = batched.synthetic_batch(10000, seed=0)
    for world in (1, 2, 4, 8):
        parts = batched.shard_by_work(sizes, world)
        assert parts[0][0] == 0 and parts[-1][1] == len(sizes)
        assert all(parts[i][1] == parts[i + 1][0] for i in range(world - 1))
        work = [float(np.sum(sizes[b:e].astype(np.float64) ** 3)) for b, e in parts]
        assert max(work) - min(work) <= 2 * 256.0 ** 3


def test_shard_edge_cases():
    assert batched.shard_by_work([], 3) == [(0, 0), (0, 0), (0, 0)]
    assert batched.shard_by_work([5], 2) in ([(0, 0), (0, 1)], [(0, 1), (1, 1)])
    with pytest.raises(ValueError):
        batched.shard_by_work([1, 2], 0)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    import torch
    import torch.distributed as dist

    import oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sizes, a, b = batched.synthetic_batch(64, seed=3, nmax=48)
    sizes[5] = 12
    begin, end = batched.shard_by_work(sizes, world)[rank]
    offs = np.concatenate([[0], np.cumsum(sizes.astype(np.int64) ** 2)])
    sing = np.full(len(sizes), -1, dtype=np.int64)
    for i in range(begin, end):
        n = int(sizes[i])
        m = a[offs[i]:offs[i] + n * n].reshape(n, n).copy()
        if i == 5:
            m[:, 4] = 0.0
        _, s = oracle.getrf(m)
        sing[i] = -1 if s is None else s
    t = torch.from_numpy(sing)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)  # each system is owned by exactly one rank
    q.put((rank, begin, end, t.numpy().tolist()))
    dist.destroy_process_group()


def test_two_gloo_ranks_solve_disjoint_shards():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    (_, b0, e0, s0), (_, b1, e1, s1) = res
    assert b0 == 0 and e0 == b1 and e1 == 64
    assert s0 == s1
    assert s0[5] == 4 and all(v == -1 for i, v in enumerate(s0) if i != 5)


def test_pack_unpack_round_trip_and_layout():
    # Packed layout of the batched ABI: A_i row-major back to back, b_i (and
    # the pivots) back to back, offsets the running sums of n_i^2 and n_i.
    rng = np.random.default_rng(5)
    sizes = [1, 3, 8, 2]
    mats = [rng.standard_normal((n, n)) for n in sizes]
    rhs = [rng.standard_normal(n) for n in sizes]
    a, b = batched.pack([np.asfortranarray(m) for m in mats], rhs, dtype=np.float32)
    assert a.dtype == np.float32 and a.size == sum(n * n for n in sizes) and b.size == sum(sizes)
    piv = np.arange(b.size, dtype=np.int32)
    off = 0
    for (ai, bi, pi), m, v, n in zip(batched.unpack(sizes, a, b, piv), mats, rhs, sizes):
        assert np.array_equal(ai, m.astype(np.float32)) and np.array_equal(bi, v.astype(np.float32))
        assert np.array_equal(pi, np.arange(off, off + n))
        off += n
    empty_a, empty_b = batched.pack([], [])
    assert empty_a.size == 0 and empty_b.size == 0


def test_synthetic_batch_is_the_benchmark_distribution():
    sizes, a, b = batched.synthetic_batch(500, seed=7, nmin=8, nmax=256)
    assert sizes.min() >= 8 and sizes.max() <= 256 and a.size == int(np.sum(sizes.astype(np.int64) ** 2))
    again = batched.synthetic_batch(500, seed=7, nmin=8, nmax=256)
    assert all(np.array_equal(x, y) for x, y in zip((sizes, a, b), again))  # seeded
    # about half the systems carry the + n I shift (their diagonal dominates)
    ao, shifted = 0, 0
    for n in sizes:
        d = a[ao:ao + n * n].reshape(n, n).diagonal()
        shifted += int(np.all(d >= n - 1))
        ao += int(n) * int(n)
    assert 0.4 * len(sizes) < shifted < 0.6 * len(sizes)
