"""Batched uneven LU solves (no lair counterpart) and their multi-GPU sharding.

``BatchSolver(sizes)`` plans one persistent, graph-captured launch that
factors and solves ``len(sizes)`` independent systems of sizes 1..256 with
lair's per-system semantics (pivots, singular step; ``mode="exact"`` gives
lair's bits).  Arrays are packed: A_i row-major back to back, b_i back to
back (see ``pack`` / ``unpack``).

``shard_by_work`` splits a batch over ranks for data-parallel solving on
several GPUs: contiguous slices balanced by sum n_i^3, no collective needed.
"""
from __future__ import annotations

import ctypes
from typing import List, Sequence, Tuple

import numpy as np

from . import _lib

BUCKET_NAMES = ("n<=16", "16<n<=32", "32<n<=64", "64<n<=96", "96<n<=128", "128<n<=160", "160<n<=192",
                "192<n<=224", "224<n<=256")


def pack(mats: Sequence[np.ndarray], rhs: Sequence[np.ndarray], dtype=np.float64) -> Tuple[np.ndarray, np.ndarray]:
    a = np.concatenate([np.ascontiguousarray(m, dtype=dtype).ravel() for m in mats]) if mats else np.zeros(0, dtype)
    b = np.concatenate([np.ascontiguousarray(v, dtype=dtype).ravel() for v in rhs]) if rhs else np.zeros(0, dtype)
    return a, b


def unpack(sizes: Sequence[int], a: np.ndarray, b: np.ndarray, piv: np.ndarray):
    out, ao, bo = [], 0, 0
    for n in sizes:
        out.append((a[ao:ao + n * n].reshape(n, n), b[bo:bo + n], piv[bo:bo + n]))
        ao += n * n
        bo += n
    return out


class BatchSolver:
    def __init__(self, sizes: Sequence[int], dtype=np.float64, mode: str = "fast"):
        self.sizes = np.ascontiguousarray(np.asarray(sizes, dtype=np.int32))
        self.dtype = np.dtype(dtype)
        if self.dtype not in (np.float64, np.float32):
            raise TypeError("batched solves support float64 and float32")
        self._lib, self._ctx = _lib.load(), _lib.context()
        h = ctypes.c_void_p()
        rc = self._lib.luhot_batch_create(self._ctx, len(self.sizes), self.sizes.ctypes.data,
                                          0 if self.dtype == np.float64 else 1, _lib.mode_id(mode), ctypes.byref(h))
        _lib.check(rc, self._ctx)
        self._h = h
        a_el, b_el = ctypes.c_int64(), ctypes.c_int64()
        self._lib.luhot_batch_layout(h, ctypes.byref(a_el), ctypes.byref(b_el))
        self.a_elems, self.b_elems = a_el.value, b_el.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and self._lib is not None:
            self._lib.luhot_batch_destroy(h)
            self._h = None

    def autotune(self, d_a: int, d_b: int) -> None:
        _lib.check(self._lib.luhot_batch_autotune(self._h, d_a, d_b), self._ctx)

    def tuning(self) -> dict:
        nb = np.zeros(9, dtype=np.int32)
        sn = ctypes.c_int32()
        self._lib.luhot_batch_tuning(self._h, nb.ctypes.data, ctypes.byref(sn))
        return {"buckets": {k: ("smem" if v == 0 else f"panel{v}") for k, v in zip(BUCKET_NAMES, nb.tolist())},
                "smem_max_n": sn.value}

    def solve_device(self, d_a: int, d_b: int, d_piv: int, d_info: int) -> None:
        _lib.check(self._lib.luhot_batch_solve(self._h, d_a, d_b, d_piv, d_info), self._ctx)

    def solve(self, a: np.ndarray, b: np.ndarray):
        """In place on packed host arrays; returns (pivots, info)."""
        if a.dtype != self.dtype or b.dtype != self.dtype or a.size != self.a_elems or b.size != self.b_elems:
            raise ValueError("packed arrays do not match the plan")
        if not (a.flags.c_contiguous and b.flags.c_contiguous):
            raise ValueError("packed arrays must be contiguous")
        piv = np.zeros(self.b_elems, dtype=np.int32)
        info = np.zeros(len(self.sizes), dtype=np.int32)
        rc = self._lib.luhot_batch_solve_host(self._h, a.ctypes.data, b.ctypes.data, piv.ctypes.data, info.ctypes.data)
        _lib.check(rc, self._ctx)
        return piv, info


def shard_by_work(sizes: Sequence[int], world: int) -> List[Tuple[int, int]]:
    """Contiguous [begin, end) slices of the batch, one per rank, with sum n^3 balanced.

    Every rank computes the same partition from the same sizes, so no
    communication is needed to agree on it.
    """
    if world < 1:
        raise ValueError("world must be >= 1")
    w = np.asarray(sizes, dtype=np.float64) ** 3
    cum = np.concatenate([[0.0], np.cumsum(w)])
    total = cum[-1]
    bounds = [0]
    for r in range(1, world):
        bounds.append(int(np.searchsorted(cum, total * r / world, side="left")))
    bounds.append(len(w))
    bounds = [min(max(b, 0), len(w)) for b in bounds]
    for i in range(1, len(bounds)):
        bounds[i] = max(bounds[i], bounds[i - 1])
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def synthetic_batch(count: int, seed: int = 0, nmin: int = 8, nmax: int = 256, dtype=np.float64):
    """The benchmark's batch: n ~ U{nmin..nmax}, A iid U[-1,1] plus n*I with
    probability 1/2, one right-hand side iid U[-1,1] (seeded)."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(nmin, nmax + 1, size=count).astype(np.int32)
    shift = rng.random(count) < 0.5
    a_el = int(np.sum(sizes.astype(np.int64) ** 2))
    a = rng.uniform(-1, 1, a_el).astype(dtype)
    b = rng.uniform(-1, 1, int(sizes.sum())).astype(dtype)
    ao = 0
    for n, s in zip(sizes, shift):
        if s:
            idx = ao + np.arange(n) * (n + 1)
            a[idx] += n
        ao += int(n) * int(n)
    return sizes, a, b
