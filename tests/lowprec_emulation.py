"""CPU emulation of the mixed-precision LU and of GMRES-IR (test infrastructure).

The low-precision factorization of ``luhot_sgetrf_mixed_dev`` has no lair
counterpart, so its checker is this emulation of the same blocked algorithm:
FP32 storage, FP32 panels with partial pivoting, FP32 triangular solve for
U12, and the Schur update A22 -= L21 U12 with each operand scaled by a power
of two (largest magnitude at 2^14) and rounded to the operand format (BF16 or
FP16 to nearest even, TF32 to nearest with ties away), products accumulated
exactly enough (FP64 here, FP32 on the GPU; both far below the operand
rounding).  ``quality`` measures what decides whether refinement converges:
the growth factor, ||I - M^-1 A||_2 and how many singular values of M^-1 A
lie far from 1 (M = P^T L U applied in FP64, as GMRES-IR applies it).
``gmres_ir`` restates the GPU's GMRES-IR (left preconditioning, restarts,
two passes of classical Gram-Schmidt, stop when the normwise backward error
reaches n 2^-53) to count iterations.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla

EPS64 = 2.0 ** -53
PANEL = {"fp32": 64, "tf32": 128, "fp16": 128, "bf16": 128}


def conditioned(n: int, kappa: float, seed: int = 0):
    """A = Q1 diag(sigma) Q2^T (Q from QR of N(0,1)), sigma geometric 1 -> 1/kappa; b N(0,1)."""
    rng = np.random.default_rng(seed)
    q1, _ = np.linalg.qr(rng.standard_normal((n, n)))
    q2, _ = np.linalg.qr(rng.standard_normal((n, n)))
    sigma = np.geomspace(1.0, 1.0 / kappa, n)
    return (q1 * sigma) @ q2.T, rng.standard_normal(n)


def _bf16(x):
    b = x.astype(np.float32).view(np.uint32)
    b = (b + (((b >> 16) & 1) + 0x7FFF)) & 0xFFFF0000
    return b.view(np.float32)


def _tf32(x):
    b = x.astype(np.float32).view(np.uint32)
    b = (b + 0x1000) & 0xFFFFE000  # to nearest, ties away from zero (13 dropped bits)
    return b.view(np.float32)


def _scale(x):
    mx = float(np.abs(x).max()) if x.size else 0.0
    if not (mx > 0.0) or not np.isfinite(mx):
        return 1.0
    _, e = np.frexp(mx)
    return float(2.0 ** (14 - int(e)))


def _round(kind, x):
    if kind == "bf16":
        return _bf16(x)
    if kind == "fp16":
        return x.astype(np.float16).astype(np.float32)
    if kind == "tf32":
        return _tf32(x)
    return x.astype(np.float32)


def factor(a: np.ndarray, kind: str):
    """Blocked LU of a (square) in the given kind -> (lu float32, perm): P A = L U with
    perm[i] the original row now at position i."""
    n = a.shape[0]
    w = PANEL[kind]
    A = a.astype(np.float32).copy()
    perm = np.arange(n)
    for k0 in range(0, n, w):
        k1 = min(n, k0 + w)
        for j in range(k0, k1):
            p = j + int(np.argmax(np.abs(A[j:, j])))
            if p != j:
                A[[j, p]] = A[[p, j]]
                perm[[j, p]] = perm[[p, j]]
            piv = A[j, j]
            if piv == 0:
                continue
            A[j + 1:, j] *= np.float32(1.0) / piv
            if j + 1 < k1:
                A[j + 1:, j + 1:k1] -= np.outer(A[j + 1:, j], A[j, j + 1:k1]).astype(np.float32)
        if k1 < n:
            L11 = np.tril(A[k0:k1, k0:k1], -1) + np.eye(k1 - k0, dtype=np.float32)
            A[k0:k1, k1:] = sla.solve_triangular(L11, A[k0:k1, k1:], lower=True, unit_diagonal=True).astype(np.float32)
            L21, U12 = A[k1:, k0:k1], A[k0:k1, k1:]
            if kind == "fp32":
                A[k1:, k1:] -= L21 @ U12
            else:
                sa, sb = _scale(L21), _scale(U12)
                prod = _round(kind, L21 * np.float32(sa)).astype(np.float64) @ \
                    _round(kind, U12 * np.float32(sb)).astype(np.float64)
                A[k1:, k1:] = (A[k1:, k1:].astype(np.float64) - prod / (sa * sb)).astype(np.float32)
    return A, perm


def perm_from_pivots(piv):
    perm = np.arange(len(piv))
    for i, p in enumerate(piv):
        if p != i:
            perm[i], perm[p] = perm[p], perm[i]
    return perm


def apply_minv(lu: np.ndarray, perm: np.ndarray, v: np.ndarray) -> np.ndarray:
    """M^-1 v = U^-1 L^-1 P v in FP64 arithmetic on the stored factors."""
    f = lu.astype(np.float64)
    y = sla.solve_triangular(f, v[perm], lower=True, unit_diagonal=True, check_finite=False)
    return sla.solve_triangular(f, y, lower=False, check_finite=False)


def quality(a: np.ndarray, lu: np.ndarray, perm: np.ndarray) -> dict:
    n = a.shape[0]
    y = apply_minv(lu, perm, a)  # M^-1 A
    s = sla.svdvals(y)
    e = np.eye(n) - y
    v = np.random.default_rng(1).standard_normal(n)
    for _ in range(40):  # power iteration for ||I - M^-1 A||_2
        v = e.T @ (e @ v)
        v /= np.linalg.norm(v)
    return {"growth": float(np.abs(np.triu(lu)).max() / np.abs(a).max()),
            "norm_I_minus_MinvA": float(np.linalg.norm(e @ v)),
            "sv_far_from_1": int(np.sum((s < 0.5) | (s > 2.0))),
            "sv_min": float(s[-1]), "sv_max": float(s[0])}


def gmres_ir(a, b, lu, perm, restart=120, max_inner=2000, max_outer=50):
    """GMRES-IR as the GPU runs it -> (outer steps, inner iterations, final backward error)."""
    n = a.shape[0]
    anorm = np.abs(a).sum(1).max()
    x = np.zeros(n)
    inner_total = 0
    berr = np.inf
    for outer in range(max_outer + 1):
        r = b - a @ x
        berr = np.abs(r).max() / (anorm * np.abs(x).max() + np.abs(b).max())
        if berr <= n * EPS64 or inner_total >= max_inner:
            return outer, inner_total, float(berr)
        t = apply_minv(lu, perm, r)
        beta = np.linalg.norm(t)
        V = np.zeros((restart + 1, n))
        V[0] = t / beta
        H = np.zeros((restart + 1, restart))
        k = 0
        for k in range(restart):
            wv = apply_minv(lu, perm, a @ V[k])
            for _ in range(2):
                h = V[:k + 1] @ wv
                wv -= h @ V[:k + 1]
                H[:k + 1, k] += h
            H[k + 1, k] = np.linalg.norm(wv)
            inner_total += 1
            g = np.zeros(k + 2)
            g[0] = beta
            yk, *_ = np.linalg.lstsq(H[:k + 2, :k + 1], g, rcond=None)
            res = np.linalg.norm(H[:k + 2, :k + 1] @ yk - g)
            if H[k + 1, k] == 0 or res <= 1e-14 * beta:
                k += 1
                break
            V[k + 1] = wv / H[k + 1, k]
        else:
            k = restart
        g = np.zeros(k + 1)
        g[0] = beta
        yk, *_ = np.linalg.lstsq(H[:k + 1, :k], g, rcond=None)
        x = x + yk @ V[:k]
    return max_outer, inner_total, float(berr)
