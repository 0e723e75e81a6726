"""Benchmark: Ax=b GFLOP/s at backward error <= n*eps64 on one GB300.

Workload (default): plain FP64 getrf + getrs, n = 16384, 16 right-hand sides,
A and B iid N(0, 1) from the seeded portable generator (lair_gb300.synthetic;
synthetic, no dataset exists for this metric), the inputs of the committed
lair reference results, so the line carries a parity key.  One step = restore A and B in HBM, factor, solve.
GFLOP/s = (2/3 n^3 + 2 n^2 nrhs) / time.  The solution's normwise backward
error ||b - Ax||_inf / (||A||_inf ||x||_inf + ||b||_inf) is checked against
n * 2^-53 after the timed steps.

Printed as one JSON line (rank 0):
  value     device-resident throughput (inputs in HBM when timing starts)
  e2e       the same solve through the C ABI with host buffers
            (luhot_dgesv: A, B copied in and X copied out every step)
  roofline  the Schur update (the dominant kernel).  With the default engine
            (--fp64-update auto) the large updates run on the FP16 tensor cores
            as exact integer-slice products (28 slice GEMMs per update): the
            executed FP16 work against the measured tensor peak, with the
            FP64-equivalent rate and C's HBM traffic beside it.  With
            --fp64-update dmma: against the FP64 tensor-core peak measured
            in this run.
  fp64_update  the engine, and one step timed with the DMMA engine for
            comparison
  resident_solve  lair's Factorized::solve with device-resident factors,
            one right-hand side per call (the block-scaled sweeps)
  parity    pivots, ||PA - LU|| and the solution error against lair's
            results for the same inputs (tests/golden fixtures)
  cpu_baseline  lair's algorithm (the CPU oracle) on a bounded sample, plus
            one complete n = 4096 run and its n^3 extrapolation (labelled)
  adjoint   the backward solve (lambda = A^-T W, dA, dB) at n = 2048, nrhs = 8
  batched   10,000 uneven systems, sharded over ranks by work when N > 1
  ir        mixed-precision LU + iterative refinement on the kappa-conditioned
            n = 16384 system, when built

--impl reference times lair's own algorithm on the host cores instead (the
oracle port: lair is Rust and cannot be built here).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Ax=b GFLOP/s at backward err ≤ n·eps64: FP64 LU vs mixed-precision IR, 1 GB300"
EPS64 = 2.0 ** -53


def flops_of(n: int, nrhs: int) -> float:
    return 2.0 / 3.0 * n ** 3 + 2.0 * n * n * nrhs


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.thread:
                self.thread.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------------
# CPU baseline: lair's getrf_row_major + getrs (the oracle) on a bounded
# slice of the same n x n system, one core (lair is single-threaded).
# --------------------------------------------------------------------------
def cpu_sample(n: int, seed: int, elim_steps: int, state=None):
    """Run `elim_steps` elimination steps (continuing from `state`) and one
    single-RHS getrs; returns (flops, seconds, state)."""
    import oracle

    if state is None:
        rng = np.random.default_rng(seed)
        a = rng.standard_normal((n, n))
        b = rng.standard_normal(n)
        piv = np.arange(n, dtype=np.uint64)
        state = {"a": a, "b": b, "piv": piv, "next": 0}
    a, piv, b = state["a"], state["piv"], state["b"]
    s0 = state["next"]
    s1 = min(n, s0 + elim_steps)
    fl = 0.0
    for ul in range(s0, s1):
        r = n - ul - 1
        fl += r + 2.0 * r * r  # scale + rank-1 update
    t0 = time.perf_counter()
    oracle.getrf_row_major_range(a, piv, s0, s1)
    t1 = time.perf_counter()
    oracle.getrs(a, piv, b)  # cost of one getrs does not depend on the values
    t2 = time.perf_counter()
    fl += 2.0 * n * n
    state["next"] = s1
    return fl, (t2 - t0), state


def cpu_full_run(n: int, nrhs: int):
    """One complete solve in lair's order on one core: getrf_row_major of an
    n x n N(0,1) matrix and lair's single-RHS getrs for each of nrhs columns."""
    import oracle
    from lair_gb300 import synthetic

    a = synthetic.normal_matrix(10 * n + 1, n, n)
    b = synthetic.normal_matrix(10 * n + 2, n, nrhs)
    t0 = time.perf_counter()
    piv, _ = oracle.getrf_row_major(a)
    for j in range(nrhs):
        oracle.getrs(a, piv, np.ascontiguousarray(b[:, j]))
    return time.perf_counter() - t0


def cpu_baseline(n: int, nrhs: int, seconds: float = 12.0, full_n: int = 4096):
    fl_total, t_total, steps, state = 0.0, 0.0, 0, None
    while t_total < seconds and (state is None or state["next"] < n):
        fl, t, state = cpu_sample(n, 1234, 2, state)
        fl_total += fl
        t_total += t
        steps += 1
    out = {"value": fl_total / t_total / 1e9, "unit": "GFLOP/s", "cores": 1, "kind": "port",
           "sample": (f"lair getrf_row_major + getrs restated in C++ (-O2 -ffp-contract=off), 1 thread: "
                      f"the first {state['next']} elimination steps of an n={n} N(0,1) matrix plus "
                      f"{steps} single-RHS getrs at n={n}; {t_total:.1f} s of CPU work"),
           "host": os.uname().machine, "host_cores_total": os.cpu_count()}
    if full_n:
        t_full = cpu_full_run(full_n, nrhs)
        scale = (n / full_n) ** 3
        out["full_run"] = {"n": full_n, "nrhs": nrhs, "seconds": t_full,
                           "gflops": flops_of(full_n, nrhs) / t_full / 1e9,
                           "what": f"complete getrf_row_major + {nrhs} single-RHS getrs at n={full_n}, 1 thread"}
        out["extrapolated"] = {"n": n, "seconds": t_full * scale,
                               "gflops": flops_of(n, nrhs) / (t_full * scale) / 1e9,
                               "how": f"EXTRAPOLATED, not measured: the n={full_n} time x (n/{full_n})^3"}
    return out


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    n = args.n
    state = None
    for _ in range(args.warmup):
        _, _, state = cpu_sample(n, 1234, args.ref_elim_steps, state)
    fl_total, t_total = 0.0, 0.0
    for _ in range(args.steps):
        fl, t, state = cpu_sample(n, 1234, args.ref_elim_steps, state)
        fl_total += fl
        t_total += t
    value = fl_total / t_total / 1e9
    sample = (f"each step: {args.ref_elim_steps} elimination steps of lair's getrf_row_major on the n={n} "
              f"N(0,1) matrix (continuing) + one single-RHS getrs at n={n}; oracle port in C++, 1 thread "
              f"(lair is single-threaded)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_total / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": workload_config(args),
            "cpu_baseline": {"value": value, "unit": "GFLOP/s", "cores": 1, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


OZ_PRODUCTS = 28  # FP16 slice GEMMs per tensor-core FP64 update (groups p + q <= 6 of 7 x 7)


def workload_config(args):
    return {"workload": f"plain FP64 getrf+getrs drop-in, n={args.n}, nrhs={args.nrhs}, A,B iid N(0,1) seeded "
                        "(portable generator, lair_gb300.synthetic)",
            "n": args.n, "nrhs": args.nrhs, "mode": args.mode,
            "fp64_update": {"auto": "FP16 tensor cores, exact integer slices (Ozaki), on trailing blocks >= 256 x 256; "
                                    "DMMA below",
                            "dmma": "FP64 tensor cores (DMMA) only",
                            "ozaki": "FP16 tensor cores, exact integer slices, on every block >= 128 x 64"}[
                                        args.fp64_update],
            "l2": "inputs larger than L2 (A is %.1f GiB vs 129 MB L2)" % (args.n * args.n * 8 / 2 ** 30),
            "parallelism": "replicas (one independent system per GPU)"}


def measured_peaks() -> dict:
    """The measured peaks of the GB300s (empty if absent)."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def measured_hbm_peak() -> float:
    """HBM copy bandwidth measured on the GB300s, else the fallback."""
    try:
        return float(measured_peaks()["hbm_gbs"])
    except (KeyError, TypeError, ValueError):
        return 6800.0


def load_parity_fixture(n: int, nrhs: int):
    """lair's results (the oracle's, committed under tests/golden) for the
    seeded N(0,1) system of order n, if there is one for this size."""
    path = os.path.join(ROOT, "tests", "golden", f"getrf_normal_n{n}.npz")
    if not os.path.exists(path):
        return None
    fx = np.load(path)
    return fx if int(fx["nrhs"]) == nrhs else None


def parity_vs_lair(torch, n, fx, A0, LU, piv, X):
    """Fast-mode results of the last timed step against lair's on the same
    inputs: pivots (or the first differing step and the candidates' margin
    there), ||PA - LU||_max / (n eps ||A||_max) on the GPU in FP64, the
    solution's relative error against lair's for columns 0 and 1, and 2048
    sampled entries of L\\U."""
    p = piv.cpu().numpy().astype(np.int64)
    ref = fx["piv"].astype(np.int64)
    diff = np.nonzero(p != ref)[0]
    first = int(diff[0]) if diff.size else -1
    perm = np.arange(n)
    for i, j in enumerate(p):
        if j != i:
            perm[i], perm[j] = perm[j], perm[i]
    L = torch.tril(LU, -1)
    L.diagonal().fill_(1.0)
    err = (A0[torch.from_numpy(perm).cuda()] - L @ torch.triu(LU)).abs().max().item()
    del L
    x = X[:, :2].cpu().numpy()
    rows = torch.from_numpy(fx["lu_rows"].astype(np.int64)).cuda()
    cols = torch.from_numpy(fx["lu_cols"].astype(np.int64)).cuda()
    lu_s = LU[rows, cols].cpu().numpy()
    out = {"reference": "lair getrf_row_major + getrs (oracle, same seeded inputs; tests/golden)",
           "pivots_identical": first < 0, "first_divergent_step": first,
           "pa_minus_lu_over_n_eps_a": err / (n * EPS64 * A0.abs().max().item()),
           "solution_rel_err_vs_lair": float(np.abs(x - fx["x01"]).max() / np.abs(fx["x01"]).max()),
           "lu_sample_rel_diff": float(np.abs(lu_s - fx["lu_vals"]).max() / np.abs(fx["lu_vals"]).max()),
           "min_relative_pivot_margin": float(np.min(fx["gap"] / fx["colmax"]))}
    if first >= 0:
        out["margin_at_divergence"] = float(fx["gap"][first])
        out["allowed_margin"] = float(64 * n * EPS64 * fx["colmax"][first])
    return out


def read_traffic(path):
    """Per-launch DRAM traffic of the GEMM from a committed ncu summary, if any."""
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


def run_ours(args):
    import ctypes

    import torch

    from lair_gb300 import _lib

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    lib = _lib.load()
    ctx = _lib.context() if local == 0 else None
    if ctx is None:  # one context per process, on this process's GPU
        h = ctypes.c_void_p()
        _lib.check(lib.luhot_create(ctypes.byref(h), local))
        ctx = h
        _lib._ctx = ctx
    # One explicit stream for torch's copies and luhot's kernels (the legacy
    # default stream would not order against luhot's non-blocking stream).
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    _lib.check(lib.luhot_set_stream(ctx, ctypes.c_void_p(stream.cuda_stream)), ctx)
    mode = _lib.mode_id(args.mode)
    _lib.check(lib.luhot_set_fp64_update(ctx, _lib.FP64_UPDATES[args.fp64_update]), ctx)

    n, nrhs = args.n, args.nrhs
    lda = n
    fixture = load_parity_fixture(n, nrhs)
    if fixture is not None:
        # the seeded inputs of lair's reference results (parity key below)
        from lair_gb300 import synthetic

        a_h = synthetic.normal_matrix(int(fixture["seed_a"]), n, n)
        b_h = synthetic.normal_matrix(int(fixture["seed_b"]), n, nrhs)
        A0 = torch.from_numpy(a_h).cuda()
        B0 = torch.from_numpy(b_h).cuda()
        inputs_match = (synthetic.digest(a_h) == str(fixture["a_digest"])
                        and synthetic.digest(b_h) == str(fixture["b_digest"]))
        del a_h, b_h
    else:
        gen = torch.Generator(device="cuda").manual_seed(args.seed + rank)
        A0 = torch.randn((n, n), dtype=torch.float64, device="cuda", generator=gen)
        B0 = torch.randn((n, nrhs), dtype=torch.float64, device="cuda", generator=gen)
        inputs_match = False
    A = torch.empty_like(A0)
    X = torch.empty_like(B0)
    piv = torch.empty(n, dtype=torch.int32, device="cuda")
    sing = ctypes.c_int64(0)

    peak = _lib.dmma_peak_tflops()

    def step():
        A.copy_(A0)
        X.copy_(B0)
        _lib.check(lib.luhot_dgetrf_dev(ctx, n, n, A.data_ptr(), lda, piv.data_ptr(), ctypes.byref(sing), mode), ctx)
        _lib.check(lib.luhot_dgetrs_dev(ctx, n, nrhs, A.data_ptr(), lda, piv.data_ptr(), X.data_ptr(), nrhs, 0, mode), ctx)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    _lib.profile_enable(True)
    launches0 = lib.luhot_launch_count(ctx)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        barrier()
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        barrier()
    launches = lib.luhot_launch_count(ctx) - launches0
    prof = _lib.profile_read()
    _lib.profile_enable(False)
    ms = ev0.elapsed_time(ev1)
    t = torch.tensor([ms], dtype=torch.float64, device="cuda")
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    ms_max = float(t.item())
    value = world * args.steps * flops_of(n, nrhs) / (ms_max * 1e-3) / 1e9

    # e2e: equation::solve through the C ABI with host buffers every step, right
    # after the device-resident steps (same GPU state as the timed region)
    e2e = None
    if not args.no_e2e:
        A_h = A0.cpu().numpy()
        B_h = B0.cpu().numpy()
        X_h = np.empty_like(B_h)
        _lib.check(lib.luhot_set_stream(ctx, None), ctx)

        def e2e_step():
            rc = lib.luhot_dgesv(ctx, n, nrhs, A_h.ctypes.data, n, 1, B_h.ctypes.data, nrhs, 1,
                                 X_h.ctypes.data, nrhs, 1, mode)
            _lib.check(rc, ctx)

        for _ in range(max(1, min(args.warmup, 2))):
            e2e_step()
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        barrier()
        dt = time.perf_counter() - t0
        tt = torch.tensor([dt], dtype=torch.float64, device="cuda")
        if world > 1:
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        dt = float(tt.item())
        e2e = {"value": world * args.steps * flops_of(n, nrhs) / dt / 1e9, "unit": "GFLOP/s",
               "h2d_bytes_per_step": int(A_h.nbytes + B_h.nbytes), "d2h_bytes_per_step": int(X_h.nbytes),
               "api": "luhot_dgesv (host A, B in; host X out; pageable numpy buffers, page-locked by the call)",
               "ms_per_step": dt / args.steps * 1e3}
        _lib.check(lib.luhot_set_stream(ctx, ctypes.c_void_p(stream.cuda_stream)), ctx)

    # backward error of the last solve (FP64 on the GPU)
    R = B0 - A0 @ X
    berr = (R.abs().max() / (A0.abs().sum(1).max() * X.abs().max() + B0.abs().max())).item()
    del R
    parity = None
    if fixture is not None and mode == _lib.MODE_FAST:
        parity = parity_vs_lair(torch, n, fixture, A0, A, piv, X) if inputs_match else {
            "error": "inputs were not reproduced bit for bit; no comparison"}

    g = prof.get("gemm", {"ms": 0.0, "flops": 0.0, "bytes": 0.0, "launches": 0})
    gemm_tflops = g["flops"] / (g["ms"] * 1e-3) / 1e12 if g["ms"] else 0.0
    total_prof_ms = sum(v["ms"] for v in prof.values())
    share = g["ms"] / total_prof_ms if total_prof_ms else None
    overall = flops_of(n, nrhs) * args.steps / (ms_max * 1e-3) / 1e12
    sliced = args.fp64_update != "dmma" and prof.get("other", {}).get("launches", 0) > 0
    if sliced:
        # Every large update is 28 FP16 slice GEMMs of the same shape (the
        # few small trailing blocks on DMMA are a negligible share).
        tensor_peak = measured_peaks().get("bf16_tflops_sustained", 1700.0)
        executed = OZ_PRODUCTS * gemm_tflops
        c_gbs = g["bytes"] / (g["ms"] * 1e-3) / 1e9 if g["ms"] else 0.0
        roofline = {"bound": "tensor", "achieved": executed, "peak": tensor_peak, "unit": "TFLOP/s",
                    "frac": executed / tensor_peak,
                    "traffic": read_traffic(os.path.join(ROOT, "profiles", "oz_gemm_fp64_slices_n16384.md")),
                    "kernel": "oz_gemm_kernel (FP64 Schur update as 28 exact FP16 slice GEMMs, tcgen05 + TMA)",
                    "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (dense FP16 = BF16 rate; the "
                                   "kernel runs inside a seconds-long step)",
                    "achieved_is": "executed FP16 tensor work: 28 slice products x 2MNK per launch / event time",
                    "fp64_equivalent_tflops": gemm_tflops,
                    "fp64_equivalent_vs_dmma_peak": gemm_tflops / peak if peak else None,
                    "hbm": {"achieved_gbs": c_gbs, "peak_gbs": args.hbm_peak_gbs,
                            "frac": c_gbs / args.hbm_peak_gbs,
                            "bytes_are": "C read + written once per update, the slices read once"},
                    "per_launch_fp64_flops": g["flops"] / max(1, g["launches"]),
                    "launches": g["launches"], "share_of_step": share,
                    "split_ms": prof["other"]["ms"] / args.steps,
                    "overall_fp64_tflops": overall}
    else:
        traffic = read_traffic(os.path.join(ROOT, "profiles", "gemm_dmma_persistent_fp64_n16384.md"))
        roofline = {"bound": "tensor", "achieved": gemm_tflops, "peak": peak, "unit": "TFLOP/s",
                    "frac": gemm_tflops / peak if peak else None, "traffic": traffic,
                    "kernel": "gemm_dmma_persistent_kernel (FP64 Schur update, mma.sync m8n8k4)",
                    "peak_source": "FP64 DMMA throughput measured in this run (register-resident "
                                   "mma.sync m8n8k4 loop); MEASURED_PEAKS.json has no FP64 figure",
                    "per_launch_flops": g["flops"] / max(1, g["launches"]),
                    "launches": g["launches"], "share_of_step": share,
                    "overall_frac_of_peak": overall / peak if peak else None}

    engine_cmp = {"engine": args.fp64_update}
    if args.fp64_update != "dmma" and not args.no_dmma_step:
        # one step with the FP64-tensor-core engine, for comparison
        _lib.check(lib.luhot_set_fp64_update(ctx, _lib.UPDATE_DMMA), ctx)
        step()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        torch.cuda.synchronize()
        _lib.check(lib.luhot_set_fp64_update(ctx, _lib.FP64_UPDATES[args.fp64_update]), ctx)
        dmma_ms = e0.elapsed_time(e1)
        engine_cmp.update({"dmma_ms_per_step": dmma_ms, "speedup_vs_dmma": dmma_ms / (ms_max / args.steps),
                           "dmma_gflops": flops_of(n, nrhs) / (dmma_ms * 1e-3) / 1e9})
        step()  # leave the factors of the default engine for the legs below
        torch.cuda.synchronize()

    resident = None
    if not args.no_resident:
        resident = run_resident_solve(args, lib, ctx, torch, A0, A, piv, peak)

    ir = None
    if not args.no_ir:
        del A, A0, X
        torch.cuda.empty_cache()
        ir = run_ir(args, lib, ctx, torch, rank)

    batched_res = None
    if not args.no_batched:
        torch.cuda.empty_cache()
        batched_res = run_batched(args, lib, ctx, torch)

    adjoint_res = None
    if not args.no_adjoint:
        torch.cuda.empty_cache()
        adjoint_res = run_adjoint(args, lib, ctx, torch)

    qr_res = None
    if not args.no_qr:
        torch.cuda.empty_cache()
        qr_res = run_qr(args, lib, ctx, torch)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(n, nrhs, args.cpu_seconds, args.cpu_full_n)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": workload_config(args), "backward_error": berr, "berr_bound": n * EPS64,
                "berr_ok": berr <= n * EPS64, "parity": parity, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "clocks": clocks.summary(), "gpu_launches": int(launches),
                "kernel_profile_ms": {k: round(v["ms"], 3) for k, v in prof.items()}, "fp64_update": engine_cmp,
                "ir": ir,
                "resident_solve": resident, "batched": batched_res, "adjoint": adjoint_res, "qr": qr_res}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def orthogonal_factors(n, seed, torch):
    """Q1, Q2 from Householder QR of seeded N(0,1) matrices (FP32 QR on the
    GPU: the orthogonality error ~1e-6 perturbs the singular values only
    relatively, so kappa is kept) and b iid N(0,1)."""
    gen = torch.Generator(device="cuda").manual_seed(seed)
    g1 = torch.randn((n, n), device="cuda", generator=gen)
    g2 = torch.randn((n, n), device="cuda", generator=gen)
    try:
        q1, _ = torch.linalg.qr(g1)
        q2, _ = torch.linalg.qr(g2)
    except RuntimeError:
        # torch's GPU linear-algebra library cannot always be loaded (e.g.
        # under a profiler's injection); the same seeded matrices then go
        # through LAPACK on the host.
        q1 = torch.from_numpy(np.linalg.qr(g1.cpu().numpy())[0]).cuda()
        q2 = torch.from_numpy(np.linalg.qr(g2.cpu().numpy())[0]).cuda()
    del g1, g2
    b = torch.randn(n, dtype=torch.float64, device="cuda", generator=gen)
    return q1, q2, b


def conditioned_matrix(q1, q2, kappa, torch):
    """A = Q1 diag(sigma) Q2^T, sigma geometric 1 -> 1/kappa, formed in FP64."""
    n = q1.shape[0]
    sigma = torch.logspace(0, -float(np.log10(kappa)), n, dtype=torch.float64, device="cuda")
    return ((q1.double() * sigma) @ q2.double().T).contiguous()


def run_ir(args, lib, ctx, torch, rank):
    """Mixed-precision LU + refinement on the kappa-conditioned n x n system,
    against the plain FP64 LU on the same system."""
    import ctypes

    from lair_gb300 import _lib

    n = args.ir_n
    kappa = args.ir_kappa
    t0 = time.perf_counter()
    q1, q2, b = orthogonal_factors(n, 7 + rank, torch)
    A = conditioned_matrix(q1, q2, kappa, torch)
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    x = torch.empty_like(b)
    stream = torch.cuda.current_stream()

    def measure(A, prec, solver, reps, warmup):
        info = _lib.IrInfo()
        status = {"rc": 0}

        def solve():
            status["rc"] = lib.luhot_dgesv_ir_dev(ctx, n, 1, A.data_ptr(), n, b.data_ptr(), 1, x.data_ptr(), 1,
                                                  _lib.PRECISIONS[prec], _lib.SOLVERS[solver], 0.0, 50,
                                                  ctypes.byref(info))
            if status["rc"] not in (0, _lib.LUHOT_ERR_NOT_CONVERGED):
                _lib.check(status["rc"], ctx)

        for _ in range(warmup):
            solve()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            solve()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        R = b - A @ x
        berr = (R.abs().max() / (A.abs().sum(1).max() * x.abs().max() + b.abs().max())).item()
        return {"ms": ms, "gflops": flops_of(n, 1) / (ms * 1e-3) / 1e9, "iterations": info.iterations,
                "inner_iterations": info.inner_iterations, "backward_error": berr, "converged": status["rc"] == 0,
                "berr_ok": berr <= n * EPS64, "factor_ms": info.factor_ms, "refine_ms": info.refine_ms}

    results = {}
    for prec, solver in (tuple(r.split("/")) for r in args.ir_runs.split(",")):
        headline = solver == "ir"
        results[f"{prec}/{solver}"] = measure(A, prec, solver, args.steps if headline else 1,
                                              args.warmup if headline else 1)
    # the other condition numbers of the workload: same Q1, Q2 and b, one timed solve each
    sweep = {}
    if not args.no_ir_sweep:
        for kap in (1e2, 1e4):
            Ak = conditioned_matrix(q1, q2, kap, torch)
            runs = {}
            for prec, solver in (("bf16x3", "ir"), ("fp32", "ir"), ("tf32", "ir"), ("fp16", "ir"), ("bf16", "gmres"),
                                 ("tf32", "gmres")):
                r = measure(Ak, prec, solver, 1, 1)
                runs[f"{prec}/{solver}"] = {k: r[k] for k in ("ms", "iterations", "inner_iterations",
                                                              "backward_error", "converged", "factor_ms")}
            ok = [k for k in runs if runs[k]["converged"] and runs[k]["backward_error"] <= n * EPS64]
            sweep[f"{kap:g}"] = {"runs": runs, "best": min(ok, key=lambda k: runs[k]["ms"]) if ok else None}
            del Ak
    del q1, q2
    # plain FP64 LU on the same system, once
    Aw = A.clone()
    piv = torch.empty(n, dtype=torch.int32, device="cuda")
    xf = b.clone().reshape(n, 1)
    sing = ctypes.c_int64(0)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    _lib.check(lib.luhot_dgetrf_dev(ctx, n, n, Aw.data_ptr(), n, piv.data_ptr(), ctypes.byref(sing), 0), ctx)
    _lib.check(lib.luhot_dgetrs_dev(ctx, n, 1, Aw.data_ptr(), n, piv.data_ptr(), xf.data_ptr(), 1, 0, 0), ctx)
    e1.record(stream)
    torch.cuda.synchronize()
    fp64_ms = e0.elapsed_time(e1)
    R = b - A @ xf[:, 0]
    fp64_berr = (R.abs().max() / (A.abs().sum(1).max() * xf.abs().max() + b.abs().max())).item()
    best = min(results, key=lambda k: results[k]["ms"] if results[k]["berr_ok"] else float("inf"))
    return {"workload": f"kappa={kappa:g} system, n={n}, nrhs=1, A=Q1 diag(sigma) Q2^T, b iid N(0,1)",
            "precisions": "fp32: FP32 LU on CUDA cores; tf32/fp16/bf16: FP32 storage, tcgen05 Schur updates "
                          "(fp16/bf16 operands scaled per panel), FP32 accumulate; FP64 residual/update",
            "n": n, "kappa": kappa, "generation_s": gen_s, "runs": results,
            "fp64_lu_ms": fp64_ms, "fp64_lu_gflops": flops_of(n, 1) / (fp64_ms * 1e-3) / 1e9,
            "fp64_backward_error": fp64_berr, "best": best, "best_gflops": results[best]["gflops"],
            "speedup_vs_fp64": fp64_ms / results[best]["ms"], "berr_bound": n * EPS64,
            "kappa_sweep": sweep}


def run_resident_solve(args, lib, ctx, torch, A0, LU, piv, dmma_peak):
    """lair's Factorized::solve with the factors kept on the device: one
    right-hand side per call (luhot_dfactor_solve_dev), after a factor made
    once from A (luhot_dfactor_create_dev).  The first solve forms the
    block-scaled tiles; the next ones are timed one by one with CUDA events
    (median).  Beside it, the plain sweeps on the same factors
    (luhot_dgetrs_dev, one right-hand side).  Algorithmic bytes per solve:
    both triangles of the factor read once, 8 n^2."""
    import ctypes

    from lair_gb300 import _lib

    n = A0.shape[0]
    stream = torch.cuda.current_stream()
    h = ctypes.c_void_p()
    pv = np.zeros(n, dtype=np.uint64)
    sing = ctypes.c_int64(0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _lib.check(lib.luhot_dfactor_create_dev(ctx, n, n, A0.data_ptr(), n, 0, pv.ctypes.data, ctypes.byref(sing),
                                            ctypes.byref(h)), ctx)
    create_s = time.perf_counter() - t0
    gen = torch.Generator(device="cuda").manual_seed(77)
    b0 = torch.randn(n, dtype=torch.float64, device="cuda", generator=gen)
    xb = torch.empty_like(b0)

    def timed(fn, reps):
        ts = []
        for _ in range(reps):
            xb.copy_(b0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    def resident():
        _lib.check(lib.luhot_dfactor_solve_dev(h, 1, xb.data_ptr(), 1, 0), ctx)

    def plain():
        _lib.check(lib.luhot_dgetrs_dev(ctx, n, 1, LU.data_ptr(), n, piv.data_ptr(), xb.data_ptr(), 1, 0, 0), ctx)

    first_ms = timed(resident, 1)  # forms W
    ms = timed(resident, max(5, args.steps))
    x = xb.clone()
    berr = ((b0 - A0 @ x).abs().max() / (A0.abs().sum(1).max() * x.abs().max() + b0.abs().max())).item()
    plain_ms = timed(plain, max(5, args.steps))
    lib.luhot_factor_destroy(h)
    byts = 8.0 * n * n
    return {"workload": f"device-resident factors (Factorized::solve), n={n}, one right-hand side per call",
            "factor_create_s": create_s, "first_solve_ms_forms_scaled_tiles": first_ms,
            "ms_per_solve": ms, "ms_per_sweep": ms / 2, "backward_error": berr,
            "achieved_gbs": byts / (ms * 1e-3) / 1e9,
            "hbm_frac_of_measured": byts / (ms * 1e-3) / 1e9 / args.hbm_peak_gbs,
            "fp64_floor_ms": 2.0 * n * n / (dmma_peak * 1e12) * 1e3,
            "fp64_floor_note": "n^2 FMAs per solve at the measured FP64 peak: the arithmetic bound, above the HBM one",
            "plain_sweeps_ms_per_solve": plain_ms,
            "timing": "median of single solves, CUDA events; the factor exceeds L2"}


def run_adjoint(args, lib, ctx, torch):
    """Adjoint of the solve at n = 2048, nrhs = 8: A = N(0,1)/sqrt(n) + I,
    B and W iid N(0,1), X = A^-1 B by getrf + getrs.  Times the FP64 backward
    with the stored factors (lambda = A^-T W by the transposed sweeps,
    dB = lambda, dA = -lambda X^T), the same including its factorization, and
    the mixed-precision form (lambda by refinement on A^T, which factors A^T
    in the low precision).  L2 (129 MB) holds the whole problem, so it is
    flushed before every timed call (a 512 MB write); each call is timed
    alone with CUDA events."""
    import ctypes

    from lair_gb300 import _lib

    n, nrhs = args.adj_n, args.adj_nrhs
    gen = torch.Generator(device="cuda").manual_seed(23)
    A = torch.randn((n, n), dtype=torch.float64, device="cuda", generator=gen) / np.sqrt(n)
    A += torch.eye(n, dtype=torch.float64, device="cuda")
    B = torch.randn((n, nrhs), dtype=torch.float64, device="cuda", generator=gen)
    W = torch.randn((n, nrhs), dtype=torch.float64, device="cuda", generator=gen)
    LU = A.clone()
    piv = torch.empty(n, dtype=torch.int32, device="cuda")
    X = B.clone()
    dB = torch.empty_like(B)
    dA = torch.empty_like(A)
    flush = torch.empty(64 << 20, dtype=torch.float64, device="cuda")
    sing = ctypes.c_int64(0)
    stream = torch.cuda.current_stream()
    _lib.check(lib.luhot_dgetrf_dev(ctx, n, n, LU.data_ptr(), n, piv.data_ptr(), ctypes.byref(sing), 0), ctx)
    _lib.check(lib.luhot_dgetrs_dev(ctx, n, nrhs, LU.data_ptr(), n, piv.data_ptr(), X.data_ptr(), nrhs, 0, 0), ctx)

    def timed(fn, reps):
        ts = []
        for _ in range(reps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    def fp64_stored():
        _lib.check(lib.luhot_dgesv_backward_dev(ctx, n, nrhs, LU.data_ptr(), n, piv.data_ptr(), X.data_ptr(), nrhs,
                                                W.data_ptr(), nrhs, dB.data_ptr(), nrhs, dA.data_ptr(), n, 0), ctx)

    LU2 = torch.empty_like(A)

    def fp64_with_factor():
        LU2.copy_(A)
        _lib.check(lib.luhot_dgetrf_dev(ctx, n, n, LU2.data_ptr(), n, piv.data_ptr(), ctypes.byref(sing), 0), ctx)
        fp64_stored()

    info = _lib.IrInfo()
    dB_ir, dA_ir = torch.empty_like(B), torch.empty_like(A)

    def ir(prec):
        def run():
            rc = lib.luhot_dgesv_backward_ir_dev(ctx, n, nrhs, A.data_ptr(), n, X.data_ptr(), nrhs, W.data_ptr(), nrhs,
                                                 dB_ir.data_ptr(), nrhs, dA_ir.data_ptr(), n,
                                                 _lib.PRECISIONS[prec], _lib.REFINE_IR, 0.0, 50, ctypes.byref(info))
            _lib.check(rc, ctx)
        return run

    reps = max(3, args.steps)
    for f in (fp64_stored, fp64_with_factor):
        f()
    ms_stored = timed(fp64_stored, reps)
    ms_factor = timed(fp64_with_factor, reps)
    lam_ref = dB.clone()
    dA_ref = dA.clone()
    out_ir = {}
    for prec in ("fp32", "bf16x3"):
        ir(prec)()
        ms = timed(ir(prec), reps)
        out_ir[prec] = {"ms": ms, "iterations": info.iterations, "backward_error_of_lambda": info.backward_error,
                        "dA_rel_diff_vs_fp64": float((dA_ir - dA_ref).abs().max() / dA_ref.abs().max()),
                        "dB_rel_diff_vs_fp64": float((dB_ir - lam_ref).abs().max() / lam_ref.abs().max())}
    # algorithmic bytes of the backward with stored factors: both triangles of
    # the factor read once (8 n^2), dA written once (8 n^2), W, X, lambda/dB
    # moved a few times (about 6 * 8 n nrhs)
    byts = 16.0 * n * n + 48.0 * n * nrhs
    del flush, LU2
    return {"workload": f"adjoint of X = A^-1 B: n={n}, nrhs={nrhs}, A = N(0,1)/sqrt(n) + I, B, W iid N(0,1)",
            "fp64_stored_factors_ms": ms_stored, "fp64_stored_factors_gbs": byts / (ms_stored * 1e-3) / 1e9,
            "hbm_frac_of_measured": byts / (ms_stored * 1e-3) / 1e9 / args.hbm_peak_gbs,
            "algorithmic_bytes": byts, "fp64_with_getrf_ms": ms_factor, "ir": out_ir,
            "timing": "median of %d calls, L2 flushed before each" % reps}


def run_qr(args, lib, ctx, torch):
    """Householder QR (lair's geqrf, fast mode) of an n x n N(0,1) matrix on the
    device, with Q formed by the same reflector kernels to check ||A - QR|| and
    ||Q^T Q - I||; GFLOP/s = (4/3 n^3) / t of the factorization."""
    import ctypes

    from lair_gb300 import _lib

    n = args.qr_n
    gen = torch.Generator(device="cuda").manual_seed(5)
    A0 = torch.randn((n, n), dtype=torch.float64, device="cuda", generator=gen)
    A = torch.empty_like(A0)
    tau = torch.empty(n, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    times = []
    for rep in range(2):
        A.copy_(A0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        _lib.check(lib.luhot_dgeqrf_dev(ctx, n, n, A.data_ptr(), n, tau.data_ptr(), 0), ctx)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = min(times)
    qr_h, tau_h = A.cpu().numpy(), tau.cpu().numpy()
    q = np.empty((n, n))
    _lib.check(lib.luhot_dqr_q(ctx, n, n, qr_h.ctypes.data, n, 1, tau_h.ctypes.data, q.ctypes.data, n, 1, 0), ctx)
    qt = torch.from_numpy(q).cuda()
    r = torch.triu(A)
    resid = float((qt @ r - A0).abs().max() / A0.abs().max())
    orth = float((qt.T @ qt - torch.eye(n, dtype=torch.float64, device="cuda")).abs().max())
    del A, A0, qt, r
    return {"workload": f"Householder QR (geqrf, fast mode) of an n x n N(0,1) matrix, n={n}", "n": n,
            "ms": ms, "gflops": 4.0 / 3.0 * n ** 3 / (ms * 1e-3) / 1e9,
            "residual_max_rel": resid, "orthogonality_max": orth,
            "bound": "FP64 pipe and HBM at the ridge (level-2 Householder, 4/3 n^3 flops over ~8 n^3 bytes)"}


def run_batched(args, lib, ctx, torch):
    """10,000 uneven systems (n ~ U{8..256}, A iid U[-1,1] + n*I with prob. 1/2,
    one rhs iid U[-1,1]) in one graph-replayed persistent launch, FP64 and
    FP32, against looping the plain single-system kernels over a sample."""
    import ctypes

    from lair_gb300 import _lib, batched

    world, rank, _ = dist_env()
    out = {}
    for name, dt, tdt in (("f64", np.float64, torch.float64), ("f32", np.float32, torch.float32)):
        sizes_all, a_all, b_all = batched.synthetic_batch(args.batch_count, seed=11, dtype=dt)
        # one contiguous slice per rank, balanced by the sum of n^3; no collective
        s0, s1 = batched.shard_by_work(sizes_all, world)[rank]
        aoff_all = np.concatenate([[0], np.cumsum(sizes_all.astype(np.int64) ** 2)])
        boff_all = np.concatenate([[0], np.cumsum(sizes_all.astype(np.int64))])
        sizes = sizes_all[s0:s1]
        a0 = a_all[aoff_all[s0]:aoff_all[s1]]
        b0 = b_all[boff_all[s0]:boff_all[s1]]
        solver = batched.BatchSolver(sizes, dtype=dt, mode="fast")
        A0 = torch.from_numpy(a0).cuda()
        B0 = torch.from_numpy(b0).cuda()
        A, B = A0.clone(), B0.clone()
        piv = torch.zeros(int(sizes.sum()), dtype=torch.int32, device="cuda")
        info = torch.zeros(len(sizes), dtype=torch.int32, device="cuda")
        t0 = time.perf_counter()
        solver.autotune(A0.data_ptr(), B0.data_ptr())
        tune_s = time.perf_counter() - t0

        def step():
            A.copy_(A0)
            B.copy_(B0)
            solver.solve_device(A.data_ptr(), B.data_ptr(), piv.data_ptr(), info.data_ptr())

        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        stream = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        ms_all = ms
        if world > 1:
            tt = torch.tensor([ms], dtype=torch.float64, device="cuda")
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            ms_all = float(tt.item())
        # worst backward error over the batch (FP64 check on the host)
        x = B.cpu().numpy()
        worst, ao, bo = 0.0, 0, 0
        for n in sizes:
            M = a0[ao:ao + n * n].reshape(n, n).astype(np.float64)
            xx, bb = x[bo:bo + n].astype(np.float64), b0[bo:bo + n].astype(np.float64)
            worst = max(worst, np.abs(bb - M @ xx).max() / (np.abs(M).sum(1).max() * np.abs(xx).max() + np.abs(bb).max()))
            ao += int(n) * int(n)
            bo += int(n)
        # baseline: plain single-system getrf + getrs per system, on a sample
        rng = np.random.default_rng(5)
        sample = rng.choice(len(sizes), size=min(args.batch_loop_sample, len(sizes)), replace=False)
        aoff = np.concatenate([[0], np.cumsum(sizes.astype(np.int64) ** 2)])
        boff = np.concatenate([[0], np.cumsum(sizes.astype(np.int64))])
        pre = "d" if dt == np.float64 else "s"
        getrf, getrs = getattr(lib, f"luhot_{pre}getrf_dev"), getattr(lib, f"luhot_{pre}getrs_dev")
        A.copy_(A0)
        B.copy_(B0)
        torch.cuda.synchronize()
        sing = ctypes.c_int64(0)
        es = A.element_size()
        t0 = time.perf_counter()
        for i in sample:
            n = int(sizes[i])
            pa = A.data_ptr() + int(aoff[i]) * es
            pb = B.data_ptr() + int(boff[i]) * es
            pp = piv.data_ptr() + int(boff[i]) * 4
            _lib.check(getrf(ctx, n, n, pa, n, pp, ctypes.byref(sing), 0), ctx)
            _lib.check(getrs(ctx, n, 1, pa, n, pp, pb, 1, 0, 0), ctx)
        torch.cuda.synchronize()
        loop_s = time.perf_counter() - t0
        loop_rate = len(sample) / loop_s
        fl = float(np.sum(2.0 / 3.0 * sizes.astype(np.float64) ** 3 + 2.0 * sizes.astype(np.float64) ** 2))
        fl_all = float(np.sum(2.0 / 3.0 * sizes_all.astype(np.float64) ** 3 + 2.0 * sizes_all.astype(np.float64) ** 2))
        out[name] = {"systems": len(sizes_all), "systems_this_rank": len(sizes), "ranks": world,
                     "ms_per_batch": ms_all, "systems_per_s": len(sizes_all) / (ms_all * 1e-3),
                     "gflops": fl_all / (ms_all * 1e-3) / 1e9, "worst_backward_error_this_rank": worst,
                     "loop_single_system_systems_per_s": loop_rate,
                     "loop_sample": f"{len(sample)} systems drawn from the batch, getrf_dev + getrs_dev each",
                     "speedup_vs_loop": (len(sizes) / (ms * 1e-3)) / loop_rate, "autotune_s": tune_s,
                     "sharding": "contiguous slices balanced by sum n^3, one per rank, no collective; "
                                 "aggregate rate = all systems / slowest rank's time",
                     "tuning": solver.tuning()}
        del A0, B0, A, B
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=16384)
    ap.add_argument("--nrhs", type=int, default=16)
    ap.add_argument("--mode", choices=["fast", "exact"], default="fast")
    ap.add_argument("--fp64-update", choices=["auto", "dmma", "ozaki"], default="auto",
                    help="Schur-update engine of fast-mode FP64 getrf")
    ap.add_argument("--no-dmma-step", action="store_true", help="skip the one comparison step with DMMA")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--cpu-full-n", type=int, default=4096,
                    help="order of the complete CPU run beside the sample (0: skip)")
    ap.add_argument("--ref-elim-steps", type=int, default=4)
    ap.add_argument("--no-ir", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-qr", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-resident", action="store_true", help="skip the device-resident single-RHS solve leg")
    ap.add_argument("--adj-n", type=int, default=2048)
    ap.add_argument("--adj-nrhs", type=int, default=8)
    ap.add_argument("--hbm-peak-gbs", type=float, default=None,
                    help="HBM roofline (default: MEASURED_PEAKS.json, else 6800)")
    ap.add_argument("--qr-n", type=int, default=4096)
    ap.add_argument("--batch-count", type=int, default=10000)
    ap.add_argument("--batch-loop-sample", type=int, default=300)
    ap.add_argument("--ir-n", type=int, default=16384)
    ap.add_argument("--ir-kappa", type=float, default=1e6)
    ap.add_argument("--ir-runs", default="fp32/ir,bf16x3/ir,bf16x3/gmres,fp32/gmres,tf32/gmres,fp16/gmres,bf16/gmres",
                    help="precision/solver pairs of the refinement leg, comma separated")
    ap.add_argument("--no-ir-sweep", action="store_true",
                    help="skip the kappa = 1e2 and 1e4 runs of the refinement leg")
    args = ap.parse_args()
    world, rank, _ = dist_env()
    if args.gpus != world and rank == 0:
        print(f"bench: --gpus {args.gpus} but WORLD_SIZE={world}; measuring {world} rank(s)", file=sys.stderr)
    if args.hbm_peak_gbs is None:
        args.hbm_peak_gbs = measured_hbm_peak()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
