"""ctypes binding of liblair_gb300.so (the luhot C ABI declared in include/luhot.h).

There is no CPU fallback: if the library is missing or no CUDA device can be
opened, every call raises.  ``load()`` only opens the shared object (works
without a GPU, so symbol checks run anywhere); ``context()`` additionally
creates the per-process luhot context on device 0 and needs a GPU.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblair_gb300.so")

LUHOT_OK = 0
LUHOT_ERR_INVALID_ARG = 1
LUHOT_ERR_CUDA = 2
LUHOT_ERR_ALLOC = 3
LUHOT_ERR_TIMEOUT = 4
LUHOT_ERR_NOT_CONVERGED = 5
LUHOT_ERR_SINGULAR = 6
LUHOT_ERR_UNSUPPORTED = 7

MODE_FAST = 0
MODE_EXACT = 1
MODES = {"fast": MODE_FAST, "exact": MODE_EXACT}

_i64 = ctypes.c_int64
_i32 = ctypes.c_int
_vp = ctypes.c_void_p
_dbl = ctypes.c_double

# name -> (restype, argtypes); mirrors include/luhot.h
SIGNATURES = {
    "luhot_version": (ctypes.c_char_p, []),
    "luhot_status_string": (ctypes.c_char_p, [_i32]),
    "luhot_create": (_i32, [ctypes.POINTER(_vp), _i32]),
    "luhot_destroy": (None, [_vp]),
    "luhot_last_error": (ctypes.c_char_p, [_vp]),
    "luhot_set_stream": (_i32, [_vp, _vp]),
    "luhot_set_block": (_i32, [_vp, _i32]),
    "luhot_launch_count": (_i64, [_vp]),
    "luhot_set_fp64_update": (_i32, [_vp, _i32]),
    "luhot_dschur_update_dev": (_i32, [_vp, _i64, _i64, _i64, _vp, _i64, _i32]),
    "luhot_selftest_wait_timeout": (_i32, [_vp, _i64]),
    "luhot_profile_enable": (_i32, [_vp, _i32]),
    "luhot_profile_read": (_i32, [_vp, _vp]),
    "luhot_measure_dmma_peak": (_i32, [_vp, ctypes.POINTER(_dbl)]),
    "luhot_dgetrf": (_i32, [_vp, _i64, _i64, _vp, _i64, _i64, _vp, _vp, _i32]),
    "luhot_sgetrf": (_i32, [_vp, _i64, _i64, _vp, _i64, _i64, _vp, _vp, _i32]),
    "luhot_dgetrs": (_i32, [_vp, _i64, _i64, _vp, _i64, _i64, _vp, _vp, _i64, _i64, _vp, _i64, _i64, _i32, _i32]),
    "luhot_sgetrs": (_i32, [_vp, _i64, _i64, _vp, _i64, _i64, _vp, _vp, _i64, _i64, _vp, _i64, _i64, _i32, _i32]),
    "luhot_dgesv": (_i32, [_vp, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _i32]),
    "luhot_dgetrf_dev": (_i32, [_vp, _i64, _i64, _vp, _i64, _vp, _vp, _i32]),
    "luhot_sgetrf_dev": (_i32, [_vp, _i64, _i64, _vp, _i64, _vp, _vp, _i32]),
    "luhot_dgetrs_dev": (_i32, [_vp, _i64, _i64, _vp, _i64, _vp, _vp, _i64, _i32, _i32]),
    "luhot_sgetrs_dev": (_i32, [_vp, _i64, _i64, _vp, _i64, _vp, _vp, _i64, _i32, _i32]),
    "luhot_dgesv_ir_dev": (_i32, [_vp, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _i32, _i32, _dbl, _i32, _vp]),
    "luhot_sgetrf_mixed_dev": (_i32, [_vp, _i64, _i64, _vp, _i64, _vp, _i32, _vp]),
    "luhot_dgesv_ir": (_i32, [_vp, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _i32, _i32, _dbl,
                              _i32, _vp]),
    "luhot_dgesv_backward": (_i32, [_vp, _i64, _i64, _vp, _i64, _i64, _vp, _vp, _i64, _i64, _vp, _i64, _i64, _vp,
                                    _i64, _i64, _vp, _i64, _i64, _i32]),
    "luhot_dgesv_backward_dev": (_i32, [_vp, _i64, _i64, _vp, _i64, _vp, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64,
                                        _i32]),
    "luhot_dgesv_backward_ir_dev": (_i32, [_vp, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64,
                                           _i32, _i32, _dbl, _i32, _vp]),
    "luhot_batch_create": (_i32, [_vp, _i64, _vp, _i32, _i32, ctypes.POINTER(_vp)]),
    "luhot_batch_destroy": (None, [_vp]),
    "luhot_batch_layout": (_i32, [_vp, _vp, _vp]),
    "luhot_batch_autotune": (_i32, [_vp, _vp, _vp]),
    "luhot_batch_tuning": (_i32, [_vp, _vp, _vp]),
    "luhot_batch_solve": (_i32, [_vp, _vp, _vp, _vp, _vp]),
    "luhot_batch_solve_host": (_i32, [_vp, _vp, _vp, _vp, _vp]),
    "luhot_dfactor_create": (_i32, [_vp, _i64, _i64, _vp, _i64, _i64, _i32, _vp, ctypes.POINTER(_i64),
                                    ctypes.POINTER(_vp)]),
    "luhot_sfactor_create": (_i32, [_vp, _i64, _i64, _vp, _i64, _i64, _i32, _vp, ctypes.POINTER(_i64),
                                    ctypes.POINTER(_vp)]),
    "luhot_dfactor_create_dev": (_i32, [_vp, _i64, _i64, _vp, _i64, _i32, _vp, ctypes.POINTER(_i64),
                                        ctypes.POINTER(_vp)]),
    "luhot_dfactor_solve": (_i32, [_vp, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _i32]),
    "luhot_sfactor_solve": (_i32, [_vp, _i64, _vp, _i64, _i64, _vp, _i64, _i64, _i32]),
    "luhot_dfactor_solve_dev": (_i32, [_vp, _i64, _vp, _i64, _i32]),
    "luhot_factor_read": (_i32, [_vp, _vp, _i64, _i64]),
    "luhot_factor_device": (_i32, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_i64), ctypes.POINTER(_vp)]),
    "luhot_factor_destroy": (None, [_vp]),
    "luhot_dgeqrf": (_i32, [_vp, _i64, _i64, _vp, _i64, _i64, _vp, _i32]),
    "luhot_sgeqrf": (_i32, [_vp, _i64, _i64, _vp, _i64, _i64, _vp, _i32]),
    "luhot_dgeqrf_dev": (_i32, [_vp, _i64, _i64, _vp, _i64, _vp, _i32]),
    "luhot_dqr_q": (_i32, [_vp, _i64, _i64, _vp, _i64, _i64, _vp, _vp, _i64, _i64, _i32]),
    "luhot_sqr_q": (_i32, [_vp, _i64, _i64, _vp, _i64, _i64, _vp, _vp, _i64, _i64, _i32]),
    "luhot_dgetrs_dev_noalloc": (_i32, [_i64, _i64, _vp, _i64, _vp, _vp, _i64, _i32, _i32, _vp]),
}

PROFILE_CLASSES = ("panel", "laswp", "trsm", "gemm", "trsv", "permute", "refine", "other")


class Profile(ctypes.Structure):
    """luhot_profile: per-class event time (ms), algorithmic flops/bytes, launches."""
    _fields_ = [("ms", _dbl * 8), ("flops", _dbl * 8), ("bytes", _dbl * 8), ("launches", _i64 * 8)]

    def as_dict(self):
        return {name: {"ms": self.ms[i], "flops": self.flops[i], "bytes": self.bytes[i],
                       "launches": int(self.launches[i])}
                for i, name in enumerate(PROFILE_CLASSES) if self.launches[i]}


UPDATE_AUTO, UPDATE_DMMA, UPDATE_OZAKI = 0, 1, 2
FP64_UPDATES = {"auto": UPDATE_AUTO, "dmma": UPDATE_DMMA, "ozaki": UPDATE_OZAKI}
PREC_FP32, PREC_BF16, PREC_FP16, PREC_TF32, PREC_BF16X3 = 0, 1, 2, 3, 4
PRECISIONS = {"fp32": PREC_FP32, "bf16": PREC_BF16, "fp16": PREC_FP16, "tf32": PREC_TF32, "bf16x3": PREC_BF16X3}
REFINE_IR, REFINE_GMRES = 0, 1
SOLVERS = {"ir": REFINE_IR, "gmres": REFINE_GMRES}


class IrInfo(ctypes.Structure):
    """luhot_ir_info"""
    _fields_ = [("iterations", _i32), ("inner_iterations", _i32), ("converged", _i32), ("precision", _i32),
                ("solver", _i32), ("backward_error", _dbl), ("factor_ms", _dbl), ("refine_ms", _dbl),
                ("singular", _i64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_lib = None
_ctx = None
_lock = threading.Lock()


class LuhotError(RuntimeError):
    """A luhot call returned a non-OK status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"luhot status {status}: {message}")
        self.status = status


def load():
    """Open the shared library (builds nothing; raises if it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "(there is no CPU fallback for the LU path)")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def context():
    """The process-wide luhot context on CUDA device 0 (created on first use)."""
    global _ctx
    with _lock:
        if _ctx is None:
            lib = load()
            handle = _vp()
            rc = lib.luhot_create(ctypes.byref(handle), 0)
            if rc != LUHOT_OK:
                raise LuhotError(rc, "luhot_create failed: " + lib.luhot_status_string(rc).decode()
                                 + " (a CUDA GPU is required; there is no CPU fallback)")
            _ctx = handle
        return _ctx


def check(rc: int, ctx=None) -> None:
    if rc != LUHOT_OK:
        lib = load()
        msg = lib.luhot_last_error(ctx).decode() if ctx is not None else ""
        raise LuhotError(rc, f"{lib.luhot_status_string(rc).decode()}: {msg}")


def launch_count() -> int:
    return int(load().luhot_launch_count(context()))


def profile_enable(on: bool = True) -> None:
    ctx = context()
    check(load().luhot_profile_enable(ctx, 1 if on else 0), ctx)


def profile_read() -> dict:
    ctx = context()
    prof = Profile()
    check(load().luhot_profile_read(ctx, ctypes.byref(prof)), ctx)
    return prof.as_dict()


def set_fp64_update(engine) -> None:
    """Schur-update engine of fast-mode FP64 getrf: "auto" (tensor-core FP64 by
    integer slices on large blocks, DMMA on small ones), "dmma" or "ozaki"."""
    ctx = context()
    eid = engine if isinstance(engine, int) else FP64_UPDATES[engine]
    check(load().luhot_set_fp64_update(ctx, eid), ctx)


def dmma_peak_tflops() -> float:
    ctx = context()
    v = _dbl(0.0)
    check(load().luhot_measure_dmma_peak(ctx, ctypes.byref(v)), ctx)
    return float(v.value)


def mode_id(mode) -> int:
    if isinstance(mode, int):
        return mode
    try:
        return MODES[mode]
    except KeyError:
        raise ValueError(f"mode must be one of {sorted(MODES)}, got {mode!r}") from None
