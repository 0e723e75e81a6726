"""The C ABI library loads and exports every symbol include/luhot.h declares (no GPU)."""
import os
import re

import pytest

from lair_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            text = open(os.path.join(ROOT, "include", f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(luhot_\w+)\s*\(", text))
    return names


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        from lair_gb300 import build

        build.build()
    return _lib.load()


def test_header_declares_core_entry_points():
    names = declared_functions()
    for must in ("luhot_dgetrf", "luhot_dgetrs", "luhot_dgesv", "luhot_create", "luhot_destroy",
                 "luhot_dgetrf_dev", "luhot_dgetrs_dev"):
        assert must in names


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_ctypes_table_matches_header():
    assert set(_lib.SIGNATURES) == declared_functions()


def declared_arity():
    """Number of parameters of every function include/*.h declares."""
    out = {}
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            text = open(os.path.join(ROOT, "include", f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            for name, params in re.findall(r"\b(luhot_\w+)\s*\(([^)]*)\)\s*;", text):
                params = params.strip()
                out[name] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_ctypes_argument_counts_match_header():
    arity = declared_arity()
    assert set(arity) == declared_functions()
    wrong = {n: (len(_lib.SIGNATURES[n][1]), arity[n]) for n in arity if len(_lib.SIGNATURES[n][1]) != arity[n]}
    assert not wrong, f"ctypes argument count differs from the header (ctypes, header): {wrong}"


def test_status_strings_without_gpu(lib):
    assert lib.luhot_status_string(0) == b"ok"
    assert lib.luhot_status_string(6) == b"matrix is singular"
    assert lib.luhot_version().startswith(b"0.")


def test_null_context_is_rejected_without_gpu(lib):
    assert lib.luhot_dgetrf(None, 2, 2, None, 2, 1, None, None, 0) == _lib.LUHOT_ERR_INVALID_ARG
    assert lib.luhot_last_error(None) == b"null context"
