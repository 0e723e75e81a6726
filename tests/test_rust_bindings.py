"""The Rust bindings (rust/lair-gb300-sys/src/lib.rs) match include/luhot.h.

No machine of this project has cargo, so the crate is not compiled here;
this CPU test keeps it in step with the C header instead: every function the
header declares is declared in the crate with the same number of parameters,
and every numeric constant has the same value.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header():
    text = open(os.path.join(ROOT, "include", "luhot.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    funcs = {}
    for name, params in re.findall(r"\b(luhot_\w+)\s*\(([^)]*)\)\s*;", text):
        params = params.strip()
        funcs[name] = 0 if params in ("", "void") else params.count(",") + 1
    consts = {k: int(v) for k, v in re.findall(r"#define (LUHOT_\w+) (\d+)\b", text)}
    return funcs, consts


def rust():
    text = open(os.path.join(ROOT, "rust", "lair-gb300-sys", "src", "lib.rs")).read()
    text = re.sub(r"//[^\n]*", "", text)
    funcs = {}
    for name, params in re.findall(r"pub fn (luhot_\w+)\s*\(([^)]*)\)", text, flags=re.S):
        params = params.strip().rstrip(",")
        funcs[name] = 0 if not params else params.count(",") + 1
    consts = {k: int(v) for k, v in re.findall(r"pub const (LUHOT_\w+): c_int = (\d+);", text)}
    return funcs, consts


def test_every_header_function_is_bound_with_the_same_arity():
    hf, _ = header()
    rf, _ = rust()
    assert set(rf) == set(hf), (set(hf) - set(rf), set(rf) - set(hf))
    wrong = {n: (rf[n], hf[n]) for n in hf if rf[n] != hf[n]}
    assert not wrong, f"parameter counts differ (rust, header): {wrong}"


def test_constants_match():
    _, hc = header()
    _, rc = rust()
    assert rc == hc
