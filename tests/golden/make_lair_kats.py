"""Extract lair's own known-answer tests for the LU path into lair_kats.json.

lair (Rust) cannot be built in this environment, so its unit tests cannot be
run; their literal inputs and expected outputs are the golden vectors that pin
the oracle.  This script reads the test modules of lair's source tree as text,
pulls every numeric literal the tests assert on, and writes them to
``lair_kats.json`` beside this file.  Run it where the lair sources are
available:

    python tests/golden/make_lair_kats.py /path/to/lair

The JSON keeps, per test function: its source file and line, the ordered
list of ``arr2``/``arr1``/plain array literals, ``vec![..]`` literals,
``Some(..)`` literals, tolerances, the view transforms applied to the input
(``swap_axes``, ``invert_axis``) and the indexed assertions
(``assert_eq!(p[(i, j)], v)`` and ``assert_relative_eq!(l[(i, j)], v, ..)``).
The tests in ``tests/test_oracle_golden.py`` interpret each entry.
"""
from __future__ import annotations

import json
import os
import re
import sys

SOURCES = {
    "getrf": "src/lapack/getrf.rs",
    "getrs": "src/lapack/getrs.rs",
    "lu": "src/decomposition/lu.rs",
    "iamax": "src/blas/iamax.rs",
    # QR (the next factorization on the path: geqrf and its reflector helpers)
    "geqrf": "src/lapack/geqrf.rs",
    "qr": "src/decomposition/qr.rs",
    "larfg": "src/lapack/larfg.rs",
    "larf": "src/lapack/larf.rs",
    "nrm2": "src/blas/nrm2.rs",
}

_NUM = r"-?\d[\d_]*(?:\.[\d_]*)?(?:e-?\d+)?(?:_f64|_f32)?"


def _num(tok: str) -> float:
    tok = tok.replace("_f64", "").replace("_f32", "").replace("_", "")
    if tok.endswith("."):
        tok = tok[:-1]
    return float(tok)


def _match_bracket(s: str, start: int) -> int:
    """Index one past the bracket closing the one at s[start]."""
    depth = 0
    for i in range(start, len(s)):
        if s[i] == "[":
            depth += 1
        elif s[i] == "]":
            depth -= 1
            if depth == 0:
                return i + 1
    raise ValueError("unbalanced brackets")


def _parse_nested(text: str):
    """Parse a Rust nested array literal of numbers into nested lists."""
    text = text.strip()
    if text.startswith("["):
        inner = text[1:-1]
        items, depth, cur = [], 0, ""
        for ch in inner:
            if ch == "[":
                depth += 1
            elif ch == "]":
                depth -= 1
            if ch == "," and depth == 0:
                if cur.strip():
                    items.append(cur)
                cur = ""
            else:
                cur += ch
        if cur.strip():
            items.append(cur)
        return [_parse_nested(it) for it in items]
    return _num(text)


def _tests(path: str):
    src = open(path).read()
    lines = src.split("\n")
    tests_at = src.find("mod tests")
    out = {}
    for m in re.finditer(r"#\[test\]\s*fn (\w+)\(\)", src[tests_at:]):
        name = m.group(1)
        begin = tests_at + m.end()
        nxt = src.find("#[test]", begin)
        body = src[begin: nxt if nxt >= 0 else len(src)]
        line = src[: tests_at + m.start()].count("\n") + 1
        end_line = src[: begin + len(body)].count("\n")
        out[name] = (body, line, end_line, lines)
    return out


def _extract(body: str):
    arrays = []
    for m in re.finditer(r"(arr2|arr1|aview1)\(&\[|let \w+ = \[", body):
        start = m.end() - 1
        stop = _match_bracket(body, start)
        lit = body[start:stop]
        if "Complex64" in lit:
            continue
        arrays.append({"kind": m.group(1) or "array", "value": _parse_nested(lit)})
    vecs = [[int(_num(t)) for t in re.findall(_NUM, m.group(1))]
            for m in re.finditer(r"vec!\[([^\]]*)\]", body)]
    somes = [int(m.group(1)) for m in re.finditer(r"Some\((\d+)\)", body)]
    eps = [_num(m.group(1)) for m in re.finditer(r"epsilon = (" + _NUM + ")", body)]
    rels = [_num(m.group(1)) for m in re.finditer(r"max_relative = (" + _NUM + ")", body)]
    transforms = re.findall(r"\.(swap_axes\(0, 1\)|invert_axis\(Axis\(\d\)\))", body)
    indexed = []
    for m in re.finditer(
        r"assert_(eq|relative_eq|abs_diff_eq)!\(\s*(\w+)\[\((\d+), (\d+)\)\](?:\.(re|im))?,\s*(" + _NUM + r")",
        body,
    ):
        indexed.append({"macro": m.group(1), "var": m.group(2), "i": int(m.group(3)),
                        "j": int(m.group(4)), "part": m.group(5), "value": _num(m.group(6))})
    scalar = []
    for m in re.finditer(r"assert_(eq|relative_eq|abs_diff_eq)!\(\s*(\w+)\[(\d+)\],\s*(" + _NUM + r")", body):
        scalar.append({"macro": m.group(1), "var": m.group(2), "i": int(m.group(3)), "value": _num(m.group(4))})
    for m in re.finditer(r"assert_eq!\((idx|max), (" + _NUM + r")\)", body):
        scalar.append({"macro": "eq", "var": m.group(1), "i": None, "value": _num(m.group(2))})
    # scalar results compared whole: assert_eq!(beta, 2.), assert_abs_diff_eq!(tau, 1.2, ..)
    for m in re.finditer(r"assert_(eq|relative_eq|abs_diff_eq)!\(\s*(\w+),\s*(" + _NUM + r")\s*[,)]", body):
        if m.group(2) not in ("idx", "max"):
            scalar.append({"macro": m.group(1), "var": m.group(2), "i": None, "value": _num(m.group(3))})
    # literal arguments of the call under test, e.g. larfg(1., x) or left(&v, 2., &mut c)
    call_args = [[_num(t) for t in re.findall(r"(?<![\w.])" + _NUM, m.group(2))]
                 for m in re.finditer(r"super::(larfg|left|right)\(([^;]*)\);", body)]
    shapes = [[int(m.group(2)), int(m.group(3))]
              for m in re.finditer(r"assert_eq!\((\w+)\.shape\(\), &\[(\d+), (\d+)\]\)", body)]
    return {
        "arrays": arrays, "vecs": vecs, "somes": somes, "epsilon": eps, "max_relative": rels,
        "call_args": call_args,
        "transforms": transforms, "indexed": indexed, "scalar": scalar, "shapes": shapes,
        "singular_none": "singular.is_none()" in body, "empty_pivots": "Vec::<usize>::new()" in body,
    }


def _doc_test(path: str):
    """The `equation::solve` doc-test (src/equation.rs)."""
    src = open(path).read()
    a = re.search(r"let a = ndarray::arr2\(&(\[.*?\]\])\);", src).group(1)
    b = re.search(r"let b = ndarray::arr1\(&(\[.*?\])\);", src).group(1)
    x = re.search(r"ndarray::aview1\(&(\[.*?\])\)", src).group(1)
    line = src[: src.find("let a = ndarray::arr2")].count("\n") + 1
    return {"file": "src/equation.rs", "line": line, "a": _parse_nested(a), "b": _parse_nested(b),
            "x": _parse_nested(x)}


def main(root: str) -> None:
    kats = {"source": "lair 0.8.0 unit tests (read as text)", "tests": {}}
    for group, rel in SOURCES.items():
        for name, (body, line, end_line, _) in _tests(os.path.join(root, rel)).items():
            entry = _extract(body)
            entry.update({"file": rel, "line": line, "end_line": end_line, "group": group, "name": name})
            kats["tests"][f"{group}::{name}"] = entry
    kats["doctest_equation_solve"] = _doc_test(os.path.join(root, "src/equation.rs"))
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lair_kats.json")
    with open(out, "w") as f:
        json.dump(kats, f, indent=1, sort_keys=True)
    print(f"wrote {len(kats['tests'])} tests to {out}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_lair_kats.py /path/to/lair (the lair source tree)")
    main(sys.argv[1])
