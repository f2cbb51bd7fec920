"""Shared test plumbing: result dicts -> rows, comparisons, golden loading."""
from __future__ import annotations

import hashlib
import json
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if GOLDEN not in sys.path:
    sys.path.insert(0, GOLDEN)


def load_known_answers() -> dict:
    with open(os.path.join(GOLDEN, "known_answers.json")) as f:
        return json.load(f)


def to_rows(result: dict) -> list:
    """{name: (values, validity)} -> list of row lists (None = NULL, DECIMAL128 -> int)."""
    names = [k for k in result if not k.startswith("__")]
    cols = []
    n = None
    for k in names:
        vals, ok = result[k]
        if vals.ndim == 2:  # DECIMAL128 words
            pairs = vals.view(np.uint64)
            conv = []
            for lo, hi in pairs:
                v = (int(hi) << 64) | int(lo)
                if v >= 1 << 127:
                    v -= 1 << 128
                conv.append(v)
            col = conv
        elif vals.dtype.kind == "f":
            col = [float(x) for x in vals]
        else:
            col = [int(x) for x in vals]
        if ok is not None:
            col = [c if o else None for c, o in zip(col, ok)]
        cols.append(col)
        n = len(col)
    return [list(r) for r in zip(*cols)] if cols else []


def canon(v):
    return repr(v) if isinstance(v, float) else v


def rows_digest(rows) -> str:
    blob = json.dumps([[canon(x) for x in r] for r in rows], separators=(",", ":"))
    return hashlib.sha256(blob.encode()).hexdigest()


def _cell_eq(a, b, tol: float, rel: float) -> bool:
    if a is None or b is None:
        return a is None and b is None
    if isinstance(a, str):
        a = float(a)
    if isinstance(b, str):
        b = float(b)
    if isinstance(a, float) or isinstance(b, float):
        a, b = float(a), float(b)
        if math.isnan(a) or math.isnan(b):
            return math.isnan(a) and math.isnan(b)
        if a == b:
            return True
        return abs(a - b) <= max(tol, rel * max(abs(a), abs(b)))
    return a == b


def rows_equal(got: list, want: list, ordered: bool, n_keys: int, tol: float = 0.0, rel: float = 0.0) -> tuple:
    """Compare result rows; unordered rows are matched by their first n_keys cells."""
    if len(got) != len(want):
        return False, f"row count {len(got)} != {len(want)}"
    if not ordered:
        key = lambda r: tuple((x is None, x if x is not None else 0) for x in r[:n_keys])
        got = sorted(got, key=key)
        want = sorted(want, key=key)
    for i, (g, w) in enumerate(zip(got, want)):
        if len(g) != len(w):
            return False, f"row {i}: width {len(g)} != {len(w)}"
        for j, (a, b) in enumerate(zip(g, w)):
            if not _cell_eq(a, b, tol, rel):
                return False, f"row {i} col {j}: {a!r} != {b!r} (got {g}, want {w})"
    return True, ""


def check_known_answer(case, q, expected: dict, result: dict) -> None:
    rows = to_rows(result)
    n_keys = len(q.request.group_cols)
    if "expected_count" in expected:
        assert len(rows) == expected["expected_count"], (case.name, q.name, len(rows))
        # per-group counts of group_by_limit: c = g % 5 + 1
        if case.name == "group_by_limit":
            for r in rows:
                assert r[1] == r[0] % 5 + 1, (q.name, r)
            assert len({r[0] for r in rows}) == len(rows)
            if q.name == "having_c5":
                assert all(r[1] == 5 for r in rows)
        return
    if "digest" in expected:
        assert len(rows) == expected["rows"], (case.name, q.name, len(rows))
        if not expected["ordered"]:  # unordered fixtures are stored sorted by key
            rows = sorted(rows, key=lambda r: tuple((x is None, x if x is not None else 0) for x in r[:n_keys]))
        assert rows_digest(rows) == expected["digest"], (case.name, q.name, "digest mismatch")
        return
    ok, msg = rows_equal(rows, expected["expected"], expected["ordered"], n_keys, tol=expected["tol"])
    assert ok, f"{case.name}/{q.name}: {msg}"


def compare_results(got: dict, want: dict, n_keys: int, ordered: bool, rel: float = 0.0, tol: float = 0.0) -> None:
    g = to_rows(got)
    w = to_rows(want)
    ok, msg = rows_equal(g, w, ordered, n_keys, tol=tol, rel=rel)
    assert ok, msg
