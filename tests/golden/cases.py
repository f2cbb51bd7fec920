"""Known-answer GROUP BY cases restated from thinDB's own integration tests.

Each case rebuilds the reference test's input from the test's closed-form
formula and states the expected result the way the test computes it (plain
Python, independent of the oracle and of the CUDA engine).  make_golden.py
writes the expectations to known_answers.json; the tests regenerate the
inputs from these formulas and compare both the oracle and the engine with
the committed answers.

Reference tests (paths in the thinDB tree):
  decimal_sum_avg        tests/integration/decimal_test.zig:424-445
  decimal_grouped        tests/integration/decimal_test.zig:447-488
  bigint_wrap            tests/integration/aggregate_test.zig:1285-1302, :1358-1486
  nullable_aggs          tests/integration/v2_group_topn_test.zig:1283-1405
  filtered_compound      tests/integration/v2_group_topn_test.zig:65-151
  wide_keys              tests/integration/v2_group_topn_test.zig:3863-3912
  distinct_double        tests/integration/v2_group_topn_test.zig:1517-1700 (the DOUBLE / INT inputs)
  between                tests/integration/between_test.zig:13-60
  group_by_limit         tests/integration/group_by_limit_test.zig:20-140

Where the reference query has no GROUP BY (decimal_sum_avg) the restatement
groups by a constant column, which yields the same single row.
"""
from __future__ import annotations

import math
import struct
from dataclasses import dataclass, field
from typing import Any, Optional

import numpy as np

from thindb_gb300 import abi
from thindb_gb300.engine import AggSpec, Column, HavingSpec, Pred, Request, SortSpec

I64_MIN, I64_MAX = -(1 << 63), (1 << 63) - 1
I32_MIN, I32_MAX = -(1 << 31), (1 << 31) - 1


def wrap64(v: int) -> int:
    v &= (1 << 64) - 1
    return v - (1 << 64) if v >= 1 << 63 else v


@dataclass
class Query:
    name: str
    request: Request
    ordered: bool = False          # compare row order (ORDER BY), else as a set keyed by the group columns
    tol: float = 0.0               # absolute tolerance on DOUBLE columns
    expected: Optional[list] = None  # filled by expectations (rows as lists, None = NULL)
    expected_count: Optional[int] = None  # when only the row count / a property is pinned


@dataclass
class Case:
    name: str
    columns: list
    row_group_rows: int
    queries: list = field(default_factory=list)


# --------------------------------------------------------------- decimals --

def decimal_sum_avg() -> Case:
    # CREATE TABLE d (id INT, a DECIMAL(16,6), b DECIMAL(10,2), q INT);
    # rows (1, 2.5, 4.0, 3), (2, 10.0, 3.0, 7), (3, 1.234567, NULL, 2)
    cols = [
        Column("id", abi.INT, np.array([1, 2, 3], np.int32)),
        Column("a", abi.DECIMAL64, np.array([2_500_000, 10_000_000, 1_234_567], np.int64), scale=6, precision=16),
        Column("b", abi.DECIMAL64, np.array([400, 300, 0], np.int64), validity=np.array([1, 1, 0], bool),
               scale=2, precision=10),
        Column("q", abi.INT, np.array([3, 7, 2], np.int32)),
        Column("one", abi.INT, np.array([1, 1, 1], np.int32)),
    ]
    c = Case("decimal_sum_avg", cols, 65536)
    # SUM(a) -> DECIMAL128(38,6) = 13_734_567 ; AVG(a) = 4.578189 (abs 1e-6)
    c.queries.append(Query("sum_avg", Request(["one"], [AggSpec("sum", "a", "s"), AggSpec("avg", "a", "av")]),
                           tol=1e-6, expected=[[1, 13_734_567, 4.578189]]))
    # the nullable DECIMAL column: SUM(b) = 7.00 (700), AVG(b) = 3.5
    c.queries.append(Query("nullable_b", Request(["one"], [AggSpec("sum", "b", "sb"), AggSpec("avg", "b", "ab"),
                                                            AggSpec("count", "b", "cb")]),
                           tol=1e-12, expected=[[1, 700, 3.5, 2]]))
    return c


def decimal_grouped() -> Case:
    # CREATE TABLE g (id INT PRIMARY KEY, grp INT NOT NULL, v DECIMAL(12,4));
    # (1,1,1.5),(2,1,2.5),(3,1,3.0),(4,2,10.0),(5,2,20.0)
    cols = [
        Column("id", abi.INT, np.array([1, 2, 3, 4, 5], np.int32)),
        Column("grp", abi.INT, np.array([1, 1, 1, 2, 2], np.int32)),
        Column("v", abi.DECIMAL64, np.array([15000, 25000, 30000, 100000, 200000], np.int64),
               validity=np.ones(5, bool), scale=4, precision=12),
    ]
    c = Case("decimal_grouped", cols, 65536)
    c.queries.append(Query("sum", Request(["grp"], [AggSpec("sum", "v", "sv")], [SortSpec("grp")]), ordered=True,
                           expected=[[1, 70_000], [2, 300_000]]))
    c.queries.append(Query("avg", Request(["grp"], [AggSpec("avg", "v", "av")], [SortSpec("grp")]), ordered=True,
                           tol=1e-5, expected=[[1, 7.0 / 3.0], [2, 15.0]]))
    c.queries.append(Query("minmax", Request(["grp"], [AggSpec("min", "v", "mn"), AggSpec("max", "v", "mx")],
                                             [SortSpec("grp")]), ordered=True,
                           expected=[[1, 15000, 30000], [2, 100000, 200000]]))
    return c


# ------------------------------------------------------------ BIGINT wrap --

WRAP_FILLER_ROWS = 70_000
WRAP_G1 = 8553255926290448384
WRAP_G2 = -8446744073709551616
WRAP_G3 = 3
WRAP_TOTAL = 106_511_852_580_896_771  # aggregate_test.zig:1302: every non-NULL v, wrapped to BIGINT


def bigint_wrap() -> Case:
    head = [(1, 1, 1, 9_000_000_000_000_000_000), (2, 1, 1, 9_000_000_000_000_000_000),
            (3, 1, 1, 9_000_000_000_000_000_000), (4, 2, 2, 5_000_000_000_000_000_000),
            (5, 2, 2, 5_000_000_000_000_000_000), (6, 3, 3, 1), (7, 3, 3, 2), (8, 3, 3, None)]
    ids = [r[0] for r in head] + [100 + i for i in range(WRAP_FILLER_ROWS)]
    g = [r[1] for r in head] + [4] * WRAP_FILLER_ROWS
    hk = [r[2] for r in head] + [100 + i for i in range(WRAP_FILLER_ROWS)]
    v = [r[3] if r[3] is not None else 0 for r in head] + [0] * WRAP_FILLER_ROWS
    ok = [r[3] is not None for r in head] + [True] * WRAP_FILLER_ROWS
    # the values are BIGINT: 9e18 fits i64 (max 9.22e18)
    cols = [Column("id", abi.BIGINT, np.array(ids, np.int64)), Column("g", abi.INT, np.array(g, np.int32)),
            Column("hk", abi.INT, np.array(hk, np.int32)),
            Column("v", abi.BIGINT, np.array(v, np.int64), validity=np.array(ok, bool))]
    c = Case("bigint_wrap", cols, 4096)
    assert wrap64(3 * 9_000_000_000_000_000_000) == WRAP_G1
    assert wrap64(2 * 5_000_000_000_000_000_000) == WRAP_G2
    assert wrap64(3 * 9_000_000_000_000_000_000 + 2 * 5_000_000_000_000_000_000 + 1 + 2) == WRAP_TOTAL
    s = [AggSpec("sum", "v", "s")]
    # SELECT SUM(v) FROM w: the global aggregate (aggregate_test.zig:1392-1398)
    c.queries.append(Query("global_sum", Request([], s), ordered=True, expected=[[WRAP_TOTAL]]))
    c.queries.append(Query("by_g", Request(["g"], s, [SortSpec("g")]), ordered=True,
                           expected=[[1, WRAP_G1], [2, WRAP_G2], [3, WRAP_G3], [4, 0]]))
    c.queries.append(Query("by_g_top2", Request(["g"], s, [SortSpec("s", True)], limit=2), ordered=True,
                           expected=[[1, WRAP_G1], [3, WRAP_G3]]))
    c.queries.append(Query("by_g_having", Request(["g"], s, having=[HavingSpec("s", "<", 0)]),
                           expected=[[2, WRAP_G2]]))
    c.queries.append(Query("by_hk_top2", Request(["hk"], s, [SortSpec("s", True)], limit=2), ordered=True,
                           expected=[[1, WRAP_G1], [3, WRAP_G3]]))
    c.queries.append(Query("by_hk_having", Request(["hk"], s, having=[HavingSpec("s", "<", 0)]),
                           expected=[[2, WRAP_G2]]))
    c.queries.append(Query("by_hk_first3", Request(["hk"], s, [SortSpec("hk")], limit=3), ordered=True,
                           expected=[[1, WRAP_G1], [2, WRAP_G2], [3, WRAP_G3]]))
    return c


# ---------------------------------------------- nullable + BIGINT aggregates --

NA_GROUPS = 20_011


def nullable_aggs_rows():
    n = NA_GROUPS * 6
    i = np.arange(n, dtype=np.int64)
    g = (i // 2) % NA_GROUPS
    all_null = g == 0
    v_ok = ~(all_null | (i % 7 == 0))
    v = ((i * 37) % 1000 - 500).astype(np.int32)
    b_ok = ~(all_null | (i % 5 == 0))
    b = i * 3_000_000_019
    d_ok = ~(all_null | (i % 3 == 0))
    d = (((i * 13) % 512).astype(np.float64) - 256) * 0.25
    return i, g.astype(np.int32), v, v_ok, b, b_ok, d, d_ok


def nullable_aggs() -> Case:
    i, g, v, v_ok, b, b_ok, d, d_ok = nullable_aggs_rows()
    cols = [Column("id", abi.BIGINT, i), Column("g", abi.INT, g, validity=np.ones(len(i), bool)),
            Column("v", abi.INT, np.where(v_ok, v, 0).astype(np.int32), validity=v_ok),
            Column("b", abi.BIGINT, np.where(b_ok, b, 0), validity=b_ok),
            Column("d", abi.DOUBLE, np.where(d_ok, d, 0.0), validity=d_ok)]
    c = Case("nullable_aggs", cols, 65536)
    int_aggs = [AggSpec("sum", "id", "si"), AggSpec("count", None, "c"), AggSpec("sum", "v", "sv"),
                AggSpec("avg", "v", "av"), AggSpec("min", "v", "mnv"), AggSpec("max", "v", "mxv"),
                AggSpec("sum", "b", "sb")]
    float_aggs = [AggSpec("sum", "id", "si"), AggSpec("avg", "b", "ab"), AggSpec("sum", "d", "sd"),
                  AggSpec("min", "d", "mnd"), AggSpec("max", "d", "mxd")]
    for lim, off in ((10, 0), (25, 7), (NA_GROUPS, 0)):
        c.queries.append(Query(f"int_l{lim}_o{off}", Request(["g"], int_aggs, [SortSpec("si", True)], limit=lim,
                                                             offset=off), ordered=True))
        c.queries.append(Query(f"float_l{lim}_o{off}", Request(["g"], float_aggs, [SortSpec("si", True)], limit=lim,
                                                               offset=off), ordered=True))
    return c


def nullable_aggs_expected(q: Query) -> list:
    """The reference test's Expected struct (v2_group_topn_test.zig:1291-1337)."""
    i, g, v, v_ok, b, b_ok, d, d_ok = nullable_aggs_rows()
    G = NA_GROUPS
    id_sum = np.bincount(g, weights=None, minlength=G) * 0  # placeholder shape
    id_sum = [0] * G
    count = [0] * G
    v_sum = [0] * G
    v_n = [0] * G
    v_min = [None] * G
    v_max = [None] * G
    b_sum = [0] * G
    b_n = [0] * G
    d_sum = [0.0] * G
    d_min = [None] * G
    d_max = [None] * G
    for r in range(len(i)):
        k = int(g[r])
        id_sum[k] += int(i[r])
        count[k] += 1
        if v_ok[r]:
            x = int(v[r])
            v_sum[k] += x
            v_n[k] += 1
            v_min[k] = x if v_min[k] is None else min(v_min[k], x)
            v_max[k] = x if v_max[k] is None else max(v_max[k], x)
        if b_ok[r]:
            b_sum[k] += int(b[r])
            b_n[k] += 1
        if d_ok[r]:
            x = float(d[r])
            d_sum[k] += x
            d_min[k] = x if d_min[k] is None else min(d_min[k], x)
            d_max[k] = x if d_max[k] is None else max(d_max[k], x)
    # SUM(id) = 12g + const: ranking by si DESC is group_count-1-rank
    order = sorted(range(G), key=lambda k: -id_sum[k])
    lim, off = q.request.limit, q.request.offset
    rows = []
    for k in order[off:off + lim]:
        if q.name.startswith("int"):
            av = None if v_n[k] == 0 else float(v_sum[k]) / float(v_n[k])
            rows.append([k, id_sum[k], count[k], None if v_n[k] == 0 else v_sum[k], av, v_min[k], v_max[k],
                         None if b_n[k] == 0 else wrap64(b_sum[k])])
        else:
            ab = None if b_n[k] == 0 else float(b_sum[k]) / float(b_n[k])
            rows.append([k, id_sum[k], ab, None if d_min[k] is None else d_sum[k], d_min[k], d_max[k]])
    return rows


# ------------------------------------------------------ filtered compound --

FC_GROUPS = 10_037


def filtered_compound() -> Case:
    n = FC_GROUPS * 3
    i = np.arange(n, dtype=np.int64)
    key = i // 3
    cols = [Column("id", abi.BIGINT, i), Column("g0", abi.INT, (key // 101).astype(np.int32)),
            Column("g1", abi.INT, (key % 101).astype(np.int32)),
            Column("kept", abi.INT, (i % 3 != 2).astype(np.int32))]
    c = Case("filtered_compound", cols, 1024)
    cnt = [AggSpec("count", None, "c")]
    c.queries.append(Query("page", Request(["g0", "g1"], cnt, [SortSpec("c", True)], limit=10, offset=10000,
                                           where=[Pred("kept", "=", 1)]), ordered=True))
    c.queries.append(Query("no_rows", Request(["g0", "g1"], cnt, [SortSpec("c", True)], limit=10, offset=10000,
                                              where=[Pred("kept", "=", 7)]), ordered=True, expected=[]))
    c.queries.append(Query("past_end", Request(["g0", "g1"], cnt, [SortSpec("c", True)], limit=10, offset=20000,
                                               where=[Pred("kept", "=", 1)]), ordered=True, expected=[]))
    return c


def filtered_compound_expected(q: Query) -> list:
    # every group keeps 2 rows (c = 2); ties break on the packed key ascending:
    # g0 in bits 0-31, g1 in bits 32-63 (v2_shape_group_topn.zig:1327-1335)
    keys = [(k // 101, k % 101) for k in range(FC_GROUPS)]
    keys.sort(key=lambda t: (t[1] << 32) | t[0])
    page = keys[q.request.offset:q.request.offset + q.request.limit]
    return [[g0, g1, 2] for g0, g1 in page]


# -------------------------------------------------------------- wide keys --

def wide_keys() -> Case:
    n = 100_000
    a_vals = [I64_MIN, -1, 0, I64_MAX]
    b_vals = [I64_MIN, I64_MIN + (1 << 32), I64_MAX, I64_MAX - (1 << 32)]
    d_vals = [I32_MIN, -1, 1, I32_MAX]
    i = np.arange(n, dtype=np.int64)
    cols = [Column("id", abi.BIGINT, i), Column("a", abi.BIGINT, np.array(a_vals, np.int64)[i % 4]),
            Column("b", abi.BIGINT, np.array(b_vals, np.int64)[(i // 4) % 4]),
            Column("c", abi.INT, np.full(n, 7, np.int32)),
            Column("d", abi.INT, np.array(d_vals, np.int32)[(i // 4) % 4])]
    c = Case("wide_keys", cols, 65536)
    cnt = [AggSpec("count", None, "n")]
    c.queries.append(Query("ab", Request(["a", "b"], cnt)))
    c.queries.append(Query("ab_top", Request(["a", "b"], cnt, [SortSpec("n", True)], limit=100), ordered=True))
    c.queries.append(Query("acd", Request(["a", "c", "d"], cnt)))
    c.queries.append(Query("acd_sum", Request(["a", "c", "d"], cnt + [AggSpec("sum", "id", "s")])))
    return c


def wide_keys_expected(q: Query) -> list:
    n = 100_000
    a_vals = [I64_MIN, -1, 0, I64_MAX]
    b_vals = [I64_MIN, I64_MIN + (1 << 32), I64_MAX, I64_MAX - (1 << 32)]
    d_vals = [I32_MIN, -1, 1, I32_MAX]
    groups: dict = {}
    for r in range(n):
        a, bb, d = a_vals[r % 4], b_vals[(r // 4) % 4], d_vals[(r // 4) % 4]
        k = (a, bb) if q.name.startswith("ab") else (a, 7, d)
        e = groups.setdefault(k, [0, 0])
        e[0] += 1
        e[1] += r
    rows = []
    for k, (cnt, s) in groups.items():
        rows.append(list(k) + [cnt] + ([s] if q.name == "acd_sum" else []))
    if q.name == "ab_top":
        # every count ties (6250): the packed key (a in bits 0-63, b in 64-127) decides
        rows.sort(key=lambda r: ((r[1] & ((1 << 64) - 1)) << 64) | (r[0] & ((1 << 64) - 1)))
    return rows


# --------------------------------------------------------- distinct double --

GD_GROUPS = 1009


def distinct_double() -> Case:
    n = 3 * 3000  # the three flushed batches
    nan_a = struct.unpack("<d", struct.pack("<Q", 0x7FF8000000000001))[0]
    nan_b = struct.unpack("<d", struct.pack("<Q", 0xFFF8000000000000))[0]
    d_pool = [-0.0, 0.0, nan_a, nan_b, 1.5, -2.25, 1e300, -1e-300]
    g = np.zeros(n, np.int32)
    d = np.zeros(n, np.float64)
    d_ok = np.zeros(n, bool)
    v = np.zeros(n, np.int32)
    v_ok = np.zeros(n, bool)
    for i in range(n):
        gi = (i // 4) % GD_GROUPS if i % 2 == 0 else (i * 7) % GD_GROUPS
        g[i] = gi
        all_null = gi == 0
        if not (all_null or i % 13 == 0):
            d_ok[i] = True
            d[i] = d_pool[i % len(d_pool)] if i % 3 == 0 else float(i % 300) * 0.5
        if not (all_null or i % 11 == 0):
            v_ok[i] = True
            v[i] = (i * 37) % 200 - 100
    cols = [Column("id", abi.BIGINT, np.arange(n, dtype=np.int64)), Column("g", abi.INT, g),
            Column("d", abi.DOUBLE, d, validity=d_ok), Column("v", abi.INT, v, validity=v_ok)]
    c = Case("distinct_double", cols, 256)
    c.queries.append(Query("dd", Request(["g"], [AggSpec("count_distinct", "d", "dd"), AggSpec("count", None, "n"),
                                                 AggSpec("count_distinct", "v", "dv")])))
    return c


def canonical_double_bits(x: float) -> int:
    if math.isnan(x):
        return 0x7FF8000000000000
    if x == 0.0:
        x = 0.0
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def distinct_double_expected(case: Case) -> list:
    g = case.columns[1].data
    d, d_ok = case.columns[2].data, case.columns[2].validity
    v, v_ok = case.columns[3].data, case.columns[3].validity
    sets_d: dict = {}
    sets_v: dict = {}
    n_by: dict = {}
    for i in range(len(g)):
        k = int(g[i])
        n_by[k] = n_by.get(k, 0) + 1
        sets_d.setdefault(k, set())
        sets_v.setdefault(k, set())
        if d_ok[i]:
            sets_d[k].add(canonical_double_bits(float(d[i])))
        if v_ok[i]:
            sets_v[k].add(int(v[i]))
    return [[k, len(sets_d[k]), n_by[k], len(sets_v[k])] for k in sorted(n_by)]


# ---------------------------------------------------------------- BETWEEN --

def between() -> Case:
    cols = [Column("id", abi.BIGINT, np.array([1, 2, 3, 4, 5], np.int64)),
            Column("qty", abi.INT, np.array([5, 15, 25, 35, 45], np.int32))]
    c = Case("between", cols, 65536)
    cnt = [AggSpec("count", None, "c")]
    c.queries.append(Query("between", Request(["id"], cnt, [SortSpec("id")], where=[Pred("qty", "between", 15, 35)]),
                           ordered=True, expected=[[2, 1], [3, 1], [4, 1]]))
    c.queries.append(Query("not_between", Request(["id"], cnt, [SortSpec("id")],
                                                  where=[Pred("qty", "not_between", 15, 35)]),
                           ordered=True, expected=[[1, 1], [5, 1]]))
    c.queries.append(Query("between_and_id", Request(["id"], cnt, [SortSpec("id")],
                                                     where=[Pred("qty", "between", 10, 30), Pred("id", ">", 2)]),
                           ordered=True, expected=[[3, 1]]))
    return c


# ------------------------------------------------------- GROUP BY ... LIMIT --

def group_by_limit() -> Case:
    ids, gs = [], []
    rid = 1
    for grp in range(50):
        for _ in range(grp % 5 + 1):
            ids.append(rid)
            gs.append(grp)
            rid += 1
    cols = [Column("id", abi.BIGINT, np.array(ids, np.int64)), Column("g", abi.INT, np.array(gs, np.int32))]
    c = Case("group_by_limit", cols, 65536)
    cnt = [AggSpec("count", None, "c")]
    # without ORDER BY the page is unspecified in thinDB; the tests pin the
    # row count and per-group counts (the engine pages in packed-key order)
    c.queries.append(Query("limit10", Request(["g"], cnt, limit=10), expected_count=10))
    c.queries.append(Query("limit5_off7", Request(["g"], cnt, limit=5, offset=7), expected_count=5))
    c.queries.append(Query("limit1000", Request(["g"], cnt, limit=1000), expected_count=50))
    c.queries.append(Query("having_c5", Request(["g"], cnt, having=[HavingSpec("c", "=", 5)], limit=3),
                           expected_count=3))
    c.queries.append(Query("all", Request(["g"], cnt), expected=[[g, g % 5 + 1] for g in range(50)]))
    return c


# --------------------------------------------- exact grouped COUNT(DISTINCT) --

def combined_distinct() -> Case:
    """aggregate_test.zig:887-940 (per-group distinct counts; a value shared
    by two groups counts in both; NULLs never count; top-2 by the count) and
    :942-990 (COUNT, SUM and COUNT(DISTINCT) side by side).  The reference
    cuts 2-row row groups, which only changes its tiling."""
    rows = [(1, 1, 100), (2, 1, 100), (3, 1, 200), (4, 1, None), (5, 2, 100), (6, 2, 300), (7, 2, 300),
            (8, 3, None), (9, 3, None), (10, 4, 500)]
    cols = [Column("id", abi.BIGINT, np.array([r[0] for r in rows], np.int64)),
            Column("r", abi.INT, np.array([r[1] for r in rows], np.int32)),
            Column("u", abi.BIGINT, np.array([r[2] or 0 for r in rows], np.int64),
                   validity=np.array([r[2] is not None for r in rows], bool))]
    c = Case("combined_distinct", cols, 65536)
    cd = [AggSpec("count_distinct", "u", "u")]
    c.queries.append(Query("per_group", Request(["r"], cd), expected=[[1, 2], [2, 2], [3, 0], [4, 1]]))
    # ORDER BY u DESC LIMIT 2: the two count-2 groups, tie broken by the packed key
    c.queries.append(Query("top2", Request(["r"], cd, [SortSpec("u", True)], limit=2), ordered=True,
                           expected=[[1, 2], [2, 2]]))
    return c


def distinct_beside_aggs() -> Case:
    """aggregate_test.zig:942-990 (Q09 shape)."""
    cols = [Column("id", abi.BIGINT, np.array([1, 2, 3, 4], np.int64)),
            Column("r", abi.INT, np.array([1, 1, 1, 2], np.int32)),
            Column("u", abi.BIGINT, np.array([7, 7, 9, 5], np.int64), validity=np.ones(4, bool))]
    c = Case("distinct_beside_aggs", cols, 65536)
    aggs = [AggSpec("count", None, "c"), AggSpec("sum", "u", "s"), AggSpec("count_distinct", "u", "nd")]
    c.queries.append(Query("q09", Request(["r"], aggs), expected=[[1, 3, 23, 2], [2, 1, 5, 1]]))
    return c


def distinct_string_group() -> Case:
    """aggregate_test.zig:1003-1040: string groups (here packed dictionary
    ids: alpha 0, beta 1, gamma 2) over an int distinct; NULLs excluded."""
    codes = [0, 0, 0, 1, 1, 2]
    u = [1, 1, 2, 1, None, None]
    cols = [Column("id", abi.BIGINT, np.arange(1, 7, dtype=np.int64)),
            Column("s", abi.DICT32, np.array(codes, np.int32)),
            Column("u", abi.BIGINT, np.array([x or 0 for x in u], np.int64),
                   validity=np.array([x is not None for x in u], bool))]
    c = Case("distinct_string_group", cols, 65536)
    c.queries.append(Query("by_string", Request(["s"], [AggSpec("count_distinct", "u", "u")]),
                           expected=[[0, 2], [1, 1], [2, 0]]))
    return c


# ------------------------------------------------- global (no GROUP BY) --

def global_stats() -> Case:
    """count_star_stats_test.zig: the scan path of two global aggregates
    (:87-130 COUNT/MIN/MAX, :166-204 SUM/AVG/COUNT over a nullable INT and a
    DOUBLE); the rows its DELETEs remove are left out by a WHERE here."""
    ids = np.arange(600, dtype=np.int64)
    v_ok = ids % 3 != 0
    cols = [Column("id", abi.BIGINT, ids), Column("k", abi.BIGINT, 1000 - ids),
            Column("k2", abi.BIGINT, 2 * ids), Column("v", abi.INT, ids.astype(np.int32), validity=v_ok),
            Column("f", abi.DOUBLE, ids + 0.5)]
    c = Case("global_stats", cols, 65536)
    cmm = [AggSpec("count", None, "c"), AggSpec("min", "k", "mn"), AggSpec("max", "id", "mx")]
    # the first test's table holds ids 0..499
    c.queries.append(Query("count_min_max", Request([], cmm, where=[Pred("id", "between", 0, 499)]), ordered=True,
                           expected=[[500, 501, 499]]))
    # after DELETE ... WHERE id >= 499
    c.queries.append(Query("count_min_max_deleted", Request([], cmm, where=[Pred("id", "between", 0, 498)]),
                           ordered=True, expected=[[499, 502, 498]]))
    sac = [AggSpec("sum", "k2", "sk"), AggSpec("avg", "v", "av"), AggSpec("count", "v", "cv"), AggSpec("sum", "f", "sf")]
    # sum 2*id = 359400; v non-NULL on 400 rows summing 120000; sum (id + 0.5) = 180000
    c.queries.append(Query("sum_avg_count", Request([], sac, where=[Pred("id", ">=", 0)]), ordered=True,
                           expected=[[359400, 300.0, 400, 180000.0]]))
    # after DELETE ... WHERE id < 9
    c.queries.append(Query("sum_avg_count_deleted", Request([], sac, where=[Pred("id", ">=", 9)]), ordered=True,
                           expected=[[359400 - 72, (120000.0 - 27.0) / 394.0, 394, 180000.0 - 40.5]]))
    return c


ALL_CASES = [decimal_sum_avg, decimal_grouped, bigint_wrap, nullable_aggs, filtered_compound, wide_keys,
             distinct_double, between, group_by_limit, global_stats, combined_distinct, distinct_beside_aggs,
             distinct_string_group]


def build_case(fn) -> Case:
    c = fn()
    for q in c.queries:
        if q.expected is None and q.expected_count is None:
            if c.name == "nullable_aggs":
                q.expected = nullable_aggs_expected(q)
            elif c.name == "filtered_compound":
                q.expected = filtered_compound_expected(q)
            elif c.name == "wide_keys":
                q.expected = wide_keys_expected(q)
            elif c.name == "distinct_double":
                q.expected = distinct_double_expected(c)
    return c
