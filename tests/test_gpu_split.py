"""The split scan (a select pass writing the surviving row numbers, then a
fold pass over them in full batches) against the oracle: the filtered
top-10 and all-groups forms, the global table, generic predicates with
NULLs, COUNT(DISTINCT) through the partitions, a WHERE that keeps nothing,
and zone-map pruning."""
import numpy as np
import pytest

from test_gpu_parity import C2_AGGS, FILTER, distinct_cols, filtered_cols, run_both
from thindb_gb300 import abi
from thindb_gb300.engine import AggSpec, Column, Pred, Request, SortSpec

pytestmark = pytest.mark.gpu
SPLIT = abi.FLAG_SPLIT_SCAN | abi.FLAG_GATHER_SCAN


def _assert_split(st):
    assert st.flags & abi.STAT_SPLIT, "the split scan did not run"


@pytest.mark.parametrize("extra", [0, abi.FLAG_FORCE_GLOBAL, abi.FLAG_NO_WARP_COMBINE])
def test_split_filtered_top10_and_all_groups(extra):
    cols = filtered_cols(2_000_000 + 77, 200_000)
    _, st = run_both(cols, Request(["k"], C2_AGGS, [SortSpec("s", True)], limit=10, where=FILTER,
                                   flags=SPLIT | extra))
    _assert_split(st)
    _, st = run_both(cols, Request(["k"], C2_AGGS, where=FILTER, flags=SPLIT | extra))
    _assert_split(st)


def test_split_generic_predicates_with_nulls():
    n = 1_500_000
    rng = np.random.default_rng(11)
    cols = [Column("k", abi.INT, rng.integers(0, 5_000, n).astype(np.int32), validity=rng.random(n) > 0.05),
            Column("a", abi.BIGINT, rng.integers(-10**9, 10**9, n).astype(np.int64), validity=rng.random(n) > 0.1),
            Column("b", abi.DOUBLE, rng.random(n)),
            Column("d", abi.DATE, rng.integers(19000, 19400, n).astype(np.int32))]
    where = [Pred("d", "between", 19100, 19250), Pred("b", "<", 0.4), Pred("a", "is_not_null")]
    req = Request(["k"], [AggSpec("count", None, "c"), AggSpec("sum", "a", "s"), AggSpec("max", "b", "mb"),
                          AggSpec("min", "a", "mn")], [SortSpec("c", True), SortSpec("k")], limit=50, where=where,
                  flags=SPLIT)
    _, st = run_both(cols, req)
    _assert_split(st)


def test_split_distinct_composite():
    cols = distinct_cols(1_000_000, 50_000)
    req = Request(["region", "url"], [AggSpec("count", None, "c"), AggSpec("count_distinct", "user_id", "u"),
                                      AggSpec("sum", "latency_ms", "lat")],
                  where=[Pred("latency_ms", "<", 300.0)], flags=SPLIT)
    _, st = run_both(cols, req)
    _assert_split(st)


def test_split_where_that_keeps_nothing():
    # a WHERE that keeps no row and that the zone maps cannot prune
    n = 300_000
    rng = np.random.default_rng(4)
    cols = [Column("k", abi.BIGINT, rng.integers(0, 1000, n).astype(np.int64)),
            Column("d", abi.DATE, (2 * rng.integers(0, 500, n)).astype(np.int32))]
    _, st = run_both(cols, Request(["k"], [AggSpec("count", None, "c")], where=[Pred("d", "=", 501)], flags=SPLIT))
    _assert_split(st)
    assert st.rows_selected == 0


def test_split_with_pruned_row_groups():
    n = 4_000_000
    rng = np.random.default_rng(6)
    d = np.sort(rng.integers(19000, 20000, n)).astype(np.int32)  # sorted: most row groups pruned
    cols = [Column("k", abi.BIGINT, rng.integers(0, 30_000, n).astype(np.int64)),
            Column("v", abi.INT, rng.integers(-1000, 1000, n).astype(np.int32)), Column("d", abi.DATE, d)]
    req = Request(["k"], [AggSpec("count", None, "c"), AggSpec("sum", "v", "s")],
                  where=[Pred("d", "between", 19400, 19450)], flags=SPLIT)
    _, st = run_both(cols, req)
    _assert_split(st)
    assert st.row_groups_pruned > 0


@pytest.mark.parametrize("col,op,lo,hi", [
    ("i", "between", -2**40, 2**40),          # clamped to the INT range: every row
    ("i", "between", -5, 5),
    ("i", "not_between", -1000, 1000),
    ("i", "between", 10, 5),                  # empty
    ("i", "not_between", 10, 5),              # every row
    ("i", "between", 2**31, 2**33),           # above every INT: no row
    ("i", ">", 2**31 - 10, 0),
    ("s", "between", -300, 300),
    ("t", "not_between", -3, 3),
    ("t", "=", -128, 0),
    ("b", "between", -2**63, -2**62),
    ("b", "<", 0, 0),
])
def test_split_range_tests_at_the_type_edges(col, op, lo, hi):
    n = 700_001
    rng = np.random.default_rng(12)
    i32 = rng.integers(-2**31, 2**31, n, dtype=np.int64).astype(np.int32)
    i32[:1000] = np.array([-2**31, 2**31 - 1, 0, -1, 1] * 200, dtype=np.int32)
    cols = [Column("k", abi.INT, rng.integers(0, 3_000, n).astype(np.int32)),
            Column("i", abi.INT, i32),
            Column("s", abi.SMALLINT, rng.integers(-2**15, 2**15, n).astype(np.int16)),
            Column("t", abi.TINYINT, rng.integers(-128, 128, n).astype(np.int8)),
            Column("b", abi.BIGINT, rng.integers(-2**63, 2**63 - 1, n, dtype=np.int64)),
            Column("v", abi.BIGINT, rng.integers(-10**6, 10**6, n).astype(np.int64))]
    req = Request(["k"], [AggSpec("count", None, "c"), AggSpec("sum", "v", "s")], where=[Pred(col, op, lo, hi)],
                  flags=SPLIT)
    _, st = run_both(cols, req)
    if st.rows_selected:
        _assert_split(st)
