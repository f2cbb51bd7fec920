"""CUDA engine parity: the reference's known answers and the oracle, bit-exact
for integers/DECIMAL, FP64 sums within 1e-12 relative (the summation order
differs from the oracle's)."""
import numpy as np
import pytest

import cases
import oracle
from helpers import check_known_answer, compare_results, load_known_answers, to_rows
from thindb_gb300 import abi, datagen
from thindb_gb300.engine import (AggSpec, Column, MemoryBudgetExceeded, Pred, QueryCancelled, Request, SortSpec,
                                 HavingSpec, Table, try_build_group_topn)

pytestmark = pytest.mark.gpu
KNOWN = load_known_answers()
FP64_REL = 1e-12


def run_gpu(cols, req, rg=65536, **kw):
    t = Table(cols, row_group_rows=rg, **kw)
    q = try_build_group_topn(t, req)
    assert q is not None, "declined"
    res = q.collect()
    st = q.stats()
    q.close()
    t.close()
    return res, st


def run_both(cols, req, rg=65536, ordered=None, rel=FP64_REL, **kw):
    got, st = run_gpu(cols, req, rg, **kw)
    want = oracle.run(oracle.HostTable(cols, rg), req, threads=1)
    if ordered is None:
        ordered = bool(req.order_specs) or req.limit is not None
    compare_results(got, want, len(req.group_cols), ordered, rel=rel)
    assert st.groups == want["__groups__"], (st.groups, want["__groups__"])
    assert st.rows_selected == want["__selected__"]
    return got, st


# ------------------------------------------------------------ known answers --

@pytest.mark.parametrize("case_fn", cases.ALL_CASES, ids=[f.__name__ for f in cases.ALL_CASES])
@pytest.mark.parametrize("flags", [0, abi.FLAG_FORCE_GLOBAL | abi.FLAG_NO_WARP_COMBINE])
def test_engine_known_answers(case_fn, flags):
    c = case_fn()
    t = Table(c.columns, row_group_rows=c.row_group_rows)
    for q in c.queries:
        q.request.flags = flags
        qq = try_build_group_topn(t, q.request)
        assert qq is not None, q.name
        check_known_answer(c, q, KNOWN[c.name][q.name], qq.collect())
        qq.close()
    t.close()


# -------------------------------------------------------- workload shapes --

def plain_cols(n):
    d = datagen.plain(n, seed=7)
    return [Column("k", abi.BIGINT, d["k"]), Column("v", abi.INT, d["v"])]


@pytest.mark.parametrize("flags", [0, abi.FLAG_FORCE_GLOBAL, abi.FLAG_NO_WARP_COMBINE,
                                   abi.FLAG_FORCE_GLOBAL | abi.FLAG_NO_WARP_COMBINE])
def test_plain_lowcard(flags):
    cols = plain_cols(1 << 20)
    req = Request(["k"], [AggSpec("count", None, "c"), AggSpec("sum", "v", "s"), AggSpec("min", "v", "mn"),
                          AggSpec("max", "v", "mx")], flags=flags)
    _, st = run_both(cols, req)
    assert st.groups == 1024
    assert st.route == (2 if flags & abi.FLAG_FORCE_GLOBAL else 1)


def filtered_cols(n, n_keys):
    d = datagen.filtered(n, seed=5, n_keys=n_keys)
    return [Column("k", abi.BIGINT, d["k"]), Column("amount", abi.DECIMAL64, d["amount"], scale=2, precision=18),
            Column("d", abi.DATE, d["d"])]


FILTER = [Pred("d", "between", datagen.FILTER_LO, datagen.FILTER_HI)]
C2_AGGS = [AggSpec("count", None, "c"), AggSpec("sum", "amount", "s"), AggSpec("avg", "amount", "a")]


@pytest.mark.parametrize("flags", [0, abi.FLAG_DENSE_SCAN, abi.FLAG_GATHER_SCAN, abi.FLAG_NO_WARP_COMBINE,
                                   abi.FLAG_FORCE_GLOBAL])
def test_filtered_top10(flags):
    cols = filtered_cols(2_000_000, 200_000)
    req = Request(["k"], C2_AGGS, [SortSpec("s", True)], limit=10, where=FILTER, flags=flags)
    got, st = run_both(cols, req)
    assert st.result_rows == 10
    # the sum is DECIMAL(38,2) and AVG is f64(sum)/count/100, bit-exact
    assert got["s"][0].shape == (10, 2)


def test_filtered_all_groups():
    cols = filtered_cols(1_000_000, 100_000)
    req = Request(["k"], C2_AGGS, where=FILTER)
    got, st = run_both(cols, req)
    assert st.route == 2


def test_filtered_sorted_page():
    cols = filtered_cols(1_000_000, 50_000)
    req = Request(["k"], C2_AGGS, [SortSpec("a", False), SortSpec("c", True)], limit=500, offset=1234, where=FILTER)
    run_both(cols, req)


def distinct_cols(n, n_users):
    d = datagen.distinct(n, seed=9, n_users=n_users)
    return [Column("region", abi.SMALLINT, d["region"]), Column("url", abi.DICT32, d["url"]),
            Column("user_id", abi.BIGINT, d["user_id"]), Column("latency_ms", abi.DOUBLE, d["latency_ms"])]


def test_distinct_composite():
    cols = distinct_cols(1_000_000, 50_000)
    req = Request(["region", "url"], [AggSpec("count", None, "c"), AggSpec("count_distinct", "user_id", "u"),
                                      AggSpec("sum", "latency_ms", "lat")])
    got, st = run_both(cols, req)
    assert st.groups > 100_000


def test_composite_key_sized_by_its_own_sketch():
    """url codes belong to one region: the product of the parts' NDVs (64 x
    50,000) overestimates the groups 8x; the composite key's own sketch
    sizes the table near the real count."""
    cols = distinct_cols(1_000_000, 50_000)
    req = Request(["region", "url"], [AggSpec("count", None, "c"), AggSpec("sum", "latency_ms", "lat")])
    _, st = run_both(cols, req)
    assert st.groups > 300_000
    assert st.table_capacity <= 4 * st.groups  # product-sized: next_pow2(2 x 1.25M rows) = 4M
    _, st0 = run_gpu(cols, req, compute_ndv=False)  # no sketches: the column domains bound it
    assert st0.groups == st.groups


def test_distinct_rerun_epochs():
    """The distinct set is reused across executions (epoch tags): results repeat."""
    cols = distinct_cols(300_000, 20_000)
    req = Request(["region"], [AggSpec("count_distinct", "user_id", "u"), AggSpec("count", None, "c")],
                  [SortSpec("region")])
    t = Table(cols)
    q = try_build_group_topn(t, req)
    first = to_rows(q.collect())
    for _ in range(3):
        q.execute()
        assert to_rows(q.collect()) == first
    q.close()
    want = oracle.run(oracle.HostTable(cols), req)
    assert to_rows(want) == first


# ------------------------------------------------------------- semantics --

def mixed_cols(n, seed=3):
    rng = np.random.default_rng(seed)
    k1 = rng.integers(-3, 4, n).astype(np.int8)
    k2 = rng.integers(-200, 200, n).astype(np.int16)
    k1_ok = rng.random(n) > 0.1
    f = rng.normal(0, 100, n).astype(np.float32)
    f_ok = rng.random(n) > 0.2
    big = rng.integers(-(1 << 62), 1 << 62, n).astype(np.int64)
    big_ok = rng.random(n) > 0.3
    dt = rng.integers(18000, 21000, n).astype(np.int32)
    b = (rng.random(n) > 0.5).astype(np.uint8)
    dbl = rng.normal(0, 1e6, n)
    return [Column("k1", abi.TINYINT, k1, validity=k1_ok), Column("k2", abi.SMALLINT, k2),
            Column("f", abi.FLOAT, f, validity=f_ok), Column("big", abi.BIGINT, big, validity=big_ok),
            Column("dt", abi.DATE, dt), Column("b", abi.BOOLEAN, b), Column("dbl", abi.DOUBLE, dbl)]


def test_mixed_types_nulls():
    cols = mixed_cols(300_000)
    # 15 of thinDB's 16 state slots (an 18-slot request declines, test_declines_like_reference)
    aggs = [AggSpec("count", None, "c"), AggSpec("count", "f", "cf"), AggSpec("sum", "big", "sb"),
            AggSpec("min", "f", "mnf"), AggSpec("max", "f", "mxf"),
            AggSpec("min", "dt", "mnd"), AggSpec("max", "big", "mxb"), AggSpec("sum", "f", "sf"),
            AggSpec("sum", "b", "sbool"), AggSpec("count_distinct", "k2", "dk2")]
    req = Request(["k1", "b"], aggs)
    run_both(cols, req, rel=1e-9)  # float32 inputs summed in f64: 1e-9 covers reordering


def test_wide_key_and_nullable_order():
    cols = mixed_cols(200_000, seed=11)
    req = Request(["big", "k1", "k2"], [AggSpec("count", None, "c"), AggSpec("max", "dbl", "m")],
                  [SortSpec("k1", True), SortSpec("m")], limit=700, offset=3)
    run_both(cols, req)


def test_order_by_key_desc_nulls_and_having():
    cols = mixed_cols(200_000, seed=5)
    req = Request(["k1"], [AggSpec("sum", "big", "s"), AggSpec("count", None, "c"), AggSpec("avg", "f", "af")],
                  [SortSpec("k1", True)], having=[HavingSpec("c", ">", 10)])
    run_both(cols, req, rel=1e-9)


def test_empty_and_all_filtered():
    cols = plain_cols(100_000)
    req = Request(["k"], [AggSpec("count", None, "c")], where=[Pred("v", ">", 10_000_000)])
    got, st = run_both(cols, req)
    assert st.result_rows == 0 and st.groups == 0
    empty = [Column("k", abi.BIGINT, np.zeros(0, np.int64)), Column("v", abi.INT, np.zeros(0, np.int32))]
    got, st = run_gpu(empty, Request(["k"], [AggSpec("count", None, "c")]))
    assert st.result_rows == 0


def test_zone_map_pruning():
    n = 1 << 20
    d = np.sort(np.random.default_rng(1).integers(0, 1000, n)).astype(np.int32)
    k = (np.arange(n) % 777).astype(np.int64)
    cols = [Column("k", abi.BIGINT, k), Column("d", abi.DATE, d)]
    req = Request(["k"], [AggSpec("count", None, "c"), AggSpec("max", "d", "md")], where=[Pred("d", "between", 300, 320)])
    got, st = run_both(cols, req)
    assert st.row_groups_pruned > 0


def test_regrow_when_estimate_too_small():
    cols = filtered_cols(500_000, 100_000)
    req = Request(["k"], C2_AGGS, expected_groups=16, flags=abi.FLAG_FORCE_GLOBAL)
    got, st = run_both(cols, req)
    assert st.retries >= 1


def test_memory_budget_and_cancel():
    cols = plain_cols(100_000)
    t = Table(cols)
    with pytest.raises(MemoryBudgetExceeded):
        try_build_group_topn(t, Request(["k"], [AggSpec("count", None, "c")], memory_budget=1024))
    q = try_build_group_topn(t, Request(["k"], [AggSpec("count", None, "c")]))
    q.cancel()
    with pytest.raises(QueryCancelled):
        q.next()
    q.close()
    t.close()


def test_declines_like_reference():
    cols = mixed_cols(1000)
    t = Table(cols)
    assert try_build_group_topn(t, Request(["dbl"], [AggSpec("count", None, "c")])) is None  # float key
    assert try_build_group_topn(t, Request(["dt"], [AggSpec("sum", "dt", "s")])) is None  # SUM(DATE)
    many = [AggSpec("sum", "big", f"s{i}") for i in range(9)]  # 9 x (2 + valid) slots > 16
    assert try_build_group_topn(t, Request(["k2"], many)) is None
    t.close()


def test_device_resident_columns():
    torch = pytest.importorskip("torch")
    d = datagen.filtered(300_000, seed=4, n_keys=30_000)
    host = [Column("k", abi.BIGINT, d["k"]), Column("amount", abi.DECIMAL64, d["amount"], scale=2),
            Column("d", abi.DATE, d["d"])]
    dev = [Column(c.name, c.type, torch.from_numpy(c.data).cuda(), scale=c.scale) for c in host]
    req = Request(["k"], C2_AGGS, [SortSpec("s", True)], limit=10, where=FILTER)
    got, _ = run_gpu(dev, req, location="device")
    want = oracle.run(oracle.HostTable(host), req)
    compare_results(got, want, 1, True)


# ------------------------------------------------------------- staged scan --
# The staged scan (tiles of every column through a shared-memory ring of bulk
# copies) runs by default only from 4M rows; these force it on small tables
# whose last tile is partial (the plain-copy tail) and compare with the oracle.

STAGED = abi.FLAG_STAGED_SCAN


def _assert_staged(st):
    assert st.flags & abi.STAT_STAGED, "the staged scan did not run"


def test_staged_filtered_top10_and_all_groups():
    cols = filtered_cols(2_000_000, 200_000)  # 2,000,000 = 1953 tiles of 1024 + 128 rows
    _, st = run_both(cols, Request(["k"], C2_AGGS, [SortSpec("s", True)], limit=10, where=FILTER, flags=STAGED))
    _assert_staged(st)
    _, st = run_both(cols, Request(["k"], C2_AGGS, where=FILTER, flags=STAGED))
    _assert_staged(st)
    _, st = run_both(cols, Request(["k"], C2_AGGS, where=FILTER, flags=STAGED | abi.FLAG_FORCE_GLOBAL |
                                   abi.FLAG_NO_WARP_COMBINE))
    _assert_staged(st)


@pytest.mark.parametrize("flags", [STAGED, STAGED | abi.FLAG_FORCE_GLOBAL])
def test_staged_plain_lowcard(flags):
    cols = plain_cols((1 << 20) + 333)
    req = Request(["k"], [AggSpec("count", None, "c"), AggSpec("sum", "v", "s"), AggSpec("min", "v", "mn"),
                          AggSpec("max", "v", "mx")], flags=flags)
    _, st = run_both(cols, req)
    _assert_staged(st)
    assert st.groups == 1024


def test_staged_distinct_composite():
    cols = distinct_cols(1_000_000, 50_000)
    req = Request(["region", "url"], [AggSpec("count", None, "c"), AggSpec("count_distinct", "user_id", "u"),
                                      AggSpec("sum", "latency_ms", "lat")], flags=STAGED)
    _, st = run_both(cols, req)
    _assert_staged(st)


def test_staged_zone_map_pruning_and_rerun():
    n = (1 << 20) + 1000
    d = np.sort(np.random.default_rng(1).integers(0, 1000, n)).astype(np.int32)
    k = (np.arange(n) % 777).astype(np.int64)
    cols = [Column("k", abi.BIGINT, k), Column("d", abi.DATE, d)]
    req = Request(["k"], [AggSpec("count", None, "c"), AggSpec("max", "d", "md")],
                  where=[Pred("d", "between", 300, 320)], flags=STAGED)
    got, st = run_both(cols, req)
    _assert_staged(st)
    assert st.row_groups_pruned > 0
    # without ORDER BY the rows come in group-slot order, and which of two
    # colliding keys claims a slot first varies: compare as sets
    t = Table(cols)
    q = try_build_group_topn(t, req)
    first = sorted(to_rows(q.collect()))
    for _ in range(2):
        q.execute()
        assert sorted(to_rows(q.collect())) == first
    q.close()
    t.close()


def test_staged_declines_to_plain_scan_for_nullable_inputs():
    """A nullable input column is not staged: the query runs the regular scan."""
    n = 300_000
    rng = np.random.default_rng(3)
    v = rng.integers(-1000, 1000, n).astype(np.int64)
    ok = rng.random(n) > 0.2
    cols = [Column("k", abi.BIGINT, (np.arange(n) % 100).astype(np.int64)), Column("v", abi.BIGINT, v, validity=ok)]
    _, st = run_both(cols, Request(["k"], [AggSpec("sum", "v", "s")], flags=STAGED))
    assert not st.flags & abi.STAT_STAGED


# ------------------------------------------------ partitioned COUNT(DISTINCT) --
# (group, value) pairs go to hash partitions, each deduplicated by one CTA in
# shared memory; the default from 2M rows, forced here on small tables.

DPART = abi.FLAG_DISTINCT_PARTITION


def test_distinct_partitioned_composite():
    cols = distinct_cols(1_000_000, 50_000)
    req = Request(["region", "url"], [AggSpec("count", None, "c"), AggSpec("count_distinct", "user_id", "u"),
                                      AggSpec("sum", "latency_ms", "lat")], flags=DPART)
    _, st = run_both(cols, req)
    assert st.flags & abi.STAT_DISTINCT_PARTITION
    assert st.groups > 100_000


def test_distinct_partitioned_region_top_and_reruns():
    cols = distinct_cols(600_000, 20_000)
    req = Request(["region"], [AggSpec("count_distinct", "user_id", "u"), AggSpec("count", None, "c")],
                  [SortSpec("u", True)], limit=10, flags=DPART)
    got, st = run_both(cols, req)
    assert st.flags & abi.STAT_DISTINCT_PARTITION
    t = Table(cols)
    q = try_build_group_topn(t, req)
    first = to_rows(q.collect())
    for _ in range(3):
        q.execute()
        assert to_rows(q.collect()) == first
    q.close()
    t.close()


def test_distinct_partitioned_nullable_and_float_values():
    """Interpreter fold (nullable / DOUBLE distinct values) through partitions."""
    n = 400_000
    rng = np.random.default_rng(21)
    k = rng.integers(0, 3000, n).astype(np.int64)
    v = rng.integers(0, 500, n).astype(np.float64) / 4.0
    v[rng.random(n) < 0.01] = -0.0
    ok = rng.random(n) > 0.1
    cols = [Column("k", abi.BIGINT, k), Column("v", abi.DOUBLE, v, validity=ok)]
    req = Request(["k"], [AggSpec("count_distinct", "v", "d"), AggSpec("count", None, "c")], flags=DPART)
    _, st = run_both(cols, req)
    assert st.flags & abi.STAT_DISTINCT_PARTITION


def test_distinct_partitioned_staged():
    """Staged scan rows reserve their pair places in the fold."""
    cols = distinct_cols(1_000_000, 50_000)
    req = Request(["region", "url"], [AggSpec("count", None, "c"), AggSpec("count_distinct", "user_id", "u"),
                                      AggSpec("sum", "latency_ms", "lat")], flags=DPART | abi.FLAG_STAGED_SCAN)
    _, st = run_both(cols, req)
    assert st.flags & abi.STAT_DISTINCT_PARTITION and st.flags & abi.STAT_STAGED


@pytest.mark.parametrize("flags", [abi.FLAG_QUEUE_SCAN, abi.FLAG_DENSE_SCAN, abi.FLAG_GATHER_SCAN])
def test_distinct_partitioned_scan_modes(flags):
    """Every scan mode under a WHERE feeds the partitions."""
    cols = distinct_cols(1_000_000, 50_000)
    req = Request(["region", "url"], [AggSpec("count", None, "c"), AggSpec("count_distinct", "user_id", "u"),
                                      AggSpec("sum", "latency_ms", "lat")],
                  where=[Pred("region", "between", 3, 40)], flags=DPART | flags)
    _, st = run_both(cols, req)
    assert st.flags & abi.STAT_DISTINCT_PARTITION


def test_distinct_partition_overflow_on_repeated_pairs():
    """One (group, value) pair repeated past a partition's capacity (all its
    copies hash to one partition): the rerun deduplicates in the global set."""
    n = 300_000
    rng = np.random.default_rng(23)
    k = (rng.random(n) < 0.5).astype(np.int64)
    v = np.where(rng.random(n) < 0.9, 7, rng.integers(0, 1000, n)).astype(np.int64)
    cols = [Column("k", abi.BIGINT, k), Column("v", abi.BIGINT, v)]
    req = Request(["k"], [AggSpec("count_distinct", "v", "d"), AggSpec("count", None, "c")], [SortSpec("k")],
                  flags=DPART)
    _, st = run_both(cols, req)
    assert not st.flags & abi.STAT_DISTINCT_PARTITION
    assert st.retries >= 1


def test_distinct_partition_overflow_on_underestimated_where():
    """A WHERE estimated to keep a few rows keeps 90%: the partitions
    overflow and the rerun sizes them for the rows that passed."""
    n = 300_000
    rng = np.random.default_rng(24)
    x = np.where(rng.random(n) < 0.9, 500_000, rng.integers(0, 1_000_000, n)).astype(np.int32)
    k = rng.integers(0, 2000, n).astype(np.int64)
    u = rng.integers(0, 100_000, n).astype(np.int64)
    cols = [Column("x", abi.INT, x), Column("k", abi.BIGINT, k), Column("u", abi.BIGINT, u)]
    req = Request(["k"], [AggSpec("count_distinct", "u", "d"), AggSpec("count", None, "c")],
                  where=[Pred("x", "between", 500_000, 500_000)], flags=DPART)
    _, st = run_both(cols, req)
    assert st.flags & abi.STAT_DISTINCT_PARTITION
    assert st.retries >= 1


# -------------------------------------------------------- global aggregate --
# No GROUP BY (thinDB's v2_global_aggregate.zig): one row, folded in each
# CTA's shared-memory table under the packed key 1; over no rows the row
# still comes back with COUNTs 0 and the rest NULL.

GLOBAL_AGGS = [AggSpec("count", None, "c"), AggSpec("sum", "amount", "s"), AggSpec("avg", "amount", "a"),
               AggSpec("min", "amount", "mn"), AggSpec("max", "d", "md")]


@pytest.mark.parametrize("where", [[], FILTER, [Pred("d", ">", 10_000_000)]], ids=["all", "filtered", "empty"])
def test_global_aggregate(where):
    cols = filtered_cols(2_000_000, 200_000)
    got, st = run_both(cols, Request([], GLOBAL_AGGS, where=where), ordered=True)
    assert len(got["c"][0]) == 1
    assert st.groups == (0 if where and where[0].op == ">" else 1)


def test_global_aggregate_nullable_float_and_distinct():
    n = 600_000
    rng = np.random.default_rng(31)
    v = rng.normal(size=n)
    ok = rng.random(n) > 0.2
    u = rng.integers(0, 50_000, n).astype(np.int64)
    w = rng.integers(-1000, 1000, n).astype(np.int32)
    cols = [Column("v", abi.DOUBLE, v, validity=ok), Column("u", abi.BIGINT, u), Column("w", abi.INT, w)]
    aggs = [AggSpec("count", "v", "cv"), AggSpec("sum", "v", "sv"), AggSpec("avg", "v", "av"),
            AggSpec("min", "w", "mn"), AggSpec("count_distinct", "u", "du"), AggSpec("sum", "w", "sw")]
    run_both(cols, Request([], aggs), ordered=True)
    run_both(cols, Request([], aggs, flags=DPART), ordered=True)
    # a narrow WHERE (a few hundred rows, some v NULL)
    run_both(cols, Request([], aggs, where=[Pred("w", "between", 5, 5)]), ordered=True)


def test_global_aggregate_pages():
    cols = filtered_cols(300_000, 10_000)
    for kw in ({"limit": 0}, {"offset": 1}, {"limit": 1}, {"limit": 5, "offset": 0}):
        got, _ = run_both(cols, Request([], GLOBAL_AGGS, **kw), ordered=True)
        assert len(got["c"][0]) == (0 if kw.get("limit") == 0 or kw.get("offset") else 1)
    got, _ = run_both(cols, Request([], GLOBAL_AGGS, [SortSpec("s", True)], where=[Pred("d", ">", 10_000_000)]),
                      ordered=True)
    assert len(got["c"][0]) == 1


def test_global_aggregate_declines_having():
    cols = filtered_cols(10_000, 100)
    t = Table(cols)
    assert try_build_group_topn(t, Request([], GLOBAL_AGGS, having=[HavingSpec("c", ">", 0)])) is None
    t.close()


# -------------------------------------------------------------- queue mode --
# Dense coalesced loads, survivors compacted into a per-warp shared-memory
# ring, full-batch folds: opt-in (TGPU_FLAG_QUEUE_SCAN), forced here.

@pytest.mark.parametrize("flags", [abi.FLAG_QUEUE_SCAN, abi.FLAG_QUEUE_SCAN | abi.FLAG_FORCE_GLOBAL,
                                   abi.FLAG_QUEUE_SCAN | abi.FLAG_NO_WARP_COMBINE])
def test_queue_mode_filtered(flags):
    cols = filtered_cols(2_000_000, 200_000)
    _, st = run_both(cols, Request(["k"], C2_AGGS, [SortSpec("s", True)], limit=10, where=FILTER, flags=flags))
    assert st.flags & abi.STAT_QUEUE
    _, st = run_both(cols, Request(["k"], C2_AGGS, where=FILTER, flags=flags))
    assert st.flags & abi.STAT_QUEUE


def test_queue_mode_sparse_and_pruned():
    cols = filtered_cols(1_500_000, 100_000)
    narrow = [Pred("d", "between", datagen.FILTER_LO, datagen.FILTER_LO)]  # one day, ~0.3%
    _, st = run_both(cols, Request(["k"], C2_AGGS, where=narrow, flags=abi.FLAG_QUEUE_SCAN))
    assert st.flags & abi.STAT_QUEUE
    n = (1 << 20) + 77
    d = np.sort(np.random.default_rng(4).integers(0, 1000, n)).astype(np.int32)
    k = (np.arange(n) % 911).astype(np.int64)
    cols = [Column("k", abi.BIGINT, k), Column("d", abi.DATE, d)]
    _, st = run_both(cols, Request(["k"], [AggSpec("count", None, "c"), AggSpec("max", "d", "md")],
                                   where=[Pred("d", "between", 300, 320)], flags=abi.FLAG_QUEUE_SCAN))
    assert st.flags & abi.STAT_QUEUE and st.row_groups_pruned > 0


def test_odd_row_count_chunks():
    """A table whose row count and chunk size leave ragged last chunks."""
    cols = filtered_cols(1_000_003, 100_000)
    for flags in (0, abi.FLAG_GATHER_SCAN, abi.FLAG_DENSE_SCAN):
        run_both(cols, Request(["k"], C2_AGGS, [SortSpec("s", True)], limit=10, where=FILTER, flags=flags))
        run_both(cols, Request(["k"], C2_AGGS, where=FILTER, flags=flags, chunk_rows=768))
