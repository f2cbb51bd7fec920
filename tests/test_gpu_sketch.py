"""ORDER BY COUNT(*) DESC LIMIT k through the two-pass count sketch (thinDB's
count_topk_sketch.zig): the tally, the threshold, the filter pass over heavy
counters only, and the rerun over every row when the filter pass cannot
prove its answer — always equal to the oracle, which groups every row."""
import numpy as np
import pytest

import oracle
from helpers import compare_results
from thindb_gb300 import abi, datagen
from thindb_gb300.engine import AggSpec, Column, Pred, Request, SortSpec, Table, try_build_group_topn


def run_both(cols, req):
    """The page against the oracle's (which groups every row).  With the
    sketch's filter pass the engine creates only the kept groups, so its
    group count is compared only when every row was grouped."""
    t = Table(cols)
    q = try_build_group_topn(t, req)
    assert q is not None
    got = q.collect()
    st = q.stats()
    q.close()
    t.close()
    want = oracle.run(oracle.HostTable(cols), req, threads=4)
    compare_results(got, want, len(req.group_cols), ordered=True)
    assert st.rows_selected == want["__selected__"]
    if not st.flags & abi.STAT_COUNT_SKETCH:
        assert st.groups == want["__groups__"]
    else:
        assert st.groups < want["__groups__"]
    return got, st

pytestmark = pytest.mark.gpu
SK = abi.FLAG_COUNT_SKETCH


def zipf_cols(n, n_keys, s=1.1, seed=5):
    d = datagen.filtered(n, seed=seed, n_keys=n_keys)
    return [Column("k", abi.BIGINT, d["k"]), Column("amount", abi.DECIMAL64, d["amount"], scale=2),
            Column("d", abi.DATE, d["d"])]


def topcount(limit=10, offset=0, where=(), flags=SK, more=()):
    return Request(["k"], [AggSpec("count", None, "c"), *more], [SortSpec("c", True)], limit=limit, offset=offset,
                   where=list(where), flags=flags)


# (LIMIT 1000 OFFSET 24 over 3M rows: the 1,024th group's count is about
# the collision noise of a counter, so most counters would be kept: declines)
@pytest.mark.parametrize("limit,offset,answered", [(10, 0, True), (1, 0, True), (100, 23, True),
                                                   (1000, 24, False)])
def test_sketch_zipf_top_counts(limit, offset, answered):
    cols = zipf_cols(3_000_000, 1_000_000)
    _, st = run_both(cols, topcount(limit, offset))
    assert bool(st.flags & abi.STAT_COUNT_SKETCH) == answered
    assert st.result_rows == limit


def test_sketch_with_where_and_other_aggregates():
    cols = zipf_cols(3_000_000, 500_000)
    req = topcount(20, where=[Pred("d", "between", datagen.FILTER_LO, datagen.FILTER_HI)],
                   more=[AggSpec("sum", "amount", "s"), AggSpec("max", "amount", "mx")])
    _, st = run_both(cols, req)
    assert st.flags & abi.STAT_COUNT_SKETCH


def test_sketch_declines_on_even_keys():
    n = 2_000_000
    rng = np.random.default_rng(8)
    cols = [Column("k", abi.BIGINT, rng.integers(0, 1 << 40, n).astype(np.int64))]
    _, st = run_both(cols, topcount(10))
    assert not st.flags & abi.STAT_COUNT_SKETCH


def test_sketch_rerun_when_the_cut_is_not_proven():
    """Two heavy keys and a long flat tail: with LIMIT 50 the 50th best kept
    group sits far below the threshold, so the filter pass cannot prove the
    page and every row is regrouped."""
    n = 2_000_000
    rng = np.random.default_rng(9)
    k = rng.integers(1000, 1000 + 40_000, n).astype(np.int64)
    k[: n // 3] = 1
    k[n // 3: n // 2] = 2
    rng.shuffle(k)
    cols = [Column("k", abi.BIGINT, k)]
    _, st = run_both(cols, topcount(50))
    assert st.flags & abi.STAT_SKETCH_RERUN or not st.flags & abi.STAT_COUNT_SKETCH


def test_sketch_ties_at_the_cut_break_on_key():
    # every key but the heavy ones holds exactly 40 rows: ties everywhere below the top
    rng = np.random.default_rng(10)
    k = np.repeat(np.arange(100, 60_100, dtype=np.int64), 40)
    k = np.concatenate([k, np.full(300_000, 7, np.int64), np.full(200_000, 9, np.int64)])
    rng.shuffle(k)
    cols = [Column("k", abi.BIGINT, k)]
    run_both(cols, topcount(5))
    run_both(cols, topcount(30))


def test_sketch_off_and_batched_shapes_unchanged():
    cols = zipf_cols(1_500_000, 300_000)
    _, st = run_both(cols, topcount(10, flags=abi.FLAG_NO_COUNT_SKETCH))
    assert not st.flags & abi.STAT_COUNT_SKETCH


@pytest.mark.parametrize("rg", [65_536, 1_001])
def test_sketch_filter_with_odd_row_groups_and_tail(rg):
    # 1,001-row groups put every other select span on an odd row (the
    # vector keep test needs 16-byte alignment) and the table ends mid-vector
    cols = zipf_cols(2_000_001, 300_000, seed=8)
    t = Table(cols, row_group_rows=rg)
    req = topcount(10)
    q = try_build_group_topn(t, req)
    got = q.collect()
    st = q.stats()
    q.close()
    t.close()
    want = oracle.run(oracle.HostTable(cols, rg), req, threads=4)
    compare_results(got, want, 1, ordered=True)
    assert st.rows_selected == want["__selected__"]
    assert st.flags & abi.STAT_COUNT_SKETCH and st.flags & abi.STAT_SPLIT
