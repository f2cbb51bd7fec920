"""The pipelined scan (producer warp + consumer warps over a ring of bulk
copies) against the oracle: filtered and unfiltered shapes, the resident
shared-memory route and the global table, a partial last tile, zone-map
pruning with reruns, COUNT(DISTINCT) through the partitions, and the
declines to the regular scan."""
import numpy as np
import pytest

from test_gpu_parity import (C2_AGGS, FILTER, distinct_cols, filtered_cols, plain_cols, run_both)
from helpers import to_rows
from thindb_gb300 import abi
from thindb_gb300.engine import AggSpec, Column, Pred, QueryCancelled, Request, SortSpec, Table, try_build_group_topn

pytestmark = pytest.mark.gpu
PIPE = abi.FLAG_PIPE_SCAN


def _assert_pipe(st):
    assert st.flags & abi.STAT_PIPE, "the pipelined scan did not run"


@pytest.mark.parametrize("extra", [0, abi.FLAG_FORCE_GLOBAL, abi.FLAG_NO_WARP_COMBINE,
                                   abi.FLAG_FORCE_GLOBAL | abi.FLAG_NO_WARP_COMBINE])
def test_pipe_filtered_top10_and_all_groups(extra):
    cols = filtered_cols(2_000_000 + 77, 200_000)  # a partial last tile
    _, st = run_both(cols, Request(["k"], C2_AGGS, [SortSpec("s", True)], limit=10, where=FILTER,
                                   flags=PIPE | extra))
    _assert_pipe(st)
    _, st = run_both(cols, Request(["k"], C2_AGGS, where=FILTER, flags=PIPE | extra))
    _assert_pipe(st)


@pytest.mark.parametrize("extra", [0, abi.FLAG_FORCE_GLOBAL])
def test_pipe_plain_lowcard(extra):
    cols = plain_cols((1 << 20) + 333)
    req = Request(["k"], [AggSpec("count", None, "c"), AggSpec("sum", "v", "s"), AggSpec("min", "v", "mn"),
                          AggSpec("max", "v", "mx")], flags=PIPE | extra)
    _, st = run_both(cols, req)
    _assert_pipe(st)
    assert st.groups == 1024
    assert st.route == (2 if extra else 1)


def test_pipe_tiny_table_and_every_row_filtered_out():
    cols = plain_cols(100)  # one partial tile, most consumer warps idle
    req = Request(["k"], [AggSpec("count", None, "c"), AggSpec("sum", "v", "s")], flags=PIPE)
    _, st = run_both(cols, req)
    _assert_pipe(st)
    # a WHERE the zone maps cannot prune that keeps no row: an odd DATE in an
    # even-only column
    n = 300_000
    rng = np.random.default_rng(4)
    cols = [Column("k", abi.BIGINT, rng.integers(0, 1000, n).astype(np.int64)),
            Column("d", abi.DATE, (2 * rng.integers(0, 500, n)).astype(np.int32))]
    _, st = run_both(cols, Request(["k"], [AggSpec("count", None, "c")], where=[Pred("d", "=", 501)], flags=PIPE))
    _assert_pipe(st)
    assert st.rows_selected == 0


def test_pipe_distinct_composite_partitions_and_set():
    cols = distinct_cols(1_000_000, 50_000)
    aggs = [AggSpec("count", None, "c"), AggSpec("count_distinct", "user_id", "u"),
            AggSpec("sum", "latency_ms", "lat")]
    _, st = run_both(cols, Request(["region", "url"], aggs, flags=PIPE | abi.FLAG_DISTINCT_PARTITION))
    _assert_pipe(st)
    assert st.flags & abi.STAT_DISTINCT_PARTITION
    _, st = run_both(cols, Request(["region", "url"], aggs, flags=PIPE | abi.FLAG_NO_DISTINCT_PARTITION))
    _assert_pipe(st)
    _, st = run_both(cols, Request(["region", "url"], aggs, where=[Pred("region", "between", 3, 40)],
                                   flags=PIPE | abi.FLAG_DISTINCT_PARTITION))
    _assert_pipe(st)


def test_pipe_zone_map_pruning_and_rerun():
    n = (1 << 20) + 1000
    d = np.sort(np.random.default_rng(1).integers(0, 1000, n)).astype(np.int32)
    k = (np.arange(n) % 777).astype(np.int64)
    cols = [Column("k", abi.BIGINT, k), Column("d", abi.DATE, d)]
    req = Request(["k"], [AggSpec("count", None, "c"), AggSpec("max", "d", "md")],
                  where=[Pred("d", "between", 300, 320)], flags=PIPE)
    _, st = run_both(cols, req)
    _assert_pipe(st)
    assert st.row_groups_pruned > 0
    t = Table(cols)
    q = try_build_group_topn(t, req)
    first = sorted(to_rows(q.collect()))
    for _ in range(2):
        q.execute()
        assert sorted(to_rows(q.collect())) == first
    q.close()
    t.close()


def test_pipe_declines_to_regular_scan():
    n = 300_000
    rng = np.random.default_rng(3)
    v = rng.integers(-1000, 1000, n).astype(np.int64)
    ok = rng.random(n) > 0.2
    cols = [Column("k", abi.BIGINT, (np.arange(n) % 100).astype(np.int64)), Column("v", abi.BIGINT, v, validity=ok)]
    _, st = run_both(cols, Request(["k"], [AggSpec("sum", "v", "s")], flags=PIPE))
    assert not st.flags & abi.STAT_PIPE  # a nullable input
    cols = filtered_cols(200_000, 1000)
    two = [Pred("d", "between", 0, 1 << 30), Pred("amount", ">", 100)]
    _, st = run_both(cols, Request(["k"], C2_AGGS, where=two, flags=PIPE))
    assert not st.flags & abi.STAT_PIPE  # two predicates


def test_pipe_cancel_before_next():
    cols = filtered_cols(1_000_000, 10_000)
    t = Table(cols)
    q = try_build_group_topn(t, Request(["k"], C2_AGGS, where=FILTER, flags=PIPE))
    q.cancel()
    with pytest.raises(QueryCancelled):
        q.collect()
    q.close()
    t.close()
