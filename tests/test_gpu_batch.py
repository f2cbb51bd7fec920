"""Batched execution (one persistent kernel over (query, tile) work items,
CUDA-graph replay) returns exactly what the plain per-query operator and the
oracle return."""
import numpy as np
import pytest

import oracle
from helpers import compare_results, to_rows
from thindb_gb300 import abi, datagen, workloads
from thindb_gb300.engine import (AggSpec, Column, EngineError, QueryBatch, QueryCancelled, Request, SortSpec, Table,
                                 try_build_group_topn)

pytestmark = pytest.mark.gpu


def batched_cols(n):
    d = datagen.filtered(n, seed=6, n_keys=200_000)
    e = datagen.extra_keys(n, seed=6)
    return [Column("k", abi.BIGINT, d["k"]), Column("amount", abi.DECIMAL64, d["amount"], scale=2),
            Column("d", abi.DATE, d["d"]), Column("k10", abi.INT, e["k10"]), Column("k1k", abi.INT, e["k1k"]),
            Column("k1m", abi.INT, e["k1m"])]


@pytest.fixture(scope="module")
def table_and_cols():
    cols = batched_cols(1_500_000)
    t = Table(cols)
    yield t, cols
    t.close()


@pytest.mark.parametrize("graph", [False, True])
def test_batch_matches_plain_and_oracle(table_and_cols, graph):
    t, cols = table_and_cols
    reqs = workloads.batched_requests(24, seed=11)
    b = QueryBatch(t, reqs, graph=graph)
    host = oracle.HostTable(cols)
    for rep in range(3):  # graph capture on the first execute, replays after
        b.execute()
        b.synchronize()
        for i, r in enumerate(reqs):
            got = b.collect(i)
            q = try_build_group_topn(t, r)
            plain = q.collect()
            q.close()
            assert to_rows(got) == to_rows(plain), (rep, i)
            if rep == 0 and i % 3 == 0:
                compare_results(got, oracle.run(host, r), 1, True)
    st = b.stats()
    assert st.n_queries == 24 and st.graph == (1 if graph else 0)
    b.close()


def test_batch_with_distinct_epochs():
    d = datagen.distinct(400_000, seed=12, n_users=30_000)
    cols = [Column("region", abi.SMALLINT, d["region"]), Column("url", abi.DICT32, d["url"]),
            Column("user_id", abi.BIGINT, d["user_id"]), Column("latency_ms", abi.DOUBLE, d["latency_ms"])]
    t = Table(cols)
    reqs = [Request(["region"], [AggSpec("count_distinct", "user_id", "u"), AggSpec("count", None, "c")],
                    [SortSpec("u", True)], limit=10),
            Request(["url"], [AggSpec("count_distinct", "user_id", "u")], [SortSpec("u", True)], limit=5)]
    b = QueryBatch(t, reqs, graph=True)
    host = oracle.HostTable(cols)
    want = [to_rows(oracle.run(host, r)) for r in reqs]
    for _ in range(3):
        b.execute()
        for i in range(len(reqs)):
            assert to_rows(b.collect(i)) == want[i]
    b.close()
    t.close()


def test_batch_declines_sorted_pages_and_cancels(table_and_cols):
    t, _ = table_and_cols
    big = Request(["k1k"], [AggSpec("count", None, "c")], [SortSpec("c", True)], limit=100)
    with pytest.raises(EngineError):
        QueryBatch(t, [big])
    b = QueryBatch(t, workloads.batched_requests(4, seed=3))
    b.cancel()
    with pytest.raises(QueryCancelled):
        b.execute()
    b.close()


def test_batch_with_global_aggregates(table_and_cols):
    """Queries without GROUP BY ride in a batch too; one keeps no row and
    still answers its single row (COUNT 0, the rest NULL)."""
    from thindb_gb300.engine import Pred

    t, cols = table_and_cols
    aggs = [AggSpec("count", None, "c"), AggSpec("sum", "amount", "s"), AggSpec("max", "amount", "m")]
    reqs = [Request([], aggs), Request([], aggs, where=[Pred("k1m", "between", 10, 5000)]),
            Request([], aggs, where=[Pred("d", ">", 10_000_000)]),
            Request(["k10"], aggs, [SortSpec("s", True)], limit=3)]
    b = QueryBatch(t, reqs, graph=True)
    host = oracle.HostTable(cols)
    for rep in range(2):
        b.execute()
        b.synchronize()
        for i, r in enumerate(reqs):
            got = b.collect(i)
            compare_results(got, oracle.run(host, r), len(r.group_cols), True)
            if not r.group_cols:
                assert len(got["c"][0]) == 1
    b.close()
