"""The served mode: requests admitted by estimated bytes, run in waves that
overlap on the device; every result is the same alone and in the mix."""
import numpy as np
import pytest

from helpers import rows_equal, to_rows
from thindb_gb300 import abi, datagen, workloads
from thindb_gb300.engine import Column, Server, Table, try_build_group_topn

pytestmark = pytest.mark.gpu


def small_tables():
    p = datagen.plain(300_000, seed=1)
    f = datagen.filtered(800_000, seed=2, n_keys=100_000)
    d = datagen.distinct(800_000, seed=3, n_users=50_000)
    e = datagen.extra_keys(800_000, seed=2)
    plain = Table([Column("k", abi.BIGINT, p["k"]), Column("v", abi.INT, p["v"])])
    filt = Table([Column("k", abi.BIGINT, f["k"]), Column("amount", abi.DECIMAL64, f["amount"], scale=2),
                  Column("d", abi.DATE, f["d"])])
    dist = Table([Column("region", abi.SMALLINT, d["region"]), Column("url", abi.DICT32, d["url"]),
                  Column("user_id", abi.BIGINT, d["user_id"]), Column("latency_ms", abi.DOUBLE, d["latency_ms"])])
    bat = Table([Column("k", abi.BIGINT, f["k"]), Column("amount", abi.DECIMAL64, f["amount"], scale=2),
                 Column("d", abi.DATE, f["d"]), Column("k10", abi.INT, e["k10"]), Column("k1k", abi.INT, e["k1k"]),
                 Column("k1m", abi.INT, e["k1m"])])
    return [plain, filt, dist, bat]


@pytest.fixture(scope="module")
def tables():
    ts = small_tables()
    yield ts
    for t in ts:
        t.close()


def alone(tables, ti, req):
    q = try_build_group_topn(tables[ti], req)
    rows = to_rows(q.collect())
    q.close()
    return rows


@pytest.mark.parametrize("mode", ["continuous-batched", "continuous", "plain"])
def test_results_same_alone_and_in_the_mix(tables, mode):
    """continuous: overlapping single executions; continuous-batched: every
    wave of same-table requests as one batched kernel (batch_min 1)."""
    mix = workloads.served_mix(36, seed=8)
    srv = Server(tables, mode="plain" if mode == "plain" else "continuous", max_batch=16, max_inflight=3,
                 batch_min=1 if mode == "continuous-batched" else 0)
    tickets = [srv.submit(ti, rq) for ti, rq in mix]  # all in flight together
    for (ti, rq), tk in zip(mix, tickets):
        got = to_rows(srv.result(tk))
        # integers exact; FP64 sums within 1e-12 relative (atomic order differs run to run)
        ok, msg = rows_equal(got, alone(tables, ti, rq), True, len(rq.group_cols), rel=1e-12)
        assert ok, (ti, rq, msg)
        srv.release(tk)
    st = srv.stats()
    assert st.completed == len(mix) and st.failed == 0
    if mode == "continuous-batched":
        assert st.waves < len(mix)  # requests shared waves
    srv.close()


def test_budget_admission_and_load(tables):
    mix = workloads.served_mix(24, seed=9)
    # a budget far below one wave's estimate still completes everything (one request at a time)
    srv = Server(tables, mode="continuous", memory_budget=1 << 20, max_batch=8)
    tickets = [srv.submit(ti, rq) for ti, rq in mix]
    for tk in tickets:
        assert srv.wait(tk, 60_000)
        srv.release(tk)
    assert srv.stats().peak_admitted_bytes > 0
    srv.close()
    srv = Server(tables, mode="continuous")
    rep = srv.run_load(mix, rate_qps=300, duration_s=0.5, seed=3)
    assert rep["completed"] == rep["submitted"] > 0 and rep["failed"] == 0
    assert 0 < rep["p50_ms"] <= rep["p99_ms"] <= rep["max_ms"]
    srv.close()
