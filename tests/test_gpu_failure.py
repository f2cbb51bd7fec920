"""The device-timeout path, made to happen without faulting anything.

The staged scan and the COUNT(DISTINCT) partition kernel wait on bulk
asynchronous copies with bounded waits.  Here the bound is set to a few SM
clocks (tgpu_debug_set_wait_limit), so the first wait of a CTA runs out while
its copy is still in flight: the kernel sets its status bit, lets its own
copies land (waiting with the built-in bound) and returns.  The query must
report TGPU_ERR_DEVICE_TIMEOUT, and the next execution on the same context —
the same query object and a fresh one — must match the oracle."""
import pytest

import oracle
from helpers import compare_results
from thindb_gb300 import abi, datagen
from thindb_gb300.engine import (AggSpec, Column, DeviceTimeout, Pred, Request, SortSpec, Table,
                                 set_device_wait_limit, try_build_group_topn)

pytestmark = pytest.mark.gpu


def filtered(n):
    d = datagen.filtered(n, seed=21, n_keys=100_000)
    return [Column("k", abi.BIGINT, d["k"]), Column("amount", abi.DECIMAL64, d["amount"], scale=2, precision=18),
            Column("d", abi.DATE, d["d"])]


def distinct(n):
    d = datagen.distinct(n, seed=22, n_users=100_000)
    return [Column("region", abi.SMALLINT, d["region"]), Column("url", abi.DICT32, d["url"]),
            Column("user_id", abi.BIGINT, d["user_id"]), Column("latency_ms", abi.DOUBLE, d["latency_ms"])]


CASES = {
    "staged_scan": (filtered, lambda: Request(
        ["k"], [AggSpec("count", None, "c"), AggSpec("sum", "amount", "s"), AggSpec("avg", "amount", "a")],
        [SortSpec("s", True)], limit=10, where=[Pred("d", "between", datagen.FILTER_LO, datagen.FILTER_HI)],
        flags=abi.FLAG_STAGED_SCAN), abi.STAT_STAGED),
    "pipe_scan": (filtered, lambda: Request(
        ["k"], [AggSpec("count", None, "c"), AggSpec("sum", "amount", "s"), AggSpec("avg", "amount", "a")],
        [SortSpec("s", True)], limit=10, where=[Pred("d", "between", datagen.FILTER_LO, datagen.FILTER_HI)],
        flags=abi.FLAG_PIPE_SCAN), abi.STAT_PIPE),
    "distinct_partitions": (distinct, lambda: Request(
        ["region", "url"], [AggSpec("count", None, "c"), AggSpec("count_distinct", "user_id", "u")],
        flags=abi.FLAG_DISTINCT_PARTITION), abi.STAT_DISTINCT_PARTITION),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_wait_timeout_reports_and_recovers(name):
    make_cols, make_req, stat_flag = CASES[name]
    cols = make_cols(2_000_000)
    t = Table(cols)
    want = oracle.run(oracle.HostTable(cols), make_req(), threads=4)
    q = try_build_group_topn(t, make_req())
    assert q is not None
    try:
        set_device_wait_limit(1)
        with pytest.raises(DeviceTimeout):
            q.collect()
    finally:
        set_device_wait_limit(0)
    # the same query object re-executed, then a fresh one, on the same context
    q.execute()
    got = q.collect()
    assert q.stats().flags & stat_flag
    ordered = bool(make_req().order_specs)
    compare_results(got, want, len(make_req().group_cols), ordered, rel=1e-12)
    q.close()
    q2 = try_build_group_topn(t, make_req())
    compare_results(q2.collect(), want, len(make_req().group_cols), ordered, rel=1e-12)
    q2.close()
    t.close()
