"""Parity at the measured sizes, with the committed GB300 tuning table on.

The benchmark runs the three single-query workloads at their full sizes with
the settings thindb_gb300/tuning/gb300.json picks for their shapes; these
tests run exactly that (same generator, sizes, seeds and tuned settings) and
compare every result with the oracle's silo mode: keys, COUNT, integer and
DECIMAL sums and AVG bit-exact, the DOUBLE sum within 1e-12 relative (the
summation order differs).  Results without ORDER BY are compared after
sorting both sides by key.
  plain     16,777,216 rows, BIGINT key over 1,024 values, COUNT/SUM/MIN/MAX
  filtered  100M rows, Zipf(1.1) key over 10M values, 36-day DATE window,
            COUNT/SUM(DECIMAL)/AVG, top-10 by SUM and the all-groups form
  distinct  200M rows, (SMALLINT, DICT32) key, COUNT/COUNT(DISTINCT)/SUM(DOUBLE)
"""
import os

import numpy as np
import pytest

import oracle
from thindb_gb300 import abi, datagen, engine, workloads
from thindb_gb300.engine import Table, try_build_group_topn

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module", autouse=True)
def tuned():
    n = engine.load_tuning()
    assert n > 0, "the committed tuning table is empty"
    yield
    engine.clear_tuning()


def host_table(workload, n):
    inputs = workloads.table_inputs(workload, n, pinned=False)
    cols = workloads.columns(inputs)
    for c in cols:
        c.data = c.data.numpy()
    return cols


def run(cols, req):
    t = Table(cols, compute_ndv=True)
    q = try_build_group_topn(t, req)
    assert q is not None, "declined"
    got = q.collect()
    st = q.stats()
    q.close()
    t.close()
    want = oracle.run(oracle.HostTable(cols), req, threads=THREADS)
    assert st.flags & abi.STAT_TUNED, "the tuned setting was not applied"
    assert st.groups == want["__groups__"]
    assert st.rows_selected == want["__selected__"]
    return got, want, st


def same_rows(got, want, keys, ordered, rel_cols=()):
    names = [k for k in want if not k.startswith("__")]
    n = len(want[names[0]][0])
    assert all(len(got[k][0]) == n for k in names), "row counts differ"
    if ordered:
        og = ow = np.arange(n)
    else:
        og = np.lexsort([np.asarray(got[k][0]) for k in reversed(keys)])
        ow = np.lexsort([np.asarray(want[k][0]) for k in reversed(keys)])
    for k in names:
        g, w = np.asarray(got[k][0])[og], np.asarray(want[k][0])[ow]
        if k in rel_cols:
            err = np.abs(g - w) / np.maximum(np.abs(w), 1e-300)
            assert float(err.max(initial=0.0)) <= 1e-12, (k, float(err.max()))
        else:
            assert np.array_equal(g, w), f"column {k} differs"
        if got[k][1] is not None or want[k][1] is not None:
            assert np.array_equal(np.asarray(got[k][1])[og], np.asarray(want[k][1])[ow]), f"validity of {k}"


def test_plain_full_size():
    cols = host_table("plain", datagen.PLAIN_ROWS)
    got, want, st = run(cols, workloads.workload_request("plain"))
    assert st.groups == 1024
    same_rows(got, want, ["k"], ordered=False)


@pytest.fixture(scope="module")
def filtered_cols():
    return host_table("filtered", datagen.FILTERED_ROWS)


def test_filtered_top10_full_size(filtered_cols):
    got, want, st = run(filtered_cols, workloads.workload_request("filtered"))
    assert st.result_rows == 10
    same_rows(got, want, ["k"], ordered=True)


def test_filtered_all_groups_full_size(filtered_cols):
    req = workloads.workload_request("filtered")
    req.order_specs = []
    req.limit = None
    got, want, st = run(filtered_cols, req)
    assert st.result_rows > 1_000_000
    same_rows(got, want, ["k"], ordered=False)


def test_distinct_full_size():
    cols = host_table("distinct", datagen.DISTINCT_ROWS)
    got, want, st = run(cols, workloads.workload_request("distinct"))
    assert st.groups > 300_000
    same_rows(got, want, ["region", "url"], ordered=False, rel_cols=("lat",))
