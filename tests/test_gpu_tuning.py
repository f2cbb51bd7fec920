"""The tuning table: a matching shape takes the tuned settings, results stay
equal to the built-in settings' and the oracle's, batched and single-query
shapes are separate classes, and the committed table loads."""
import os

import pytest

import oracle
from helpers import compare_results
from test_gpu_parity import C2_AGGS, FILTER, filtered_cols
from thindb_gb300 import abi, engine
from thindb_gb300.engine import Request, SortSpec, Table, request_shape, try_build_group_topn

pytestmark = pytest.mark.gpu


def _install(entries):
    arr = (abi.Tuning * max(1, len(entries)))()
    for i, (shape, knobs) in enumerate(entries):
        for k, v in shape.items():
            setattr(arr[i].shape, k, v)
        for k, v in knobs.items():
            setattr(arr[i], k, v)
    assert engine.lib().tgpu_tuning_set(arr, len(entries)) == abi.OK


@pytest.fixture
def clean_tuning():
    saved = engine.tuning_entries()
    yield
    engine.clear_tuning()
    if saved:
        _install([(e["shape"], {k: e[k] for k in ("chunk_rows", "cache_slots", "table_load_pct", "flags")})
                  for e in saved])


@pytest.mark.parametrize("knobs", [
    {"chunk_rows": 512, "cache_slots": -1, "table_load_pct": 25, "flags": abi.FLAG_GATHER_SCAN},
    {"chunk_rows": 4096, "cache_slots": 256, "table_load_pct": 70, "flags": abi.FLAG_DENSE_SCAN},
    {"chunk_rows": 1024, "cache_slots": 0, "table_load_pct": 0, "flags": abi.FLAG_NO_WARP_COMBINE},
])
def test_tuned_settings_apply_and_match(clean_tuning, knobs):
    cols = filtered_cols(2_000_000, 200_000)
    t = Table(cols)
    req = Request(["k"], C2_AGGS, [SortSpec("s", True)], limit=10, where=FILTER)
    shape = request_shape(t, req)
    assert shape["filtered"] == 1 and shape["sel_log2"] < 0 and shape["batched"] == 0
    assert request_shape(t, req, batched=True) == dict(shape, batched=1)
    _install([(shape, knobs)])
    q = try_build_group_topn(t, req)
    got = q.collect()
    st = q.stats()
    q.close()
    assert st.flags & abi.STAT_TUNED
    if knobs["flags"] & abi.FLAG_GATHER_SCAN:
        assert st.flags & abi.STAT_GATHER
    if knobs["flags"] & abi.FLAG_DENSE_SCAN:
        assert not st.flags & abi.STAT_GATHER
    # a request that sets its own knobs is not tuned
    q = try_build_group_topn(t, Request(["k"], C2_AGGS, [SortSpec("s", True)], limit=10, where=FILTER,
                                        chunk_rows=256))
    q.collect()
    assert not q.stats().flags & abi.STAT_TUNED
    q.close()
    t.close()
    want = oracle.run(oracle.HostTable(cols, 65536), req, threads=1)
    compare_results(got, want, 1, True, rel=1e-12)


def test_committed_table_loads(clean_tuning):
    if not os.path.exists(engine.TUNING_PATH):
        pytest.skip("no tuning table committed")
    n = engine.load_tuning(engine.TUNING_PATH)
    assert n == len(engine.tuning_entries()) and n > 0
