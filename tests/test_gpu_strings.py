"""String group keys carried as dictionary codes (TGPU_DICT32).

thinDB groups a string column by its table id and reads the strings back at
emit (v2_shape_group_topn.zig:1741; its DESIGN.md §4.6 "Packed ids"); an
ORDER BY on the string key ranks the emitted strings (finish_after_emit,
v2_shape_group_topn.zig:302-325).  These dictionaries are built so that code
order and string order disagree: ordering by code would fail every check."""
import numpy as np
import pytest

import oracle
from helpers import compare_results, to_rows
from thindb_gb300 import abi
from thindb_gb300.engine import AggSpec, Column, Request, SortSpec, Table, try_build_group_topn

pytestmark = pytest.mark.gpu


def shuffled_dictionary(n, seed):
    rng = np.random.default_rng(seed)
    alpha = np.array(list(b"abcdefghijklmnopqrstuvwxyz0123456789/."))
    words = set()
    while len(words) < n:
        ln = int(rng.integers(1, 12))
        words.add(bytes(alpha[rng.integers(0, len(alpha), ln)]).decode())
    words = sorted(words)
    perm = rng.permutation(n)  # code i holds words[perm[i]]: code order != string order
    return [words[p] for p in perm]


def table(n_rows, n_words, seed, nullable=False):
    rng = np.random.default_rng(seed)
    dic = shuffled_dictionary(n_words, seed)
    url = rng.integers(0, n_words, n_rows).astype(np.int32)
    region = rng.integers(0, 4, n_rows).astype(np.int16)
    v = rng.integers(-1000, 1000, n_rows).astype(np.int64)
    valid = rng.random(n_rows) > 0.05 if nullable else None
    cols = [Column("url", abi.DICT32, url, validity=valid, dictionary=dic), Column("region", abi.SMALLINT, region),
            Column("v", abi.BIGINT, v)]
    return cols, dic


@pytest.mark.parametrize("limit", [None, 7, 500])
@pytest.mark.parametrize("desc", [False, True])
def test_order_by_string_key(limit, desc):
    cols, dic = table(300_000, 2_000, 1)
    req = Request(["url"], [AggSpec("count", None, "c"), AggSpec("sum", "v", "s")], [SortSpec("url", desc)],
                  limit=limit)
    t = Table(cols)
    q = try_build_group_topn(t, req)
    assert q is not None
    got = q.collect()
    want = oracle.run(oracle.HostTable(cols), req)
    compare_results(got, want, 1, ordered=True)
    # the strings come back in string order
    strs = q.key_strings(0, got["url"][0])
    assert strs == sorted(strs, reverse=desc)
    assert strs == [dic[c] for c in got["url"][0]]
    q.close()
    t.close()


def test_string_key_in_composite_order_and_nulls():
    cols, dic = table(200_000, 700, 2, nullable=True)
    req = Request(["region", "url"], [AggSpec("count", None, "c"), AggSpec("max", "v", "mx")],
                  [SortSpec("url", False), SortSpec("region", True)], limit=300, offset=11)
    t = Table(cols)
    q = try_build_group_topn(t, req)
    got = q.collect()
    want = oracle.run(oracle.HostTable(cols), req)
    compare_results(got, want, 2, ordered=True)
    q.execute()  # collect drained the result: run again for the strings
    s = q.collect_strings()
    rows = list(zip(s["url"][0], s["region"][0]))
    assert rows[0][0] is None or all(r[0] is not None for r in rows)  # NULL keys first
    named = [r[0] for r in rows if r[0] is not None]
    assert named == sorted(named)
    q.close()
    t.close()


def test_order_by_aggregate_ties_break_on_packed_code():
    # equal counts tie; the packed key (the code) breaks the tie as in thinDB
    cols, _ = table(50_000, 50, 3)
    req = Request(["url"], [AggSpec("count", None, "c")], [SortSpec("c", True)], limit=20)
    t = Table(cols)
    q = try_build_group_topn(t, req)
    compare_results(q.collect(), oracle.run(oracle.HostTable(cols), req), 1, ordered=True)
    q.close()
    t.close()


def test_repeated_dictionary_string_declines():
    cols, dic = table(10_000, 20, 4)
    dic2 = list(dic)
    dic2[5] = dic2[6]
    cols[0] = Column("url", abi.DICT32, cols[0].data, dictionary=dic2)
    req = Request(["url"], [AggSpec("count", None, "c")])
    t = Table(cols)
    assert try_build_group_topn(t, req) is None
    with pytest.raises(oracle.OracleDecline):
        oracle.run(oracle.HostTable(cols), req)
    t.close()


def test_order_by_string_key_without_dictionary_declines():
    cols, _ = table(10_000, 20, 5)
    cols[0] = Column("url", abi.DICT32, cols[0].data)
    t = Table(cols)
    assert try_build_group_topn(t, Request(["url"], [AggSpec("count", None, "c")], [SortSpec("url")])) is None
    # grouping without ordering by it still runs (codes out)
    q = try_build_group_topn(t, Request(["url"], [AggSpec("count", None, "c")]))
    assert q is not None
    assert len(to_rows(q.collect())) == 20
    q.close()
    t.close()
