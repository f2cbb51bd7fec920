"""The oracle against the reference's known answers (CPU; pins the oracle)."""
import pytest

import cases
import oracle
from helpers import check_known_answer, load_known_answers

KNOWN = load_known_answers()


@pytest.mark.parametrize("case_fn", cases.ALL_CASES, ids=[f.__name__ for f in cases.ALL_CASES])
@pytest.mark.parametrize("threads", [1, 4])
def test_oracle_known_answers(case_fn, threads):
    c = case_fn()
    t = oracle.HostTable(c.columns, c.row_group_rows)
    for q in c.queries:
        res = oracle.run(t, q.request, threads=threads)
        check_known_answer(c, q, KNOWN[c.name][q.name], res)


def test_golden_fixture_is_current():
    """known_answers.json matches what make_golden.py derives from the formulas."""
    from helpers import rows_digest

    for fn in cases.ALL_CASES:
        c = cases.build_case(fn)
        for q in c.queries:
            e = KNOWN[c.name][q.name]
            if q.expected is not None:
                assert e["rows"] == len(q.expected)
                if "digest" in e:
                    assert e["digest"] == rows_digest(q.expected)


def test_oracle_global_aggregate_over_no_rows():
    """No GROUP BY and a WHERE that keeps nothing: still one row, COUNTs 0 and
    the other aggregates NULL (v2_global_aggregate.zig emitRow :1839-1905)."""
    import numpy as np

    from thindb_gb300 import abi
    from thindb_gb300.engine import AggSpec, Column, Pred, Request

    x = np.arange(1000, dtype=np.int32)
    cols = [Column("x", abi.INT, x), Column("d", abi.DECIMAL64, x.astype(np.int64) * 7, scale=2)]
    aggs = [AggSpec("count", None, "c"), AggSpec("count", "x", "cx"), AggSpec("sum", "x", "s"),
            AggSpec("avg", "d", "a"), AggSpec("min", "x", "mn"), AggSpec("max", "x", "mx"),
            AggSpec("count_distinct", "x", "u")]
    host = oracle.HostTable(cols, 256)
    res = oracle.run(host, Request([], aggs, where=[Pred("x", ">", 5000)]))
    assert res["__groups__"] == 0 and res["__selected__"] == 0
    for name in ("c", "cx", "u"):
        vals, ok = res[name]
        assert list(vals) == [0] and (ok is None or list(ok) == [True])
    for name in ("s", "a", "mn", "mx"):
        vals, ok = res[name]
        assert len(vals) == 1 and list(ok) == [False]
    # with rows: one group; the DECIMAL AVG divides the sum by count x 10^scale
    res = oracle.run(host, Request([], aggs, where=[Pred("x", "<", 10)]))
    assert res["__groups__"] == 1
    assert res["a"][0][0] == float(sum(range(10)) * 7) / (10 * 100.0)
    assert res["s"][0][0] == 45 and res["mx"][0][0] == 9 and res["u"][0][0] == 10
    # OFFSET past the row, or LIMIT 0: nothing
    assert oracle.run(host, Request([], aggs, limit=0))["c"][0].size == 0
    assert oracle.run(host, Request([], aggs, offset=1))["c"][0].size == 0


def test_oracle_orders_string_keys_by_their_strings():
    """ORDER BY a DICT32 key ranks strings bytewise (thinDB's post-emit sort,
    v2_shape_group_topn.zig:302-325), not codes; a dictionary holding a string
    twice declines."""
    import numpy as np

    from thindb_gb300 import abi
    from thindb_gb300.engine import AggSpec, Column, Request, SortSpec

    dic = ["pear", "apple", "b", "ab", "a", "zz", "a/b", "a.b"]
    codes = np.array([0, 1, 2, 3, 4, 5, 6, 7, 1, 1, 4], dtype=np.int32)
    cols = [Column("s", abi.DICT32, codes, dictionary=dic), Column("v", abi.BIGINT, np.arange(11, dtype=np.int64))]
    for desc in (False, True):
        r = oracle.run(oracle.HostTable(cols), Request(["s"], [AggSpec("count", None, "c")], [SortSpec("s", desc)]))
        got = [dic[c] for c in r["s"][0]]
        assert got == sorted(dic, reverse=desc)
    dup = list(dic)
    dup[2] = "pear"
    with pytest.raises(oracle.OracleDecline):
        oracle.run(oracle.HostTable([Column("s", abi.DICT32, codes, dictionary=dup), cols[1]]),
                   Request(["s"], [AggSpec("count", None, "c")]))


def test_oracle_groups_varchar_keys_by_bytes():
    """A VARCHAR key is hashed (a digest places it, the bytes decide): the
    oracle's groups equal a Python dict's over the same strings, NULLs in one
    group, and ORDER BY the string key declines."""
    import numpy as np

    from thindb_gb300 import abi
    from thindb_gb300.engine import AggSpec, Column, Request, SortSpec

    rng = np.random.default_rng(3)
    pool = ["", "a", "ab", "abc", "b", "ba", "zz/x.y", "a" * 40, "a" * 41, "0123456789abcdef"]
    vals = [pool[i] for i in rng.integers(0, len(pool), 5000)]
    ok = rng.random(5000) > 0.1
    v = rng.integers(-100, 100, 5000).astype(np.int64)
    cols = [Column("s", abi.VARCHAR, vals, validity=ok), Column("v", abi.BIGINT, v)]
    r = oracle.run(oracle.HostTable(cols), Request(["s"], [AggSpec("count", None, "c"), AggSpec("sum", "v", "t")]),
                   threads=4)
    got = {}
    for row, valid, c, t in zip(r["s"][0], r["s"][1], r["c"][0], r["t"][0]):
        got[vals[row] if valid else None] = (int(c), int(t))
    want = {}
    for s, o, x in zip(vals, ok, v):
        k = s if o else None
        c, t = want.get(k, (0, 0))
        want[k] = (c + 1, t + int(x))
    assert got == want
    with pytest.raises(oracle.OracleDecline):
        oracle.run(oracle.HostTable(cols), Request(["s"], [AggSpec("count", None, "c")], [SortSpec("s")]))
