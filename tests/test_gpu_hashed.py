"""Hashed group keys (§8(f) row 3): a VARCHAR key, alone or beside integer
parts, and integer parts wider than 128 packed bits, grouped by a 64-bit
digest with an exact check of the key's bytes (thinDB's ExactKey,
silo_group_core.zig:6337), the strings read back from each group's
representative row (emitResultStageHashed, v2_shape_group_topn.zig:1741).
The engine and the oracle may pick different representative rows of a
group, so results are compared with the string keys materialised."""
import numpy as np
import pytest

import oracle
import math
from thindb_gb300 import abi
from thindb_gb300.engine import AggSpec, Column, Pred, Request, SortSpec, Table, try_build_group_topn

pytestmark = pytest.mark.gpu


def string_pool(n, seed):
    rng = np.random.default_rng(seed)
    alpha = np.array(list(b"abcdefghijklmnopqrstuvwxyz0123456789/."))
    out = {""}
    while len(out) < n:
        out.add(bytes(alpha[rng.integers(0, len(alpha), int(rng.integers(1, 48)))]).decode())
    return sorted(out)


def materialise(res, cols, keys):
    """Result rows with every VARCHAR key's row index replaced by its string."""
    by_name = {c.name: c for c in cols}
    names = [k for k in res if not k.startswith("__")]
    rows = []
    n = len(res[names[0]][0])
    for i in range(n):
        row = []
        for nm in names:
            vals, ok = res[nm]
            if ok is not None and not ok[i]:
                row.append(None)
                continue
            x = vals[i]
            if nm in keys and by_name[nm].type == abi.VARCHAR:
                row.append(by_name[nm].data[int(x)])
            elif np.ndim(x):
                row.append(tuple(int(y) for y in x))
            else:
                row.append(x.item() if hasattr(x, "item") else x)
        rows.append(row)
    return rows


def check(cols, req, ordered=None):
    t = Table(cols)
    q = try_build_group_topn(t, req)
    assert q is not None, "declined"
    got = q.collect()
    st = q.stats()
    q.close()
    t.close()
    want = oracle.run(oracle.HostTable(cols), req, threads=4)
    keys = set(req.group_cols)
    g, w = materialise(got, cols, keys), materialise(want, cols, keys)
    if ordered is None:
        ordered = bool(req.order_specs)
    same_rows(g, w, ordered, len(req.group_cols))
    assert st.groups == want["__groups__"]
    return got, st


def same_rows(g, w, ordered, n_keys):
    """Equal rows (strings and integers exact, DOUBLE within 1e-12 relative);
    unordered results are matched by their key cells."""
    assert len(g) == len(w), (len(g), len(w))
    if not ordered:
        order = lambda r: tuple((0, "") if x is None else (1, str(x)) for x in r[:n_keys])
        g, w = sorted(g, key=order), sorted(w, key=order)
    for i, (a, b) in enumerate(zip(g, w)):
        for x, y in zip(a, b):
            if isinstance(x, float) or isinstance(y, float):
                assert math.isclose(x, y, rel_tol=1e-12, abs_tol=0.0), (i, a, b)
            else:
                assert x == y, (i, a, b)


def table(n, n_strings, seed, nullable=False):
    rng = np.random.default_rng(seed)
    pool = string_pool(n_strings, seed)
    s = [pool[i] for i in rng.integers(0, len(pool), n)]
    valid = rng.random(n) > 0.05 if nullable else None
    r = rng.integers(0, 16, n).astype(np.int32)
    v = rng.integers(-1_000_000, 1_000_000, n).astype(np.int64)
    u = rng.integers(0, 5000, n).astype(np.int64)
    return [Column("s", abi.VARCHAR, s, validity=valid), Column("r", abi.INT, r), Column("v", abi.BIGINT, v),
            Column("u", abi.BIGINT, u)]


AGGS = [AggSpec("count", None, "c"), AggSpec("sum", "v", "sv"), AggSpec("min", "v", "mn"), AggSpec("max", "v", "mx"),
        AggSpec("avg", "v", "av")]


def test_varchar_key_alone():
    cols = table(600_000, 20_000, 1)
    _, st = check(cols, Request(["s"], AGGS))
    assert st.groups == 20_000


def test_varchar_key_composite_nullable_and_page():
    cols = table(400_000, 3_000, 2, nullable=True)
    check(cols, Request(["r", "s"], AGGS))
    check(cols, Request(["s", "r"], AGGS, [SortSpec("sv", True), SortSpec("c", False)], limit=25, offset=3))


def test_varchar_key_with_where_distinct_and_regrow():
    cols = table(500_000, 8_000, 3)
    req = Request(["s"], [AggSpec("count", None, "c"), AggSpec("count_distinct", "u", "du")],
                  where=[Pred("r", "between", 2, 9)], expected_groups=64)
    _, st = check(cols, req)
    assert st.retries >= 1  # the 64-group hint was far too small: the table regrew


def test_keys_wider_than_128_bits():
    rng = np.random.default_rng(4)
    n = 300_000
    base = rng.integers(0, 4000, n)
    cols = [Column("a", abi.BIGINT, (base * 7919).astype(np.int64)), Column("b", abi.BIGINT, (base % 97).astype(np.int64)),
            Column("c", abi.BIGINT, (-base).astype(np.int64)), Column("v", abi.INT, rng.integers(-9, 9, n).astype(np.int32))]
    _, st = check(cols, Request(["a", "b", "c"], [AggSpec("count", None, "n"), AggSpec("sum", "v", "s")]))
    assert st.groups == len(np.unique(base))


def test_key_strings_of_the_result():
    cols = table(100_000, 500, 5)
    t = Table(cols)
    q = try_build_group_topn(t, Request(["s"], [AggSpec("count", None, "c")], [SortSpec("c", True)], limit=7))
    got = q.collect_strings()
    q.execute()
    raw = q.collect()
    assert got["s"][0] == [cols[0].data[int(i)] for i in raw["s"][0]]
    q.close()
    t.close()


@pytest.mark.parametrize("req", [
    Request(["s"], [AggSpec("count", None, "c")], [SortSpec("s")]),
    Request(["s"], [AggSpec("count", None, "c")], where=[Pred("s", "=", 1)]),
    Request(["r"], [AggSpec("min", "s", "m")]),
    Request(["r"], [AggSpec("count_distinct", "s", "d")]),
], ids=["order_by_key", "where_on_string", "string_min", "string_distinct"])
def test_hashed_declines(req):
    cols = table(10_000, 100, 6)
    t = Table(cols)
    assert try_build_group_topn(t, req) is None
    with pytest.raises(oracle.OracleDecline):
        oracle.run(oracle.HostTable(cols), req)
    t.close()

