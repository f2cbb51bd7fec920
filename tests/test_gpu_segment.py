"""Tables registered from thinDB segment images: the blocks decode on the
device (raw, FOR, RLE, validity bitmaps) and every query over the decoded
table matches the oracle over the original arrays.  The images come from the
restated segment writer in tests/golden/segments.py."""
import numpy as np
import pytest

import oracle
from golden.segments import write_segment
from helpers import compare_results
from thindb_gb300 import abi
from thindb_gb300.engine import AggSpec, Column, Pred, Request, SortSpec, Table, try_build_group_topn

pytestmark = pytest.mark.gpu


def columns(n, seed, nullable=True):
    rng = np.random.default_rng(seed)
    region = np.repeat(rng.integers(0, 6, n // 500 + 1), 500)[:n].astype(np.int16)   # long runs: RLE
    day = (19000 + np.arange(n) // 997).astype(np.int32)                              # sorted: FOR / RLE
    user = rng.integers(0, 50_000, n).astype(np.int64)                                # FOR width 2
    amount = rng.integers(-10**9, 10**9, n).astype(np.int64)                          # FOR width 4
    price = np.round(rng.random(n) * 1000, 2)                                         # raw double
    flag = (rng.random(n) > 0.7).astype(np.uint8)
    tiny = rng.integers(-100, 100, n).astype(np.int8)
    cents = rng.integers(-10**6, 10**6, n).astype(np.int64)
    v = (lambda p: rng.random(n) > p) if nullable else (lambda p: None)
    return [Column("region", abi.SMALLINT, region), Column("day", abi.DATE, day, validity=v(0.02)),
            Column("user", abi.BIGINT, user, validity=v(0.05)), Column("amount", abi.BIGINT, amount),
            Column("price", abi.DOUBLE, price, validity=v(0.1)), Column("flag", abi.BOOLEAN, flag),
            Column("tiny", abi.TINYINT, tiny, validity=v(0.2)),
            Column("cents", abi.DECIMAL64, cents, scale=2, precision=12)]


def from_segment(cols, **kw):
    image, _ = write_segment([c.type for c in cols], [c.data for c in cols], [c.validity for c in cols], **kw)
    schema = [Column(c.name, c.type, None, scale=c.scale, precision=c.precision) for c in cols]
    return Table.from_segment(image, schema)


REQUESTS = [
    Request(["region"], [AggSpec("count", None, "c"), AggSpec("sum", "amount", "s"), AggSpec("min", "day", "mn"),
                         AggSpec("max", "user", "mx"), AggSpec("avg", "price", "ap"), AggSpec("sum", "cents", "sc")]),
    Request(["day", "flag"], [AggSpec("count", "user", "cu"), AggSpec("sum", "tiny", "st")],
            [SortSpec("cu", True)], limit=25, where=[Pred("amount", "between", -10**8, 5 * 10**8)]),
    Request(["user"], [AggSpec("count", None, "c"), AggSpec("max", "price", "mp")], [SortSpec("c", True)], limit=100),
    Request(["tiny", "region"], [AggSpec("count_distinct", "user", "du"), AggSpec("min", "amount", "ma")]),
]


def run_and_compare(t, cols, req, ordered):
    q = try_build_group_topn(t, req)
    assert q is not None
    got = q.collect()
    want = oracle.run(oracle.HostTable(cols), req)
    compare_results(got, want, len(req.group_cols), ordered=ordered, rel=1e-12)
    q.close()


@pytest.mark.parametrize("encoding", [None, "raw", "for", "for8", "rle"])
def test_segment_queries_match_the_oracle(encoding):
    cols = columns(200_003, 1)
    t = from_segment(cols, row_group_rows=16_384, encoding=encoding)
    assert t.n_rows == 200_003 and t.n_row_groups == 13
    for i, req in enumerate(REQUESTS):
        run_and_compare(t, cols, req, ordered=bool(req.order_specs))
    t.close()


def test_rle_everywhere_integer_columns():
    # every integer column forced to RLE, runs of one row included
    cols = [c for c in columns(50_001, 2) if c.type != abi.DOUBLE]
    t = from_segment(cols, row_group_rows=4096, encoding="rle")
    run_and_compare(t, cols, REQUESTS[3], ordered=False)
    run_and_compare(t, cols, Request(["region", "flag"], [AggSpec("sum", "amount", "s"), AggSpec("avg", "cents", "a")]),
                    ordered=False)
    t.close()


def test_zone_maps_prune_row_groups_of_a_segment_table():
    cols = columns(300_000, 3, nullable=False)
    t = from_segment(cols, row_group_rows=10_000)
    req = Request(["region"], [AggSpec("count", None, "c"), AggSpec("sum", "amount", "s")],
                  where=[Pred("day", "between", 19050, 19100)])
    q = try_build_group_topn(t, req)
    got = q.collect()
    assert q.stats().row_groups_pruned > 0
    compare_results(got, oracle.run(oracle.HostTable(cols), req), 1, ordered=False)
    q.close()
    t.close()


def test_empty_and_single_row_segments():
    for n in (0, 1):
        cols = columns(n, 4)
        t = from_segment(cols)
        assert t.n_rows == n
        run_and_compare(t, cols, REQUESTS[0], ordered=False)
        t.close()


def test_ten_million_rows_auto_encodings():
    cols = columns(10_000_000, 5)
    t = from_segment(cols, row_group_rows=65_536)
    for req in REQUESTS[:3]:
        run_and_compare(t, cols, req, ordered=bool(req.order_specs))
    t.close()


@pytest.mark.parametrize("encoding", [None, "raw", "for", "for8", "rle"])
@pytest.mark.parametrize("rg", [65_536, 1_000, 37])
def test_decoded_columns_are_bit_exact_with_the_oracle_decode(encoding, rg):
    # row groups of 1,000 and 37 rows put block boundaries inside validity words
    cols = columns(150_001 if rg > 37 else 20_001, 6)
    image, _ = write_segment([c.type for c in cols], [c.data for c in cols], [c.validity for c in cols],
                             row_group_rows=rg, encoding=encoding)
    t = Table.from_segment(image, [Column(c.name, c.type, None, scale=c.scale, precision=c.precision) for c in cols])
    want = oracle.decode_segment(image, [c.type for c in cols], [c.validity is not None for c in cols])
    for c, (wv, wok) in zip(cols, want):
        gv, gok = t.read_column(c.name)
        assert np.array_equal(gv.view(np.uint8), wv.view(np.uint8)), c.name
        if wok is None:
            assert gok.all()
        else:
            assert np.array_equal(gok, wok), c.name
    st = t.load_stats()
    assert st.image_bytes == len(image) and st.blocks == len(cols) * -(-t.n_rows // rg)
    assert 1 <= st.chunks <= 16 and st.kernel_launches >= st.chunks
    t.close()


def test_row_groups_of_differing_sizes():
    # 1,000-row groups, then 700, then 1,000 again: the table keeps 1,000-row
    # groups of its own, so the statistics are taken after the whole decode
    from golden.segments import concat
    parts = [columns(3_000, 7), columns(700, 8), columns(2_000, 9)]
    images = [write_segment([c.type for c in p], [c.data for c in p], [c.validity for c in p],
                            row_group_rows=1000)[0] for p in parts]
    image = concat(images, len(parts[0]))
    cols = [Column(c.name, c.type, np.concatenate([p[i].data for p in parts]),
                   validity=None if c.validity is None else np.concatenate([p[i].validity for p in parts]),
                   scale=c.scale, precision=c.precision) for i, c in enumerate(parts[0])]
    t = Table.from_segment(image, [Column(c.name, c.type, None, scale=c.scale, precision=c.precision) for c in cols])
    assert t.n_rows == 5_700 and t.load_stats().chunks == 1
    for req in REQUESTS:
        run_and_compare(t, cols, req, ordered=bool(req.order_specs))
    q = try_build_group_topn(t, Request(["region"], [AggSpec("count", None, "c")],
                                        where=[Pred("day", "between", 19000, 19001)]))
    compare_results(q.collect(), oracle.run(oracle.HostTable(cols), Request(["region"], [AggSpec("count", None, "c")],
                    where=[Pred("day", "between", 19000, 19001)])), 1, ordered=False)
    q.close()
    t.close()


@pytest.mark.parametrize("rg", [65_536, 10_000])
def test_statistics_match_a_table_registered_from_columns(rg):
    # the decode's zone maps and sketches equal those taken from resident columns
    cols = columns(400_000, 10)
    seg = from_segment(cols, row_group_rows=rg)
    ref = Table(cols, row_group_rows=rg)
    for c in cols:
        assert seg.ndv(c.name) == ref.ndv(c.name), c.name
    for where in ([Pred("day", "between", 19100, 19150)], [Pred("user", "<", 100)], [Pred("price", ">", 999.5)],
                  [Pred("amount", "between", -10**9, -10**9 + 10**6)]):
        req = Request(["region"], [AggSpec("count", None, "c")], where=where)
        pruned = []
        for t in (seg, ref):
            q = try_build_group_topn(t, req)
            q.collect()
            pruned.append(q.stats().row_groups_pruned)
            q.close()
        assert pruned[0] == pruned[1], where
    seg.close()
    ref.close()
