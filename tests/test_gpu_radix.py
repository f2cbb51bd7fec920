"""The radix-partitioned route (rows scattered by key hash into partitions
whose groups one CTA folds in shared memory) against the oracle: the
composite-key COUNT(DISTINCT) shape it serves by default, with and without a
WHERE, through the distinct partitions and the global set, skewed keys whose
heaviest partition overflows its buffer (resize and rerun), low-cardinality
keys, and the all-zero key."""
import numpy as np
import pytest

from test_gpu_parity import C2_AGGS, FILTER, distinct_cols, filtered_cols, plain_cols, run_both
from thindb_gb300 import abi
from thindb_gb300.engine import AggSpec, Column, Pred, Request, SortSpec

pytestmark = pytest.mark.gpu
RX = abi.FLAG_RADIX
DIST_AGGS = [AggSpec("count", None, "c"), AggSpec("count_distinct", "user_id", "u"),
             AggSpec("sum", "latency_ms", "lat")]


def _radix(st):
    assert st.flags & abi.STAT_RADIX, "the radix route did not run"


@pytest.mark.parametrize("extra", [abi.FLAG_DISTINCT_PARTITION, abi.FLAG_NO_DISTINCT_PARTITION,
                                   abi.FLAG_DISTINCT_PARTITION | abi.FLAG_NO_WARP_COMBINE])
def test_radix_distinct_composite(extra):
    cols = distinct_cols(1_500_000, 60_000)
    _, st = run_both(cols, Request(["region", "url"], DIST_AGGS, flags=RX | extra))
    _radix(st)


def test_radix_distinct_with_where_and_top10():
    cols = distinct_cols(1_000_000, 40_000)
    req = Request(["region", "url"], DIST_AGGS, [SortSpec("u", True)], limit=10,
                  where=[Pred("region", "between", 5, 50)], flags=RX | abi.FLAG_DISTINCT_PARTITION)
    _, st = run_both(cols, req)
    _radix(st)


def test_radix_skewed_keys_overflow_and_rerun():
    # Zipf keys: the heaviest key's partition holds far more than an even share
    cols = filtered_cols(2_000_000, 200_000)
    _, st = run_both(cols, Request(["k"], C2_AGGS, [SortSpec("s", True)], limit=10, flags=RX))
    _radix(st)
    assert st.retries >= 1, "the heaviest partition should have overflowed its first buffer"
    _, st = run_both(cols, Request(["k"], C2_AGGS, where=FILTER, flags=RX))
    _radix(st)


def test_radix_low_cardinality_and_zero_key():
    cols = plain_cols((1 << 20) + 77)
    k = np.asarray(cols[0].data).copy()
    k[::1000] = 0  # the all-zero key lives in the global table's extra slot
    cols[0] = Column("k", abi.BIGINT, k)
    req = Request(["k"], [AggSpec("count", None, "c"), AggSpec("sum", "v", "s"), AggSpec("min", "v", "mn"),
                          AggSpec("max", "v", "mx")], flags=RX)
    _, st = run_both(cols, req)
    _radix(st)


def test_radix_declines_for_wide_keys():
    # a two-word packed key is not a radix shape: the regular scan runs
    n = 200_000
    rng = np.random.default_rng(2)
    cols = [Column("a", abi.BIGINT, rng.integers(0, 1000, n).astype(np.int64)),
            Column("b", abi.BIGINT, rng.integers(0, 1000, n).astype(np.int64))]
    _, st = run_both(cols, Request(["a", "b"], [AggSpec("count", None, "c")], flags=RX))
    assert not st.flags & abi.STAT_RADIX
