"""The scan loop with one inlined fold call site (TGPU_FLAG_INLINE_FOLD)
against the oracle: survivor gather under a WHERE, in-place folds without
one (shared-memory resident route and global table), COUNT(DISTINCT) through
the pair partitions, a partial last chunk, and the count sketch's filter pass."""
import pytest

from test_gpu_parity import C2_AGGS, FILTER, distinct_cols, filtered_cols, plain_cols, run_both
from thindb_gb300 import abi
from thindb_gb300.engine import AggSpec, Request, SortSpec

pytestmark = pytest.mark.gpu
IN = abi.FLAG_INLINE_FOLD


@pytest.mark.parametrize("extra", [0, abi.FLAG_NO_WARP_COMBINE, abi.FLAG_FORCE_GLOBAL, abi.FLAG_DENSE_SCAN])
def test_inline_filtered(extra):
    cols = filtered_cols(2_000_000 + 13, 200_000)
    run_both(cols, Request(["k"], C2_AGGS, [SortSpec("s", True)], limit=10, where=FILTER, flags=IN | extra))
    run_both(cols, Request(["k"], C2_AGGS, where=FILTER, flags=IN | extra))


@pytest.mark.parametrize("extra", [0, abi.FLAG_FORCE_GLOBAL])
def test_inline_plain(extra):
    cols = plain_cols((1 << 20) + 333)
    req = Request(["k"], [AggSpec("count", None, "c"), AggSpec("sum", "v", "s"), AggSpec("min", "v", "mn"),
                          AggSpec("max", "v", "mx")], flags=IN | extra)
    _, st = run_both(cols, req)
    assert st.groups == 1024


def test_inline_distinct_partitions():
    cols = distinct_cols(1_000_000, 50_000)
    req = Request(["region", "url"], [AggSpec("count", None, "c"), AggSpec("count_distinct", "user_id", "u"),
                                      AggSpec("sum", "latency_ms", "lat")], flags=IN | abi.FLAG_DISTINCT_PARTITION)
    _, st = run_both(cols, req)
    assert st.flags & abi.STAT_DISTINCT_PARTITION


def test_inline_count_sketch():
    from test_gpu_sketch import run_both as run_sketch, topcount, zipf_cols

    cols = zipf_cols(3_000_000, 1_000_000)
    _, st = run_sketch(cols, topcount(10, flags=abi.FLAG_COUNT_SKETCH | IN))
    assert st.flags & abi.STAT_COUNT_SKETCH
