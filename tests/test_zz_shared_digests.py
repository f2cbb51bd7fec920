"""Hashed group keys under shared digests (after thinDB's
tests/integration/exact_group_keys_test.zig, which narrows the key digest
with THINDB_V2_KEY_DIGEST_BITS): distinct keys that share a digest each keep
a group of their own, decided by the exact check of the key's parts against
the group's representative row.  The digest width is process-wide state, so
this file runs last and puts it back."""
import numpy as np
import pytest

from test_gpu_hashed import AGGS, check, table
from thindb_gb300 import abi
from thindb_gb300.engine import AggSpec, Column, Pred, Request, set_digest_bits

pytestmark = pytest.mark.gpu


def test_exact_check_decides_under_shared_digests():
    """The digest keeps 8 bits (3,000 strings over 256 digests) and 6 bits
    for integer keys over 128 bits; every result still equals the oracle's,
    which compares keys exactly."""
    cols = table(200_000, 3_000, 7, nullable=True)
    rng = np.random.default_rng(8)
    n = 100_000
    base = rng.integers(0, 2000, n)
    wide = [Column("a", abi.BIGINT, (base * 7919).astype(np.int64)), Column("b", abi.BIGINT, (base % 97).astype(np.int64)),
            Column("c", abi.BIGINT, (-base).astype(np.int64)), Column("v", abi.INT, rng.integers(-9, 9, n).astype(np.int32))]
    try:
        set_digest_bits(8)
        check(cols, Request(["s"], AGGS))
        check(cols, Request(["r", "s"], [AggSpec("count", None, "c"), AggSpec("count_distinct", "u", "du")],
                            where=[Pred("r", "between", 2, 9)]))
        set_digest_bits(6)
        _, st = check(wide, Request(["a", "b", "c"], [AggSpec("count", None, "n"), AggSpec("sum", "v", "s")]))
        assert st.groups == len(np.unique(base))
    finally:
        set_digest_bits(0)
