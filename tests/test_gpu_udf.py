"""A request naming a user-defined aggregate: thinDB's silo runs registered
aggregates on the host (v2_shape_group_topn.zig:86, :170-177), so this
operator declines one that is registered and refuses an unknown name."""
import numpy as np
import pytest

from thindb_gb300 import abi, engine
from thindb_gb300.engine import AggSpec, Column, EngineError, Request, Table, try_build_group_topn

pytestmark = pytest.mark.gpu


def test_registered_aggregate_declines_unknown_is_refused():
    rng = np.random.default_rng(1)
    t = Table([Column("k", abi.BIGINT, rng.integers(0, 10, 10_000).astype(np.int64)),
               Column("v", abi.DOUBLE, rng.random(10_000))])
    req = Request(["k"], [AggSpec("count", None, "c"), AggSpec("udf", "v", "g", udf_name="geo_mean")])
    with pytest.raises(EngineError) as e:
        try_build_group_topn(t, req)
    assert e.value.status == abi.ERR_INVALID_ARGUMENT
    engine.register_aggregate("geo_mean")
    try:
        assert try_build_group_topn(t, req) is None  # declined: the caller's executor runs it
        # the same table and a built-in request still run here
        q = try_build_group_topn(t, Request(["k"], [AggSpec("count", None, "c")]))
        assert q is not None and int(q.collect()["c"][0].sum()) == 10_000
        q.close()
    finally:
        engine.unregister_aggregate("geo_mean")
    t.close()
