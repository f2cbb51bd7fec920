"""The sharded N-GPU design on CPU: two gloo ranks each aggregate their own row
groups (the oracle stands in for the per-GPU operator), exchange partial
group states by key hash, merge per owner and merge the owners' pages on
rank 0 — the answer equals the single-node oracle's."""
import math
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

RG = 65_536
N = 7 * RG + 1234  # ragged last row group


def _cols():
    from thindb_gb300 import abi
    from thindb_gb300.engine import Column

    rng = np.random.default_rng(77)
    k = (rng.zipf(1.3, N) % 5000).astype(np.int64)
    g = rng.integers(-3, 9, N).astype(np.int32)
    amount = rng.integers(-10_000, 1_000_000, N).astype(np.int64)
    d = rng.integers(18_000, 18_365, N).astype(np.int32)
    u = rng.integers(0, 3000, N).astype(np.int32)
    v = rng.normal(size=N)
    v_ok = rng.random(N) > 0.1
    u_ok = rng.random(N) > 0.05
    return [Column("k", abi.BIGINT, k), Column("g", abi.INT, g), Column("amount", abi.DECIMAL64, amount, scale=2),
            Column("d", abi.DATE, d), Column("u", abi.INT, u, validity=u_ok), Column("k32", abi.INT, k.astype(np.int32)),
            Column("v", abi.DOUBLE, v, validity=v_ok)]


def _subset(cols, rows):
    from thindb_gb300.engine import Column

    return [Column(c.name, c.type, np.ascontiguousarray(c.data[rows]), scale=c.scale,
                   validity=None if c.validity is None else np.ascontiguousarray(c.validity[rows])) for c in cols]


def _requests():
    from thindb_gb300.engine import AggSpec, HavingSpec, Pred, Request, SortSpec

    c2 = [AggSpec("count", None, "c"), AggSpec("sum", "amount", "s"), AggSpec("avg", "amount", "a")]
    return [
        Request(["k"], c2, [SortSpec("s", True)], limit=10, where=[Pred("d", "between", 18_050, 18_086)]),
        Request(["g", "k32"], [AggSpec("count", None, "c"), AggSpec("min", "v", "mn"), AggSpec("max", "amount", "mx"),
                               AggSpec("count_distinct", "u", "du")], [SortSpec("g"), SortSpec("k32")], limit=50, offset=7),
        Request(["g"], [AggSpec("count", None, "c"), AggSpec("sum", "amount", "s")], [SortSpec("g", True)],
                having=[HavingSpec("c", ">", 40_000)]),
        Request(["g"], [AggSpec("avg", "v", "av"), AggSpec("count", "v", "cv"), AggSpec("count_distinct", "u", "du")],
                [SortSpec("du", True), SortSpec("g")]),
        # a page without ORDER BY is taken in packed-key order: negative g and
        # the nullable u's validity bit decide it
        Request(["g", "u"], [AggSpec("count", None, "c")], limit=40, offset=3),
    ]


def _types(cols, req):
    from thindb_gb300 import abi

    by = {c.name: c for c in cols}
    key_types = [by[k].type for k in req.group_cols]
    key_null = [by[k].validity is not None for k in req.group_cols]
    agg_types = {a.col: (by[a.col].type, by[a.col].scale or 0) for a in req.aggs if a.col}
    return key_types, key_null, agg_types


def _as_rows(res, req):
    from thindb_gb300.shard import _cell, _rows

    keys = _rows(res, list(req.group_cols))
    aggs = [[_cell(*res[a.as_], i) for a in req.aggs] for i in range(len(keys))]
    return keys, aggs


def _close(a, b):
    if a is None or b is None:
        return a is b
    if isinstance(a, float) or isinstance(b, float):
        return (math.isnan(a) and math.isnan(b)) or a == pytest.approx(b, rel=1e-12, abs=1e-12)
    return a == b


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle
    from thindb_gb300.shard import sharded_group_by

    cols = _cols()
    rgs = np.arange((N + RG - 1) // RG)
    mine = np.concatenate([np.arange(r * RG, min(N, (r + 1) * RG)) for r in rgs[rank::world]])
    host = oracle.HostTable(_subset(cols, mine), RG)
    results = []
    for req in _requests():
        kt, kn, at = _types(cols, req)
        results.append(sharded_group_by(req, lambda r: oracle.run(host, r), kt, kn, at, dist))
    if rank == 0:
        out[0] = results
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_aggregation_matches_one_node(world):
    import oracle

    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        got = out[0]
    cols = _cols()
    host = oracle.HostTable(cols, RG)
    for req, res in zip(_requests(), got):
        keys, aggs = _as_rows(oracle.run(host, req), req)
        assert res["keys"] == keys, req
        assert len(res["aggs"]) == len(aggs)
        for ga, wa in zip(res["aggs"], aggs):
            assert all(_close(x, y) for x, y in zip(ga, wa)), (req, ga, wa)


def test_single_rank_is_the_plain_answer():
    import oracle
    from thindb_gb300.shard import sharded_group_by

    cols = _cols()
    host = oracle.HostTable(cols, RG)
    for req in _requests():
        kt, kn, at = _types(cols, req)
        res = sharded_group_by(req, lambda r: oracle.run(host, r), kt, kn, at)
        keys, aggs = _as_rows(oracle.run(host, req), req)
        assert res["keys"] == keys
        for ga, wa in zip(res["aggs"], aggs):
            assert all(_close(x, y) for x, y in zip(ga, wa)), (req, ga, wa)
