"""Sharded grouped aggregation over N ranks: the host side of the N-GPU design.

Each rank runs the plain operator over its own row groups and returns
partial group states (COUNT, SUM, MIN, MAX; AVG as its SUM and count); one
hash exchange sends every group's partial to its owner rank (a hash of the
group key modulo N); each owner merges what it owns and keeps its best
OFFSET + LIMIT groups; rank 0 merges the owners' pages into the answer.
COUNT(DISTINCT) cannot merge counts, so it shards the distinct (group,
value) pairs by their own hash: each owner counts the pairs it alone holds
and the per-group counts add up.

Limits: COUNT(DISTINCT) over an integer or DICT32 column whose bits and the
key's fit the packed 128 (its pairs are groups of the operator), and AVG
over an integer column whose per-shard sum fits BIGINT (the shard's SUM
output wraps there).

thinDB runs on one node; the owner role here is the one its silo buckets
play (silo_group_core.zig runSiloGrid :11493, rows routed to buckets by the
key hash :5226-5235, each bucket folded by one worker).  The per-rank
aggregation is any engine that takes a Request and returns
{column: (values, validity)}; the exchange goes through torch.distributed
(object collectives, so gloo on CPU works as well as NCCL).  Result
semantics follow the single-node operator: ORDER BY keys then the packed
key ascending (rowOrderBefore, v2_shape_group_topn.zig:1327-1335), NULLs
first, AVG = f64(sum) / f64(count) / 10^scale (avgValue :1438-1446), SUM
over integers wrapping to BIGINT (aggregate.zig:3700-3742).
"""
from __future__ import annotations

import math
from dataclasses import replace
from typing import Callable, Optional, Sequence

import numpy as np

from . import abi
from .engine import AggSpec, Request

TYPE_BITS = {abi.BOOLEAN: 8, abi.TINYINT: 8, abi.SMALLINT: 16, abi.INT: 32, abi.DATE: 32, abi.DICT32: 32,
             abi.BIGINT: 64, abi.DATETIME: 64, abi.DECIMAL64: 64}
MASK64 = (1 << 64) - 1


def _wrap64(v: int) -> int:
    v &= MASK64
    return v - (1 << 64) if v >> 63 else v


def packed_key(values: Sequence, types: Sequence[int], nullable: Sequence[bool]) -> int:
    """The operator's packed key: parts LSB-first, a nullable part's validity
    bit right above its payload (v2_shape_group_topn.zig KeyLayout :105-119)."""
    key, off = 0, 0
    for v, t, nl in zip(values, types, nullable):
        bits = TYPE_BITS[t]
        if v is not None:
            key |= ((int(v) & ((1 << bits) - 1)) | ((1 << bits) if nl else 0)) << off
        off += bits + (1 if nl else 0)
    return key


def _owner(key: tuple, world: int) -> int:
    h = 0x9E3779B97F4A7C15
    for v in key:
        x = (h ^ (0 if v is None else (int(v) & MASK64))) & MASK64
        x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9 & MASK64
        x = (x ^ (x >> 27)) * 0x94D049BB133111EB & MASK64
        h = x ^ (x >> 31)
    return h % world


def _cell(vals: np.ndarray, ok: Optional[np.ndarray], i: int):
    if ok is not None and not ok[i]:
        return None
    v = vals[i]
    if vals.ndim == 2:  # DECIMAL128: (lo, hi)
        return (int(v[1]) << 64) | (int(v[0]) & MASK64)
    return v.item()


# ----------------------------------------------------------- partial plan --

def partial_requests(req: Request) -> tuple[Request, list[Request]]:
    """(the per-shard request of mergeable states, one per-shard pair request
    per COUNT(DISTINCT)): no ORDER BY, LIMIT, OFFSET or HAVING; AVG becomes
    its SUM and COUNT(col); a COUNT(DISTINCT col) becomes GROUP BY (keys...,
    col) over the same WHERE, whose groups are the shard's distinct pairs."""
    aggs: list[AggSpec] = []
    for i, a in enumerate(req.aggs):
        if a.func == "avg":
            aggs += [AggSpec("sum", a.col, f"__s{i}"), AggSpec("count", a.col, f"__n{i}")]
        elif a.func != "count_distinct":
            aggs.append(AggSpec(a.func, a.col, f"__p{i}"))
    if not aggs:
        aggs.append(AggSpec("count", None, "__rows"))
    base = replace(req, aggs=aggs, order_specs=(), limit=None, offset=0, having=())
    pairs = [replace(req, group_cols=list(req.group_cols) + [a.col], aggs=[AggSpec("count", None, "__c")],
                     order_specs=(), limit=None, offset=0, having=())
             for a in req.aggs if a.func == "count_distinct"]
    return base, pairs


def _rows(res: dict, keys: Sequence[str]) -> list[tuple]:
    n = len(next(iter(res.values()))[0]) if res else 0
    return [tuple(_cell(*res[k], i) for k in keys) for i in range(n)]


# ------------------------------------------------------------- the merge --

def _merge_state(func: str, a, b):
    if a is None:
        return b
    if b is None:
        return a
    if func in ("count", "sum"):
        return a + b
    # MIN / MAX: a NaN anywhere makes the result NaN, as on one node
    if (isinstance(a, float) and math.isnan(a)) or (isinstance(b, float) and math.isnan(b)):
        return math.nan
    return min(a, b) if func == "min" else max(a, b)


def _exchange(items: list, world: int, key_of: Callable, dist) -> list:
    """Every item to its owner: object all-gather, keep what this rank owns."""
    if dist is None or world == 1:
        return items
    parts: list = [None] * world
    dist.all_gather_object(parts, items)
    me = dist.get_rank()
    return [it for p in parts for it in p if _owner(key_of(it), world) == me]


def sharded_group_by(req: Request, run_shard: Callable[[Request], dict], key_types: Sequence[int],
                     key_nullable: Sequence[bool], agg_types: dict, dist=None) -> Optional[dict]:
    """The answer of `req` over all ranks' shards, on rank 0 (None elsewhere).

    run_shard(request) runs a request over this rank's rows and returns
    {column: (values, validity)}; key_types / key_nullable describe the group
    columns; agg_types maps an aggregate's input column to (type, scale) for
    output typing (DECIMAL SUM stays exact, AVG divides by 10^scale)."""
    world = dist.get_world_size() if dist is not None and dist.is_initialized() else 1
    rank = dist.get_rank() if world > 1 else 0
    keys = list(req.group_cols)
    base, pair_reqs = partial_requests(req)

    # 1. partial states, keyed by group, to their owners
    res = run_shard(base)
    items = [(kt, {a.as_: _cell(*res[a.as_], i) for a in base.aggs}) for i, kt in enumerate(_rows(res, keys))]
    owned = _exchange(items, world, lambda it: it[0], dist)
    groups: dict = {}
    funcs = {a.as_: a.func for a in base.aggs}
    for kt, st in owned:
        cur = groups.get(kt)
        if cur is None:
            groups[kt] = dict(st)
        else:
            for name, v in st.items():
                cur[name] = _merge_state(funcs[name], cur[name], v)

    # 2. COUNT(DISTINCT): distinct pairs to the pair's owner, counts to the group's
    for j, pr in enumerate(pair_reqs):
        pairs = [t for t in _rows(run_shard(pr), list(pr.group_cols)) if t[-1] is not None]  # NULLs never count
        mine = set(_exchange(pairs, world, lambda t: t, dist))
        counts: dict = {}
        for t in mine:
            counts[t[:-1]] = counts.get(t[:-1], 0) + 1
        owned_counts = _exchange(list(counts.items()), world, lambda it: it[0], dist)
        for kt, c in owned_counts:
            groups.setdefault(kt, {})
            groups[kt][f"__d{j}"] = groups[kt].get(f"__d{j}", 0) + c

    # 3. final values, HAVING, this owner's page
    rows = []
    for kt, st in groups.items():
        out, dj = [], 0
        for i, a in enumerate(req.aggs):
            if a.func == "avg":
                s, n = st.get(f"__s{i}"), st.get(f"__n{i}") or 0
                t, scale = agg_types.get(a.col, (abi.BIGINT, 0))
                if s is None or n == 0:
                    out.append(None)
                elif t in (abi.FLOAT, abi.DOUBLE):
                    out.append(s / n)
                else:
                    out.append(float(s) / float(n) / (10.0 ** scale))
            elif a.func == "count_distinct":
                out.append(st.get(f"__d{dj}", 0))
                dj += 1
            else:
                v = st.get(f"__p{i}")
                t, _ = agg_types.get(a.col, (abi.BIGINT, 0))
                if a.func == "sum" and v is not None and t not in (abi.FLOAT, abi.DOUBLE, abi.DECIMAL64):
                    v = _wrap64(v)
                out.append(0 if (v is None and a.func == "count") else v)
        rows.append((kt, packed_key(kt, key_types, key_nullable), out))
    names = [a.as_ for a in req.aggs]
    for h in req.having:
        rows = [r for r in rows if _having(r[2][names.index(h.agg)], h.op, h.value)]
    rows = _page(rows, req, keys, names, keep_offset=True)

    # 4. rank 0 merges the owners' pages
    if world > 1:
        parts: list = [None] * world
        dist.all_gather_object(parts, rows)
        rows = [r for p in parts for r in p]
    if rank != 0:
        return None
    rows = _page(rows, req, keys, names, keep_offset=False)
    return {"keys": [r[0] for r in rows], "aggs": [r[2] for r in rows]}


def _having(v, op: str, x) -> bool:
    if v is None:
        return False
    return {"=": v == x, "!=": v != x, "<": v < x, "<=": v <= x, ">": v > x, ">=": v >= x}[op]


def _order_value(v):
    # NULLs first; NaN orders as the largest value
    if v is None:
        return (0, 0)
    if isinstance(v, float) and math.isnan(v):
        return (2, 0)
    return (1, v)


def _page(rows: list, req: Request, keys: list, names: list, keep_offset: bool) -> list:
    """ORDER BY then the packed key; an owner keeps OFFSET + LIMIT rows, the
    final merge applies OFFSET and LIMIT."""
    import functools

    def cmp(x, y):
        for s in req.order_specs:
            if s.col in keys:
                a, b = x[0][keys.index(s.col)], y[0][keys.index(s.col)]
            else:
                a, b = x[2][names.index(s.col)], y[2][names.index(s.col)]
            a, b = _order_value(a), _order_value(b)
            if a != b:
                return (-1 if a < b else 1) * (-1 if s.desc else 1)
        return -1 if x[1] < y[1] else (1 if x[1] > y[1] else 0)

    rows = sorted(rows, key=functools.cmp_to_key(cmp))
    if req.limit is None:
        return rows if keep_offset else rows[req.offset:]
    if keep_offset:
        return rows[:req.offset + req.limit]
    return rows[req.offset:req.offset + req.limit]
