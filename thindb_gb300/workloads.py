"""The benchmark workloads: their tables and queries.

table_inputs(workload, n) / workload_request(workload): the tables and
queries of the plain (16M rows, BIGINT key over 1,024 values), filtered
(100M rows, Zipf key, DECIMAL amount, DATE filter), distinct (200M rows,
(SMALLINT, DICT32) key, COUNT(DISTINCT)) and batched (the filtered table plus
three INT keys) workloads, generated by the seeded native generator.

Synthetic query mixes for the batched and served modes:

batched_requests(n, seed): n GROUP BY queries over the batched table (the
filtered table's k / amount / d plus INT keys k10, k1k, k1m with 10, 1,000
and 1,000,000 uniform values).  Per query, drawn from a generator seeded
with (seed, query index):
  * selectivity s log-uniform in [0.1%, 50%]; s >= 2/365 becomes a DATE window
    of round(s * 365) days, smaller s a range of width round(s * 1e6) on the
    uniform k1m column (a 365-day DATE window cannot express 0.1%);
  * the group key: one of k (Zipf over 10M), k10, k1k, k1m;
  * a non-empty random subset of COUNT(*), SUM(amount), MIN(amount),
    MAX(amount);
  * ORDER BY the first aggregate DESC LIMIT 10 (ties broken by the key).
"""
from __future__ import annotations

import math

import numpy as np

from . import abi, datagen
from .engine import AggSpec, Column, Pred, Request, SortSpec

# ------------------------------------------------------------------ tables --

def table_inputs(workload: str, n: int, pinned: bool = True) -> list:
    """Host columns of a workload's table: (name, type, tensor, scale) tuples
    (pinned torch tensors when asked)."""
    import torch

    def buf(count, dtype):
        return torch.empty(count, dtype=dtype, pin_memory=pinned)

    if workload == "topcount":
        return table_inputs("filtered", n, pinned)[:1]
    if workload in ("filtered", "batched"):
        k, a, d = buf(n, torch.int64), buf(n, torch.int64), buf(n, torch.int32)
        datagen.filtered_into(n, 2, datagen.FILTERED_KEYS, k.data_ptr(), a.data_ptr(), d.data_ptr())
        cols = [("k", abi.BIGINT, k, 0), ("amount", abi.DECIMAL64, a, 2), ("d", abi.DATE, d, 0)]
        if workload == "batched":
            k10, k1k, k1m = (buf(n, torch.int32) for _ in range(3))
            datagen.lib().tdg_extra_keys(n, 2, k10.data_ptr(), k1k.data_ptr(), k1m.data_ptr(), 0)
            cols += [("k10", abi.INT, k10, 0), ("k1k", abi.INT, k1k, 0), ("k1m", abi.INT, k1m, 0)]
        return cols
    if workload == "plain":
        k, v = buf(n, torch.int64), buf(n, torch.int32)
        datagen.lib().tdg_plain(n, 1, k.data_ptr(), v.data_ptr(), 0)
        return [("k", abi.BIGINT, k, 0), ("v", abi.INT, v, 0)]
    if workload == "distinct":
        r, u, us, lat = buf(n, torch.int16), buf(n, torch.int32), buf(n, torch.int64), buf(n, torch.float64)
        datagen.lib().tdg_distinct(n, 3, datagen.DISTINCT_USERS, r.data_ptr(), u.data_ptr(), us.data_ptr(),
                                   lat.data_ptr(), 0)
        return [("region", abi.SMALLINT, r, 0), ("url", abi.DICT32, u, 0), ("user_id", abi.BIGINT, us, 0),
                ("latency_ms", abi.DOUBLE, lat, 0)]
    raise ValueError(f"unknown workload {workload!r}")


def columns(inputs, ndv=None) -> list:
    """engine.Column objects over table_inputs() tuples."""
    return [Column(nm, ty, t, scale=sc, ndv_hint=(ndv or {}).get(nm, 0)) for nm, ty, t, sc in inputs]


def workload_request(workload: str, flags: int = 0, stream: int = 0) -> Request:
    """The query a single-query workload runs."""
    if workload == "filtered":
        return Request(["k"], [AggSpec("count", None, "c"), AggSpec("sum", "amount", "s"),
                               AggSpec("avg", "amount", "a")], [SortSpec("s", True)], limit=10,
                       where=[Pred("d", "between", datagen.FILTER_LO, datagen.FILTER_HI)], flags=flags, stream=stream)
    if workload == "topcount":
        # the filtered table's Zipf key, every row: the heaviest ten groups
        return Request(["k"], [AggSpec("count", None, "c")], [SortSpec("c", True)], limit=10, flags=flags,
                       stream=stream)
    if workload == "plain":
        return Request(["k"], [AggSpec("count", None, "c"), AggSpec("sum", "v", "s"), AggSpec("min", "v", "mn"),
                               AggSpec("max", "v", "mx")], flags=flags, stream=stream)
    if workload == "distinct":
        return Request(["region", "url"], [AggSpec("count", None, "c"), AggSpec("count_distinct", "user_id", "u"),
                                           AggSpec("sum", "latency_ms", "lat")], flags=flags, stream=stream)
    raise ValueError(f"unknown workload {workload!r}")


# ------------------------------------------------------------ query mixes --

KEYS = ["k", "k10", "k1k", "k1m"]
AGGS = [("count", None), ("sum", "amount"), ("min", "amount"), ("max", "amount")]


def batched_request(seed: int, i: int, flags: int = 0) -> Request:
    rng = np.random.default_rng([seed, i])
    s = math.exp(rng.uniform(math.log(0.001), math.log(0.5)))
    if s >= 2.0 / 365.0:
        days = max(1, int(round(s * 365)))
        start = int(rng.integers(0, 365 - days + 1))
        where = [Pred("d", "between", datagen.DATE_BASE + start, datagen.DATE_BASE + start + days - 1)]
    else:
        width = max(1, int(round(s * 1_000_000)))
        start = int(rng.integers(0, 1_000_000 - width + 1))
        where = [Pred("k1m", "between", start, start + width - 1)]
    key = KEYS[int(rng.integers(0, len(KEYS)))]
    mask = int(rng.integers(1, 16))
    aggs = [AggSpec(f, c, f"{f}_{c or 'star'}") for b, (f, c) in enumerate(AGGS) if mask >> b & 1]
    return Request([key], aggs, [SortSpec(aggs[0].as_, True)], limit=10, where=where, flags=flags)


def batched_requests(n: int = 256, seed: int = 4, flags: int = 0) -> list:
    return [batched_request(seed, i, flags) for i in range(n)]


# Served mix: tables are [plain, filtered, distinct, batched]; shapes come from
# the filtered, distinct and batched families (one third each).
SERVED_TABLES = ["plain", "filtered", "distinct", "batched"]


def served_request(seed: int, i: int) -> tuple:
    """(table index, Request) of served request template i."""
    rng = np.random.default_rng([seed, 7, i])
    fam = i % 3
    if fam == 0:  # filtered DECIMAL top-10 over a random DATE window of 1-36 days
        days = int(rng.integers(1, 37))
        start = int(rng.integers(0, 365 - days + 1))
        where = [Pred("d", "between", datagen.DATE_BASE + start, datagen.DATE_BASE + start + days - 1)]
        return 1, Request(["k"], [AggSpec("count", None, "c"), AggSpec("sum", "amount", "s"),
                                  AggSpec("avg", "amount", "a")], [SortSpec("s", True)], limit=10, where=where)
    if fam == 1:  # composite key + COUNT(DISTINCT) for one region, top-10 by distinct users
        r = int(rng.integers(0, 64))
        return 2, Request(["region", "url"], [AggSpec("count", None, "c"), AggSpec("count_distinct", "user_id", "u"),
                                              AggSpec("sum", "latency_ms", "lat")], [SortSpec("u", True)], limit=10,
                          where=[Pred("region", "=", r)])
    return 3, batched_request(seed, 100_000 + i)


def served_mix(n: int = 96, seed: int = 5) -> list:
    return [served_request(seed, i) for i in range(n)]
