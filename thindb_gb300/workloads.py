"""Synthetic query mixes for the batched and served modes.

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

from . import datagen
from .engine import AggSpec, Pred, Request, SortSpec

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
