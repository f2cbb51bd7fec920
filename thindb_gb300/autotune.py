"""Autotuner: measures the engine's settings per request shape and writes the
tuning table the library installs at load (thindb_gb300/tuning/gb300.json).

thinDB fixes its engine knobs as defaults overridable from the environment
(v2_group_topn_engine.zig:25-33: DOP, bucket count, scan tile row groups,
route block rows, raw chunk rows; :521-626 paramsFromEnv).  This engine's
knobs are

    chunk_rows      rows per warp chunk (the scan tile)
    cache_slots     shared-memory table slots per CTA, -1 = none (the
                    pre-aggregation tier that takes the place of the bucket
                    partition: hot keys fold on chip)
    table_load_pct  global group-table load target (table sizing)
    groups_shift    size the group table for (estimated groups >> shift): the
                    estimate from NDV sketches and selectivity can be far above
                    the real count (a table that proves too small regrows)
    flags           scan mode: the staged scan (column tiles through a
                    shared-memory ring of bulk copies), dense loads or survivor
                    gathers; the in-warp pre-combine on or off; which L2
                    prefetches run (table slots, next chunks, distinct entries);
                    the split scan off; the radix-partitioned route (its
                    partition bits follow the group estimate, so groups_shift
                    moves them too)

For each shape class (tgpu_shape: key width, fold signature, aggregate count,
distinct, selectivity class, group-count class, batched or not) a coordinate
descent over the knobs keeps the setting with the lowest median device time
whose results equal the built-in setting's (integers and keys bit for bit,
FP64 sums within 1e-12 relative).  A batch is tuned as a whole (one setting
for all of its queries), and every shape in it gets that setting.

    python -m thindb_gb300.autotune [--out PATH] [--workloads plain,filtered,distinct,batched]
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import statistics
import sys
import time

import numpy as np

from . import abi, datagen, workloads
from .engine import EngineError, QueryBatch, Request, Table, request_shape, try_build_group_topn
from .engine import lib as engine_lib
from .engine import tuning_entries as engine_tuning_entries

KNOBS = {
    "flags": [0, abi.FLAG_STAGED_SCAN, abi.FLAG_DENSE_SCAN, abi.FLAG_GATHER_SCAN, abi.FLAG_QUEUE_SCAN,
              abi.FLAG_NO_WARP_COMBINE,
              abi.FLAG_NO_PREFETCH, abi.FLAG_NO_CHUNK_PREFETCH, abi.FLAG_NO_PREFETCH | abi.FLAG_NO_CHUNK_PREFETCH,
              abi.FLAG_DISTINCT_PREFETCH, abi.FLAG_NO_DISTINCT_PARTITION,
              abi.FLAG_NO_SPLIT | abi.FLAG_NO_PREFETCH | abi.FLAG_NO_CHUNK_PREFETCH, abi.FLAG_RADIX],
    "chunk_rows": [0, 512, 1024, 2048, 4096],
    "cache_slots": [0, -1, 256, 1024, 4096],
    "table_load_pct": [0, 25, 70],
    "groups_shift": [0, 2, 3, 4],
}
DEFAULT = {"flags": 0, "chunk_rows": 0, "cache_slots": 0, "table_load_pct": 0, "groups_shift": 0}
GAIN = 0.97  # a setting must beat the current best by 3% to replace it


def _install(shapes: list, knobs: dict) -> None:
    """Make `knobs` the tuning-table entry of every shape in `shapes` (only)."""
    arr = (abi.Tuning * max(1, len(shapes)))()
    for i, sh in enumerate(shapes):
        for k, v in sh.items():
            setattr(arr[i].shape, k, int(v))
        for k, v in knobs.items():
            setattr(arr[i], k, int(v))
    engine_lib().tgpu_tuning_set(arr, len(shapes))


def _timed(req: Request) -> Request:
    return dataclasses.replace(req, flags=req.flags | abi.FLAG_TIMING)


def _same(a: dict, b: dict) -> bool:
    """Results equal: exact, except FP64 values within 1e-12 relative."""
    if a.keys() != b.keys():
        return False
    for name in a:
        va, oka = a[name]
        vb, okb = b[name]
        if (oka is None) != (okb is None) or (oka is not None and not np.array_equal(oka, okb)):
            return False
        if va.shape != vb.shape:
            return False
        if va.dtype.kind == "f":
            if not np.allclose(va, vb, rtol=1e-12, atol=0.0, equal_nan=True):
                return False
        elif not np.array_equal(va, vb):
            return False
    return True


def _sorted_result(res: dict) -> dict:
    """A result in a canonical row order (all-groups results come in table order)."""
    keys = [np.asarray(v).reshape(len(v), -1) for v, _ in res.values()]
    if not keys or len(keys[0]) == 0:
        return res
    order = np.lexsort(tuple(k[:, j] for k in reversed(keys) for j in reversed(range(k.shape[1]))))
    return {n: (np.asarray(v)[order], None if ok is None else np.asarray(ok)[order]) for n, (v, ok) in res.items()}


def _fatal(e: Exception) -> bool:
    """A CUDA error can leave the context unusable: tuning stops there
    instead of rejecting every later candidate."""
    return isinstance(e, EngineError) and e.status in (abi.ERR_CUDA, abi.ERR_NO_DEVICE)


def time_query(table: Table, req: Request, knobs: dict, reps: int):
    """(median device ms, result) of `req` run with `knobs` as its shape's
    tuning entry; None if it fails."""
    _install([request_shape(table, req)], knobs)
    try:
        q = try_build_group_topn(table, _timed(req))
    except Exception as e:
        if _fatal(e):
            raise
        return None
    if q is None:
        return None
    try:
        times = []
        res = None
        for i in range(reps + 1):
            q.execute()
            q.synchronize()
            if i:
                times.append(q.stats().total_ms)
            res = q.collect()
        return statistics.median(times), _sorted_result(res)
    except Exception as e:
        if _fatal(e):
            raise
        return None
    finally:
        q.close()


def time_batch(table: Table, reqs: list, knobs: dict, reps: int, stream: int):
    shapes = {json.dumps(request_shape(table, r, batched=True), sort_keys=True) for r in reqs}
    _install([json.loads(x) for x in sorted(shapes)], knobs)
    try:
        b = QueryBatch(table, [_timed(r) for r in reqs], graph=True, stream=stream)
    except Exception as e:
        if _fatal(e):
            raise
        return None
    try:
        times = []
        for i in range(reps + 1):
            b.execute()
            b.synchronize()
            if i:
                times.append(b.stats().total_ms)
        res = [_sorted_result(b.collect(i)) for i in range(len(reqs))]
        return statistics.median(times), res
    except Exception as e:
        if _fatal(e):
            raise
        return None
    finally:
        b.close()


GRID = [(c, k, f) for c in (512, 1024, 2048, 4096) for k in (0, -1, 256, 1024)
        for f in (0, abi.FLAG_NO_PREFETCH | abi.FLAG_NO_CHUNK_PREFETCH)]


def descend(measure, same, log=print, rounds: int = 3, starts=()):
    """A joint grid over rows per chunk x shared-table slots x prefetching
    (the knobs interact), then coordinate descent over KNOBS from
    the best of that, the built-in setting and `starts` (e.g. the installed
    table's entry for the shape)."""
    base = measure(DEFAULT)
    if base is None:
        raise RuntimeError("the built-in setting failed")
    best, (best_ms, ref) = dict(DEFAULT), base
    default_ms = best_ms
    log(f"  built-in: {best_ms:.3f} ms")
    for st in list(starts) + [dict(DEFAULT, chunk_rows=c, cache_slots=k, flags=f) for c, k, f in GRID]:
        r = measure(st)
        if r is not None and same(r[1], ref):
            log(f"  start {st}: {r[0]:.3f} ms")
            if r[0] < best_ms:
                best, best_ms = dict(st), r[0]
    for _ in range(rounds):
        improved = False
        for knob, values in KNOBS.items():
            for v in values:
                if v == best[knob]:
                    continue
                cand = dict(best, **{knob: v})
                r = measure(cand)
                if r is None or not same(r[1], ref):
                    log(f"  {cand}: rejected")
                    continue
                log(f"  {cand}: {r[0]:.3f} ms")
                if r[0] < best_ms * GAIN:
                    best, best_ms, improved = cand, r[0], True
        if not improved:
            break
    return best, default_ms, best_ms


def _incumbent(shape: dict, table: list) -> list:
    """The installed table's setting for `shape`, as a starting point."""
    for e in table:
        if e["shape"] == shape:
            return [{k: int(e.get(k, 0)) for k in DEFAULT}]
    return []


def tune_served(scale: float, stream: int, reps: int, log=print, previous=(), max_shapes: int = 12) -> list:
    """Entries for the served mix's shapes (single executions: the continuous
    server runs short backlogs as separate queries): the most frequent shapes,
    each tuned on its first request."""
    sizes = {"plain": datagen.PLAIN_ROWS, "filtered": datagen.FILTERED_ROWS, "distinct": datagen.DISTINCT_ROWS,
             "batched": datagen.FILTERED_ROWS}
    tables = []
    for wl in workloads.SERVED_TABLES:
        inputs = workloads.table_inputs(wl, max(1 << 16, int(sizes[wl] * scale)), pinned=True)
        tables.append(Table(workloads.columns(inputs), compute_ndv=True, stream=stream))
        del inputs
    entries = []
    try:
        by_shape = {}
        for ti, req in workloads.served_mix(96, seed=5):
            req.stream = stream
            key = json.dumps(request_shape(tables[ti], req), sort_keys=True)
            by_shape.setdefault(key, []).append((ti, req))
        ranked = sorted(by_shape.items(), key=lambda kv: -len(kv[1]))[:max_shapes]
        for key, reqs in ranked:
            ti, req = reqs[0]
            shape = json.loads(key)
            log(f"served shape {shape} ({len(reqs)} of 96 requests)")
            best, d_ms, b_ms = descend(lambda k: time_query(tables[ti], req, k, reps), _same, log,
                                       starts=_incumbent(shape, previous))
            entries.append({"shape": shape, **best, "workload": f"served ({len(reqs)} of 96 requests)",
                            "ms_builtin": d_ms, "ms_tuned": b_ms})
    finally:
        for t in tables:
            t.close()
    return entries


def tune_workload(name: str, n: int, stream: int, reps: int, log=print, previous=()) -> list:
    """Tuning entries for one workload's shapes."""
    inputs = workloads.table_inputs(name, n, pinned=True)
    table = Table(workloads.columns(inputs), compute_ndv=True, stream=stream)
    del inputs
    entries = []
    try:
        if name == "batched":
            reqs = workloads.batched_requests(256, seed=4)
            for r in reqs:
                r.stream = stream
            shapes = {json.dumps(request_shape(table, r, batched=True), sort_keys=True) for r in reqs}
            starts = _incumbent(json.loads(sorted(shapes)[0]), previous)
            best, d_ms, b_ms = descend(lambda k: time_batch(table, reqs, k, reps, stream),
                                       lambda a, b: all(_same(x, y) for x, y in zip(a, b)), log, starts=starts)
            for sh in sorted(shapes):
                entries.append({"shape": json.loads(sh), **best, "workload": "batched (256 queries, tuned as one)",
                                "ms_builtin": d_ms, "ms_tuned": b_ms})
        else:
            req = workloads.workload_request(name, stream=stream)
            starts = _incumbent(request_shape(table, req), previous)
            best, d_ms, b_ms = descend(lambda k: time_query(table, req, k, reps), _same, log, starts=starts)
            entries.append({"shape": request_shape(table, req), **best, "workload": name,
                            "ms_builtin": d_ms, "ms_tuned": b_ms})
    finally:
        table.close()
    return entries


def merge_tables(old: dict, entries: list, command: str, seconds: float):
    """(entries, generated_by, seconds) of a tuning table `old` updated with
    freshly tuned `entries`: a shape tuned again takes the new entry, every
    other shape keeps its old one; the provenance lists both commands."""
    tuned = {json.dumps(e["shape"], sort_keys=True) for e in entries}
    kept = [e for e in old["entries"] if json.dumps(e["shape"], sort_keys=True) not in tuned]
    before = old["generated_by"] if isinstance(old["generated_by"], list) else [old["generated_by"]]
    return kept + entries, before + [command + " --merge <this file>"], round(old.get("seconds", 0) + seconds, 1)


def main(argv=None) -> int:
    import torch

    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--out", default=None, help="tuning JSON to write (default: print only)")
    ap.add_argument("--workloads", default="plain,filtered,distinct,batched,served")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--scale", type=float, default=1.0, help="fraction of each workload's full row count")
    ap.add_argument("--merge", default=None,
                    help="tuning JSON whose entries to keep, except the shapes this run tunes again")
    args = ap.parse_args(argv)
    sizes = {"plain": datagen.PLAIN_ROWS, "filtered": datagen.FILTERED_ROWS, "distinct": datagen.DISTINCT_ROWS,
             "batched": datagen.FILTERED_ROWS}
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    t0 = time.time()
    previous = engine_tuning_entries()  # the installed table: warm starts
    entries = []
    log = lambda m: print(m, file=sys.stderr, flush=True)  # noqa: E731
    for name in args.workloads.split(","):
        if name == "served":
            log("served: the four served tables")
            new = tune_served(args.scale, stream.cuda_stream, args.reps, log=log, previous=previous)
        else:
            n = max(1 << 16, int(sizes[name] * args.scale))
            log(f"{name}: {n:,} rows")
            new = tune_workload(name, n, stream.cuda_stream, args.reps, log=log, previous=previous)
        # a shape two workloads tuned keeps the faster setting
        index = {json.dumps(e["shape"], sort_keys=True): i for i, e in enumerate(entries)}
        for e in new:
            k = json.dumps(e["shape"], sort_keys=True)
            if k not in index:
                index[k] = len(entries)
                entries.append(e)
            elif e["ms_tuned"] < entries[index[k]]["ms_tuned"]:
                entries[index[k]] = e
    command = f"python -m thindb_gb300.autotune --workloads {args.workloads} --reps {args.reps}"
    seconds = round(time.time() - t0, 1)
    if args.merge:
        with open(args.merge) as f:
            entries, command, seconds = merge_tables(json.load(f), entries, command, seconds)
    doc = {
        "device": torch.cuda.get_device_name(0),
        "generated_by": command,
        "seconds": seconds,
        "knobs": KNOBS,
        "entries": entries,
    }
    text = json.dumps(doc, indent=1)
    if args.out:
        with open(args.out, "w") as f:
            f.write(text + "\n")
    print(text)
    return 0


if __name__ == "__main__":
    sys.exit(main())
