"""Benchmark of the GB300 grouped-aggregation path.

Default workload (the filtered high-cardinality DECIMAL aggregate, 100M rows):
    SELECT k, COUNT(*), SUM(amount), AVG(amount) FROM t
    WHERE d BETWEEN 2026-04-11 AND 2026-05-16 GROUP BY k ORDER BY SUM(amount) DESC LIMIT 10
k BIGINT Zipf(1.1) over 10M values, amount DECIMAL(18,2), d DATE over 365 days.

One step = one execution of that query over the whole table.
  value  rows/s with the table resident in HBM (CUDA events on the query's stream)
  e2e    rows/s through the C ABI from pinned HOST buffers: table registration
         (H2D copy of the three columns + zone maps) + plan + execute + next
         (D2H of the result) inside the timed region
Inputs (2.0 GB) are larger than L2 (129 MB), so no flush between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--workload filtered|plain|topcount|distinct|batched|served|segment]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from thindb_gb300 import abi, datagen  # noqa: E402

WORKLOADS = {
    "filtered": {
        "name": "filtered high-cardinality DECIMAL aggregate: 100M rows, k BIGINT Zipf(1.1) over 10M, "
                "amount DECIMAL(18,2) log-normal, d DATE 365 days, WHERE d BETWEEN (36 days, ~9.9%), "
                "COUNT/SUM(int128)/AVG, ORDER BY SUM DESC LIMIT 10",
        "rows": datagen.FILTERED_ROWS, "bytes_per_row": 20, "dtype": "int64/int128",
    },
    "plain": {
        "name": "plain GROUP BY: 16,777,216 rows, k BIGINT over 1,024 values, v INT, COUNT/SUM/MIN/MAX",
        "rows": datagen.PLAIN_ROWS, "bytes_per_row": 12, "dtype": "int64",
    },
    "topcount": {
        "name": "ORDER BY COUNT(*) DESC LIMIT 10: 100M rows, k BIGINT Zipf(1.1) over 10M (the filtered table's key), "
                "no WHERE; the two-pass count sketch",
        "rows": datagen.FILTERED_ROWS, "bytes_per_row": 8, "dtype": "int64",
    },
    "distinct": {
        "name": "composite key + COUNT(DISTINCT): 200M rows, (region SMALLINT, url DICT32), user_id BIGINT "
                "Zipf(0.9) over 5M, latency DOUBLE, COUNT/COUNT(DISTINCT)/SUM(f64)",
        "rows": datagen.DISTINCT_ROWS, "bytes_per_row": 22, "dtype": "int64/f64",
    },
}


def load_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_traffic(workload, kernel="scan"):
    """dram bytes per launch of the dominant kernel from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", f"{kernel}_{workload}_traffic.json")
    try:
        with open(p) as f:
            return json.load(f).get("dram_bytes_per_launch")
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------- inputs --

def make_inputs(workload: str, n: int, pinned: bool):
    from thindb_gb300 import workloads

    return workloads.table_inputs(workload, n, pinned)


KNOBS = {}  # explicit engine settings (--chunk-rows / --cache-slots / --table-load / --flags)


def make_request(workload: str, flags: int = 0, stream: int = 0):
    from thindb_gb300 import workloads

    req = workloads.workload_request(workload, flags | KNOBS.get("flags", 0), stream)
    for k in ("chunk_rows", "cache_slots", "table_load_pct"):
        if k in KNOBS:
            setattr(req, k, KNOBS[k])
    return req


def rows_of(result: dict) -> list:
    """A result dict as a list of exact rows (bytes per column), for equality checks."""
    cols = []
    for name, (vals, ok) in result.items():
        cols.append((name, np.ascontiguousarray(vals).tobytes(), None if ok is None else ok.tobytes()))
    return cols


def columns_of(inputs, ndv=None):
    from thindb_gb300 import workloads

    return workloads.columns(inputs, ndv)


# ------------------------------------------------------------ CPU legs --

DOP1_SAMPLE_ROWS = 10_000_000  # single-thread figure: a bounded prefix of the workload


def oracle_columns(workload: str, inputs):
    """engine.Column objects over host numpy views of the workload's columns."""
    cols = columns_of(inputs)
    for c in cols:
        c.data = c.data.numpy() if hasattr(c.data, "numpy") else c.data
    return cols


def run_oracle(workload: str, cols, threads: int):
    """The oracle (C++ restatement of thinDB's silo executor) over `cols`;
    returns (result, seconds)."""
    import oracle

    t = oracle.HostTable(cols)
    req = make_request(workload)
    t0 = time.perf_counter()
    res = oracle.run(t, req, threads=threads)
    return res, time.perf_counter() - t0


def prefix_columns(cols, n):
    from thindb_gb300.engine import Column

    return [Column(c.name, c.type, c.data[:n], scale=c.scale) for c in cols]


def same_result(got: dict, want: dict, keys: list, ordered: bool, rel_cols=()) -> bool:
    """Bit-exact equality of two result dicts (DOUBLE sums in rel_cols within
    1e-12 relative); unordered results are compared sorted by key."""
    names = [k for k in want if not k.startswith("__")]
    n = len(want[names[0]][0])
    if any(len(got[k][0]) != n for k in names):
        return False
    og = ow = np.arange(n)
    if not ordered:
        og = np.lexsort([np.asarray(got[k][0]) for k in reversed(keys)])
        ow = np.lexsort([np.asarray(want[k][0]) for k in reversed(keys)])
    for k in names:
        g, w = np.asarray(got[k][0])[og], np.asarray(want[k][0])[ow]
        if k in rel_cols:
            if n and float((np.abs(g - w) / np.maximum(np.abs(w), 1e-300)).max()) > 1e-12:
                return False
        elif not np.array_equal(g, w):
            return False
    return True


PARITY = {  # group keys, ordered result, DOUBLE-sum columns
    "filtered": (["k"], True, ()),
    "plain": (["k"], False, ()),
    "distinct": (["region", "url"], False, ("lat",)),
    "topcount": (["k"], True, ()),
}


def reference_arm(args, wl):
    """thinDB's CPU executor, restated (oracle/, C++; the Zig toolchain is
    absent), over the same full workload as the GPU arm, all host threads."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    inputs = make_inputs(args.workload, wl["rows"], pinned=False)
    cols = oracle_columns(args.workload, inputs)
    for _ in range(max(0, min(args.warmup, 1))):
        run_oracle(args.workload, prefix_columns(cols, min(wl["rows"], 2_000_000)), threads)
    secs = []
    for _ in range(args.steps):
        _, dt = run_oracle(args.workload, cols, threads)
        secs.append(dt)
    ms = statistics.median(secs) * 1e3
    value = wl["rows"] / (ms / 1e3)
    line = {
        "impl": "reference", "metric": "GROUP BY rows/s", "value": value, "unit": "rows/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": wl["dtype"],
        "data": "synthetic (seeded generator)",
        "config": {"workload": wl["name"], "rows": wl["rows"]},
        "cpu_baseline": {"value": value, "unit": "rows/s", "cores": threads, "kind": "port",
                         "sample": f"the whole workload ({wl['rows']:,} rows) per step, {threads} host threads; "
                                   "C++ restatement of thinDB's silo executor (Zig toolchain absent)"},
        "e2e": {"value": value, "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------- GPU arm --

def gpu_arm(args, wl):
    import torch

    from thindb_gb300 import engine
    from thindb_gb300.engine import Table, try_build_group_topn

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    n = wl["rows"]
    inputs = make_inputs(args.workload, n, pinned=True)
    h2d_bytes = sum(t.numel() * t.element_size() for _, _, t, _ in inputs)

    stream = torch.cuda.Stream()
    table = Table(columns_of(inputs), compute_ndv=True, stream=stream.cuda_stream)
    req = make_request(args.workload, flags=abi.FLAG_TIMING, stream=stream.cuda_stream)
    q = try_build_group_topn(table, req)
    assert q is not None
    out_schema = q.output_schema()

    for _ in range(args.warmup):
        q.execute()
        q.synchronize()
    scan_ms, launches = [], 0
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        q.execute()
        q.synchronize()  # reads the status word (table-overflow retry check) each step
        st = q.stats()
        scan_ms.append(st.scan_ms)
        launches += st.kernel_launches
    ev1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    total_ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    st = q.stats()
    res = q.collect()
    from thindb_gb300 import replicas

    ms_per_step = replicas.slowest_ms(total_ms / args.steps, dist, device="cuda")
    value = replicas.job_rows_per_s(n, world, ms_per_step)
    q.close()

    # end to end through the C ABI from pinned host buffers: registration
    # (H2D copies, zone maps, NDV sketches), plan, execute, next (D2H)
    e2e_steps = max(1, min(args.steps, 5))
    d2h = sum(c.elem_bytes for c in out_schema) * st.result_rows
    e2e_times = []
    for i in range(e2e_steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        t2 = Table(columns_of(inputs), compute_ndv=True, stream=stream.cuda_stream)
        q2 = try_build_group_topn(t2, make_request(args.workload, stream=stream.cuda_stream))
        r2 = q2.collect()
        q2.close()
        t2.close()
        dt = time.perf_counter() - t0
        if i > 0:  # the first pass warms the column pool
            e2e_times.append(dt)
    e2e_value = n / statistics.median(e2e_times)
    # the ceiling e2e is bounded by: the same bytes copied from the same
    # pinned buffers by plain cudaMemcpyAsync, one per column; the fastest of
    # six passes (the host link's rate varies between passes on a shared host)
    dev_bufs = [torch.empty(t.numel() * t.element_size(), dtype=torch.uint8, device="cuda") for _, _, t, _ in inputs]
    h2d_ms = []
    for i in range(7):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for b, (_, _, t, _) in zip(dev_bufs, inputs):
                b.copy_(t.view(torch.uint8).reshape(-1), non_blocking=True)
            e1.record(stream)
        e1.synchronize()
        if i:
            h2d_ms.append(e0.elapsed_time(e1))
    del dev_bufs
    h2d_best = min(h2d_ms)
    h2d_gbs = h2d_bytes / (h2d_best / 1e3) / 1e9

    peak, peak_kind = load_peak()
    scan_avg = statistics.mean(scan_ms)
    alg_bytes = n * wl["bytes_per_row"]
    achieved = alg_bytes / (scan_avg / 1e3) / 1e9
    traffic = load_traffic(args.workload)
    scan_kernel = ("staged_scan_kernel" if st.flags & abi.STAT_STAGED else
                   "pipe_scan_kernel" if st.flags & abi.STAT_PIPE else
                   "select_rows_kernel + fold_rows_staged_kernel" if st.flags & abi.STAT_SPLIT else "scan_group_kernel")

    # the CPU baseline over the same table, whose result doubles as the
    # parity check of the GPU result (outside the timed region)
    cpu, parity = None, None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        ocols = oracle_columns(args.workload, inputs)
        want, dt_all = run_oracle(args.workload, ocols, threads)
        keys, ordered, rel = PARITY[args.workload]
        parity = same_result(res, want, keys, ordered, rel)
        n1 = min(n, DOP1_SAMPLE_ROWS)
        _, dt1 = run_oracle(args.workload, prefix_columns(ocols, n1), 1)
        cpu = {"value": n / dt_all, "unit": "rows/s", "cores": threads, "kind": "port",
               "sample": f"the whole workload ({n:,} rows, {dt_all:.2f} s) on {threads} threads; C++ restatement "
                         "of thinDB's silo executor (Zig toolchain absent)",
               "dop1": {"value": n1 / dt1, "unit": "rows/s", "cores": 1,
                        "sample": f"first {n1:,} rows of the workload ({dt1:.2f} s) on 1 thread"},
               "dop_all": {"value": n / dt_all, "unit": "rows/s", "cores": threads}}

    if rank == 0:
        line = {
            "metric": "GROUP BY rows/s", "value": value, "unit": "rows/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": wl["dtype"], "data": "synthetic (seeded generator)",
            "config": {"workload": wl["name"], "rows": n, "l2": "inputs larger than L2 (no flush)",
                       "selectivity": st.rows_selected / max(1, st.rows_scanned), "groups": st.groups,
                       "table_capacity": st.table_capacity,
                       "route": "shared-memory" if st.route == 1 else "global table",
                       "scan": ("staged" if st.flags & abi.STAT_STAGED else "pipelined" if st.flags & abi.STAT_PIPE
                                else "survivor gather, split (select pass, fold pass)" if st.flags & abi.STAT_SPLIT
                                else "queue" if st.flags & abi.STAT_QUEUE
                                else "survivor gather" if st.flags & abi.STAT_GATHER else "in place"),
                       "count_sketch": bool(st.flags & abi.STAT_COUNT_SKETCH),
                       "tuned": bool(st.flags & abi.STAT_TUNED),
                       "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": scan_kernel, "kernel_ms": scan_avg,
                         "algorithmic_bytes": alg_bytes, "peak_kind": peak_kind,
                         "step_achieved": alg_bytes / (ms_per_step / 1e3) / 1e9,
                         "step_frac": alg_bytes / (ms_per_step / 1e3) / 1e9 / peak},
            "e2e": {"value": e2e_value, "unit": "rows/s", "h2d_bytes_per_step": h2d_bytes,
                    "d2h_bytes_per_step": d2h, "ms_per_step": statistics.median(e2e_times) * 1e3,
                    "h2d_ceiling_gbs": h2d_gbs, "h2d_ceiling_ms": h2d_best,
                    "frac_of_h2d_ceiling": h2d_best / (statistics.median(e2e_times) * 1e3)},
            "parity": parity,
            "gpu_launches": launches,
            "clocks": clk,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    table.close()
    if dist:
        dist.destroy_process_group()


def batched_arm(args):
    """256 GROUP BY queries over one resident 100M-row table: one batched
    persistent kernel replayed from a CUDA graph vs 256 plain sequential
    operator executions; identical results required."""
    import torch

    from thindb_gb300 import workloads
    from thindb_gb300.engine import QueryBatch, Table, try_build_group_topn

    n = args.rows or datagen.FILTERED_ROWS
    torch.cuda.set_device(0)
    inputs = make_inputs("batched", n, pinned=True)
    stream = torch.cuda.Stream()
    table = Table(columns_of(inputs), compute_ndv=True, stream=stream.cuda_stream)
    nq = args.queries
    reqs = workloads.batched_requests(nq, seed=4)
    for r in reqs:
        r.stream = stream.cuda_stream

    b = QueryBatch(table, reqs, graph=True, stream=stream.cuda_stream)
    for _ in range(args.warmup):
        b.execute()
        b.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        b.execute()
        b.synchronize()
        batched_rows = [rows_of(b.collect(i)) for i in range(nq)]
    batched_s = (time.perf_counter() - t0) / args.steps
    clk = clocks.stop()
    bst = b.stats()
    b.close()

    qs = [try_build_group_topn(table, r) for r in reqs]
    for q in qs:  # warm every plain operator once
        q.execute()
        q.synchronize()
    t0 = time.perf_counter()
    plain_rows = []
    for q in qs:
        q.execute()
        plain_rows.append(rows_of(q.collect()))
    plain_s = time.perf_counter() - t0
    for q in qs:
        q.close()
    identical = plain_rows == batched_rows
    value = nq / batched_s
    line = {
        "metric": "batched GROUP BY queries/s", "value": value, "unit": "queries/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": batched_s * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int64/int128", "data": "synthetic (seeded generator)",
        "config": {"workload": f"{nq} concurrent GROUP BY queries over one resident {n:,}-row table "
                               "(k Zipf 10M, k10, k1k, k1m keys; selectivity log-uniform 0.1%-50%; random "
                               "COUNT/SUM/MIN/MAX subsets; ORDER BY first aggregate DESC LIMIT 10)",
                   "step": "one batched execute (CUDA graph replay) + results of every query to the host"},
        "plain": {"value": nq / plain_s, "unit": "queries/s",
                  "how": f"{nq} plain operators executed one after another (execute + next each)"},
        "speedup_vs_plain": plain_s / batched_s,
        "identical_results": identical,
        "batch": {"kernel_launches": bst.kernel_launches, "graph": bool(bst.graph), "work_items": bst.work_items,
                  "device_ms": bst.total_ms, "rerun_queries": bst.rerun_queries},
        "gpu_launches": bst.kernel_launches * args.steps,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    table.close()


def served_arm(args):
    """Open-loop Poisson arrivals against the four resident tables, continuous
    batching vs the plain one-query-at-a-time operator on the same GPU."""
    import torch

    from thindb_gb300 import workloads
    from thindb_gb300.engine import Server, Table

    torch.cuda.set_device(0)
    scale = args.rows / datagen.FILTERED_ROWS if args.rows else 1.0
    n_plain = max(1 << 16, int(datagen.PLAIN_ROWS * scale))
    n_filt = max(1 << 16, int(datagen.FILTERED_ROWS * scale))
    n_dist = max(1 << 16, int(datagen.DISTINCT_ROWS * scale))
    stream = torch.cuda.Stream()
    tables = []
    for wl, n in (("plain", n_plain), ("filtered", n_filt), ("distinct", n_dist)):
        inp = make_inputs(wl, n, pinned=True)
        tables.append(Table(columns_of(inp), compute_ndv=True, stream=stream.cuda_stream))
        del inp
    inp = make_inputs("batched", n_filt, pinned=True)
    tables.append(Table(columns_of(inp), compute_ndv=True, stream=stream.cuda_stream))
    del inp
    resident = torch.cuda.memory_allocated()  # torch's own; the tables live in the engine's allocations
    mix = workloads.served_mix(96, seed=5)
    rates = [float(r) for r in args.rates.split(",")]
    results = {}
    for mode in ("continuous", "plain"):
        srv = Server(tables, mode=mode, memory_budget=120 << 30)
        srv.run_load(mix, rate_qps=200, duration_s=0.5, seed=99)  # warm the workspace pool
        results[mode] = []
        for rate in rates:
            dur = args.duration if mode == "continuous" else min(args.duration, 2.0)
            rep = srv.run_load(mix, rate_qps=rate, duration_s=dur, seed=int(rate))
            rep["offered_qps"] = rate
            results[mode].append(rep)
            print(json.dumps({"mode": mode, **rep}), file=sys.stderr, flush=True)
        srv.close()
    best = max((r for r in results["continuous"] if r["p99_ms"] <= 50.0), key=lambda r: r["achieved_qps"],
               default=None)
    plain_max = max(r["achieved_qps"] for r in results["plain"])
    line = {
        "metric": "served GROUP BY queries/s at p99 <= 50 ms", "value": best["achieved_qps"] if best else 0.0,
        "unit": "queries/s", "n_gpus": 1, "steps": len(rates), "warmup": 1,
        "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int64/int128/f64", "data": "synthetic (seeded generator)",
        "config": {"workload": "served mix: open-loop Poisson arrivals over 4 resident tables (plain, filtered, "
                               "distinct, batched); request shapes from the filtered / distinct / batched families",
                   "rows": {"plain": n_plain, "filtered": n_filt, "distinct": n_dist, "batched": n_filt},
                   "admission_budget_bytes": 120 << 30},
        "rates": results,
        "plain_max_qps": plain_max,
        "speedup_vs_plain": (best["achieved_qps"] / plain_max) if best and plain_max else None,
    }
    print(json.dumps(line), flush=True)
    for t in tables:
        t.close()


# ------------------------------------------------------ segment ingest --

SEGMENT_RG_ROWS = 65_536
SEGMENT_BASE_GROUPS = 64      # rows written by the segment writer, then repeated
SEGMENT_TIMES = 25            # 64 x 25 row groups of 65,536 rows = 104,857,600 rows
SEGMENT_NAME = ("segment ingest: a thinDB segment image (version 17, no block compression) of 1,600 row groups "
                "x 65,536 rows (104,857,600 rows), 8 columns: SMALLINT/DATE runs (RLE), BIGINT x2 and DECIMAL64 "
                "(FOR widths 2/4/4), DOUBLE, BOOLEAN, TINYINT (raw); 4 nullable columns (validity bitmaps)")


def segment_image(rows: int = 0):
    """A seeded segment image: the writer's first 64 row groups, repeated."""
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from segments import replicate, sample_table, write_segment

    base = SEGMENT_BASE_GROUPS * SEGMENT_RG_ROWS
    times = SEGMENT_TIMES
    if rows:
        base = min(base, rows)
        times = max(1, -(-rows // base))
    names, types, values, validity = sample_table(base)
    image, _ = write_segment(types, values, validity, row_group_rows=SEGMENT_RG_ROWS)
    if times > 1:
        image = replicate(image, len(types), times)
    return names, types, validity, image, base * times


def segment_schema(names, types):
    from thindb_gb300.engine import Column
    return [Column(nm, ty, None, scale=2 if ty == abi.DECIMAL64 else 0, precision=12)
            for nm, ty in zip(names, types)]


def segment_oracle(image, types, validity, threads):
    import oracle
    t0 = time.perf_counter()
    out = oracle.decode_segment(image, types, [v is not None for v in validity], threads=threads)
    return out, time.perf_counter() - t0


def segment_reference_arm(args):
    """The CPU decode of the same image (oracle/segment.cpp, a C++
    restatement of thinDB's segment reader; the Zig toolchain is absent), all
    host threads."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    names, types, validity, image, n = segment_image(args.rows)
    threads = os.cpu_count() or 1
    segment_oracle(image, types, validity, threads)
    secs = [segment_oracle(image, types, validity, threads)[1] for _ in range(args.steps)]
    ms = statistics.median(secs) * 1e3
    value = n / (ms / 1e3)
    print(json.dumps({
        "impl": "reference", "metric": "segment ingest rows/s", "value": value, "unit": "rows/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/int64",
        "data": "synthetic (seeded generator)", "config": {"workload": SEGMENT_NAME, "rows": n},
        "cpu_baseline": {"value": value, "unit": "rows/s", "cores": threads, "kind": "port",
                         "sample": f"the whole image ({len(image) / 1e9:.2f} GB) decoded per step on {threads} "
                                   "threads; C++ restatement of thinDB's segment reader (Zig toolchain absent)"},
        "e2e": {"value": value, "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def segment_arm(args):
    """Register the image as a table, K times: host walk, then the image
    copied in chunks of row groups, each chunk decoded and its zone maps and
    NDV sketches taken while the next copies.  value: rows/s of that device
    work (the decode and statistics launches' summed durations); e2e: rows/s
    of the whole call from a pinned host image."""
    import torch

    from thindb_gb300.engine import Table

    torch.cuda.set_device(0)
    names, types, validity, image, n = segment_image(args.rows)
    host = torch.empty(len(image), dtype=torch.uint8, pin_memory=True)
    host.numpy()[:] = np.frombuffer(image, dtype=np.uint8)
    schema = segment_schema(names, types)
    stream = torch.cuda.Stream()
    for _ in range(args.warmup):
        Table.from_segment(host, schema, stream=stream.cuda_stream).close()
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    torch.cuda.synchronize()
    stats, wall = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        t = Table.from_segment(host, schema, stream=stream.cuda_stream)
        wall.append(time.perf_counter() - t0)
        st = t.load_stats()
        stats.append((st.h2d_ms, st.decode_ms, st.stats_ms, st.total_ms, st.pipeline_ms))
        t.close()
    torch.cuda.synchronize()
    clk = clocks.stop()
    decode_ms = statistics.mean(s[1] for s in stats)
    device_ms = statistics.median(s[1] + s[2] for s in stats)
    e2e_ms = statistics.median(wall) * 1e3
    t = Table.from_segment(host, schema, stream=stream.cuda_stream)
    st = t.load_stats()
    alg = st.image_bytes + st.decoded_bytes
    peak, peak_kind = load_peak()
    achieved = alg / (decode_ms / 1e3) / 1e9
    # parity: every decoded column bit-exact with the CPU decode of the image
    cpu, parity = None, None
    threads = os.cpu_count() or 1
    if not args.no_cpu:
        want, dt_all = segment_oracle(image, types, validity, threads)
        parity = True
        for nm, (wv, wok) in zip(names, want):
            gv, gok = t.read_column(nm)
            parity = parity and bool(np.array_equal(gv.view(np.uint8), wv.view(np.uint8)))
            parity = parity and (bool(gok.all()) if wok is None else bool(np.array_equal(gok, wok)))
        del want
        base_rows = SEGMENT_BASE_GROUPS * SEGMENT_RG_ROWS
        _, types1, valid1, image1, n1 = segment_image(min(n, base_rows))
        _, dt1 = segment_oracle(image1, types1, valid1, 1)
        cpu = {"value": n / dt_all, "unit": "rows/s", "cores": threads, "kind": "port",
               "sample": f"the whole image ({len(image) / 1e9:.2f} GB, {dt_all:.2f} s) on {threads} threads; "
                         "C++ restatement of thinDB's segment reader (Zig toolchain absent)",
               "dop1": {"value": n1 / dt1, "unit": "rows/s", "cores": 1,
                        "sample": f"the first {n1:,} rows ({dt1:.2f} s) on 1 thread"}}
    t.close()
    line = {
        "metric": "segment ingest rows/s", "value": n / (device_ms / 1e3), "unit": "rows/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": device_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8/int64", "data": "synthetic (seeded generator)",
        "config": {"workload": SEGMENT_NAME, "rows": n, "image_bytes": st.image_bytes,
                   "decoded_bytes": st.decoded_bytes, "blocks": st.blocks,
                   "l2": "image and columns larger than L2 (no flush)",
                   "value_covers": "decode launches + zone-map / NDV-sketch launches (device time, summed)",
                   "decode_ms": decode_ms, "stats_ms": statistics.mean(s[2] for s in stats)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": load_traffic("ingest", "decode"), "kernel": "decode_blocks_kernel", "kernel_ms": decode_ms,
                     "algorithmic_bytes": alg, "peak_kind": peak_kind},
        "e2e": {"value": n / (e2e_ms / 1e3), "unit": "rows/s", "h2d_bytes_per_step": st.image_bytes,
                "d2h_bytes_per_step": 0, "ms_per_step": e2e_ms,
                "h2d_ms": statistics.median(s[0] for s in stats),
                "pipeline_ms": statistics.median(s[4] for s in stats),
                "chunks": st.chunks,
                "how": "the image copied in chunks of row groups; each chunk decoded and its statistics taken "
                       "while the next one copies"},
        "parity": parity,
        "gpu_launches": args.steps * st.kernel_launches,
        "clocks": clk,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="filtered", choices=sorted(WORKLOADS) + ["batched", "served", "segment"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--rows", type=int, default=0, help="rows of the workload (default: its full size)")
    ap.add_argument("--queries", type=int, default=256, help="queries of the batched workload")
    ap.add_argument("--rates", default="500,750,1000,1250,2500,5000",
                    help="offered loads of the served workload (q/s): the configured rates and points between")
    ap.add_argument("--duration", type=float, default=4.0, help="seconds of arrivals per served rate")
    ap.add_argument("--chunk-rows", type=int, default=None, help="pin rows per warp chunk (profiling a small case)")
    ap.add_argument("--cache-slots", type=int, default=None, help="pin shared-memory table slots (-1 none)")
    ap.add_argument("--table-load", type=int, default=None, help="pin the group-table load target (%%)")
    ap.add_argument("--flags", type=int, default=None, help="extra TGPU_FLAG_* bits for the request")
    args = ap.parse_args()
    for name, key in (("chunk_rows", "chunk_rows"), ("cache_slots", "cache_slots"), ("table_load", "table_load_pct"),
                      ("flags", "flags")):
        if getattr(args, name) is not None:
            KNOBS[key] = getattr(args, name)
    if args.workload == "served":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the served mode has no CPU reference arm; "
                              "run the default workload"}))
            return
        served_arm(args)
        return
    if args.workload == "segment":
        if args.impl == "reference":
            segment_reference_arm(args)
        else:
            segment_arm(args)
        return
    if args.workload == "batched":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the batched mode has no CPU reference arm; "
                              "run the default workload"}))
            return
        batched_arm(args)
        return
    wl = dict(WORKLOADS[args.workload])
    if args.rows:
        wl["rows"] = args.rows
        wl["name"] += f" (run at {args.rows:,} rows)"
    if args.impl == "reference":
        reference_arm(args, wl)
    else:
        gpu_arm(args, wl)


if __name__ == "__main__":
    main()
