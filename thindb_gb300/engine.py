"""Host-side mirror of thinDB's grouped-aggregation operator interface.

The names follow the reference so tests read like its own:

    Table            a registered immutable table (an `api.Table` snapshot in HBM)
    AggSpec          exec.AggSpec {func, col, as}          (src/exec/aggregate.zig:237)
    SortSpec         sort.SortSpec {col, desc}             (src/exec/sort.zig:28)
    Request          GroupTopNRequest                      (src/exec/v2_shape_group_topn.zig:63)
    try_build_group_topn(table, request) -> Query | None  (v2_pipeline.tryBuildGroupTopN:
                     None means "decline", exactly as the Zig routing point returns null)
    Query.next() -> Batch | None                           (exec.Query.next, src/exec/exec.zig:913)

Every call goes through the C ABI of libthindb_gpu.so (include/thindb_gpu.h);
there is no CPU path: without the built extension, importing the library
raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from typing import Any, Optional, Sequence

import numpy as np

from . import abi

_LIB: Optional[C.CDLL] = None
LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libthindb_gpu.so")


def lib() -> C.CDLL:
    """Load libthindb_gpu.so (built in-tree by thindb_gb300.build)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"thindb_gb300 CUDA extension missing at {LIB_PATH}: run thindb_gb300.build first")
        L = C.CDLL(LIB_PATH)
        for name, res, args in abi.SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
        # the measured settings for this GPU (THINDB_GPU_TUNING=off: built-in
        # rules only; =<path>: another table)
        choice = os.environ.get("THINDB_GPU_TUNING", "")
        if choice != "off":
            path = choice or TUNING_PATH
            if os.path.exists(path):
                load_tuning(path)
    return _LIB


TUNING_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning", "gb300.json")


def load_tuning(path: str = TUNING_PATH) -> int:
    """Install the tuning table a JSON file written by thindb_gb300.autotune holds;
    returns the number of entries."""
    import json
    with open(path) as f:
        doc = json.load(f)
    entries = doc.get("entries", [])
    arr = (abi.Tuning * max(1, len(entries)))()
    for i, e in enumerate(entries):
        for k, v in e["shape"].items():
            setattr(arr[i].shape, k, int(v))
        arr[i].chunk_rows = int(e.get("chunk_rows", 0))
        arr[i].cache_slots = int(e.get("cache_slots", 0))
        arr[i].table_load_pct = int(e.get("table_load_pct", 0))
        arr[i].flags = int(e.get("flags", 0))
        arr[i].groups_shift = int(e.get("groups_shift", 0))
    _check(lib().tgpu_tuning_set(arr, len(entries)))
    return len(entries)


def set_device_wait_limit(sm_cycles: int) -> None:
    """Bound of the device's bulk-copy waits in SM clocks for queries executed
    from now on (0 = the built-in ~2 s); a test hook for the timeout path."""
    _check(lib().tgpu_debug_set_wait_limit(sm_cycles))


def set_digest_bits(bits: int) -> None:
    """Keep only the low `bits` of hashed keys' digests for queries planned
    from now on (0 = all 64): a test hook that makes distinct keys share
    digests, so the exact key check decides every match."""
    _check(lib().tgpu_debug_set_digest_bits(bits))


def register_aggregate(name: str) -> None:
    """Record a host user-defined aggregate's name (thinDB's registerAggregate):
    requests naming it decline to the caller's executor."""
    _check(lib().tgpu_aggregate_register(name.encode()))


def unregister_aggregate(name: str) -> None:
    _check(lib().tgpu_aggregate_unregister(name.encode()))


def aggregate_registered(name: str) -> bool:
    return bool(lib().tgpu_aggregate_registered(name.encode()))


def clear_tuning() -> None:
    _check(lib().tgpu_tuning_set(None, 0))


def tuning_entries() -> list:
    n = lib().tgpu_tuning_get(None, 0)
    arr = (abi.Tuning * max(1, n))()
    lib().tgpu_tuning_get(arr, n)
    return [{"shape": arr[i].shape.as_dict(), "chunk_rows": arr[i].chunk_rows, "cache_slots": arr[i].cache_slots,
             "table_load_pct": arr[i].table_load_pct, "flags": arr[i].flags, "groups_shift": arr[i].groups_shift}
            for i in range(n)]


class EngineError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class MemoryBudgetExceeded(EngineError):
    pass


class DeviceTimeout(EngineError):
    """A bounded device wait ran out (TGPU_ERR_DEVICE_TIMEOUT)."""


class QueryCancelled(EngineError):
    pass


def _check(status: int) -> None:
    if status == abi.OK:
        return
    msg = (lib().tgpu_last_error_message() or b"").decode(errors="replace")
    if status == abi.ERR_MEMORY_BUDGET:
        raise MemoryBudgetExceeded(status, msg)
    if status == abi.ERR_CANCELLED:
        raise QueryCancelled(status, msg)
    if status == abi.ERR_DEVICE_TIMEOUT:
        raise DeviceTimeout(status, msg)
    raise EngineError(status, msg)


NP_DTYPES = {abi.BOOLEAN: np.uint8, abi.TINYINT: np.int8, abi.SMALLINT: np.int16, abi.INT: np.int32,
             abi.DATE: np.int32, abi.BIGINT: np.int64, abi.DATETIME: np.int64, abi.DECIMAL64: np.int64,
             abi.FLOAT: np.float32, abi.DOUBLE: np.float64, abi.DICT32: np.int32, abi.VARCHAR: np.int64}


def varchar_buffers(values) -> tuple:
    """A VARCHAR column's (u32 offsets of n + 1, u8 bytes) from a list of
    str/bytes values (None for NULL: an empty string under a validity bit)."""
    enc = [b"" if v is None else (v.encode() if isinstance(v, str) else bytes(v)) for v in values]
    offs = np.zeros(len(enc) + 1, dtype=np.uint32)
    offs[1:] = np.cumsum([len(e) for e in enc], dtype=np.uint64).astype(np.uint32)
    blob = np.frombuffer(b"".join(enc) or b"\0", dtype=np.uint8).copy()
    return offs, blob


def decimal128_to_ints(raw: np.ndarray) -> list[int]:
    """(n, 2) little-endian words of an i128 column -> Python ints."""
    pairs = np.asarray(raw).reshape(-1, 2).view(np.uint64)
    out = []
    for lo, hi in pairs:
        v = (int(hi) << 64) | int(lo)
        if v >= 1 << 127:
            v -= 1 << 128
        out.append(v)
    return out


@dataclass
class Column:
    """One input column: host numpy array or device tensor (anything with data_ptr())."""
    name: str
    type: int
    data: Any
    validity: Optional[np.ndarray] = None   # bool per row (True = value), None = NOT NULL
    scale: int = 0
    precision: int = 18
    dictionary: Optional[Sequence[str]] = None  # DICT32 strings
    ndv_hint: int = 0


def _ptr(x: Any) -> int:
    if hasattr(x, "data_ptr"):
        return int(x.data_ptr())
    return int(x.ctypes.data)


class Table:
    """An immutable, HBM-resident table with zone maps and NDV sketches."""

    def __init__(self, columns: Sequence[Column], row_group_rows: int = 65536, location: str = "host",
                 compute_ndv: bool = True, stream: int = 0):
        self.columns = list(columns)
        if not self.columns:
            raise ValueError("a table needs columns")
        n = len(self.columns[0].data) if not hasattr(self.columns[0].data, "numel") else int(self.columns[0].data.numel())
        self.n_rows = n
        self._keep: list[Any] = []
        descs = (abi.ColumnDesc * len(self.columns))()
        for i, c in enumerate(self.columns):
            cn = len(c.data) if not hasattr(c.data, "numel") else int(c.data.numel())
            if cn != n:
                raise ValueError(f"column {c.name} has {cn} rows, expected {n}")
            d = descs[i]
            nm = c.name.encode()
            self._keep.append(nm)
            d.name = nm
            d.type = c.type
            d.decimal_precision = c.precision
            d.decimal_scale = c.scale
            if c.type == abi.VARCHAR:
                if location != "host":
                    raise ValueError("VARCHAR columns register from host values")
                offs, blob = varchar_buffers(c.data)
                self._keep += [offs, blob]
                d.data = _ptr(offs)
                d.dict_bytes = _ptr(blob)
            elif location == "host":
                arr = np.ascontiguousarray(c.data, dtype=NP_DTYPES[c.type]) if not hasattr(c.data, "data_ptr") else c.data
                self._keep.append(arr)
                d.data = _ptr(arr)
            else:
                d.data = _ptr(c.data)
            if c.validity is not None:
                bm = np.packbits(np.asarray(c.validity, dtype=bool), bitorder="little")
                if location == "device":
                    import torch
                    bm = torch.from_numpy(bm).cuda()
                self._keep.append(bm)
                d.validity = _ptr(bm)
            if c.type == abi.DICT32 and c.dictionary is not None:
                enc = [s.encode() if isinstance(s, str) else bytes(s) for s in c.dictionary]
                offs = np.zeros(len(enc) + 1, dtype=np.uint32)
                offs[1:] = np.cumsum([len(s) for s in enc])
                blob = np.frombuffer(b"".join(enc) or b"\0", dtype=np.uint8).copy()
                self._keep += [offs, blob]
                d.dict_offsets = _ptr(offs)
                d.dict_bytes = _ptr(blob)
                d.dict_size = len(enc)
            d.ndv_hint = c.ndv_hint
        td = abi.TableDesc()
        td.columns = descs
        td.n_columns = len(self.columns)
        td.row_group_rows = row_group_rows
        td.n_rows = n
        td.location = abi.LOC_HOST if location == "host" else abi.LOC_DEVICE
        td.compute_ndv = 1 if compute_ndv else 0
        td.stream = stream or None
        h = C.c_void_p()
        _check(lib().tgpu_table_register(C.byref(td), C.byref(h)))
        self.handle = h
        if location == "host":
            self._keep = []  # copied into HBM
        self.row_group_rows = row_group_rows

    @classmethod
    def from_segment(cls, image: bytes, columns: Sequence[Column], compute_ndv: bool = True,
                     stream: int = 0) -> "Table":
        """Register a thinDB segment file image (src/storage/format.zig layout;
        bytes, a uint8 numpy array or a host tensor): `columns` name the
        schema in order (name, type, decimal scale and precision; `data`
        unused).  The blocks decode on the device; the row
        groups keep the segment's size."""
        self = cls.__new__(cls)
        self.columns = list(columns)
        if not self.columns:
            raise ValueError("a table needs columns")
        if hasattr(image, "data_ptr"):  # a (pinned) host tensor
            ptr, size = int(image.data_ptr()), int(image.numel() * image.element_size())
        else:
            buf = image if isinstance(image, np.ndarray) else np.frombuffer(image, dtype=np.uint8)
            ptr, size = int(buf.ctypes.data), int(buf.nbytes)
        names = [c.name.encode() for c in self.columns]
        descs = (abi.SegmentColumn * len(self.columns))()
        for i, c in enumerate(self.columns):
            descs[i].name = names[i]
            descs[i].type = c.type
            descs[i].decimal_precision = c.precision
            descs[i].decimal_scale = c.scale
        h = C.c_void_p()
        _check(lib().tgpu_table_register_segment(ptr if size else None, size, descs,
                                                 len(self.columns), 1 if compute_ndv else 0, stream or None,
                                                 C.byref(h)))
        self.handle = h
        self._keep = []
        rows, groups = C.c_uint64(), C.c_uint32()
        _check(lib().tgpu_table_info(h, -1, C.byref(rows), C.byref(groups), None))
        self.n_rows = rows.value
        self.row_group_rows = 0
        self.n_row_groups = groups.value
        return self

    def read_column(self, name: str) -> tuple:
        """A column's values and validity (bool per row) copied back to the host."""
        i = self.col_index(name)
        ty = self.columns[i].type
        vals = np.empty(self.n_rows, dtype=NP_DTYPES[ty])
        bm = np.empty((self.n_rows + 7) // 8 + 1, dtype=np.uint8)
        _check(lib().tgpu_table_read_column(self.handle, i, vals.ctypes.data, bm.ctypes.data))
        return vals, np.unpackbits(bm, bitorder="little")[:self.n_rows].astype(bool)

    def load_stats(self) -> abi.LoadStats:
        """Timings and byte counts of a registration from a segment image."""
        st = abi.LoadStats()
        _check(lib().tgpu_table_load_stats(self.handle, C.byref(st)))
        return st

    def col_index(self, name: str) -> int:
        for i, c in enumerate(self.columns):
            if c.name.lower() == name.lower():
                return i
        raise KeyError(name)

    def ndv(self, name: str) -> int:
        v = C.c_uint64()
        _check(lib().tgpu_table_info(self.handle, self.col_index(name), None, None, C.byref(v)))
        return v.value

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().tgpu_table_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class AggSpec:
    func: str            # count | sum | avg | min | max | count_distinct | udf
    col: Optional[str] = None
    as_: str = ""
    udf_name: Optional[str] = None   # func "udf": the registered aggregate's name


@dataclass
class SortSpec:
    col: str             # a group column or an aggregate's output name
    desc: bool = False


@dataclass
class Pred:
    col: str
    op: str              # between | not_between | = | != | < | <= | > | >= | is_null | is_not_null
    lo: Any = 0
    hi: Any = 0


@dataclass
class HavingSpec:
    agg: str             # aggregate output name
    op: str              # = != < <= > >=
    value: Any = 0


@dataclass
class Request:
    group_cols: Sequence[str]
    aggs: Sequence[AggSpec]
    order_specs: Sequence[SortSpec] = ()
    limit: Optional[int] = None
    offset: int = 0
    where: Sequence[Pred] = ()
    having: Sequence[HavingSpec] = ()
    expected_groups: int = 0
    memory_budget: int = 0
    flags: int = 0
    stream: int = 0
    chunk_rows: int = 0
    cache_slots: int = 0
    table_load_pct: int = 0


def build_request(table: Table, req: Request) -> tuple[abi.Request, list]:
    """Translate a name-based Request into the C struct (keeps the arrays alive)."""
    keep: list = []
    g = (C.c_int32 * len(req.group_cols))(*[table.col_index(c) for c in req.group_cols])
    aggs = (abi.AggSpec * len(req.aggs))()
    for i, a in enumerate(req.aggs):
        aggs[i].func = abi.AGG_BY_NAME[a.func]
        aggs[i].column = -1 if a.col is None else table.col_index(a.col)
        nm = (a.as_ or f"{a.func}_{a.col or 'star'}").encode()
        keep.append(nm)
        aggs[i].as_ = nm
        if a.udf_name is not None:
            un = a.udf_name.encode()
            keep.append(un)
            aggs[i].udf_name = un
    where = (abi.Predicate * max(1, len(req.where)))()
    for i, p in enumerate(req.where):
        ci = table.col_index(p.col)
        where[i].column = ci
        where[i].op = abi.PRED_BY_NAME[p.op]
        if table.columns[ci].type in (abi.FLOAT, abi.DOUBLE):
            where[i].flo, where[i].fhi = float(p.lo), float(p.hi)
        else:
            where[i].lo, where[i].hi = int(p.lo), int(p.hi)
    names = [a.as_ or f"{a.func}_{a.col or 'star'}" for a in req.aggs]
    having = (abi.Having * max(1, len(req.having)))()
    for i, h in enumerate(req.having):
        having[i].agg = names.index(h.agg)
        having[i].op = abi.PRED_BY_NAME[h.op]
        having[i].ival = int(h.value) if not isinstance(h.value, float) else int(h.value)
        having[i].fval = float(h.value)
    order = (abi.SortSpec * max(1, len(req.order_specs)))()
    lower_keys = [c.lower() for c in req.group_cols]
    lower_aggs = [n.lower() for n in names]
    for i, s in enumerate(req.order_specs):
        if s.col.lower() in lower_aggs:
            order[i].target, order[i].index = abi.SORT_AGG, lower_aggs.index(s.col.lower())
        elif s.col.lower() in lower_keys:
            order[i].target, order[i].index = abi.SORT_KEY, lower_keys.index(s.col.lower())
        else:
            raise KeyError(f"ORDER BY {s.col}: not an output column")
        order[i].desc = 1 if s.desc else 0
    r = abi.Request()
    r.group_cols, r.n_group_cols = g, len(req.group_cols)
    r.aggs, r.n_aggs = aggs, len(req.aggs)
    r.where, r.n_where = where, len(req.where)
    r.having, r.n_having = having, len(req.having)
    r.order, r.n_order = order, len(req.order_specs)
    r.limit = abi.NO_LIMIT if req.limit is None else int(req.limit)
    r.offset = int(req.offset)
    r.expected_groups = int(req.expected_groups)
    r.memory_budget_bytes = int(req.memory_budget)
    r.stream = req.stream or None
    r.flags = int(req.flags)
    r.chunk_rows = int(req.chunk_rows)
    r.cache_slots = int(req.cache_slots)
    r.table_load_pct = int(req.table_load_pct)
    keep += [g, aggs, where, having, order]
    return r, keep


@dataclass
class Batch:
    """One result batch: schema + column arrays (+ validity as bool arrays, None = NOT NULL)."""
    schema: list
    values: list
    validity: list
    row_count: int


@dataclass
class OutCol:
    name: str
    type: int
    nullable: bool
    elem_bytes: int
    precision: int = 0
    scale: int = 0


class Query:
    """A planned GPU GROUP BY operator (the `exec.Query` the shim would wrap)."""

    def __init__(self, handle: C.c_void_p, table: Table):
        self.handle = handle
        self.table = table
        n = C.c_uint32()
        _check(lib().tgpu_query_output_schema(handle, None, 0, C.byref(n)))
        cols = (abi.OutputColumn * n.value)()
        _check(lib().tgpu_query_output_schema(handle, cols, n.value, C.byref(n)))
        self.schema = _schema(cols)

    def _next_c(self, b, done) -> None:
        _check(lib().tgpu_query_next(self.handle, C.byref(b), C.byref(done)))

    def output_schema(self) -> list:
        return self.schema

    def execute(self) -> None:
        _check(lib().tgpu_query_execute(self.handle))

    def synchronize(self) -> None:
        _check(lib().tgpu_query_synchronize(self.handle))

    def next(self, capacity: int = 1 << 16) -> Optional[Batch]:
        vals = []
        valid = []
        for c in self.schema:
            if c.type == abi.DECIMAL128:
                vals.append(np.empty((capacity, 2), dtype=np.int64))
            else:
                vals.append(np.empty(capacity, dtype=NP_DTYPES[c.type]))
            valid.append(np.empty((capacity + 7) // 8, dtype=np.uint8))
        b = abi.Batch()
        b.n_columns = len(self.schema)
        vp = (C.c_void_p * len(vals))(*[v.ctypes.data for v in vals])
        bp = (C.c_void_p * len(valid))(*[v.ctypes.data for v in valid])
        b.values = vp
        b.validity = bp
        b.capacity_rows = capacity
        done = C.c_int32()
        self._next_c(b, done)
        n = b.row_count
        if n == 0 and done.value:
            return None
        out_v = [v[:n] for v in vals]
        out_ok = [np.unpackbits(bm, bitorder="little")[:n].astype(bool) if c.nullable else None
                  for bm, c in zip(valid, self.schema)]
        return Batch(self.schema, out_v, out_ok, n)

    def collect(self, capacity: int = 1 << 20) -> dict:
        """Drain the query: {column name: (values, validity or None)} in result order."""
        parts: list[Batch] = []
        rows = self._result_rows()
        if rows is not None:
            capacity = max(1, min(capacity, rows))
        while True:
            b = self.next(capacity)
            if b is None:
                break
            parts.append(b)
            if b.row_count < capacity:
                # the next call returns the end marker
                continue
        out = {}
        for i, c in enumerate(self.schema):
            if parts:
                v = np.concatenate([p.values[i] for p in parts])
                ok = np.concatenate([p.validity[i] for p in parts]) if c.nullable else None
            else:
                v = np.zeros((0, 2) if c.type == abi.DECIMAL128 else 0,
                             dtype=np.int64 if c.type == abi.DECIMAL128 else NP_DTYPES[c.type])
                ok = np.zeros(0, dtype=bool) if c.nullable else None
            out[c.name] = (v, ok)
        return out

    def key_strings(self, column: int, codes: np.ndarray) -> list:
        """The strings of DICT32 key codes (late materialisation through
        tgpu_query_key_strings); column is the output column index."""
        codes = np.ascontiguousarray(codes, dtype=np.int64 if self.schema[column].type == abi.VARCHAR else np.int32)
        n = len(codes)
        offs = np.zeros(n + 1, dtype=np.uint64)
        need = C.c_uint64()
        _check(lib().tgpu_query_key_strings(self.handle, column, codes.ctypes.data, n, offs.ctypes.data, None, 0,
                                            C.byref(need)))
        blob = np.zeros(max(1, need.value), dtype=np.uint8)
        _check(lib().tgpu_query_key_strings(self.handle, column, codes.ctypes.data, n, offs.ctypes.data,
                                            blob.ctypes.data, need.value, C.byref(need)))
        raw = blob.tobytes()
        return [raw[int(offs[i]):int(offs[i + 1])].decode() for i in range(n)]

    def collect_strings(self, capacity: int = 1 << 20) -> dict:
        """collect() with every DICT32 key column's codes replaced by its
        strings (None for a NULL key)."""
        out = self.collect(capacity)
        for i, c in enumerate(self.schema):
            if c.type not in (abi.DICT32, abi.VARCHAR):  # only group keys come out as strings
                continue
            vals, ok = out[c.name]
            strs = self.key_strings(i, np.where(ok, vals, 0) if ok is not None else vals)
            if ok is not None:
                strs = [s if o else None for s, o in zip(strs, ok)]
            out[c.name] = (strs, ok)
        return out

    def _result_rows(self) -> Optional[int]:
        """Rows the current execution emits (a zero-row next runs or waits for
        it), so collect sizes its buffers to the result."""
        if self.next(0) is None:
            return 0
        return int(self.stats().result_rows)

    def cancel(self) -> None:
        _check(lib().tgpu_query_cancel(self.handle))

    def stats(self) -> abi.QueryStats:
        s = abi.QueryStats()
        _check(lib().tgpu_query_get_stats(self.handle, C.byref(s)))
        return s

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().tgpu_query_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _schema(cols) -> list:
    return [OutCol(c.name.decode(), c.type, bool(c.nullable), c.elem_bytes, c.decimal_precision, c.decimal_scale)
            for c in cols]


def request_shape(table: Table, req: Request, batched: bool = False) -> dict:
    """The shape class (tuning-table key) of `req` on `table`."""
    creq, _keep = build_request(table, req)
    out = abi.Shape()
    _check(lib().tgpu_request_shape(table.handle, C.byref(creq), 1 if batched else 0, C.byref(out)))
    return out.as_dict()


def try_build_group_topn(table: Table, req: Request) -> Optional[Query]:
    """v2_pipeline.tryBuildGroupTopN: a Query, or None when the shape declines."""
    r, keep = build_request(table, req)
    h = C.c_void_p()
    st = lib().tgpu_query_create(table.handle, C.byref(r), C.byref(h))
    del keep
    if st == abi.DECLINE:
        return None
    _check(st)
    return Query(h, table)


class _BatchMember(Query):
    """Result view of one query of a QueryBatch (same next/collect as Query)."""

    def __init__(self, batch: "QueryBatch", index: int):
        self.batch = batch
        self.index = index
        self.handle = None
        self.table = batch.table
        n = C.c_uint32()
        _check(lib().tgpu_batch_output_schema(batch.handle, index, None, 0, C.byref(n)))
        cols = (abi.OutputColumn * n.value)()
        _check(lib().tgpu_batch_output_schema(batch.handle, index, cols, n.value, C.byref(n)))
        self.schema = _schema(cols)

    def _next_c(self, b, done) -> None:
        _check(lib().tgpu_batch_next(self.batch.handle, self.index, C.byref(b), C.byref(done)))

    def _result_rows(self) -> Optional[int]:
        return None

    def close(self) -> None:
        pass


class QueryBatch:
    """Many GROUP BY queries over one table in one persistent kernel
    (optionally replayed from a captured CUDA graph)."""

    def __init__(self, table: Table, requests: Sequence[Request], graph: bool = True, stream: int = 0):
        self.table = table
        reqs = (abi.Request * len(requests))()
        keep = []
        for i, rq in enumerate(requests):
            r, k = build_request(table, rq)
            reqs[i] = r
            keep.append(k)
        h = C.c_void_p()
        st = lib().tgpu_batch_create(table.handle, reqs, len(requests), abi.BATCH_GRAPH if graph else 0,
                                     stream or None, C.byref(h))
        del keep
        if st == abi.DECLINE:
            raise EngineError(st, (lib().tgpu_last_error_message() or b"").decode())
        _check(st)
        self.handle = h
        self.members = [_BatchMember(self, i) for i in range(len(requests))]

    def execute(self) -> None:
        _check(lib().tgpu_batch_execute(self.handle))

    def synchronize(self) -> None:
        _check(lib().tgpu_batch_synchronize(self.handle))

    def collect(self, i: int, capacity: int = 1 << 20) -> dict:
        return self.members[i].collect(capacity)

    def cancel(self) -> None:
        _check(lib().tgpu_batch_cancel(self.handle))

    def stats(self) -> abi.BatchStats:
        s = abi.BatchStats()
        _check(lib().tgpu_batch_get_stats(self.handle, C.addressof(s)))
        return s

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().tgpu_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _ServerResult(Query):
    """Result view of one finished server ticket (same next/collect as Query)."""

    def __init__(self, server: "Server", ticket: int):
        self.server = server
        self.ticket = ticket
        self.handle = None
        self.table = None
        n = C.c_uint32()
        _check(lib().tgpu_server_output_schema(server.handle, ticket, None, 0, C.byref(n)))
        cols = (abi.OutputColumn * n.value)()
        _check(lib().tgpu_server_output_schema(server.handle, ticket, cols, n.value, C.byref(n)))
        self.schema = _schema(cols)

    def _next_c(self, b, done) -> None:
        _check(lib().tgpu_server_next(self.server.handle, self.ticket, C.byref(b), C.byref(done)))

    def _result_rows(self) -> Optional[int]:
        return None

    def close(self) -> None:
        pass


class Server:
    """Continuous-batching request loop over resident tables (native dispatcher)."""

    def __init__(self, tables: Sequence[Table], mode: str = "continuous", memory_budget: int = 0,
                 max_batch: int = 0, max_inflight: int = 0, batch_min: int = 0):
        self.tables = list(tables)
        arr = (C.c_void_p * len(self.tables))(*[t.handle.value for t in self.tables])
        o = abi.ServerOptions()
        o.memory_budget_bytes = memory_budget
        o.max_batch = max_batch
        o.max_inflight = max_inflight
        o.batch_min = batch_min
        o.mode = abi.SERVE_PLAIN if mode == "plain" else abi.SERVE_CONTINUOUS
        h = C.c_void_p()
        _check(lib().tgpu_server_create(arr, len(self.tables), C.byref(o), C.byref(h)))
        self.handle = h

    def submit(self, table_index: int, req: Request) -> int:
        r, keep = build_request(self.tables[table_index], req)
        t = C.c_uint64()
        _check(lib().tgpu_server_submit(self.handle, table_index, C.byref(r), C.byref(t)))
        del keep
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1) -> bool:
        d = C.c_int32()
        _check(lib().tgpu_server_wait(self.handle, ticket, timeout_ms, C.byref(d)))
        return bool(d.value)

    def result(self, ticket: int) -> dict:
        self.wait(ticket)
        return _ServerResult(self, ticket).collect()

    def release(self, ticket: int) -> None:
        _check(lib().tgpu_server_release(self.handle, ticket))

    def stats(self) -> abi.ServerStats:
        s = abi.ServerStats()
        _check(lib().tgpu_server_get_stats(self.handle, C.byref(s)))
        return s

    def run_load(self, mix: Sequence[tuple], rate_qps: float, duration_s: float, seed: int = 1) -> dict:
        """Open-loop Poisson load over `mix` = [(table index, Request)]; latency percentiles in ms."""
        reqs = (abi.Request * len(mix))()
        tabs = (C.c_uint32 * len(mix))()
        keep = []
        for i, (ti, rq) in enumerate(mix):
            r, k = build_request(self.tables[ti], rq)
            reqs[i] = r
            tabs[i] = ti
            keep.append(k)
        spec = abi.LoadSpec()
        spec.table_of = tabs
        spec.requests = reqs
        spec.n_requests = len(mix)
        spec.rate_qps = rate_qps
        spec.duration_s = duration_s
        spec.seed = seed
        rep = abi.LoadReport()
        _check(lib().tgpu_server_run_load(self.handle, C.byref(spec), C.byref(rep)))
        del keep
        return {f: getattr(rep, f) for f, _ in abi.LoadReport._fields_}

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().tgpu_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
