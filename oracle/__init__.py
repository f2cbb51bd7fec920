"""Python binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this;
the product never imports it.  `run(columns, request)` evaluates a GROUP BY
with the C++ restatement of thinDB's semantics (oracle.cpp) over host numpy
columns and returns {output name: (values, validity or None)}.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

from thindb_gb300 import abi
from thindb_gb300.engine import NP_DTYPES, Column, Request, build_request, varchar_buffers

from . import build as _build

_LIB: Optional[C.CDLL] = None


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        so = _build.SO
        if not os.path.exists(so):
            _build.build()
        L = C.CDLL(so)
        L.orc_group_by.restype = C.c_int
        L.orc_group_by.argtypes = [C.POINTER(abi.TableDesc), C.POINTER(abi.Request), C.c_int, C.POINTER(C.c_void_p)]
        L.orc_result_rows.restype = C.c_uint64
        L.orc_result_rows.argtypes = [C.c_void_p]
        L.orc_result_cols.restype = C.c_uint32
        L.orc_result_cols.argtypes = [C.c_void_p]
        L.orc_result_groups.restype = C.c_uint64
        L.orc_result_groups.argtypes = [C.c_void_p]
        L.orc_result_selected.restype = C.c_uint64
        L.orc_result_selected.argtypes = [C.c_void_p]
        L.orc_result_data.restype = C.c_void_p
        L.orc_result_data.argtypes = [C.c_void_p, C.c_uint32]
        L.orc_result_valid.restype = C.c_void_p
        L.orc_result_valid.argtypes = [C.c_void_p, C.c_uint32]
        L.orc_result_schema.restype = C.c_int
        L.orc_result_schema.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(abi.OutputColumn)]
        L.orc_result_free.argtypes = [C.c_void_p]
        L.orc_last_error.restype = C.c_char_p
        L.orc_i128_to_f64.restype = C.c_double
        L.orc_i128_to_f64.argtypes = [C.c_uint64, C.c_int64]
        L.orc_avg_decimal.restype = C.c_double
        L.orc_avg_decimal.argtypes = [C.c_uint64, C.c_int64, C.c_uint64, C.c_int32]
        _LIB = L
    return _LIB


class HostTable:
    """Host columns described like engine.Table (names, types, validity)."""

    def __init__(self, columns: Sequence[Column], row_group_rows: int = 65536):
        self.columns = list(columns)
        self.row_group_rows = row_group_rows
        self.n_rows = len(self.columns[0].data)
        self._keep: list = []
        self.descs = (abi.ColumnDesc * len(self.columns))()
        for i, c in enumerate(self.columns):
            d = self.descs[i]
            nm = c.name.encode()
            d.name = nm
            d.type = c.type
            d.decimal_precision = c.precision
            d.decimal_scale = c.scale
            if c.type == abi.VARCHAR:
                offs, blob = varchar_buffers(c.data)
                self._keep += [nm, offs, blob]
                d.data = offs.ctypes.data
                d.dict_bytes = blob.ctypes.data
            else:
                arr = np.ascontiguousarray(c.data, dtype=NP_DTYPES[c.type])
                self._keep += [nm, arr]
                d.data = arr.ctypes.data
            if c.validity is not None:
                bm = np.packbits(np.asarray(c.validity, dtype=bool), bitorder="little")
                self._keep.append(bm)
                d.validity = bm.ctypes.data
            if c.type == abi.DICT32 and c.dictionary is not None:
                enc = [s.encode() if isinstance(s, str) else bytes(s) for s in c.dictionary]
                offs = np.zeros(len(enc) + 1, dtype=np.uint32)
                offs[1:] = np.cumsum([len(e) for e in enc], dtype=np.uint64).astype(np.uint32)
                blob = np.frombuffer(b"".join(enc) or b"\0", dtype=np.uint8).copy()
                self._keep += [offs, blob]
                d.dict_offsets = offs.ctypes.data
                d.dict_bytes = blob.ctypes.data
                d.dict_size = len(enc)
        self.desc = abi.TableDesc()
        self.desc.columns = self.descs
        self.desc.n_columns = len(self.columns)
        self.desc.row_group_rows = row_group_rows
        self.desc.n_rows = self.n_rows
        self.desc.location = abi.LOC_HOST

    def col_index(self, name: str) -> int:
        for i, c in enumerate(self.columns):
            if c.name.lower() == name.lower():
                return i
        raise KeyError(name)


class OracleDecline(Exception):
    pass


def run(table: HostTable, req: Request, threads: int = 1) -> dict:
    """Evaluate `req`; raises OracleDecline for shapes the engine declines."""
    r, keep = build_request(table, req)
    h = C.c_void_p()
    st = lib().orc_group_by(C.byref(table.desc), C.byref(r), threads, C.byref(h))
    if st == abi.DECLINE:
        raise OracleDecline(lib().orc_last_error().decode())
    if st != abi.OK:
        raise RuntimeError(f"oracle status {st}: {lib().orc_last_error().decode()}")
    try:
        rows = lib().orc_result_rows(h)
        out = {}
        for c in range(lib().orc_result_cols(h)):
            oc = abi.OutputColumn()
            lib().orc_result_schema(h, c, C.byref(oc))
            eb = oc.elem_bytes
            raw = C.string_at(lib().orc_result_data(h, c), rows * eb) if rows else b""
            if oc.type == abi.DECIMAL128:
                vals = np.frombuffer(raw, dtype=np.int64).reshape(-1, 2).copy()
            else:
                vals = np.frombuffer(raw, dtype=NP_DTYPES[oc.type]).copy()
            ok = np.frombuffer(C.string_at(lib().orc_result_valid(h, c), rows) if rows else b"",
                               dtype=np.uint8).astype(bool)
            out[oc.name.decode()] = (vals, ok if oc.nullable else None)
        out["__groups__"] = lib().orc_result_groups(h)
        out["__selected__"] = lib().orc_result_selected(h)
        return out
    finally:
        lib().orc_result_free(h)
        del keep


def i128_to_f64(lo: int, hi: int) -> float:
    return lib().orc_i128_to_f64(lo & ((1 << 64) - 1), hi)


class SegmentError(Exception):
    def __init__(self, status: int, message: str):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def decode_segment(image: bytes, types: Sequence[int], nullable: Sequence[bool], threads: int = 1) -> list:
    """Decode a segment image (segment.cpp) into [(values, validity or None)]
    per column; `nullable[c]` asks for column c's validity."""
    L = lib()
    if not hasattr(L, "_seg_bound"):
        L.orc_segment_decode.restype = C.c_int
        L.orc_segment_decode.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(C.c_uint32), C.c_uint32,
                                         C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_int]
        L.orc_segment_error.restype = C.c_char_p
        L._seg_bound = True
    buf = np.frombuffer(bytes(image), dtype=np.uint8)
    n = int(buf[24:32].view(np.uint64)[0]) if buf.size >= 32 else 0
    nc = len(types)
    elem = (C.c_uint32 * nc)(*[abi.TYPE_BYTES[t] for t in types])
    vals = [np.zeros(n, dtype=NP_DTYPES[t]) for t in types]
    bms = [np.zeros((n + 7) // 8 + 1, dtype=np.uint8) if nullable[c] else None for c, t in enumerate(types)]
    outs = (C.c_void_p * nc)(*[v.ctypes.data for v in vals])
    valid = (C.c_void_p * nc)(*[b.ctypes.data if b is not None else None for b in bms])
    st = L.orc_segment_decode(buf.ctypes.data, buf.size, elem, nc, outs, valid, threads)
    if st != abi.OK:
        raise SegmentError(st, L.orc_segment_error().decode())
    return [(v, None if b is None else np.unpackbits(b, bitorder="little")[:n].astype(bool)) for v, b in zip(vals, bms)]
