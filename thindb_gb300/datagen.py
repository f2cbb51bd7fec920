"""Seeded synthetic inputs (libthindb_datagen.so): see csrc/datagen.cpp for the
distributions.  Each function fills numpy arrays, or caller buffers given as
raw pointers (e.g. pinned host tensors)."""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

_LIB: Optional[C.CDLL] = None
LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libthindb_datagen.so")

P = C.c_void_p
U64 = C.c_uint64


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"datagen library missing at {LIB_PATH}: run thindb_gb300.build first")
        L = C.CDLL(LIB_PATH)
        L.tdg_splitmix_at.restype = U64
        L.tdg_splitmix_at.argtypes = [U64, U64]
        L.tdg_mix64.restype = U64
        L.tdg_mix64.argtypes = [U64]
        L.tdg_plain.argtypes = [U64, U64, P, P, C.c_int]
        L.tdg_filtered.argtypes = [U64, U64, U64, P, P, P, C.c_int]
        L.tdg_extra_keys.argtypes = [U64, U64, P, P, P, C.c_int]
        L.tdg_distinct.argtypes = [U64, U64, U64, P, P, P, P, C.c_int]
        L.tdg_url_dictionary.restype = U64
        L.tdg_url_dictionary.argtypes = [U64, C.c_uint32, P, P, U64]
        _LIB = L
    return _LIB


PLAIN_ROWS = 16_777_216
FILTERED_ROWS = 100_000_000
FILTERED_KEYS = 10_000_000
DISTINCT_ROWS = 200_000_000
DISTINCT_USERS = 5_000_000
DATE_BASE = 20454          # 2026-01-01 in days since 1970-01-01
FILTER_LO = DATE_BASE + 100
FILTER_HI = DATE_BASE + 135


def plain(n: int = PLAIN_ROWS, seed: int = 1, threads: int = 0) -> dict:
    k = np.empty(n, np.int64)
    v = np.empty(n, np.int32)
    lib().tdg_plain(n, seed, k.ctypes.data, v.ctypes.data, threads)
    return {"k": k, "v": v}


def filtered(n: int = FILTERED_ROWS, seed: int = 2, n_keys: int = FILTERED_KEYS, threads: int = 0) -> dict:
    k = np.empty(n, np.int64)
    a = np.empty(n, np.int64)
    d = np.empty(n, np.int32)
    lib().tdg_filtered(n, seed, n_keys, k.ctypes.data, a.ctypes.data, d.ctypes.data, threads)
    return {"k": k, "amount": a, "d": d}


def filtered_into(n: int, seed: int, n_keys: int, k_ptr: int, a_ptr: int, d_ptr: int, threads: int = 0) -> None:
    lib().tdg_filtered(n, seed, n_keys, k_ptr, a_ptr, d_ptr, threads)


def extra_keys(n: int = FILTERED_ROWS, seed: int = 2, threads: int = 0) -> dict:
    a = np.empty(n, np.int32)
    b = np.empty(n, np.int32)
    c = np.empty(n, np.int32)
    lib().tdg_extra_keys(n, seed, a.ctypes.data, b.ctypes.data, c.ctypes.data, threads)
    return {"k10": a, "k1k": b, "k1m": c}


def distinct(n: int = DISTINCT_ROWS, seed: int = 3, n_users: int = DISTINCT_USERS, threads: int = 0) -> dict:
    r = np.empty(n, np.int16)
    u = np.empty(n, np.int32)
    us = np.empty(n, np.int64)
    lat = np.empty(n, np.float64)
    lib().tdg_distinct(n, seed, n_users, r.ctypes.data, u.ctypes.data, us.ctypes.data, lat.ctypes.data, threads)
    return {"region": r, "url": u, "user_id": us, "latency_ms": lat}


def url_dictionary(seed: int = 3, count: int = 50_000) -> list[str]:
    need = lib().tdg_url_dictionary(seed, count, None, None, 0)
    offs = np.empty(count + 1, np.uint32)
    blob = np.empty(max(1, need), np.uint8)
    lib().tdg_url_dictionary(seed, count, offs.ctypes.data, blob.ctypes.data, need)
    raw = blob.tobytes()
    return [raw[offs[i]:offs[i + 1]].decode() for i in range(count)]


def splitmix_at(seed: int, i: int) -> int:
    return int(lib().tdg_splitmix_at(seed, i))
