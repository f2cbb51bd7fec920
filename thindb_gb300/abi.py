"""ctypes mirror of include/thindb_gpu.h (types only; no library is loaded here)."""
from __future__ import annotations

import ctypes as C

ABI_VERSION = 2

# tgpu_status
OK, DECLINE, ERR_INVALID_ARGUMENT, ERR_MEMORY_BUDGET, ERR_UNSUPPORTED_TYPE, ERR_CANCELLED, ERR_CUDA, \
    ERR_DEVICE_TIMEOUT, ERR_INTERNAL, ERR_NO_DEVICE = range(10)
STATUS_NAMES = {
    OK: "OK", DECLINE: "DECLINE", ERR_INVALID_ARGUMENT: "INVALID_ARGUMENT", ERR_MEMORY_BUDGET: "MEMORY_BUDGET",
    ERR_UNSUPPORTED_TYPE: "UNSUPPORTED_TYPE", ERR_CANCELLED: "CANCELLED", ERR_CUDA: "CUDA",
    ERR_DEVICE_TIMEOUT: "DEVICE_TIMEOUT", ERR_INTERNAL: "INTERNAL", ERR_NO_DEVICE: "NO_DEVICE",
}

# tgpu_type
BOOLEAN, TINYINT, SMALLINT, INT, DATE, BIGINT, DATETIME, DECIMAL64, FLOAT, DOUBLE, DECIMAL128, DICT32, VARCHAR = \
    range(1, 14)
TYPE_NAMES = {BOOLEAN: "BOOLEAN", TINYINT: "TINYINT", SMALLINT: "SMALLINT", INT: "INT", DATE: "DATE",
              BIGINT: "BIGINT", DATETIME: "DATETIME", DECIMAL64: "DECIMAL64", FLOAT: "FLOAT", DOUBLE: "DOUBLE",
              DECIMAL128: "DECIMAL128", DICT32: "DICT32", VARCHAR: "VARCHAR"}
# (a VARCHAR output column holds one i64 row index per group)
TYPE_BYTES = {BOOLEAN: 1, TINYINT: 1, SMALLINT: 2, INT: 4, DATE: 4, BIGINT: 8, DATETIME: 8, DECIMAL64: 8,
              FLOAT: 4, DOUBLE: 8, DECIMAL128: 16, DICT32: 4, VARCHAR: 8}

LOC_HOST, LOC_DEVICE = 0, 1

# tgpu_agg_func
AGG_COUNT, AGG_SUM, AGG_AVG, AGG_MIN, AGG_MAX, AGG_COUNT_DISTINCT, AGG_UDF = range(1, 8)
AGG_BY_NAME = {"count": AGG_COUNT, "sum": AGG_SUM, "avg": AGG_AVG, "min": AGG_MIN, "max": AGG_MAX,
               "count_distinct": AGG_COUNT_DISTINCT, "udf": AGG_UDF}

# tgpu_pred_op
PRED_BETWEEN, PRED_NOT_BETWEEN, PRED_EQ, PRED_NE, PRED_LT, PRED_LE, PRED_GT, PRED_GE, PRED_IS_NULL, \
    PRED_IS_NOT_NULL = range(1, 11)
PRED_BY_NAME = {"between": PRED_BETWEEN, "not_between": PRED_NOT_BETWEEN, "=": PRED_EQ, "!=": PRED_NE,
                "<": PRED_LT, "<=": PRED_LE, ">": PRED_GT, ">=": PRED_GE, "is_null": PRED_IS_NULL,
                "is_not_null": PRED_IS_NOT_NULL}

SORT_KEY, SORT_AGG = 1, 2
NO_LIMIT = (1 << 64) - 1

FLAG_TIMING = 0x1
FLAG_FORCE_GLOBAL = 0x2
FLAG_DENSE_SCAN = 0x4
FLAG_NO_WARP_COMBINE = 0x8
FLAG_GATHER_SCAN = 0x10
FLAG_NO_TUNING = 0x20
FLAG_STAGED_SCAN = 0x40
FLAG_NO_STAGED = 0x80
FLAG_NO_PREFETCH = 0x100
FLAG_NO_CHUNK_PREFETCH = 0x200
FLAG_DISTINCT_PREFETCH = 0x400
FLAG_DISTINCT_PARTITION = 0x800
FLAG_NO_DISTINCT_PARTITION = 0x1000
FLAG_QUEUE_SCAN = 0x2000
FLAG_PIPE_SCAN = 0x4000
FLAG_NO_PIPE = 0x8000
FLAG_COUNT_SKETCH = 0x10000
FLAG_NO_COUNT_SKETCH = 0x20000
FLAG_RADIX = 0x40000
FLAG_NO_RADIX = 0x80000
FLAG_INLINE_FOLD = 0x100000
FLAG_SPLIT_SCAN = 0x200000
FLAG_NO_SPLIT = 0x400000
STAT_TUNED = 0x1
STAT_GATHER = 0x2
STAT_STAGED = 0x4
STAT_DISTINCT_PARTITION = 0x8
STAT_QUEUE = 0x10
STAT_PIPE = 0x20
STAT_COUNT_SKETCH = 0x40
STAT_SKETCH_RERUN = 0x80
STAT_RADIX = 0x100
STAT_SPLIT = 0x200


class ColumnDesc(C.Structure):
    _fields_ = [("name", C.c_char_p), ("type", C.c_int32), ("decimal_precision", C.c_uint8),
                ("decimal_scale", C.c_uint8), ("reserved", C.c_uint8 * 2), ("data", C.c_void_p),
                ("validity", C.c_void_p), ("dict_offsets", C.c_void_p), ("dict_bytes", C.c_void_p),
                ("dict_size", C.c_uint32), ("reserved2", C.c_uint32), ("ndv_hint", C.c_uint64)]


class TableDesc(C.Structure):
    _fields_ = [("columns", C.POINTER(ColumnDesc)), ("n_columns", C.c_uint32), ("row_group_rows", C.c_uint32),
                ("n_rows", C.c_uint64), ("location", C.c_int32), ("compute_ndv", C.c_int32),
                ("stream", C.c_void_p)]


class AggSpec(C.Structure):
    _fields_ = [("func", C.c_int32), ("column", C.c_int32), ("as_", C.c_char_p), ("udf_name", C.c_char_p)]


class Predicate(C.Structure):
    _fields_ = [("column", C.c_int32), ("op", C.c_int32), ("lo", C.c_int64), ("hi", C.c_int64),
                ("flo", C.c_double), ("fhi", C.c_double)]


class Having(C.Structure):
    _fields_ = [("agg", C.c_int32), ("op", C.c_int32), ("ival", C.c_int64), ("fval", C.c_double)]


class SortSpec(C.Structure):
    _fields_ = [("target", C.c_int32), ("index", C.c_int32), ("desc", C.c_int32), ("reserved", C.c_int32)]


class Request(C.Structure):
    _fields_ = [("group_cols", C.POINTER(C.c_int32)), ("n_group_cols", C.c_uint32),
                ("aggs", C.POINTER(AggSpec)), ("n_aggs", C.c_uint32),
                ("where", C.POINTER(Predicate)), ("n_where", C.c_uint32),
                ("having", C.POINTER(Having)), ("n_having", C.c_uint32),
                ("order", C.POINTER(SortSpec)), ("n_order", C.c_uint32),
                ("limit", C.c_uint64), ("offset", C.c_uint64), ("expected_groups", C.c_uint64),
                ("memory_budget_bytes", C.c_uint64), ("stream", C.c_void_p), ("flags", C.c_int32),
                ("chunk_rows", C.c_int32), ("cache_slots", C.c_int32), ("table_load_pct", C.c_int32)]


class OutputColumn(C.Structure):
    _fields_ = [("name", C.c_char * 64), ("type", C.c_int32), ("decimal_precision", C.c_uint8),
                ("decimal_scale", C.c_uint8), ("nullable", C.c_uint8), ("reserved", C.c_uint8),
                ("elem_bytes", C.c_uint32), ("reserved2", C.c_uint32)]


class Batch(C.Structure):
    _fields_ = [("n_columns", C.c_uint32), ("reserved", C.c_uint32), ("values", C.POINTER(C.c_void_p)),
                ("validity", C.POINTER(C.c_void_p)), ("capacity_rows", C.c_uint64), ("row_count", C.c_uint64)]


class QueryStats(C.Structure):
    _fields_ = [("rows_scanned", C.c_uint64), ("rows_selected", C.c_uint64), ("groups", C.c_uint64),
                ("result_rows", C.c_uint64), ("table_capacity", C.c_uint64), ("distinct_capacity", C.c_uint64),
                ("row_groups_total", C.c_uint32), ("row_groups_pruned", C.c_uint32), ("route", C.c_uint32),
                ("retries", C.c_uint32), ("kernel_launches", C.c_uint32), ("flags", C.c_uint32),
                ("scan_ms", C.c_double), ("finalize_ms", C.c_double), ("total_ms", C.c_double),
                ("device_bytes", C.c_uint64)]


# Every entry point include/thindb_gpu.h declares: (name, restype, argtypes).
SIGNATURES = [
    ("tgpu_abi_version", C.c_uint32, []),
    ("tgpu_build_info", C.c_char_p, []),
    ("tgpu_last_error_message", C.c_char_p, []),
    ("tgpu_table_register", C.c_int, [C.POINTER(TableDesc), C.POINTER(C.c_void_p)]),
    ("tgpu_table_destroy", C.c_int, [C.c_void_p]),
    ("tgpu_table_info", C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32),
                                  C.POINTER(C.c_uint64)]),
    ("tgpu_query_create", C.c_int, [C.c_void_p, C.POINTER(Request), C.POINTER(C.c_void_p)]),
    ("tgpu_query_output_schema", C.c_int, [C.c_void_p, C.POINTER(OutputColumn), C.c_uint32,
                                           C.POINTER(C.c_uint32)]),
    ("tgpu_query_execute", C.c_int, [C.c_void_p]),
    ("tgpu_query_next", C.c_int, [C.c_void_p, C.POINTER(Batch), C.POINTER(C.c_int32)]),
    ("tgpu_query_cancel", C.c_int, [C.c_void_p]),
    ("tgpu_query_key_strings", C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p,
                                         C.c_uint64, C.POINTER(C.c_uint64)]),
    ("tgpu_query_get_stats", C.c_int, [C.c_void_p, C.POINTER(QueryStats)]),
    ("tgpu_query_destroy", C.c_int, [C.c_void_p]),
    ("tgpu_query_synchronize", C.c_int, [C.c_void_p]),
    ("tgpu_batch_create", C.c_int, [C.c_void_p, C.POINTER(Request), C.c_uint32, C.c_int32, C.c_void_p,
                                    C.POINTER(C.c_void_p)]),
    ("tgpu_batch_execute", C.c_int, [C.c_void_p]),
    ("tgpu_batch_synchronize", C.c_int, [C.c_void_p]),
    ("tgpu_batch_output_schema", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(OutputColumn), C.c_uint32,
                                           C.POINTER(C.c_uint32)]),
    ("tgpu_batch_next", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(Batch), C.POINTER(C.c_int32)]),
    ("tgpu_batch_cancel", C.c_int, [C.c_void_p]),
    ("tgpu_batch_get_stats", C.c_int, [C.c_void_p, C.c_void_p]),
    ("tgpu_batch_destroy", C.c_int, [C.c_void_p]),
]

BATCH_GRAPH = 0x1
SERVE_CONTINUOUS, SERVE_PLAIN = 0, 1


class ServerOptions(C.Structure):
    _fields_ = [("memory_budget_bytes", C.c_uint64), ("max_batch", C.c_uint32), ("max_inflight", C.c_uint32),
                ("mode", C.c_int32), ("batch_min", C.c_int32)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("waves", C.c_uint64), ("peak_admitted_bytes", C.c_uint64), ("peak_queued", C.c_uint64)]


class LoadSpec(C.Structure):
    _fields_ = [("table_of", C.POINTER(C.c_uint32)), ("requests", C.POINTER(Request)), ("n_requests", C.c_uint32),
                ("reserved", C.c_uint32), ("rate_qps", C.c_double), ("duration_s", C.c_double),
                ("seed", C.c_uint64)]


class LoadReport(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("elapsed_s", C.c_double), ("achieved_qps", C.c_double), ("p50_ms", C.c_double),
                ("p99_ms", C.c_double), ("p999_ms", C.c_double), ("max_ms", C.c_double), ("mean_ms", C.c_double)]


SIGNATURES += [
    ("tgpu_server_create", C.c_int, [C.POINTER(C.c_void_p), C.c_uint32, C.POINTER(ServerOptions),
                                     C.POINTER(C.c_void_p)]),
    ("tgpu_server_submit", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(Request), C.POINTER(C.c_uint64)]),
    ("tgpu_server_wait", C.c_int, [C.c_void_p, C.c_uint64, C.c_int32, C.POINTER(C.c_int32)]),
    ("tgpu_server_output_schema", C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(OutputColumn), C.c_uint32,
                                            C.POINTER(C.c_uint32)]),
    ("tgpu_server_next", C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(Batch), C.POINTER(C.c_int32)]),
    ("tgpu_server_release", C.c_int, [C.c_void_p, C.c_uint64]),
    ("tgpu_server_get_stats", C.c_int, [C.c_void_p, C.POINTER(ServerStats)]),
    ("tgpu_server_destroy", C.c_int, [C.c_void_p]),
    ("tgpu_server_run_load", C.c_int, [C.c_void_p, C.POINTER(LoadSpec), C.POINTER(LoadReport)]),
]


class BatchStats(C.Structure):
    _fields_ = [("n_queries", C.c_uint32), ("kernel_launches", C.c_uint32), ("graph", C.c_uint32),
                ("rerun_queries", C.c_uint32), ("work_items", C.c_uint64), ("total_ms", C.c_double)]


class Shape(C.Structure):
    _fields_ = [("key_words", C.c_int32), ("fold", C.c_int32), ("n_aggs", C.c_int32), ("distinct", C.c_int32),
                ("filtered", C.c_int32), ("sel_log2", C.c_int32), ("groups_log2", C.c_int32),
                ("batched", C.c_int32)]

    def as_dict(self):
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


class Tuning(C.Structure):
    _fields_ = [("shape", Shape), ("chunk_rows", C.c_int32), ("cache_slots", C.c_int32),
                ("table_load_pct", C.c_int32), ("flags", C.c_int32), ("groups_shift", C.c_int32),
                ("reserved", C.c_int32)]


SIGNATURES += [
    ("tgpu_request_shape", C.c_int, [C.c_void_p, C.POINTER(Request), C.c_int32, C.POINTER(Shape)]),
    ("tgpu_tuning_set", C.c_int, [C.POINTER(Tuning), C.c_uint32]),
    ("tgpu_tuning_get", C.c_uint32, [C.POINTER(Tuning), C.c_uint32]),
    ("tgpu_debug_set_wait_limit", C.c_int, [C.c_uint64]),
    ("tgpu_debug_set_digest_bits", C.c_int, [C.c_uint32]),
]


class SegmentColumn(C.Structure):
    _fields_ = [("name", C.c_char_p), ("type", C.c_int32), ("decimal_precision", C.c_uint8),
                ("decimal_scale", C.c_uint8), ("reserved", C.c_uint8 * 2)]


class LoadStats(C.Structure):
    _fields_ = [("image_bytes", C.c_uint64), ("decoded_bytes", C.c_uint64), ("blocks", C.c_uint32),
                ("kernel_launches", C.c_uint32), ("chunks", C.c_uint32), ("reserved", C.c_uint32),
                ("h2d_ms", C.c_double), ("decode_ms", C.c_double), ("stats_ms", C.c_double),
                ("pipeline_ms", C.c_double), ("first_decode_ms", C.c_double), ("total_ms", C.c_double)]


SIGNATURES += [
    ("tgpu_table_load_stats", C.c_int, [C.c_void_p, C.POINTER(LoadStats)]),
    ("tgpu_aggregate_register", C.c_int, [C.c_char_p]),
    ("tgpu_aggregate_unregister", C.c_int, [C.c_char_p]),
    ("tgpu_aggregate_registered", C.c_int32, [C.c_char_p]),
    ("tgpu_table_read_column", C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    ("tgpu_table_register_segment", C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(SegmentColumn), C.c_uint32,
                                              C.c_int32, C.c_void_p, C.POINTER(C.c_void_p)]),
]
