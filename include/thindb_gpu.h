/*
 * thindb_gpu.h — plain-C boundary of the GB300 grouped-aggregation operator.
 *
 * This header is the whole interface between thinDB's Zig host and the CUDA
 * engine: it uses only C scalar types, fixed-size structs and opaque handles,
 * so Zig can `@cImport` it unchanged (no C++ and no torch types appear here).
 *
 * Reference interfaces replaced (paths inside the thinDB source tree):
 *   - the operator handle `exec.Query` + `VTable`      src/exec/exec.zig:299-373, :903-1218
 *   - `makeQuery` (operator -> Query)                  src/exec/exec.zig:1221-1239
 *   - the routing points `tryBuildGroupTopN` /
 *     `tryBuildLowCardGroup` (null = decline)          src/exec/v2_pipeline.zig:17-34,
 *                                                      called from src/exec/engine_v2.zig:968-972
 *   - the request `GroupTopNRequest`                   src/exec/v2_shape_group_topn.zig:63-101
 *   - `AggSpec` / `AggFunc`                            src/exec/aggregate.zig:88, :237-267
 *   - `SortSpec` (ORDER BY key + direction)            src/exec/sort.zig:28-31
 *   - `Batch` / `ColumnView` output (bit 1 = valid)    src/exec/exec.zig:175-236,
 *                                                      src/storage/column.zig:28-46, :207-210
 *   - error set `exec.Error` (MemoryBudgetExceeded,
 *     UnsupportedOperatorForType, QueryCancelled)      src/exec/exec.zig:87-110, :913-920,
 *                                                      src/memory.zig:665
 *
 * Ownership: every handle is created and destroyed through this API.  Input
 * columns may live on the host (copied into HBM at registration) or already on
 * the device.  Output batches are written into CALLER-OWNED host buffers.
 *
 * Threading: all calls on one handle come from one thread at a time, except
 * tgpu_query_cancel, which may be called from any thread at any time (it only
 * sets a flag that kernels poll between scan tiles).
 */
#ifndef THINDB_GPU_H
#define THINDB_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TGPU_ABI_VERSION 2

/* ---------------------------------------------------------------- status -- */

typedef enum tgpu_status {
    TGPU_OK = 0,
    /* The shape is outside what this operator runs: the caller tries its next
     * route, exactly as a `tryBuild*` returning null (v2_pipeline.zig:17-34). */
    TGPU_DECLINE = 1,
    TGPU_ERR_INVALID_ARGUMENT = 2,
    /* exec.Error.MemoryBudgetExceeded (exec.zig:915-919). */
    TGPU_ERR_MEMORY_BUDGET = 3,
    /* exec.Error.UnsupportedOperatorForType. */
    TGPU_ERR_UNSUPPORTED_TYPE = 4,
    /* error.QueryCancelled (memory.zig:665). */
    TGPU_ERR_CANCELLED = 5,
    /* A CUDA runtime call failed; tgpu_last_error_message() names it. */
    TGPU_ERR_CUDA = 6,
    /* A bounded device-side wait ran out; the context stays usable. */
    TGPU_ERR_DEVICE_TIMEOUT = 7,
    TGPU_ERR_INTERNAL = 8,
    /* The CUDA extension found no usable GPU. */
    TGPU_ERR_NO_DEVICE = 9
} tgpu_status;

/* ----------------------------------------------------------------- types -- */

/* Column types, named after thinDB's `types.Type` (src/types.zig:375-383,
 * :617): DECIMAL(p<=18,s) is a `decimal64` i64 mantissa, DATE is i32 days since
 * 1970-01-01, DATETIME is i64 microseconds.  TGPU_DICT32 is a string column
 * carried as int32 codes into a table-level dictionary (thinDB's packed table
 * ids, src/exec/silo_group_core.zig:523-538); TGPU_DECIMAL128 only appears in
 * outputs (SUM over a DECIMAL). */
typedef enum tgpu_type {
    TGPU_BOOLEAN = 1,    /* u8 0/1 */
    TGPU_TINYINT = 2,    /* i8  */
    TGPU_SMALLINT = 3,   /* i16 */
    TGPU_INT = 4,        /* i32 */
    TGPU_DATE = 5,       /* i32 days */
    TGPU_BIGINT = 6,     /* i64 */
    TGPU_DATETIME = 7,   /* i64 us */
    TGPU_DECIMAL64 = 8,  /* i64 mantissa, scale in the column descriptor */
    TGPU_FLOAT = 9,      /* f32 */
    TGPU_DOUBLE = 10,    /* f64 */
    TGPU_DECIMAL128 = 11,/* i128 little-endian (lo u64, hi i64): outputs only */
    TGPU_DICT32 = 12,    /* i32 code into the column's dictionary */
    TGPU_VARCHAR = 13    /* strings: `data` holds n_rows + 1 u32 offsets, `dict_bytes` the bytes;
                          * row r is dict_bytes[data[r] .. data[r + 1]).  A group key only
                          * (hashed: digest + exact byte check); in outputs an i64 row index
                          * whose string tgpu_query_key_strings returns */
} tgpu_type;

typedef enum tgpu_location {
    TGPU_LOC_HOST = 0,   /* pointers are host memory: copied into HBM */
    TGPU_LOC_DEVICE = 1  /* pointers are device memory on the current device: used in place */
} tgpu_location;

/* One input column.  `validity` follows thinDB's ColumnView.nulls: NULL means
 * NOT NULL; otherwise bit (row & 7) of byte (row >> 3) is 1 when the row holds
 * a value (src/storage/column.zig:28-46, :207-210). */
typedef struct tgpu_column_desc {
    const char *name;
    int32_t type;               /* tgpu_type */
    uint8_t decimal_precision;  /* DECIMAL64 only */
    uint8_t decimal_scale;      /* DECIMAL64 only */
    uint8_t reserved[2];
    const void *data;           /* n_rows elements of the type's width */
    const uint8_t *validity;    /* optional validity bitmap */
    /* DICT32 only: dictionary strings i live at dict_bytes[dict_offsets[i] ..
     * dict_offsets[i+1]) (host memory, dict_size + 1 offsets). */
    const uint32_t *dict_offsets;
    const uint8_t *dict_bytes;
    uint32_t dict_size;
    uint32_t reserved2;
    /* Optional distinct-count hint (thinDB keeps HLL NDV stats per segment);
     * 0 = estimate it at registration with a device HyperLogLog pass. */
    uint64_t ndv_hint;
} tgpu_column_desc;

/* An immutable table: one segment of `n_rows` rows cut into row groups of
 * `row_group_rows` (thinDB's default 65,536, src/api/api.zig:140). */
typedef struct tgpu_table_desc {
    const tgpu_column_desc *columns;
    uint32_t n_columns;
    uint32_t row_group_rows;    /* 0 = 65536 */
    uint64_t n_rows;
    int32_t location;           /* tgpu_location */
    int32_t compute_ndv;        /* 1 = run the HLL pass for columns without ndv_hint, and let
                                   plans sketch a composite group key once (kept with the table) */
    void *stream;               /* cudaStream_t for the copies / stats, NULL = library stream */
} tgpu_table_desc;

typedef struct tgpu_table tgpu_table;
typedef struct tgpu_query tgpu_query;

/* ------------------------------------------------------------- requests -- */

/* thinDB AggFunc members this operator folds (src/exec/aggregate.zig:88). */
typedef enum tgpu_agg_func {
    TGPU_AGG_COUNT = 1,          /* COUNT(*) when column < 0, else COUNT(col) */
    TGPU_AGG_SUM = 2,
    TGPU_AGG_AVG = 3,
    TGPU_AGG_MIN = 4,
    TGPU_AGG_MAX = 5,
    TGPU_AGG_COUNT_DISTINCT = 6,
    TGPU_AGG_UDF = 7             /* a registered user-defined aggregate (AggFunc.udf), named by udf_name */
} tgpu_agg_func;

typedef struct tgpu_agg_spec {
    int32_t func;                /* tgpu_agg_func */
    int32_t column;              /* input column index, -1 for COUNT(*) */
    const char *as;              /* output column name (may be NULL) */
    const char *udf_name;        /* TGPU_AGG_UDF: the registry name (AggSpec.udf_name, aggregate.zig:240) */
} tgpu_agg_spec;

/* One conjunct of the fused WHERE (thinDB's scan fuses the conjunction of
 * column-vs-constant leaves, src/exec/scan.zig:2808; BETWEEN lowers to two
 * inclusive leaves, src/sql/parse_predicate.zig:671).  Integer, DATE and
 * DECIMAL64 columns compare as i64 against lo/hi (DECIMAL bounds are
 * mantissas at the column's scale); FLOAT/DOUBLE columns compare against
 * flo/fhi.  A NULL row never satisfies a comparison. */
typedef enum tgpu_pred_op {
    TGPU_PRED_BETWEEN = 1,       /* lo <= x <= hi */
    TGPU_PRED_NOT_BETWEEN = 2,   /* x < lo or x > hi */
    TGPU_PRED_EQ = 3,            /* x == lo */
    TGPU_PRED_NE = 4,            /* x != lo */
    TGPU_PRED_LT = 5,            /* x <  lo */
    TGPU_PRED_LE = 6,            /* x <= lo */
    TGPU_PRED_GT = 7,            /* x >  lo */
    TGPU_PRED_GE = 8,            /* x >= lo */
    TGPU_PRED_IS_NULL = 9,
    TGPU_PRED_IS_NOT_NULL = 10
} tgpu_pred_op;

typedef struct tgpu_predicate {
    int32_t column;
    int32_t op;                  /* tgpu_pred_op */
    int64_t lo, hi;
    double flo, fhi;
} tgpu_predicate;

/* HAVING conjunct over an aggregate's EMITTED value (a BIGINT SUM compares
 * wrapped, v2_shape_group_topn.zig:1448-1453).  Integer-valued outputs compare
 * as i128 against `ival`; DOUBLE outputs against `fval`.  A NULL aggregate
 * never satisfies it. */
typedef struct tgpu_having {
    int32_t agg;                 /* index into the request's aggs */
    int32_t op;                  /* TGPU_PRED_EQ .. TGPU_PRED_GE */
    int64_t ival;
    double fval;
} tgpu_having;

typedef enum tgpu_sort_target {
    TGPU_SORT_KEY = 1,           /* index = position in group_cols */
    TGPU_SORT_AGG = 2            /* index = position in aggs */
} tgpu_sort_target;

typedef struct tgpu_sort_spec {
    int32_t target;              /* tgpu_sort_target */
    int32_t index;
    int32_t desc;
    int32_t reserved;
} tgpu_sort_spec;

#define TGPU_NO_LIMIT UINT64_MAX

/* Mirror of GroupTopNRequest (v2_shape_group_topn.zig:63-101) in plain C.
 * n_group_cols = 0 is the global aggregate (v2_global_aggregate.zig Request,
 * :51-65): exactly one row (COUNTs 0 and other aggregates NULL when no row
 * passes), HAVING declined. */
typedef struct tgpu_request {
    const int32_t *group_cols;   uint32_t n_group_cols;
    const tgpu_agg_spec *aggs;   uint32_t n_aggs;
    const tgpu_predicate *where; uint32_t n_where;
    const tgpu_having *having;   uint32_t n_having;
    const tgpu_sort_spec *order; uint32_t n_order;
    uint64_t limit;              /* TGPU_NO_LIMIT for none */
    uint64_t offset;
    uint64_t expected_groups;    /* allocation hint, 0 = estimate from stats */
    uint64_t memory_budget_bytes;/* 0 = unlimited */
    void *stream;                /* cudaStream_t, NULL = library stream */
    int32_t flags;               /* TGPU_FLAG_* */
    /* Tuning knobs (0 = engine default; the autotuner sets them per shape):
     * rows per warp chunk of the scan (a multiple of 256, at most 65,536;
     * default: about eight chunks per warp of the persistent grid),
     * shared-memory table slots (power of two; -1 = no shared-memory table),
     * group-table load in percent (capacity = expected groups * 100 / load;
     * default 50). */
    int32_t chunk_rows;
    int32_t cache_slots;
    int32_t table_load_pct;
} tgpu_request;

/* Record per-phase CUDA event times (tgpu_query_stats.*_ms). */
#define TGPU_FLAG_TIMING 0x1
/* Force the global-table route even when the groups fit a CTA's shared memory. */
#define TGPU_FLAG_FORCE_GLOBAL 0x2
/* Fold rows in place (every needed column loaded densely, a fold per 32
 * scanned rows) instead of the queue or gather modes. */
#define TGPU_FLAG_DENSE_SCAN 0x4
/* Disable the in-warp __match_any_sync pre-combine (tuning / tests). */
#define TGPU_FLAG_NO_WARP_COMBINE 0x8
/* Gather only the survivors' keys and inputs (late materialisation) whatever
 * the estimated selectivity. */
#define TGPU_FLAG_GATHER_SCAN 0x10
/* Run the staged scan (every column through a shared-memory ring of bulk
 * asynchronous copies) when the plan qualifies (compiled fold, NOT NULL
 * columns, a single range WHERE or none).  TGPU_FLAG_NO_STAGED: never. */
#define TGPU_FLAG_STAGED_SCAN 0x40
#define TGPU_FLAG_NO_STAGED 0x80
/* Prefetch control: no L2 prefetch of group-table slots; no bulk L2
 * prefetch of each warp's next chunk; also prefetch distinct-set entries. */
#define TGPU_FLAG_NO_PREFETCH 0x100
#define TGPU_FLAG_NO_CHUNK_PREFETCH 0x200
#define TGPU_FLAG_DISTINCT_PREFETCH 0x400
/* COUNT(DISTINCT) through hash partitions of (group, value) pairs, each
 * deduplicated in one CTA's shared memory (the default for one distinct
 * aggregate over 2M rows or more outside batches), or never. */
#define TGPU_FLAG_DISTINCT_PARTITION 0x800
#define TGPU_FLAG_NO_DISTINCT_PARTITION 0x1000
/* Queue mode for a WHERE (compiled folds): every row's key and inputs loaded
 * densely, the survivors compacted into a per-warp shared-memory ring and
 * folded in full batches. */
#define TGPU_FLAG_QUEUE_SCAN 0x2000
/* The pipelined scan: a producer warp per CTA streams every scanned column
 * by bulk asynchronous copies into shared-memory ring slots owned by
 * consumer warps, which filter and fold from there (compiled fold, NOT NULL
 * columns, one range WHERE on an integer column or none).
 * TGPU_FLAG_NO_PIPE: never. */
#define TGPU_FLAG_PIPE_SCAN 0x4000
#define TGPU_FLAG_NO_PIPE 0x8000
/* ORDER BY COUNT(*) DESC LIMIT k (k + OFFSET <= 1024, no HAVING, no
 * COUNT(DISTINCT)) runs thinDB's two-pass count top-K
 * (src/exec/count_topk_sketch.zig): a tally of 2^14 counters by key hash,
 * then a grouping pass over the rows of the heavy counters only, exact (a
 * filter pass that cannot prove its answer reruns over every row).  By
 * default from 1M scanned rows; TGPU_FLAG_COUNT_SKETCH forces it on smaller
 * inputs, TGPU_FLAG_NO_COUNT_SKETCH turns it off. */
#define TGPU_FLAG_COUNT_SKETCH 0x10000
#define TGPU_FLAG_NO_COUNT_SKETCH 0x20000
/* Radix-partitioned route for high-cardinality keys (thinDB's bucket
 * staging, silo_group_core.zig:9228, :9348): rows scattered by the top bits
 * of their key hash into partitions whose groups fit one CTA's shared
 * memory, then folded there (compiled fold, a key of at most 64 packed
 * bits), on request: TGPU_FLAG_RADIX; TGPU_FLAG_NO_RADIX never. */
#define TGPU_FLAG_RADIX 0x40000
#define TGPU_FLAG_NO_RADIX 0x80000
/* Scan loop with one inlined fold call site (compiled folds; survivor
 * gather or in place): batch i + 1 loads while batch i folds, instead of
 * several batches folded through an out-of-line call. */
#define TGPU_FLAG_INLINE_FOLD 0x100000
/* Split scan for a filtered survivor gather (the default for one): the
 * WHERE as a streaming pass that writes the surviving row numbers (4 bytes
 * each), then a fold pass over that list in full batches.
 * TGPU_FLAG_NO_SPLIT keeps the fused scan; TGPU_FLAG_SPLIT_SCAN is
 * accepted for requests that name it. */
#define TGPU_FLAG_SPLIT_SCAN 0x200000
#define TGPU_FLAG_NO_SPLIT 0x400000

/* ----------------------------------------------------------------- output -- */

typedef struct tgpu_output_column {
    char name[64];
    int32_t type;                /* tgpu_type of the emitted column */
    uint8_t decimal_precision;
    uint8_t decimal_scale;
    uint8_t nullable;
    uint8_t reserved;
    uint32_t elem_bytes;         /* width of one value in the data buffer */
    uint32_t reserved2;
} tgpu_output_column;

/* Caller-owned host buffers for one `next()`.  values[c] holds capacity_rows
 * values of column c; validity[c] (optional, may be NULL) receives a thinDB
 * validity bitmap (bit 1 = valid) of ceil(capacity_rows / 8) bytes. */
typedef struct tgpu_batch {
    uint32_t n_columns;
    uint32_t reserved;
    void **values;
    uint8_t **validity;
    uint64_t capacity_rows;
    uint64_t row_count;          /* filled by tgpu_query_next */
} tgpu_batch;

typedef struct tgpu_query_stats {
    uint64_t rows_scanned;       /* rows in row groups that survived zone maps */
    uint64_t rows_selected;      /* rows that passed the WHERE */
    uint64_t groups;             /* groups before HAVING */
    uint64_t result_rows;        /* rows the query emits (after OFFSET/LIMIT) */
    uint64_t table_capacity;     /* global group-table slots */
    uint64_t distinct_capacity;  /* (group, value) set slots, 0 if none */
    uint32_t row_groups_total;
    uint32_t row_groups_pruned;
    uint32_t route;              /* 1 = shared-memory (lowcard) route, 2 = global table */
    uint32_t retries;            /* group-table regrowths */
    uint32_t kernel_launches;    /* kernels the last execute launched */
    uint32_t flags;              /* TGPU_STAT_* */
    double scan_ms;              /* filter + group + fold kernel (TGPU_FLAG_TIMING) */
    double finalize_ms;          /* compaction + ranking + output gather */
    double total_ms;             /* whole execute on the device */
    uint64_t device_bytes;       /* workspace bytes held by the query */
} tgpu_query_stats;

#define TGPU_STAT_TUNED 0x1     /* settings came from the tuning table */
#define TGPU_STAT_GATHER 0x2    /* survivors gathered (late materialisation) */
#define TGPU_STAT_STAGED 0x4    /* the staged (bulk-copy ring) scan ran */
#define TGPU_STAT_DISTINCT_PARTITION 0x8  /* COUNT(DISTINCT) went through partitions */
#define TGPU_STAT_QUEUE 0x10    /* queue mode (dense loads, per-warp survivor ring) */
#define TGPU_STAT_PIPE 0x20     /* the pipelined (producer/consumer bulk-copy) scan ran */
#define TGPU_STAT_COUNT_SKETCH 0x40  /* the count sketch's filter pass gave the answer */
#define TGPU_STAT_SKETCH_RERUN 0x80  /* its filter pass could not prove the answer: every row regrouped */
#define TGPU_STAT_RADIX 0x100   /* the radix-partitioned route ran */
#define TGPU_STAT_SPLIT 0x200   /* the survivor gather ran as the split scan (select pass, fold pass) */

/* -------------------------------------------------------------- the API -- */

/* ABI version and a short build string (arch, CUDA version). */
uint32_t tgpu_abi_version(void);
const char *tgpu_build_info(void);

/* Message of the last failing call on this thread ("" if none). */
const char *tgpu_last_error_message(void);

/* Register an immutable table: copies host columns into HBM (or adopts device
 * pointers), builds per-row-group zone maps (min/max) and NDV estimates.
 * Replaces opening an `api.Table` snapshot for the scan (scan.zig:470). */
tgpu_status tgpu_table_register(const tgpu_table_desc *desc, tgpu_table **out);
tgpu_status tgpu_table_destroy(tgpu_table *table);

/* One column of a segment's schema, in schema order. */
typedef struct tgpu_segment_column {
    const char *name;
    int32_t type;               /* tgpu_type: integer family, DATE/DATETIME, DECIMAL64, FLOAT, DOUBLE */
    uint8_t decimal_precision;
    uint8_t decimal_scale;
    uint8_t reserved[2];
} tgpu_segment_column;

/* Register a table from a thinDB segment file image (host memory, `bytes`
 * long; src/storage/format.zig layout, version 17 as
 * segment_reader.zig:1388 requires): the header and each
 * row group's 12-byte column-block headers are checked on the host, the
 * image is copied to the device once, and the column blocks are decoded
 * there — raw, frame-of-reference (FOR) and run-length (RLE) payloads with
 * their validity bitmaps (segment_reader.zig decodeColumnPayload :1730,
 * forBlockOf :1809, rleBlockOf :2133) — straight into the resident columns;
 * zone maps and NDV sketches follow as in tgpu_table_register.  Row groups
 * keep the segment's size.  Blocks stored zstd- or lz4-compressed or with
 * integer-stream transforms, string columns and dictionary / FSST blocks
 * return TGPU_ERR_UNSUPPORTED_TYPE; a malformed image
 * TGPU_ERR_INVALID_ARGUMENT. */
tgpu_status tgpu_table_register_segment(const uint8_t *image, uint64_t bytes, const tgpu_segment_column *columns,
                                        uint32_t n_columns, int32_t compute_ndv, void *stream, tgpu_table **out);
/* What registering a table from a segment image took (all zero for tables
 * registered from columns). */
typedef struct tgpu_load_stats {
    uint64_t image_bytes;       /* segment image copied to the device */
    uint64_t decoded_bytes;     /* column values and validity bytes the decode wrote */
    uint32_t blocks;            /* column blocks decoded */
    uint32_t kernel_launches;   /* decode and statistics launches */
    uint32_t chunks;            /* the image's copies, each decoded as it lands */
    uint32_t reserved;
    double h2d_ms;              /* first copy start to the last copy's end (device clock) */
    double decode_ms;           /* the decode launches, summed (device clock) */
    double stats_ms;            /* the zone-map / NDV-sketch launches, summed (device clock) */
    double pipeline_ms;         /* first copy start to the last chunk's work done (device clock) */
    double first_decode_ms;     /* first copy start to the first decode start (device clock) */
    double total_ms;            /* the whole call (host clock) */
} tgpu_load_stats;
tgpu_status tgpu_table_load_stats(const tgpu_table *table, tgpu_load_stats *out);
/* Copy a registered column back to host memory: `values` receives n_rows
 * values of the column's type, `validity` (may be null) (n_rows + 7) / 8
 * bitmap bytes, bit set = value (all set for a NOT NULL column; the bits past
 * the last row of the last byte are unspecified).  VARCHAR columns return
 * TGPU_ERR_UNSUPPORTED_TYPE. */
tgpu_status tgpu_table_read_column(const tgpu_table *table, uint32_t column, void *values, uint8_t *validity);
/* thinDB's aggregate registry (udf.zig UdfRegistry.registerAggregate :870):
 * the names of the host's user-defined aggregates, so that a request can
 * name one (TGPU_AGG_UDF).  A name is case-insensitive, 1-63 characters of
 * [A-Za-z0-9_] not starting with a digit, and not a built-in aggregate's
 * (count, sum, avg, min, max, count_distinct, ...): those return
 * TGPU_ERR_INVALID_ARGUMENT, as does registering a name twice.  The
 * aggregate's code (AggregateUdf init / update / combine / finalize,
 * udf.zig:88-102) is host code this operator does not run: a request with a
 * registered TGPU_AGG_UDF aggregate returns TGPU_DECLINE from
 * tgpu_query_create (the caller keeps thinDB's executor, whose silo runs
 * registered aggregates, v2_shape_group_topn.zig:86, :170-177); an
 * unregistered name returns TGPU_ERR_INVALID_ARGUMENT. */
tgpu_status tgpu_aggregate_register(const char *name);
tgpu_status tgpu_aggregate_unregister(const char *name);
/* 1 when `name` is registered, else 0. */
int32_t tgpu_aggregate_registered(const char *name);
/* Row count, row-group count and a column's NDV estimate (-1 column = none). */
tgpu_status tgpu_table_info(const tgpu_table *table, int32_t column,
                            uint64_t *n_rows, uint32_t *n_row_groups, uint64_t *ndv);

/* tryBuildLowCardGroup / tryBuildGroupTopN in one call: validates the shape
 * (validateShape, v2_shape_group_topn.zig:2051-2370), plans key packing and
 * state slots, sizes the workspace.  Returns TGPU_DECLINE for shapes thinDB's
 * V2 core also declines or that this engine leaves to another route. */
tgpu_status tgpu_query_create(tgpu_table *table, const tgpu_request *request, tgpu_query **out);

/* The result schema (`outputSchema`).  Writes up to `cap` columns. */
tgpu_status tgpu_query_output_schema(const tgpu_query *q, tgpu_output_column *cols,
                                     uint32_t cap, uint32_t *n_columns);

/* Run the whole query on its stream (asynchronous; results stay in HBM).
 * `next` calls this on first use, as GroupTopNPipeline.execute runs on the
 * first `next()` (v2_shape_group_topn.zig:646-681).  Executing again reruns
 * the query over the same table. */
tgpu_status tgpu_query_execute(tgpu_query *q);

/* `Query.next`: copies up to batch->capacity_rows result rows into the
 * caller's buffers; *done = 1 once every row has been returned. */
tgpu_status tgpu_query_next(tgpu_query *q, tgpu_batch *batch, int32_t *done);

/* Late materialisation of a string group key.  A TGPU_DICT32 key groups by
 * its 32-bit code and `next` returns codes; thinDB groups a string column by
 * its table id the same way and reads the strings back at emit
 * (v2_group_topn_engine.zig packedIdKeys; v2_shape_group_topn.zig:1741
 * emitResultStageHashed; DESIGN.md §4.6 "Packed ids").  A TGPU_VARCHAR key
 * is hashed (a digest places the group, the bytes decide equality) and
 * `next` returns, per group, the i64 index of one of its rows (thinDB's
 * rowref).  For output column `column` (such a key), writes the strings of
 * values[0..n) — int32 codes for DICT32, int64 row indices for VARCHAR —
 * contiguously into `bytes` with offsets[0] = 0 and string i at
 * [offsets[i], offsets[i + 1]); *bytes_needed receives the total.  bytes may
 * be NULL (size query).  A row whose key is NULL carries 0 in `next`'s
 * buffer: skip it by its validity.  A code outside the dictionary, a row
 * outside the table, or a column that is not such a key returns
 * TGPU_ERR_INVALID_ARGUMENT.  ORDER BY a DICT32 key orders by the strings
 * (bytewise, a proper prefix first), as thinDB's post-emit sort does
 * (v2_shape_group_topn.zig:302-325); ORDER BY a hashed key declines; a
 * DICT32 key whose dictionary holds a string twice declines. */
tgpu_status tgpu_query_key_strings(const tgpu_query *q, uint32_t column, const void *values, uint64_t n,
                                   uint64_t *offsets, uint8_t *bytes, uint64_t bytes_cap, uint64_t *bytes_needed);

/* Async-safe cancellation flag; the next tile boundary or `next` returns
 * TGPU_ERR_CANCELLED. */
tgpu_status tgpu_query_cancel(tgpu_query *q);

tgpu_status tgpu_query_get_stats(const tgpu_query *q, tgpu_query_stats *out);
tgpu_status tgpu_query_destroy(tgpu_query *q);

/* Synchronise the library stream / the query's stream (tests and benches). */
tgpu_status tgpu_query_synchronize(tgpu_query *q);

/* ------------------------------------------------------ batched execution -- */

/* Many GROUP BY queries over one table run as ONE persistent kernel that
 * drains a work queue of (query, row-group tile) items, then one set of
 * batched compaction / top-k / gather / clear kernels (grid.y = query).  With
 * TGPU_BATCH_GRAPH the whole sequence is captured once into a CUDA graph and
 * every later execute replays it.  thinDB runs such queries one operator at a
 * time (one `Query` per statement, exec.zig:903); this has no direct
 * counterpart and produces, per query, exactly the rows `tgpu_query_next`
 * would.  Each request must return all groups or a top-k page with
 * offset + limit <= 32; other shapes decline the batch. */
typedef struct tgpu_query_batch tgpu_query_batch;

#define TGPU_BATCH_GRAPH 0x1

typedef struct tgpu_batch_stats {
    uint32_t n_queries;
    uint32_t kernel_launches;    /* kernels one execute launches */
    uint32_t graph;              /* 1 when executes replay a captured CUDA graph */
    uint32_t rerun_queries;      /* queries rerun alone after a table overflow */
    uint64_t work_items;         /* (query, tile) items of one execute */
    double total_ms;             /* last execute on the device (CUDA events) */
} tgpu_batch_stats;

tgpu_status tgpu_batch_create(tgpu_table *table, const tgpu_request *requests, uint32_t n_requests,
                              int32_t flags, void *stream, tgpu_query_batch **out);
tgpu_status tgpu_batch_execute(tgpu_query_batch *b);
tgpu_status tgpu_batch_synchronize(tgpu_query_batch *b);
tgpu_status tgpu_batch_output_schema(const tgpu_query_batch *b, uint32_t query, tgpu_output_column *cols,
                                     uint32_t cap, uint32_t *n_columns);
/* `next` of query `query` of the last execute. */
tgpu_status tgpu_batch_next(tgpu_query_batch *b, uint32_t query, tgpu_batch *batch, int32_t *done);
tgpu_status tgpu_batch_cancel(tgpu_query_batch *b);
tgpu_status tgpu_batch_get_stats(const tgpu_query_batch *b, tgpu_batch_stats *out);
tgpu_status tgpu_batch_destroy(tgpu_query_batch *b);

/* --------------------------------------------------------------- serving -- */

/* A request loop over resident tables (the serving side thinDB's
 * thindb-server runs per connection, src/cmd/server.zig; here one native
 * dispatcher thread).  Submitted requests are admitted while the sum of their
 * estimated group-table + distinct-set + buffer bytes stays under
 * `memory_budget_bytes` (thinDB's MemoryAccountant, src/memory.zig:626);
 * admitted requests of one table are launched together as a wave (the
 * batched persistent kernel) on one of several streams, so waves overlap on
 * the device and requests that arrive while others run join the next wave.
 * TGPU_SERVE_PLAIN instead runs one plain operator at a time, in arrival
 * order (the baseline the continuous mode is compared with). */
typedef struct tgpu_server tgpu_server;

#define TGPU_SERVE_CONTINUOUS 0
#define TGPU_SERVE_PLAIN 1

typedef struct tgpu_server_options {
    uint64_t memory_budget_bytes;  /* 0 = 120 GB */
    uint32_t max_batch;            /* requests per wave, 0 = 256 */
    uint32_t max_inflight;         /* waves on the device at once, 0 = 8 */
    int32_t mode;                  /* TGPU_SERVE_* */
    int32_t batch_min;             /* continuous mode: waiting requests on one table that
                                    * make a wave one batched kernel (0 = never: every request
                                    * runs as its own execution, overlapping on the wave streams) */
} tgpu_server_options;

typedef struct tgpu_server_stats {
    uint64_t submitted, completed, failed;
    uint64_t waves;                /* launches (waves or plain queries) */
    uint64_t peak_admitted_bytes;
    uint64_t peak_queued;          /* most requests waiting for admission at once */
} tgpu_server_stats;

tgpu_status tgpu_server_create(tgpu_table *const *tables, uint32_t n_tables, const tgpu_server_options *opts,
                               tgpu_server **out);
/* Thread-safe; copies the request.  *ticket identifies the result. */
tgpu_status tgpu_server_submit(tgpu_server *s, uint32_t table, const tgpu_request *req, uint64_t *ticket);
/* Wait up to timeout_ms (-1 = no limit) for a ticket; *done = 1 when its result is ready. */
tgpu_status tgpu_server_wait(tgpu_server *s, uint64_t ticket, int32_t timeout_ms, int32_t *done);
tgpu_status tgpu_server_output_schema(tgpu_server *s, uint64_t ticket, tgpu_output_column *cols, uint32_t cap,
                                      uint32_t *n_columns);
/* Rows of a finished ticket (status of the request if it failed). */
tgpu_status tgpu_server_next(tgpu_server *s, uint64_t ticket, tgpu_batch *batch, int32_t *done);
tgpu_status tgpu_server_release(tgpu_server *s, uint64_t ticket);
tgpu_status tgpu_server_get_stats(tgpu_server *s, tgpu_server_stats *out);
tgpu_status tgpu_server_destroy(tgpu_server *s);

/* Open-loop load: Poisson arrivals at `rate_qps` for `duration_s`, request i
 * drawn as requests[j], j uniform (seeded), against table tables_of[j];
 * latency = submit to result ready.  Waits for every submitted request. */
typedef struct tgpu_load_spec {
    const uint32_t *table_of;
    const tgpu_request *requests;
    uint32_t n_requests;
    uint32_t reserved;
    double rate_qps;
    double duration_s;
    uint64_t seed;
} tgpu_load_spec;

typedef struct tgpu_load_report {
    uint64_t submitted, completed, failed;
    double elapsed_s;              /* first submit to last completion */
    double achieved_qps;           /* completed / elapsed_s */
    double p50_ms, p99_ms, p999_ms, max_ms, mean_ms;
} tgpu_load_report;

tgpu_status tgpu_server_run_load(tgpu_server *s, const tgpu_load_spec *spec, tgpu_load_report *out);

/* ----------------------------------------------------------------- tuning -- */

/* Measured engine settings per request shape.  thinDB fixes its engine knobs
 * (scan tile rows, route block rows, bucket count) as defaults overridable from
 * the environment (v2_group_topn_engine.zig:25-33, :521-626 paramsFromEnv);
 * here an autotuner (thindb_gb300/autotune.py) measures them per shape class
 * and installs the table with tgpu_tuning_set.  A request that sets
 * chunk_rows, cache_slots, table_load_pct, a scan-mode flag or
 * TGPU_FLAG_NO_TUNING keeps its own settings. */
#define TGPU_FLAG_NO_TUNING 0x20

typedef struct tgpu_shape {
    int32_t key_words;    /* packed key words: 1 or 2 */
    int32_t fold;         /* compiled fold signature, -1 = interpreter */
    int32_t n_aggs;       /* aggregates requested */
    int32_t distinct;     /* 1 if any COUNT(DISTINCT) */
    int32_t filtered;     /* 1 if a WHERE is present */
    int32_t sel_log2;     /* floor(log2(estimated kept fraction)); 0 without WHERE */
    int32_t groups_log2;  /* ceil(log2(estimated groups)) */
    int32_t batched;      /* 1 inside tgpu_batch_create */
} tgpu_shape;

typedef struct tgpu_tuning {
    tgpu_shape shape;
    int32_t chunk_rows;      /* 0 = built-in rule */
    int32_t cache_slots;     /* 0 = built-in rule, -1 = no shared-memory table */
    int32_t table_load_pct;  /* 0 = 50 */
    int32_t flags;           /* scan-mode and prefetch TGPU_FLAG_* bits */
    int32_t groups_shift;    /* size the group table for (estimated groups >> groups_shift),
                              * 0..8; an estimate found too small regrows the table x4 */
    int32_t reserved;
} tgpu_tuning;

/* The shape class `req` falls in on `table` (plans the request; allocates nothing). */
tgpu_status tgpu_request_shape(tgpu_table *table, const tgpu_request *req, int32_t batched, tgpu_shape *out);
/* Replace the process-wide tuning table (n = 0 clears it). */
tgpu_status tgpu_tuning_set(const tgpu_tuning *entries, uint32_t n);
/* Copy up to `cap` entries out; returns the table size. */
uint32_t tgpu_tuning_get(tgpu_tuning *entries, uint32_t cap);

/* ------------------------------------------------------ failure testing -- */

/* No counterpart in thinDB (its executor has no device waits).  The staged
 * scan and the COUNT(DISTINCT) partition kernel wait on bulk asynchronous
 * copies with a bounded wait (default about 2 s of SM clock); a wait that
 * runs out sets a status bit, the kernel lets its own copies land and
 * returns, and the query reports TGPU_ERR_DEVICE_TIMEOUT.  This sets that
 * bound in SM clocks for queries executed from now on (0 = the default), so
 * a test can make the waits run out and check that the status comes back
 * and that the next query on the same context is correct.  Process-wide. */
tgpu_status tgpu_debug_set_wait_limit(uint64_t sm_cycles);

/* Test hook for hashed group keys, after thinDB's THINDB_V2_KEY_DIGEST_BITS
 * (tests/integration/exact_group_keys_test.zig): queries planned from now on
 * keep only the low `bits` of a hashed key's 64-bit digest (0 = all), so
 * distinct keys share digests and the exact check of the key's parts
 * against each group's representative row decides every match.  Results do
 * not change; probes get longer.  Process-wide. */
tgpu_status tgpu_debug_set_digest_bits(uint32_t bits);

/* ------------------------------------------------- allocation-free call -- */

/* No counterpart in thinDB.  For callers that cannot let the library
 * allocate device memory (a host that reserves the GPU's memory for its own
 * arena up front, a plugin running inside another runtime's memory pool, a
 * latency-critical loop that must not block in cudaMalloc/cudaFree):
 *
 *   SELECT key, COUNT(*), SUM(value), MIN(value), MAX(value) GROUP BY key
 *
 * over two NOT NULL BIGINT device columns of n_rows rows, with the same
 * kernels as tgpu_query_create.  Nothing is allocated: the group table lives
 * in one fixed array of about 9.6 MB inside the library (held on every GPU
 * that loads it until the process exits).  Outputs are caller-provided device
 * buffers of TGPU_NOALLOC_MAX_GROUPS values each; *out_groups (device memory)
 * receives the number of groups.  SUM is BIGINT and wraps, as thinDB's.
 * More than TGPU_NOALLOC_MAX_GROUPS distinct keys returns
 * TGPU_ERR_INVALID_ARGUMENT; a group-table probe that runs past its limit
 * with fewer groups (clustered key hashes) returns TGPU_ERR_INTERNAL.  When
 * the call returns an error, *out_groups and the output buffers are
 * undefined.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress): make that first call before any stream
 * capture.  Every call clears the parts of the array it reads on `stream`
 * (any stream, blocking or not); the call is synchronous (it reads back a
 * status word).  All calls share the array: calls that overlap on the GPU
 * race. */
#define TGPU_NOALLOC_MAX_GROUPS 65536
tgpu_status tgpu_group_by_i64_noalloc(const int64_t *keys, const int64_t *values, uint64_t n_rows,
                                      int64_t *out_keys, int64_t *out_count, int64_t *out_sum,
                                      int64_t *out_min, int64_t *out_max, uint64_t *out_groups,
                                      void *stream);

#ifdef __cplusplus
}
#endif

#endif /* THINDB_GPU_H */
