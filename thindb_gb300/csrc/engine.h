// engine.h — internal plan, device descriptors and launch entry points of the
// GB300 grouped-aggregation engine (behind include/thindb_gpu.h).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/thindb_gpu.h"

namespace tgpu {

constexpr int MAX_GROUP_KEYS = 8;   // thinDB MAX_GROUP_KEYS (v2_shape_group_topn.zig:50)
// Composite keys whose parts' NDV product exceeds this get their own sketch.
constexpr uint64_t COMPOSITE_SKETCH_MIN = 1ULL << 16;
constexpr int MAX_AGGS = 16;        // thinDB MAX_AGGS (v2_shape_group_topn.zig:54)
constexpr int MAX_STATE_WORDS = 17; // the row count + 16 numeric slots
constexpr int MAX_DISTINCT = 8;     // thinDB MAX_DISTINCT_AGG_SLOTS (v2_shape_group_topn.zig:62)
constexpr int MAX_PREDS = 8;
constexpr int MAX_QCOLS = 24;       // distinct columns one query reads
constexpr int MAX_ORDER = 6;
constexpr int MAX_SORT_WORDS = 2 * MAX_ORDER + 2;

// Key-width class of the top-k kernels for an encoded sort key of `sw` words
// (one to six ORDER BY entries): the candidate buffers hold this many words
// per entry.
__host__ __device__ constexpr int topk_width(int sw) { return sw <= 4 ? 4 : sw <= 6 ? 6 : sw <= 8 ? 8 : 14; }
constexpr uint32_t TOPK_W4 = 1, TOPK_W6 = 2, TOPK_W8 = 4, TOPK_W14 = 8;
__host__ __device__ constexpr uint32_t topk_width_bit(int sw) {
    return sw <= 4 ? TOPK_W4 : sw <= 6 ? TOPK_W6 : sw <= 8 ? TOPK_W8 : TOPK_W14;
}

// Scan geometry: persistent CTAs of SCAN_WARPS warps; each warp folds a
// static, strided set of chunks of chunk_rows rows.
constexpr int SCAN_THREADS = 512;
constexpr int SCAN_WARPS = SCAN_THREADS / 32;
constexpr int CHUNK_ALIGN = 256;
constexpr int WQ_RING_ROWS = 64;  // queue mode: fold rows per warp ring (scan_impl.cuh WQ_ROWS)

// Status bits the kernels OR into the query's device status word.
constexpr unsigned ST_TABLE_FULL = 1u;      // a probe ran past MAX_PROBE: regrow and rerun
constexpr unsigned ST_DISTINCT_FULL = 2u;   // a distinct set probe ran past MAX_PROBE
constexpr unsigned ST_CANCELLED = 4u;       // the host cancel flag was seen
constexpr unsigned ST_BAD_INDEX = 8u;       // a bounds check caught an index (never expected)
constexpr unsigned ST_WAIT_TIMEOUT = 16u;   // a bounded wait on an asynchronous copy gave up
constexpr unsigned ST_PART_FULL = 32u;      // a radix partition buffer overflowed: resize and rerun
constexpr unsigned MAX_PROBE = 4096;

// DevQuery::prefetch bits
constexpr int PF_SLOT = 1;      // a gathered row's group-table slot, as soon as its key is loaded
constexpr int PF_NEXT = 2;      // the warp's next chunk of every scanned column (bulk L2 prefetch)
constexpr int PF_DISTINCT = 4;  // a gathered row's distinct-set entries

// Aggregate fold kinds (one state word each unless noted).
enum AggKind : int32_t {
    AK_COUNT_ROWS = 0,   // COUNT(*) / non-nullable COUNT(col): word 0
    AK_COUNT_VALID = 1,  // nullable COUNT(col): own word
    AK_SUM_I64 = 2,      // SUM/AVG over 8/16/32-bit ints: wrapping u64 word
    AK_SUM_I128 = 3,     // SUM/AVG over 64-bit ints / DECIMAL64: two carry-free words,
                         // sum of low 32-bit halves (u64) and of high halves (i64);
                         // exact while a group folds < 2^32 values (i128_of_split)
    AK_SUM_F64 = 4,      // SUM/AVG over FLOAT/DOUBLE: f64 word
    AK_MIN_I = 5,        // ~enc_i64 word, folded by atomicMax
    AK_MAX_I = 6,        // enc_i64 word
    AK_MIN_F = 7,        // ~enc_f64 word
    AK_MAX_F = 8,        // enc_f64 word
    AK_DISTINCT = 9,     // count word + a (group, value) set
    AK_SUM_I128C = 10    // as AK_SUM_I128 for tables of 2^32 rows or more: i128 lo, hi
                         // words, the carry taken from the low word's atomicAdd
};

struct DevCol {
    const void *data;       // values; TGPU_VARCHAR: the string bytes
    const uint32_t *valid;  // validity bitmap as little-endian u32 words, nullptr = NOT NULL
    const uint32_t *offs;   // TGPU_VARCHAR: row r's bytes at [offs[r], offs[r + 1]); else nullptr
    int32_t type;           // tgpu_type
    int32_t bytes;          // element width (TGPU_VARCHAR: 0)
};

struct DevPred {
    int32_t col;            // index into DevQuery::cols
    int32_t op;             // tgpu_pred_op
    int32_t is_float;
    int32_t pad;
    int64_t lo, hi;
    double flo, fhi;
};

struct DevKeyPart {
    int32_t col;
    int32_t offset;         // bit offset in the packed key
    int32_t payload;        // payload bits (type width)
    int32_t nullable;       // validity bit at offset + payload
};

struct DevAgg {
    int32_t kind;           // AggKind
    int32_t col;            // DevQuery::cols index, -1 for COUNT(*)
    int32_t word;           // first state word
    int32_t vword;          // valid-count word, -1 = none
    int32_t dset;           // distinct set index (AK_DISTINCT)
    int32_t is_float_in;    // input column is FLOAT/DOUBLE
    int32_t owner;          // folds its state words (0 when an earlier aggregate shares them)
    int32_t needs_value;    // the fold reads the input value (not only its validity)
};

// Everything a scan launch needs, passed by value (kernel parameter).
struct DevQuery {
    // rows
    uint64_t n_rows;
    const uint32_t *rg_list;  // surviving row groups, nullptr = every row group
    uint32_t n_rg;            // row groups iterated (list length or total)
    uint32_t rg_rows;
    uint32_t chunks_per_rg;
    uint32_t n_chunks;        // warp-sized units of work
    uint32_t chunk_rows;      // rows per chunk (multiple of 256)
    uint32_t shared_scan;     // 1: other queries of a batch read the same rows (keep them in L2)
    // columns / predicates / key / aggregates
    DevCol cols[MAX_QCOLS];
    int32_t n_cols;
    int32_t n_preds;
    DevPred preds[MAX_PREDS];
    // A WHERE that is one range test on a NOT NULL integer column:
    // (fp_lo <= x <= fp_hi) != fp_negate, read with width-specialised loads.
    const void *fp_data;
    int64_t fp_lo, fp_hi;
    int32_t fp_bytes;        // 0 = no fast predicate
    int32_t fp_negate;
    DevKeyPart parts[MAX_GROUP_KEYS];
    int32_t n_parts;
    int32_t key_words;        // 1 or 2
    // hashed keys (a string part, or parts wider than 128 bits): word 1 is
    // the parts' digest, word 0 the representative row + 1; equal digests
    // are told apart by comparing the rows' key parts
    int32_t hashed;
    uint32_t digest_bits;     // 0: the full 64-bit digest; else only its low bits (set for tests of the exact check)
    uint64_t key_or;          // OR'ed into every packed key: 1 for a global aggregate (its one group), else 0
    DevAgg aggs[MAX_AGGS];
    int32_t n_aggs;
    // compiled fast fold: key mode (0 = none, 1 = one NOT NULL part, 2 = several
    // NOT NULL parts) and the owner aggregates it folds, in plan order
    int32_t fast_km;
    int32_t n_faggs;
    DevAgg faggs[4];
    int32_t fast_id;          // index of the matching compiled fold, -1 = interpreter
    int32_t inline_fold;      // scan loop with one inlined fold call site (scan_inline.cu)
    int32_t state_words;      // row count + slots
    int32_t slot_words;       // key_words + state_words rounded to a power of two
    int32_t needs_gid;        // a distinct aggregate needs each row's group slot
    // global group table: capacity + 1 slots (the last one holds the all-zero key)
    unsigned long long *table;
    uint64_t cap;             // power of two
    uint32_t *occ;            // occupancy bitmap, cap + 1 bits
    // distinct sets: entries of {value u64, gid u32 | epoch << 32}
    unsigned long long *dset[MAX_DISTINCT];
    uint64_t dset_cap[MAX_DISTINCT];
    uint32_t epoch;
    int32_t n_dsets;
    // shared-memory pre-aggregation (0 slots = off)
    int32_t cache_slots;      // power of two
    int32_t cache_probe;      // probe limit (cache_slots when the table holds every group)
    int32_t warp_combine;     // __match_any_sync pre-combine on/off
    int32_t gather;           // 1 = compact survivors, then gather; 0 = process rows in place
    // partitioned COUNT(DISTINCT) (one distinct aggregate): the scan appends
    // (value, gid) pairs to 2^dpart_bits hash partitions of dpart_cap
    // entries; dpart_bits == 0: inserts go straight to the distinct set
    int32_t dpart_bits;
    uint32_t dpart_cap;
    uint32_t *dpart_cursor;          // per partition
    ulonglong2 *dpart_buf;           // partition p at [p * dpart_cap, (p + 1) * dpart_cap)
    // prefetching: PF_* bits, and the columns whose next chunk a warp pulls
    // into L2 with one bulk prefetch per column before scanning its chunk
    int32_t prefetch;
    int32_t n_pf;
    int32_t pf_cols[8];
    // ORDER BY COUNT(*) DESC LIMIT k through the count sketch (sketch.cu):
    // when *sk_on, only rows whose counter hash(key) >> (64 - SK_BITS) has
    // its bit set in sk_keep fold; nullptr = every row folds
    const uint32_t *sk_keep;
    const uint32_t *sk_on;
    // control
    long long wait_cycles;                // bound of the bulk-copy waits in SM clocks, 0 = WAIT_CYCLES
    unsigned int *tile_counter;
    unsigned int *status;
    const volatile int *cancel;           // host-mapped cancel flag (may be nullptr)
    unsigned long long *selected_rows;    // rows that passed WHERE
};

// Ranking / emit descriptors -------------------------------------------------

struct DevOrder {
    int32_t target;           // TGPU_SORT_KEY / TGPU_SORT_AGG
    int32_t index;            // key part / aggregate index
    int32_t desc;
    int32_t pad;
};

// How one output aggregate column is finalised from the state words.
struct DevOut {
    int32_t func;             // tgpu_agg_func
    int32_t kind;             // AggKind of the state
    int32_t word;
    int32_t vword;
    int32_t out_type;         // tgpu_type of the emitted column
    int32_t in_type;
    int32_t scale;            // DECIMAL input scale (AVG divides by 10^scale)
    int32_t nullable;         // all-NULL input groups emit NULL
};

struct DevHaving {
    int32_t agg;
    int32_t op;
    int64_t ival;
    double fval;
};

struct DevFinal {
    const unsigned long long *table;
    uint64_t cap;
    const uint32_t *occ;
    int32_t key_words;
    int32_t slot_words;
    int32_t n_parts;
    int32_t n_aggs;
    int32_t n_order;
    int32_t n_having;
    int32_t sort_words;       // words of one encoded sort key
    int32_t global_avg;       // a global aggregate's AVG: sum / (n * 10^scale), else sum / n / 10^scale
    int32_t hashed;           // hashed keys: key parts are read from part_cols at the representative row
    int32_t pad_h;
    DevCol part_cols[MAX_GROUP_KEYS];
    DevKeyPart parts[MAX_GROUP_KEYS];
    int32_t part_types[MAX_GROUP_KEYS];
    // ORDER BY a DICT32 key: code c ranks as part_rank[c] (its string's place
    // in bytewise order) when c < part_rank_n, else after every string
    const uint32_t *part_rank[MAX_GROUP_KEYS];
    uint32_t part_rank_n[MAX_GROUP_KEYS];
    DevOut outs[MAX_AGGS];
    DevOrder order[MAX_ORDER];
    DevHaving having[MAX_AGGS];
};

// Per-query finalize buffers of a batch (device array, one per query).
struct DevFinalBufs {
    uint32_t *block_counts;
    uint32_t *gids;
    unsigned long long *counts;      // [0] groups [1] kept [2] result rows [3] selection size [4] selected rows
    unsigned long long *cand_keys;
    uint32_t *cand_gids;
    uint32_t *sel;                   // selection list read by gather (gids or the top-k)
    void **out_cols;
    uint8_t **out_valid;
    uint64_t offset;
    uint64_t gather_rows;
    uint32_t n_cpt_blocks;
    uint32_t n_cand_blocks;
    uint32_t k;
    int32_t rank;                    // 0 all groups, 1 top-k (k <= 32)
    // result packing into mapped host memory (pack_rows == 0: not packed):
    // [u64 rows][column c: pack_rows * elem_bytes[c]]...[column c validity: pack_rows bytes]...
    uint8_t *pack_dst;
    uint64_t pack_rows;
    uint32_t n_out;
    uint32_t out_bytes[MAX_GROUP_KEYS + MAX_AGGS];
};

// The staged scan (scan_staged.cu): tiles of tile_rows rows of every staged
// column, brought into an S-deep shared-memory ring by bulk asynchronous
// copies.  Tile t covers rows [row0, row0 + tile_rows) of surviving row group
// t / tiles_per_rg.
constexpr int STAGE_THREADS = 512;
constexpr uint32_t STAGE_TILE = 1024;
constexpr uint32_t STAGE_FOLD_AT = 512;                    // queued rows that start a fold round
constexpr uint32_t STAGE_QCAP = STAGE_FOLD_AT + STAGE_TILE;  // fold-queue rows
struct StagePlan {
    uint32_t n_tiles;
    uint32_t tiles_per_rg;
    uint32_t stages;             // ring depth S
    uint32_t stage_bytes;        // bytes of one tile of every staged column
    uint32_t n_cols;             // staged columns
    uint32_t row_bytes;          // bytes of one fold-queue entry
    int32_t col[MAX_QCOLS];      // query column of staged column i
    uint32_t off[MAX_QCOLS];     // its byte offset inside a stage
    int32_t slot[MAX_QCOLS];     // staged index of query column c, -1 = not staged
    uint32_t cache_off, queue_off, ring_off, smem_bytes;
};
// Plan the staged scan for q (its cache_slots may shrink to fit); false if
// the query does not qualify.
bool stage_plan(DevQuery &q, uint64_t tile_count, StagePlan *sp);
cudaError_t launch_staged_scan(const DevQuery &q, const StagePlan &sp, int grid, cudaStream_t s);

// The pipelined scan (scan_pipe.cu): one producer warp streams tiles of
// PIPE_TILE rows of every scanned column by bulk copies into ring slots owned
// by PIPE_CWARPS consumer warps (`depth` slots each), which filter and fold
// from shared memory.  Tile t covers rows [row0, row0 + PIPE_TILE) of
// surviving row group t / tiles_per_rg.
constexpr int PIPE_CWARPS = 16;
constexpr int PIPE_THREADS = (PIPE_CWARPS + 1) * 32;
constexpr uint32_t PIPE_TILE = 256;
struct PipePlan {
    uint32_t n_tiles;
    uint32_t tiles_per_rg;
    uint32_t log_depth;          // log2 of the ring slots per consumer warp (1 or 2)
    uint32_t stage_bytes;        // bytes of one tile of every scanned column
    uint32_t n_cols;
    int32_t col[MAX_QCOLS];      // query column of staged column i
    uint32_t off[MAX_QCOLS];     // its byte offset inside a stage
    int32_t slot[MAX_QCOLS];     // staged index of query column c, -1 = not staged
    uint32_t ctl_off, bar_off, cache_off, queue_off, list_off, ring_off, smem_bytes;
};
// Plan the pipelined scan for q (its cache_slots may shrink to fit); false
// if the query does not qualify (compiled fold, NOT NULL 16-byte aligned
// columns, one range WHERE on an integer column or none).
bool pipe_plan(DevQuery &q, uint64_t tile_count, PipePlan *pp);
cudaError_t launch_pipe_scan(const DevQuery &q, const PipePlan &pp, int grid, cudaStream_t s);
// The split scan (scan_split.cu): select pass writing the surviving row
// numbers to `rows` (count at n_rows), then the fold pass over them.
cudaError_t launch_split_scan(const DevQuery &q, uint32_t *rows, unsigned long long *n_rows, int sms, cudaStream_t s);

// The two-pass COUNT top-K sketch (sketch.cu): 2^SK_BITS counters, served
// for OFFSET + LIMIT up to SK_MAX_NEED over at least SK_MIN_ROWS rows.
constexpr int SK_BITS = 14;
constexpr uint32_t SK_MAX_NEED = 1024;     // MAX_NEED, count_topk_sketch.zig:64
constexpr uint64_t SK_MIN_ROWS = 1u << 20;
// counts: 2^SK_BITS u32; keep: 2^SK_BITS bits; ctl: 8 u32 ([0] on, [1] threshold, ...)
cudaError_t launch_count_sketch(const DevQuery &q, uint32_t need, uint32_t *counts, uint32_t *keep, uint32_t *ctl,
                                int sms, cudaStream_t s);

// The radix-partitioned route (radix.cu): rows are scattered by the top
// `bits` of their key hash into 2^bits partition buffers of `cap` records
// (packed key + the compiled fold's inputs), then each partition's groups
// are folded by one CTA in a shared-memory table of cache_slots entries.
constexpr uint32_t RX_TILE = 2048;
constexpr uint32_t RX_SLOTS = 4096;       // shared-memory group slots per partition
constexpr uint32_t RX_MAX_BITS = 10;
struct RadixPlan {
    uint32_t bits;                // 2^bits partitions
    uint32_t sub_bits;            // COUNT(DISTINCT): pair sub-partitions per partition
    uint64_t cap;                 // records per partition buffer
    uint32_t n_tiles, tiles_per_rg;
    unsigned long long *buf;      // partition p's records at [p * cap, (p + 1) * cap), (1 + n_faggs) words each
    uint32_t *cursor;             // records per partition (may pass cap: ST_PART_FULL)
    uint32_t dcur_off;            // aggregate kernel: shared-memory offset of the sub-partition cursors
    uint32_t agg_smem;
    uint32_t agg_per_sm;
    uint32_t pad;
};
size_t radix_scatter_smem(const DevQuery &q, uint32_t bits);
cudaError_t launch_radix(const DevQuery &q, const RadixPlan &rp, int sms, cudaStream_t s);

// One column block of a thinDB segment image (segment.cu): rows
// [row0, row0 + rows) of its column, payload at image offset `payload`, the
// value region `values` bytes into it (past the validity bitmap).
struct SegBlock {
    uint64_t row0;       // the block's first row in the table
    uint64_t payload;    // byte offset of the payload in the image
    void *out;           // the decoded column (elem bytes per row)
    uint32_t *valid;     // the column's validity words (null: NOT NULL)
    uint32_t values;     // payload offset of the values (past the validity bitmap)
    uint32_t rows;
    uint32_t encoding;   // 0 raw, 1 FOR, 3 RLE (format.Encoding)
    uint32_t width;      // FOR delta / RLE value / raw element width in bytes
    uint32_t runs;       // RLE runs
    uint32_t run0;       // RLE: index of its first run start in the run-start array
    uint32_t elem;       // decoded element bytes (1, 2, 4, 8)
    uint32_t has_nulls;  // a validity bitmap prefixes the payload
    // statistics taken while decoding (the block is one row group of the table)
    uint32_t col;        // the column's statistics slice
    uint32_t rg;         // the row group's zone-map entry
    int32_t type;        // tgpu_type of the column
    uint32_t flags;      // SEG_ZONE, SEG_SKETCH
    uint32_t part_row;   // its HLL register row in the scratch
    uint32_t pad;
};
constexpr uint32_t SEG_ZONE = 1, SEG_SKETCH = 2;
// Where decode_blocks_kernel leaves statistics: column c's slice at
// stats + c * slice holds imin, imax (i64), fmin, fmax (f64) and NULL counts
// (u32) of nrg row groups, and 2^HLL_P u32 registers at reg_off; part holds a
// row of 2^HLL_P byte registers per block.
struct SegStats {
    unsigned char *stats;
    uint64_t slice, reg_off, nrg;
    uint8_t *part;
};
constexpr uint32_t SEG_IMAGE_PAD = 16;
// A segment image goes to the device in about this many chunks of row groups.
constexpr uint32_t SEG_CHUNKS = 16;
cudaError_t launch_decode_blocks(const uint8_t *image, const SegBlock *blocks, uint32_t n_blocks,
                                 const uint32_t *run_starts, const SegStats &st, cudaStream_t s);
// Raise each column's registers to the maximum over its `rows` part rows
// (column c's rows start at row c * stride).
cudaError_t launch_seg_hll_merge(const SegStats &st, uint32_t n_cols, uint32_t rows, uint32_t stride, cudaStream_t s);

// Partitioned COUNT(DISTINCT): pairs per partition (one CTA deduplicates a
// partition in shared memory) and the partition's index-table slots.
constexpr uint32_t DPART_CAP = 4096;     // 64 KB of pairs per ring stage; three stages + 32 KB of slots per SM
constexpr uint32_t DPART_SLOTS = 8192;
constexpr int DPART_MAX_BITS = 20;      // 2^20 partitions: 64 GB of pairs for 3.2G rows
// Deduplicate every partition's pairs and add each new pair to its group's
// distinct count (table word `word` of slot gid).
cudaError_t launch_distinct_partitions(const DevQuery &q, int word, cudaStream_t s);

// Bound of the device's bulk-copy waits for queries planned from now on, in
// SM clocks (0 = the built-in ~2 s); set by tgpu_debug_set_wait_limit.
long long device_wait_limit();

// Low bits of a hashed key's digest that queries planned from now on keep
// (0 = all 64); set by tgpu_debug_set_digest_bits.
uint32_t hashed_digest_bits();

// Message returned by tgpu_last_error_message() on this thread (api.cpp).
void set_error(const char *msg);

// Launchers (scan.cu / finalize.cu / table.cu) --------------------------------

int scan_grid_size(const DevQuery &q, int device_sms);
// index of the compiled fast fold matching the plan (-1: the interpreter runs it)
int fast_fold_id(const DevQuery &q);
size_t scan_smem_bytes(const DevQuery &q);
cudaError_t launch_scan(const DevQuery &q, int grid, cudaStream_t s);
// the scan loop with one inlined fold call site (compiled folds; scan_inline.cu)
const void *inline_scan_kernel(const DevQuery &q);
cudaError_t launch_scan_inline(const DevQuery &q, int grid, size_t smem, cudaStream_t s);
// many queries, one persistent kernel per fold class over (query, row group)
// work items: class = the compiled fold's id, or the interpreter for up to 4
// or up to 16 aggregates
constexpr int BATCH_GENERIC4 = 12;
constexpr int BATCH_GENERIC16 = 13;
constexpr int BATCH_CLASSES = 14;
// A batch work item: one query's kept row groups within a window of about
// this many rows.
constexpr uint64_t BATCH_WINDOW_ROWS = 1ull << 20;
int batch_fold_class(const DevQuery &q);
int batch_scan_grid(int cls, size_t smem, int sms);
// items[i] = {query, first chunk of one of its row groups}, every query of class cls
cudaError_t launch_batch_scan(int cls, const DevQuery *qs, const uint4 *items, uint32_t n_items, size_t smem,
                              int grid, const volatile int *cancel, unsigned int *status, cudaStream_t s);
// compaction, top-k / all-groups selection, gather and clear for every query of a batch
// single-query top-k straight from the occupancy bitmap (counts[0] groups,
// [1] kept, [3] selected); `done` is a zeroed counter
cudaError_t launch_topk_scan(const DevFinal &f, unsigned long long *counts, uint32_t k, unsigned long long *cand_keys,
                             uint32_t *cand_gids, uint32_t n_cand_blocks, uint32_t *sel_out, unsigned int *done,
                             cudaStream_t s);
// topk_widths: TOPK_W* bits of the key-width classes of the batch's top-k queries
cudaError_t launch_finalize_batch(const DevFinal *fs, const DevFinalBufs *bs, uint32_t n_queries,
                                  uint32_t max_cpt_blocks, uint32_t max_cand_blocks, uint32_t topk_widths,
                                  uint64_t max_rows, uint64_t max_words, cudaStream_t s);

// compaction: dense list of occupied slots that pass HAVING
cudaError_t launch_compact(const DevFinal &f, uint32_t *block_counts, uint32_t n_blocks,
                           uint32_t *gids_out, unsigned long long *counts /*[0]=groups,[1]=kept*/,
                           cudaStream_t s);
uint32_t compact_blocks(uint64_t cap);
// counts[] (device): [0] groups, [1] groups kept by HAVING, [2] result rows,
// [3] entries in the selection list.
// top-k (k <= 32) over the dense list -> sel_out, counts[3]
cudaError_t launch_topk(const DevFinal &f, const uint32_t *gids, unsigned long long *counts, uint32_t k,
                        unsigned long long *cand_keys, uint32_t *cand_gids, uint32_t n_cand_blocks,
                        uint32_t *sel_out, cudaStream_t s);
// full sort of the dense list (ORDER BY without a small LIMIT) -> *sorted_out, counts[3]
cudaError_t launch_sort(const DevFinal &f, const uint32_t *gids, unsigned long long *counts, uint64_t max_n,
                        unsigned long long *keys_a, unsigned long long *keys_b, uint32_t *ids_a, uint32_t *ids_b,
                        uint32_t **sorted_out, cudaStream_t s);
// the dense list itself is the selection: counts[3] = counts[1]
cudaError_t launch_sel_all(unsigned long long *counts, cudaStream_t s);
// output columns for rows [offset, offset + max_rows) of `sel` -> counts[2]
cudaError_t launch_gather(const DevFinal &f, const uint32_t *sel, unsigned long long *counts, uint64_t offset,
                          uint64_t max_rows, void *const *out_cols, uint8_t *const *out_valid, cudaStream_t s);
// zero the occupied slots and the bitmap (leaves the table ready for reuse)
cudaError_t launch_clear(unsigned long long *table, uint64_t cap, int32_t slot_words, uint32_t *occ, cudaStream_t s);

// table statistics
cudaError_t launch_hll(const void *data, const uint32_t *valid, int32_t type, uint64_t n_rows, uint32_t *regs,
                       cudaStream_t s, const uint32_t *offs = nullptr);
// Zone maps of row groups [g0, g1) and (regs non-null) the HLL registers of
// their rows, for a fixed-width column in one pass; the registers are
// replaced, or raised when `accumulate`.  `part` is scratch of
// STATS_GRID_MAX x 2^HLL_P bytes.
constexpr uint32_t STATS_GRID_MAX = 512;
cudaError_t launch_column_stats(const void *data, const uint32_t *valid, int32_t type, uint64_t n_rows,
                                uint32_t rg_rows, uint32_t g0, uint32_t g1, int64_t *imin, int64_t *imax, double *fmin,
                                double *fmax, uint32_t *nulls, uint32_t *regs, uint8_t *part, int accumulate,
                                cudaStream_t s);
// Columns of a composite key for its HyperLogLog sketch.
struct KeySketchCols {
    const void *data[MAX_GROUP_KEYS];
    const uint32_t *valid[MAX_GROUP_KEYS];
    const uint32_t *offs[MAX_GROUP_KEYS];  // TGPU_VARCHAR parts
    int32_t type[MAX_GROUP_KEYS];
    int32_t n;
};
cudaError_t launch_key_hll(const KeySketchCols &k, uint64_t n_rows, uint32_t *regs, cudaStream_t s);
constexpr int HLL_P = 14;

}  // namespace tgpu
