// api.cpp — host runtime behind include/thindb_gpu.h.
//
// Table registration (HBM residency, zone maps, NDV), query planning (thinDB's
// validateShape: key packing and state slots, v2_shape_group_topn.zig:2051-2370),
// group-table sizing (expectedTotalGroups, silo_group_core.zig:11398), a
// workspace pool of self-cleaning group tables and epoch-tagged distinct sets,
// and the execute / next / cancel life cycle of thinDB's `exec.Query`
// (exec.zig:903-1218).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <random>
#include <set>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "engine.h"

using namespace tgpu;

namespace {

thread_local std::string g_err;

tgpu_status fail(tgpu_status s, const std::string &msg) {
    g_err = msg;
    return s;
}

}  // namespace

void tgpu::set_error(const char *msg) { g_err = msg ? msg : ""; }

namespace {
std::atomic<long long> g_wait_limit{0};
}
long long tgpu::device_wait_limit() { return g_wait_limit.load(std::memory_order_relaxed); }
std::atomic<uint32_t> g_digest_bits{0};
uint32_t tgpu::hashed_digest_bits() { return g_digest_bits.load(std::memory_order_relaxed); }

namespace {

#define CU(call)                                                                                 \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess) {                                                                 \
            cudaGetLastError(); /* a non-sticky error must not resurface in a later launch */    \
            return fail(TGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));      \
        }                                                                                        \
    } while (0)

int type_bytes(int t) {
    switch (t) {
        case TGPU_BOOLEAN: case TGPU_TINYINT: return 1;
        case TGPU_SMALLINT: return 2;
        case TGPU_INT: case TGPU_DATE: case TGPU_DICT32: case TGPU_FLOAT: return 4;
        case TGPU_DECIMAL128: return 16;
        default: return 8;
    }
}
// intTypeBits (v2_shape_group_topn.zig:2698-2706) plus packed string ids.
int type_bits(int t) {
    switch (t) {
        case TGPU_BOOLEAN: case TGPU_TINYINT: return 8;
        case TGPU_SMALLINT: return 16;
        case TGPU_INT: case TGPU_DATE: case TGPU_DICT32: return 32;
        case TGPU_BIGINT: case TGPU_DATETIME: case TGPU_DECIMAL64: return 64;
        default: return 0;
    }
}
bool is_float_t(int t) { return t == TGPU_FLOAT || t == TGPU_DOUBLE; }
bool is_temporal(int t) { return t == TGPU_DATE || t == TGPU_DATETIME; }
bool is_i64_phys(int t) { return t == TGPU_BIGINT || t == TGPU_DATETIME || t == TGPU_DECIMAL64; }

uint64_t next_pow2(uint64_t x) {
    uint64_t p = 1;
    while (p < x) p <<= 1;
    return p;
}
uint64_t ceil_div(uint64_t a, uint64_t b) { return (a + b - 1) / b; }
uint64_t round_up(uint64_t a, uint64_t b) { return ceil_div(a, b) * b; }

// ------------------------------------------------------------ device --

struct DeviceCtx {
    int id = -1;
    int sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t stats_stream = nullptr;  // registration statistics, beside the column copies
    cudaMemPool_t col_pool = nullptr;     // table columns: stream-ordered, kept after free
};

std::mutex g_dev_mu;
DeviceCtx g_dev;

tgpu_status device_ctx(DeviceCtx **out) {
    std::lock_guard<std::mutex> lk(g_dev_mu);
    if (g_dev.id < 0) {
        int n = 0;
        cudaError_t e = cudaGetDeviceCount(&n);
        if (e != cudaSuccess || n == 0)
            return fail(TGPU_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
        int id = 0;
        CU(cudaGetDevice(&id));
        CU(cudaDeviceGetAttribute(&g_dev.sms, cudaDevAttrMultiProcessorCount, id));
        CU(cudaStreamCreateWithFlags(&g_dev.stream, cudaStreamNonBlocking));
        CU(cudaStreamCreateWithFlags(&g_dev.stats_stream, cudaStreamNonBlocking));
        // Table columns come from a pool of our own that keeps freed memory
        // (release threshold: never), so registering and dropping tables
        // repeatedly does not pay cudaMalloc/cudaFree each time.
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = id;
        CU(cudaMemPoolCreate(&g_dev.col_pool, &props));
        uint64_t keep = UINT64_MAX;
        CU(cudaMemPoolSetAttribute(g_dev.col_pool, cudaMemPoolAttrReleaseThreshold, &keep));
        g_dev.id = id;
    }
    *out = &g_dev;
    return TGPU_OK;
}

// ------------------------------------------------------- workspace pool --

// Group tables come back all-zero (the clear kernel zeroes every slot it
// used), distinct sets carry an epoch so old entries read as free: neither
// needs a memset between queries.
struct Buffer {
    void *p = nullptr;
    size_t bytes = 0;
    bool dirty = false;     // contents unknown: must be zeroed before use
    uint32_t epoch = 0;     // distinct sets: last epoch written
};

void trim_all();

struct Pool {
    explicit Pool(bool zero_) : zero(zero_) {}
    const bool zero;  // hands out zeroed buffers (group tables, bitmaps, sets)
    std::mutex mu;
    std::vector<Buffer> free_;
    tgpu_status take(size_t bytes, cudaStream_t s, Buffer *out) {
        {
            std::lock_guard<std::mutex> lk(mu);
            int best = -1;
            for (size_t i = 0; i < free_.size(); ++i)
                if (free_[i].bytes >= bytes && free_[i].bytes <= 2 * bytes + (1u << 20) &&
                    (best < 0 || free_[i].bytes < free_[best].bytes))
                    best = (int)i;
            if (best >= 0) {
                *out = free_[best];
                free_.erase(free_.begin() + best);
                if (out->dirty && zero) {
                    CU(cudaMemsetAsync(out->p, 0, out->bytes, s));
                    out->dirty = false;
                    out->epoch = 0;
                }
                return TGPU_OK;
            }
        }
        Buffer b;
        b.bytes = bytes;
        cudaError_t e = cudaMalloc(&b.p, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            // release cached buffers and retry once
            trim_all();
            e = cudaMalloc(&b.p, bytes);
            if (e != cudaSuccess) {
                cudaGetLastError();
                return fail(TGPU_ERR_MEMORY_BUDGET, "device allocation of " + std::to_string(bytes) + " bytes failed");
            }
        }
        if (zero) CU(cudaMemsetAsync(b.p, 0, bytes, s));
        *out = b;
        return TGPU_OK;
    }
    void give(Buffer b) {
        if (!b.p) return;
        std::lock_guard<std::mutex> lk(mu);
        free_.push_back(b);
    }
    void trim() {
        std::lock_guard<std::mutex> lk(mu);
        for (auto &b : free_) cudaFree(b.p);
        free_.clear();
    }
};

// Zero-clean buffers (group tables, occupancy bitmaps) and epoch-tagged
// distinct sets never mix: a set's stale entries are not zero.
Pool g_pool(true);
Pool g_set_pool(true);
// Per-query and per-batch scratch (counters, candidate lists, outputs,
// descriptors): reused as is, so creating a query calls no cudaMalloc and
// destroying one no cudaFree (both of which would stall the whole device).
Pool g_scratch_pool(false);

void trim_all() {
    g_pool.trim();
    g_set_pool.trim();
    g_scratch_pool.trim();
}

// Small pinned, device-mapped host blocks (a query's counters and cancel
// flag): carved from 64 KiB cudaHostAlloc chunks and recycled, so creating a
// query allocates no pinned memory.
struct HostSlab {
    static constexpr size_t BLOCK = 128, CHUNK = 64 * 1024;
    std::mutex mu;
    std::vector<char *> free_;
    tgpu_status take(char **out) {
        std::lock_guard<std::mutex> lk(mu);
        if (free_.empty()) {
            char *c = nullptr;
            CU(cudaHostAlloc((void **)&c, CHUNK, cudaHostAllocMapped));
            for (size_t o = 0; o < CHUNK; o += BLOCK) free_.push_back(c + o);
        }
        *out = free_.back();
        free_.pop_back();
        std::memset(*out, 0, BLOCK);
        return TGPU_OK;
    }
    void give(char *p) {
        if (!p) return;
        std::lock_guard<std::mutex> lk(mu);
        free_.push_back(p);
    }
};
HostSlab g_slab;

// Larger pinned, device-mapped host buffers (a batch's packed results and
// counters), best fit from a free list.
struct PinnedPool {
    std::mutex mu;
    std::vector<std::pair<char *, size_t>> free_;
    tgpu_status take(size_t bytes, char **out, size_t *got) {
        {
            std::lock_guard<std::mutex> lk(mu);
            int best = -1;
            for (size_t i = 0; i < free_.size(); ++i)
                if (free_[i].second >= bytes && free_[i].second <= 2 * bytes + 65536 &&
                    (best < 0 || free_[i].second < free_[best].second))
                    best = (int)i;
            if (best >= 0) {
                *out = free_[best].first;
                *got = free_[best].second;
                free_.erase(free_.begin() + best);
                return TGPU_OK;
            }
        }
        CU(cudaHostAlloc((void **)out, bytes, cudaHostAllocMapped));
        *got = bytes;
        return TGPU_OK;
    }
    void give(char *p, size_t bytes) {
        if (!p) return;
        std::lock_guard<std::mutex> lk(mu);
        free_.emplace_back(p, bytes);
    }
};
PinnedPool g_pinned;

// ----------------------------------------------------------------- table --

struct Column {
    std::string name;
    int type = 0;
    int precision = 0, scale = 0;
    void *d_data = nullptr;
    uint32_t *d_valid = nullptr;
    bool owned = false;
    bool nullable = false;
    uint64_t ndv = 0;
    std::vector<int64_t> zmin, zmax;
    std::vector<double> zfmin, zfmax;
    std::vector<uint32_t> znull;
    std::vector<uint32_t> dict_offsets;
    std::vector<uint8_t> dict_bytes;
    // DICT32 with a dictionary: whether every string is there once, and each
    // code's rank in the strings' bytewise order (device, dict size entries)
    bool dict_unique = true;
    uint32_t *d_rank = nullptr;
    std::vector<uint32_t> h_rank;
    // TGPU_VARCHAR: d_data holds the string bytes, d_offs the n_rows + 1
    // offsets; host copies for late materialisation
    uint32_t *d_offs = nullptr;
    std::vector<uint32_t> str_offs;
    std::vector<uint8_t> str_bytes;
    uint32_t dict_size() const { return dict_offsets.size() > 1 ? (uint32_t)dict_offsets.size() - 1 : 0; }
};

// Bytewise order of dictionary strings a and b, a proper prefix first.
int dict_cmp(const Column &c, uint32_t a, uint32_t b) {
    const uint32_t la = c.dict_offsets[a + 1] - c.dict_offsets[a], lb = c.dict_offsets[b + 1] - c.dict_offsets[b];
    const uint32_t n = std::min(la, lb);
    const int r = n ? std::memcmp(c.dict_bytes.data() + c.dict_offsets[a], c.dict_bytes.data() + c.dict_offsets[b], n)
                    : 0;
    if (r) return r < 0 ? -1 : 1;
    return la == lb ? 0 : (la < lb ? -1 : 1);
}

}  // namespace

struct tgpu_table {
    uint64_t n_rows = 0;
    uint32_t rg_rows = 65536;
    uint32_t n_rg = 0;
    std::vector<Column> cols;
    bool sketches = false;  // registered with compute_ndv: plans may sketch composite keys
    cudaStream_t stream = nullptr;  // registration stream: the columns are freed on it
    mutable std::mutex key_mu;
    mutable std::map<std::vector<int32_t>, uint64_t> key_ndv;  // composite-key NDV per group-column list
    tgpu_load_stats load{};  // registration from a segment image
    ~tgpu_table() {
        // Queries on other streams that read the table have finished (a
        // query's next/synchronize waits for it; destroying a table under a
        // running query is a caller error).  Frees return the memory to the
        // column pool in stream order.
        for (auto &c : cols) {
            if (c.owned) cudaFreeAsync(c.d_data, stream);
            if (c.d_valid) cudaFreeAsync(c.d_valid, stream);
            if (c.d_rank) cudaFreeAsync(c.d_rank, stream);
            if (c.d_offs) cudaFreeAsync(c.d_offs, stream);
        }
        cudaStreamSynchronize(stream);
    }
};

namespace {

double hll_estimate(const std::vector<uint32_t> &regs) {
    const double m = (double)regs.size();
    double sum = 0;
    int zeros = 0;
    for (uint32_t r : regs) {
        sum += std::ldexp(1.0, -(int)r);
        if (r == 0) ++zeros;
    }
    double alpha = 0.7213 / (1.0 + 1.079 / m);
    double e = alpha * m * m / sum;
    if (e <= 2.5 * m && zeros > 0) e = m * std::log(m / zeros);  // linear counting
    return e;
}

}  // namespace

// Distinct composite keys of the group columns over all of t's rows: a
// HyperLogLog sketch computed on the device once per column list and kept
// with the table (thinDB sizes its group tables from NDV estimates,
// silo_group_core.zig expectedTotalGroups :11398).
tgpu_status composite_ndv(const tgpu_table *t, const int32_t *cols, uint32_t n, uint64_t *out) {
    const std::vector<int32_t> key(cols, cols + n);
    {
        std::lock_guard<std::mutex> lk(t->key_mu);
        auto it = t->key_ndv.find(key);
        if (it != t->key_ndv.end()) {
            *out = it->second;
            return TGPU_OK;
        }
    }
    DeviceCtx *dev;
    tgpu_status st = device_ctx(&dev);
    if (st != TGPU_OK) return st;
    const cudaStream_t s = dev->stream;
    KeySketchCols k{};
    k.n = (int32_t)n;
    for (uint32_t i = 0; i < n; ++i) {
        const Column &c = t->cols[cols[i]];
        k.data[i] = c.d_data;
        k.valid[i] = c.d_valid;
        k.offs[i] = c.d_offs;
        k.type[i] = c.type;
    }
    std::vector<uint32_t> regs(1u << HLL_P);
    uint32_t *d_regs = nullptr;
    CU(cudaMallocAsync((void **)&d_regs, regs.size() * 4, s));
    cudaError_t e = cudaMemsetAsync(d_regs, 0, regs.size() * 4, s);
    if (e == cudaSuccess) e = launch_key_hll(k, t->n_rows, d_regs, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(regs.data(), d_regs, regs.size() * 4, cudaMemcpyDeviceToHost, s);
    const cudaError_t f = cudaFreeAsync(d_regs, s);
    if (e == cudaSuccess) e = f;
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    CU(e);
    const uint64_t nd = (uint64_t)std::llround(hll_estimate(regs));
    std::lock_guard<std::mutex> lk(t->key_mu);
    t->key_ndv[key] = nd;
    *out = nd;
    return TGPU_OK;
}


// ----------------------------------------------------------------- query --

namespace {

enum RankMode { RANK_NONE = 0, RANK_TOPK = 1, RANK_SORT = 2 };

}  // namespace

struct tgpu_query {
    tgpu_table *t = nullptr;
    cudaStream_t stream = nullptr;
    int flags = 0;
    uint64_t limit = TGPU_NO_LIMIT, offset = 0;
    uint64_t budget = 0;
    std::vector<tgpu_output_column> schema;
    std::vector<int> key_cols;  // table column of each group key (output column i < key_cols.size())
    DevQuery dq{};
    DevFinal df{};
    std::vector<int> out_types;
    int route = 0;
    uint64_t groups_est = 0, sel_est = 0, rows_scanned = 0;
    uint32_t rg_total = 0, rg_pruned = 0;
    int rank = RANK_NONE;
    uint32_t k = 0;
    uint64_t out_rows_max = 0;
    int grid = 0;
    int cache_req = 0;            // requested shared-memory slots (0 auto, -1 off)
    uint32_t chunk_req = 0;       // requested rows per warp chunk (0 auto)
    int load_pct = 50;            // group-table load target
    bool tuned = false;           // settings taken from the tuning table
    bool staged = false;          // the staged (bulk-copy ring) scan runs this query
    bool piped = false;           // the pipelined (producer/consumer) scan runs this query
    bool split = false;           // the split scan (select pass, fold pass) runs this query
    Buffer split_buf;             // its row list and count
    bool radix = false;           // the radix-partitioned route runs this query
    RadixPlan rp{};
    uint64_t radix_cap_req = 0;   // records per partition after an overflow (0 = from the estimate)
    Buffer radix_buf;
    bool sketch = false;          // ORDER BY COUNT(*) DESC LIMIT k: the count sketch runs first
    bool sketch_off = false;      // an inexact filter pass switched it off for this query
    int sketch_order_agg = 0;     // the COUNT(*) aggregate it ranks by
    uint32_t sketch_reruns = 0;
    uint32_t *d_sketch = nullptr; // counts | keep bits | control
    PipePlan pp{};
    int pipe_grid = 0;
    bool batched = false;         // created for a batch (runs inside the batched kernel)
    uint64_t dpart_rows = 0;      // rows that passed when the partitions overflowed
    bool dpart_off = false;       // repeated pairs overflowed a partition: global set
    Buffer dpart_cursor_buf, dpart_pairs_buf;
    int dpart_word = -1;          // the distinct aggregate's state word
    StagePlan sp{};
    int stage_grid = 0;
    // workspace
    Buffer table_buf, occ_buf;
    std::vector<Buffer> dset_bufs;
    std::vector<uint64_t> dset_need;   // distinct entries estimated per set
    Buffer scratch_buf;                // per-query small buffers (one pooled allocation)
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    uint32_t *d_rg_list = nullptr;
    unsigned int *d_ctrl = nullptr;            // [0] tile counter, [1] status
    unsigned long long *d_counts = nullptr;    // [0..3] counts, [4] selected rows
    uint32_t *d_block_counts = nullptr;
    uint32_t n_cpt_blocks = 0;
    uint32_t *d_gids = nullptr;
    unsigned long long *d_cand_keys = nullptr;
    uint32_t *d_cand_gids = nullptr;
    uint32_t n_cand_blocks = 0;
    uint32_t *d_sel = nullptr;
    unsigned long long *d_sort_keys[2] = {nullptr, nullptr};
    uint32_t *d_sort_ids[2] = {nullptr, nullptr};
    std::vector<void *> d_out;
    std::vector<uint8_t *> d_outvalid;
    void **d_out_ptrs = nullptr;
    uint8_t **d_valid_ptrs = nullptr;
    std::vector<uint32_t> rg_list;
    // host pinned (one slab block: counts at 0, cancel flag at 96)
    char *h_block = nullptr;
    int *h_cancel = nullptr;
    int *d_cancel = nullptr;
    unsigned long long *h_counts = nullptr;   // [0..4] counts + selected, [5] status
    // results packed into host memory by a batch (nullptr: read the device outputs)
    const uint8_t *h_packed = nullptr;
    uint64_t pack_rows = 0;
    // state
    bool executed = false, synced = false;
    uint64_t returned = 0, result_rows = 0;
    bool global_agg = false;   // no GROUP BY: exactly one row before OFFSET/LIMIT
    bool synth_empty = false;  // that row, with no rows passing, is written on the host
    uint32_t retries = 0;
    uint32_t launches = 0;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    tgpu_query_stats stats{};

    ~tgpu_query() {
        if (stream) cudaStreamSynchronize(stream);
        release_workspace();
        g_scratch_pool.give(scratch_buf);
        g_slab.give(h_block);
        for (auto e : ev)
            if (e) cudaEventDestroy(e);
    }
    void release_workspace() {
        // a table the clear kernel never ran on (failed/cancelled execute) is dirty
        g_pool.give(table_buf);
        g_pool.give(occ_buf);
        table_buf = occ_buf = Buffer();
        g_scratch_pool.give(dpart_cursor_buf);
        g_scratch_pool.give(dpart_pairs_buf);
        dpart_cursor_buf = dpart_pairs_buf = Buffer();
        g_scratch_pool.give(radix_buf);
        radix_buf = Buffer();
        g_scratch_pool.give(split_buf);
        split_buf = Buffer();
        for (auto &b : dset_bufs) g_set_pool.give(b);
        dset_bufs.clear();
    }
};

namespace {

// Could row group `rg` hold a row satisfying `p`?  (statsOverlapPredicate,
// predicate.zig:3380; rowGroupCanMatch, scan.zig:3539)
bool rg_may_match(const tgpu_table *t, const Column &c, uint32_t rg, const tgpu_predicate &p) {
    uint64_t rows = std::min<uint64_t>(t->rg_rows, t->n_rows - (uint64_t)rg * t->rg_rows);
    uint64_t nulls = c.znull[rg];
    uint64_t valid = rows - nulls;
    if (p.op == TGPU_PRED_IS_NULL) return nulls > 0;
    if (p.op == TGPU_PRED_IS_NOT_NULL) return valid > 0;
    if (valid == 0) return false;
    if (is_float_t(c.type)) {
        double mn = c.zfmin[rg], mx = c.zfmax[rg];
        switch (p.op) {
            case TGPU_PRED_BETWEEN: return mx >= p.flo && mn <= p.fhi;
            case TGPU_PRED_NOT_BETWEEN: return mn < p.flo || mx > p.fhi;
            case TGPU_PRED_EQ: return p.flo >= mn && p.flo <= mx;
            case TGPU_PRED_NE: return true;
            case TGPU_PRED_LT: return mn < p.flo;
            case TGPU_PRED_LE: return mn <= p.flo;
            case TGPU_PRED_GT: return mx > p.flo;
            default: return mx >= p.flo;
        }
    }
    int64_t mn = c.zmin[rg], mx = c.zmax[rg];
    switch (p.op) {
        case TGPU_PRED_BETWEEN: return mx >= p.lo && mn <= p.hi;
        case TGPU_PRED_NOT_BETWEEN: return mn < p.lo || mx > p.hi;
        case TGPU_PRED_EQ: return p.lo >= mn && p.lo <= mx;
        case TGPU_PRED_NE: return !(mn == mx && mn == p.lo);
        case TGPU_PRED_LT: return mn < p.lo;
        case TGPU_PRED_LE: return mn <= p.lo;
        case TGPU_PRED_GT: return mx > p.lo;
        default: return mx >= p.lo;
    }
}

// Fraction of a column's values a predicate keeps, assuming values spread
// uniformly between the column's global min and max (an allocation hint).
double pred_selectivity(const tgpu_table *t, const Column &c, const tgpu_predicate &p) {
    uint64_t nulls = 0;
    for (uint32_t v : c.znull) nulls += v;
    double valid_frac = t->n_rows ? 1.0 - (double)nulls / (double)t->n_rows : 1.0;
    if (p.op == TGPU_PRED_IS_NULL) return 1.0 - valid_frac;
    if (p.op == TGPU_PRED_IS_NOT_NULL) return valid_frac;
    double lo, hi;
    bool have = false;
    double gmin = 0, gmax = 0;
    for (uint32_t rg = 0; rg < t->n_rg; ++rg) {
        uint64_t rows = std::min<uint64_t>(t->rg_rows, t->n_rows - (uint64_t)rg * t->rg_rows);
        if (c.znull[rg] >= rows) continue;
        double mn = is_float_t(c.type) ? c.zfmin[rg] : (double)c.zmin[rg];
        double mx = is_float_t(c.type) ? c.zfmax[rg] : (double)c.zmax[rg];
        if (!have) {
            gmin = mn;
            gmax = mx;
            have = true;
        } else {
            gmin = std::min(gmin, mn);
            gmax = std::max(gmax, mx);
        }
    }
    if (!have) return 0.0;
    const bool f = is_float_t(c.type);
    lo = f ? p.flo : (double)p.lo;
    hi = f ? p.fhi : (double)p.hi;
    double span = gmax - gmin + (f ? 0.0 : 1.0);
    if (span <= 0) span = 1.0;
    auto frac = [&](double a, double b) {
        double x = std::max(a, gmin), y = std::min(b, gmax);
        if (y < x) return 0.0;
        return std::min(1.0, (y - x + (f ? 0.0 : 1.0)) / span);
    };
    double s;
    switch (p.op) {
        case TGPU_PRED_BETWEEN: s = frac(lo, hi); break;
        case TGPU_PRED_NOT_BETWEEN: s = 1.0 - frac(lo, hi); break;
        case TGPU_PRED_EQ: s = 1.0 / (double)std::max<uint64_t>(1, c.ndv); break;
        case TGPU_PRED_NE: s = 1.0; break;
        case TGPU_PRED_LT: case TGPU_PRED_LE: s = frac(gmin, lo); break;
        default: s = frac(lo, gmax); break;
    }
    return std::max(0.0, std::min(1.0, s)) * valid_frac;
}

int used_col(DevQuery &dq, std::vector<int> &map, const tgpu_table *t, int c) {
    if (map[c] >= 0) return map[c];
    if (dq.n_cols >= MAX_QCOLS) return -1;
    const Column &col = t->cols[c];
    DevCol &d = dq.cols[dq.n_cols];
    d.data = col.d_data;
    d.valid = col.d_valid;
    d.offs = col.d_offs;
    d.type = col.type;
    d.bytes = type_bytes(col.type);
    map[c] = dq.n_cols++;
    return map[c];
}

// validateShape (v2_shape_group_topn.zig:2051-2370) for this engine: integer /
// DATE / DECIMAL64 / packed-id keys up to 128 packed bits, COUNT/SUM/AVG/MIN/
// MAX/COUNT(DISTINCT) within thinDB's 16 state slots.  Strings other than
// packed ids (hashed keys) decline to the next route.
// The registered user-defined aggregates' names, lower-cased.
std::mutex g_udf_mu;
std::set<std::string> g_udfs;

// A registry name as thinDB's validateName / lowerName take it, or "" when invalid.
std::string udf_key(const char *name) {
    if (!name) return "";
    std::string k;
    for (const char *c = name; *c; ++c) {
        const unsigned char ch = (unsigned char)*c;
        const bool ok = (ch >= 'a' && ch <= 'z') || (ch >= 'A' && ch <= 'Z') || ch == '_' || (ch >= '0' && ch <= '9');
        if (!ok || k.size() >= 63) return "";
        k.push_back((char)((ch >= 'A' && ch <= 'Z') ? ch - 'A' + 'a' : ch));
    }
    if (k.empty() || (k[0] >= '0' && k[0] <= '9')) return "";
    return k;
}

// Built-in aggregate names a registration may not take (isReservedAggregateName).
bool udf_reserved(const std::string &k) {
    static const char *const names[] = {"count", "sum", "avg", "min", "max", "count_distinct", "sum_distinct",
                                        "avg_distinct", "any_value", "first", "last", "max_by", "min_by",
                                        "percentile", "percentile_disc", "percentile_approx", "group_concat",
                                        "approx_top_k", "stddev", "variance", "median"};
    for (const char *n : names)
        if (k == n) return true;
    return false;
}

tgpu_status plan_query(tgpu_query *q, const tgpu_table *t, const tgpu_request *req) {
    // a user-defined aggregate runs on the host: decline it by name
    for (uint32_t i = 0; i < req->n_aggs; ++i) {
        if (req->aggs[i].func != TGPU_AGG_UDF) continue;
        const std::string k = udf_key(req->aggs[i].udf_name);
        std::lock_guard<std::mutex> lk(g_udf_mu);
        if (k.empty() || !g_udfs.count(k))
            return fail(TGPU_ERR_INVALID_ARGUMENT, std::string("unknown aggregate ") + (req->aggs[i].udf_name ? req->aggs[i].udf_name : "(null)"));
        return fail(TGPU_DECLINE, "user-defined aggregate " + k + " runs on the host");
    }
    DevQuery &dq = q->dq;
    DevFinal &df = q->df;
    std::memset(&dq, 0, sizeof(dq));
    std::memset(&df, 0, sizeof(df));
    std::vector<int> map(t->cols.size(), -1);

    // no GROUP BY: thinDB's global aggregate (v2_global_aggregate.zig), one
    // row; it declines HAVING (:1191)
    if (req->n_group_cols > (uint32_t)MAX_GROUP_KEYS) return fail(TGPU_DECLINE, "group key count");
    q->global_agg = req->n_group_cols == 0;
    if (q->global_agg && req->n_having) return fail(TGPU_DECLINE, "HAVING on a global aggregate");
    if (req->n_aggs == 0 || req->n_aggs > (uint32_t)MAX_AGGS) return fail(TGPU_DECLINE, "aggregate count");
    if (req->n_where > (uint32_t)MAX_PREDS) return fail(TGPU_DECLINE, "too many WHERE conjuncts");
    if (req->n_order > (uint32_t)MAX_ORDER) return fail(TGPU_DECLINE, "too many ORDER BY keys");
    if (req->n_having > (uint32_t)MAX_AGGS) return fail(TGPU_DECLINE, "too many HAVING conjuncts");

    // WHERE
    for (uint32_t i = 0; i < req->n_where; ++i) {
        const tgpu_predicate &w = req->where[i];
        if (w.column < 0 || (size_t)w.column >= t->cols.size())
            return fail(TGPU_ERR_INVALID_ARGUMENT, "predicate column index");
        if (w.op < TGPU_PRED_BETWEEN || w.op > TGPU_PRED_IS_NOT_NULL) return fail(TGPU_DECLINE, "predicate op");
        const Column &c = t->cols[w.column];
        if (c.type == TGPU_VARCHAR) return fail(TGPU_DECLINE, "predicate on a string column");
        if (c.type == TGPU_DICT32 && !(w.op == TGPU_PRED_EQ || w.op == TGPU_PRED_NE || w.op == TGPU_PRED_IS_NULL ||
                                       w.op == TGPU_PRED_IS_NOT_NULL))
            return fail(TGPU_DECLINE, "string range predicate");
        DevPred &p = dq.preds[dq.n_preds++];
        p.col = used_col(dq, map, t, w.column);
        if (p.col < 0) return fail(TGPU_DECLINE, "too many columns");
        p.op = w.op;
        p.is_float = is_float_t(c.type);
        p.lo = w.lo;
        p.hi = w.hi;
        p.flo = w.flo;
        p.fhi = w.fhi;
    }

    // one NOT NULL integer range test: the scan's width-specialised fast filter
    dq.fp_bytes = 0;
    if (req->n_where == 1) {
        const tgpu_predicate &w = req->where[0];
        const Column &c = t->cols[w.column];
        if (!c.nullable && !is_float_t(c.type) && w.op >= TGPU_PRED_BETWEEN && w.op <= TGPU_PRED_GE) {
            const int64_t MN = INT64_MIN, MX = INT64_MAX;
            int64_t lo = 1, hi = 0;  // empty
            int neg = 0;
            switch (w.op) {
                case TGPU_PRED_BETWEEN: lo = w.lo; hi = w.hi; break;
                case TGPU_PRED_NOT_BETWEEN: lo = w.lo; hi = w.hi; neg = 1; break;
                case TGPU_PRED_EQ: lo = hi = w.lo; break;
                case TGPU_PRED_NE: lo = hi = w.lo; neg = 1; break;
                case TGPU_PRED_LT: if (w.lo != MN) { lo = MN; hi = w.lo - 1; } break;
                case TGPU_PRED_LE: lo = MN; hi = w.lo; break;
                case TGPU_PRED_GT: if (w.lo != MX) { lo = w.lo + 1; hi = MX; } break;
                default: lo = w.lo; hi = MX; break;
            }
            dq.fp_data = c.d_data;
            dq.fp_lo = lo;
            dq.fp_hi = hi;
            dq.fp_negate = neg;
            dq.fp_bytes = type_bytes(c.type);
        }
    }

    // key layout: packed (LSB-first parts) up to 128 bits; a string part or
    // wider parts make the key hashed (validateShape, v2_shape_group_topn.zig:
    // 2055-2070: a digest placing the group, its bytes deciding equality)
    int off = 0;
    bool hashed = false;
    {
        int total = 0;
        for (uint32_t i = 0; i < req->n_group_cols; ++i) {
            const int c = req->group_cols[i];
            if (c < 0 || (size_t)c >= t->cols.size()) return fail(TGPU_ERR_INVALID_ARGUMENT, "group column index");
            const Column &col = t->cols[c];
            if (col.type == TGPU_VARCHAR) hashed = true;
            else if (type_bits(col.type) == 0) return fail(TGPU_DECLINE, "group key type");
            else total += type_bits(col.type) + (col.nullable ? 1 : 0);
        }
        if (total > 128) hashed = true;
    }
    for (uint32_t i = 0; i < req->n_group_cols; ++i) {
        int c = req->group_cols[i];
        const Column &col = t->cols[c];
        int bits = col.type == TGPU_VARCHAR ? 0 : type_bits(col.type);
        // a packed code stands for its string only when no string has two
        // codes (thinDB's table ids are one per value)
        if (col.type == TGPU_DICT32 && !col.dict_unique) return fail(TGPU_DECLINE, "dictionary repeats a string");
        DevKeyPart &kp = dq.parts[dq.n_parts];
        kp.col = used_col(dq, map, t, c);
        if (kp.col < 0) return fail(TGPU_DECLINE, "too many columns");
        kp.offset = off;
        kp.payload = bits;
        kp.nullable = col.nullable ? 1 : 0;
        df.parts[dq.n_parts] = kp;
        df.part_types[dq.n_parts] = col.type;
        df.part_cols[dq.n_parts] = dq.cols[kp.col];
        dq.n_parts++;
        off += bits + kp.nullable;
        tgpu_output_column oc{};
        std::snprintf(oc.name, sizeof(oc.name), "%s", col.name.c_str());
        oc.type = col.type;
        oc.decimal_precision = (uint8_t)col.precision;
        oc.decimal_scale = (uint8_t)col.scale;
        oc.nullable = col.nullable;
        oc.elem_bytes = col.type == TGPU_VARCHAR ? 8 : type_bytes(col.type);  // a string key: its row
        q->schema.push_back(oc);
        q->key_cols.push_back(c);
    }
    dq.hashed = df.hashed = hashed ? 1 : 0;
    dq.digest_bits = hashed ? hashed_digest_bits() : 0;
    dq.key_words = hashed || off > 64 ? 2 : 1;
    // a global aggregate's one group takes the packed key 1, not the empty
    // marker 0, so it lives in each CTA's shared-memory table
    dq.key_or = q->global_agg ? 1 : 0;
    df.global_avg = q->global_agg ? 1 : 0;

    // aggregates and state words (word 0 = the group's row count).  `next`
    // counts slots exactly as thinDB does (its 16-slot limit decides
    // declines); `phys` allocates the device words, where SUM and AVG of one
    // column share their sum (and valid-count) words.
    int next = 1, phys = 1;
    struct Shared {
        int col, kind, word, vword;
    };
    std::vector<Shared> shared;
    for (uint32_t i = 0; i < req->n_aggs; ++i) {
        const tgpu_agg_spec &a = req->aggs[i];
        DevAgg &g = dq.aggs[dq.n_aggs];
        DevOut &o = df.outs[dq.n_aggs];
        g.col = -1;
        g.vword = -1;
        g.owner = 1;
        o.vword = -1;
        o.func = a.func;
        int in_type = 0, scale = 0;
        bool nullable = false;
        if (a.column >= 0) {
            if ((size_t)a.column >= t->cols.size()) return fail(TGPU_ERR_INVALID_ARGUMENT, "aggregate column index");
            const Column &col = t->cols[a.column];
            in_type = col.type;
            nullable = col.nullable;
            scale = col.type == TGPU_DECIMAL64 ? col.scale : 0;
            g.col = used_col(dq, map, t, a.column);
            if (g.col < 0) return fail(TGPU_DECLINE, "too many columns");
            g.is_float_in = is_float_t(in_type);
        }
        int out_type = TGPU_BIGINT;
        switch (a.func) {
            case TGPU_AGG_COUNT:
                if (nullable) {
                    if (next > MAX_AGGS) return fail(TGPU_DECLINE, "aggregate state count");
                    g.kind = AK_COUNT_VALID;
                    next++;
                    g.word = phys++;
                } else {
                    g.kind = AK_COUNT_ROWS;
                    g.word = 0;
                }
                break;
            case TGPU_AGG_SUM: case TGPU_AGG_AVG: case TGPU_AGG_MIN: case TGPU_AGG_MAX: {
                if (a.column < 0) return fail(TGPU_ERR_INVALID_ARGUMENT, "aggregate column");
                if (in_type == TGPU_DICT32 || in_type == TGPU_VARCHAR) return fail(TGPU_DECLINE, "string aggregate");
                bool sum = a.func == TGPU_AGG_SUM || a.func == TGPU_AGG_AVG;
                if (sum && is_temporal(in_type)) return fail(TGPU_DECLINE, "temporal read as a number");
                bool wide = sum && is_i64_phys(in_type);
                int width = (wide ? 2 : 1) + (nullable ? 1 : 0);
                if (next + width - 1 > MAX_AGGS) return fail(TGPU_DECLINE, "aggregate state count");
                next += width;
                // a group of a table under 2^32 rows folds fewer than 2^32 values: carry-free words
                const int wide_kind = t->n_rows < (1ULL << 32) ? AK_SUM_I128 : AK_SUM_I128C;
                if (sum) g.kind = is_float_t(in_type) ? AK_SUM_F64 : (wide ? wide_kind : AK_SUM_I64);
                else {
                    bool mn = a.func == TGPU_AGG_MIN;
                    g.kind = is_float_t(in_type) ? (mn ? AK_MIN_F : AK_MAX_F) : (mn ? AK_MIN_I : AK_MAX_I);
                }
                const Shared *sh = nullptr;
                for (const Shared &s2 : shared)
                    if (s2.col == a.column && s2.kind == g.kind) sh = &s2;
                if (sh) {
                    g.word = sh->word;
                    g.vword = sh->vword;
                    g.owner = 0;
                } else {
                    g.word = phys;
                    g.vword = nullable ? phys + width - 1 : -1;
                    phys += width;
                    shared.push_back(Shared{a.column, g.kind, g.word, g.vword});
                }
                if (sum) {
                    if (a.func == TGPU_AGG_SUM)
                        out_type = in_type == TGPU_DECIMAL64 ? TGPU_DECIMAL128 : (is_float_t(in_type) ? TGPU_DOUBLE : TGPU_BIGINT);
                    else
                        out_type = TGPU_DOUBLE;
                } else {
                    out_type = in_type;
                }
                break;
            }
            case TGPU_AGG_COUNT_DISTINCT:
                if (a.column < 0) return fail(TGPU_ERR_INVALID_ARGUMENT, "count distinct column");
                if (in_type == TGPU_VARCHAR) return fail(TGPU_DECLINE, "COUNT(DISTINCT) over a string column");
                if (dq.n_dsets >= MAX_DISTINCT) return fail(TGPU_DECLINE, "count distinct slot count");
                if (next > MAX_AGGS) return fail(TGPU_DECLINE, "aggregate state count");
                g.kind = AK_DISTINCT;
                next++;
                g.word = phys++;
                g.dset = dq.n_dsets++;
                dq.needs_gid = 1;
                break;
            default:
                return fail(TGPU_DECLINE, "aggregate func");
        }
        g.needs_value = (g.kind == AK_DISTINCT || (g.owner && g.kind != AK_COUNT_ROWS && g.kind != AK_COUNT_VALID)) ? 1 : 0;
        o.kind = g.kind;
        o.word = g.word;
        o.vword = g.vword;
        o.out_type = out_type;
        o.in_type = in_type;
        o.scale = scale;
        o.nullable = (nullable && (a.func == TGPU_AGG_SUM || a.func == TGPU_AGG_AVG || a.func == TGPU_AGG_MIN ||
                                   a.func == TGPU_AGG_MAX)) ? 1 : 0;
        dq.n_aggs++;
        q->out_types.push_back(out_type);
        tgpu_output_column oc{};
        std::snprintf(oc.name, sizeof(oc.name), "%s", a.as ? a.as : "");
        oc.type = out_type;
        // a global aggregate over no rows still emits its row: SUM, AVG, MIN
        // and MAX are NULL there (v2_global_aggregate.zig:1853-1855)
        oc.nullable = o.nullable || (q->global_agg && (a.func == TGPU_AGG_SUM || a.func == TGPU_AGG_AVG ||
                                                       a.func == TGPU_AGG_MIN || a.func == TGPU_AGG_MAX));
        if (out_type == TGPU_DECIMAL128) {
            oc.decimal_precision = 38;
            oc.decimal_scale = (uint8_t)scale;
        } else if (out_type == TGPU_DECIMAL64) {
            oc.decimal_precision = (uint8_t)t->cols[a.column].precision;
            oc.decimal_scale = (uint8_t)scale;
        }
        oc.elem_bytes = type_bytes(out_type);
        q->schema.push_back(oc);
    }
    dq.state_words = phys;
    dq.slot_words = (int)next_pow2((uint64_t)(dq.key_words + dq.state_words));

    // compiled fast fold: NOT NULL key parts and inputs, at most four owner
    // aggregates (the scan falls back to the interpreter when no compiled
    // signature matches)
    dq.fast_km = 0;
    dq.n_faggs = 0;
    {
        bool ok = dq.n_parts > 0 && !dq.hashed;  // the compiled folds read at least one packed key part
        for (int i = 0; i < dq.n_parts; ++i) ok = ok && !dq.parts[i].nullable;
        for (int a = 0; a < dq.n_aggs && ok; ++a) {
            const DevAgg &g = dq.aggs[a];
            if (g.kind == AK_COUNT_ROWS || !g.owner) continue;
            if (g.kind == AK_COUNT_VALID || g.vword >= 0 || (g.kind == AK_DISTINCT && g.is_float_in) ||
                dq.n_faggs >= 4) {
                ok = false;
                break;
            }
            dq.faggs[dq.n_faggs++] = g;
        }
        if (ok) dq.fast_km = dq.n_parts == 1 ? 1 : 2;
        else dq.n_faggs = 0;
        dq.fast_id = fast_fold_id(dq);
    }

    for (uint32_t i = 0; i < req->n_order; ++i) {
        const tgpu_sort_spec &s = req->order[i];
        if (!((s.target == TGPU_SORT_KEY && s.index >= 0 && (uint32_t)s.index < req->n_group_cols) ||
              (s.target == TGPU_SORT_AGG && s.index >= 0 && (uint32_t)s.index < req->n_aggs)))
            return fail(TGPU_DECLINE, "order key");
        df.order[i] = DevOrder{s.target, s.index, s.desc ? 1 : 0, 0};
        // thinDB ranks a hashed key's parts after the emit (finish_after_emit,
        // v2_shape_group_topn.zig:302-325); this operator does not
        if (s.target == TGPU_SORT_KEY && dq.hashed) return fail(TGPU_DECLINE, "ORDER BY a hashed key");
        if (s.target == TGPU_SORT_KEY && df.part_types[s.index] == TGPU_DICT32) {
            // thinDB ranks a string key on its emitted strings
            // (v2_shape_group_topn.zig:302-325): here on each code's rank
            const Column &col = t->cols[req->group_cols[s.index]];
            if (!col.d_rank) return fail(TGPU_DECLINE, "ORDER BY a string key without its dictionary");
            df.part_rank[s.index] = col.d_rank;
            df.part_rank_n[s.index] = col.dict_size();
        }
    }
    for (uint32_t i = 0; i < req->n_having; ++i) {
        const tgpu_having &h = req->having[i];
        if (h.agg < 0 || (uint32_t)h.agg >= req->n_aggs || h.op < TGPU_PRED_EQ || h.op > TGPU_PRED_GE)
            return fail(TGPU_DECLINE, "having");
        df.having[i] = DevHaving{h.agg, h.op, h.ival, h.fval};
    }
    df.n_parts = dq.n_parts;
    df.n_aggs = dq.n_aggs;
    df.n_order = (int32_t)req->n_order;
    df.n_having = (int32_t)req->n_having;
    df.key_words = dq.key_words;
    df.slot_words = dq.slot_words;
    df.sort_words = 2 * (int32_t)req->n_order + 2;

    // zone-map pruning -> the row groups the scan visits
    q->rg_total = t->n_rg;
    q->rg_list.clear();
    uint64_t rows_scanned = 0;
    for (uint32_t rg = 0; rg < t->n_rg; ++rg) {
        bool keep = true;
        for (uint32_t i = 0; i < req->n_where && keep; ++i)
            keep = rg_may_match(t, t->cols[req->where[i].column], rg, req->where[i]);
        if (keep) {
            q->rg_list.push_back(rg);
            rows_scanned += std::min<uint64_t>(t->rg_rows, t->n_rows - (uint64_t)rg * t->rg_rows);
        }
    }
    q->rg_pruned = t->n_rg - (uint32_t)q->rg_list.size();
    q->rows_scanned = rows_scanned;

    double sel = 1.0;
    for (uint32_t i = 0; i < req->n_where; ++i) sel *= pred_selectivity(t, t->cols[req->where[i].column], req->where[i]);
    uint64_t sel_rows = (uint64_t)std::ceil((double)rows_scanned * std::min(1.0, sel * 1.25));
    q->sel_est = sel_rows;
    uint64_t groups = 1;
    for (uint32_t i = 0; i < req->n_group_cols; ++i) {
        const Column &c = t->cols[req->group_cols[i]];
        uint64_t nd = std::max<uint64_t>(1, c.ndv) + (c.nullable ? 1 : 0);
        groups = (groups > (1ULL << 40) / nd) ? (1ULL << 40) : groups * nd;
    }
    if (req->n_group_cols >= 2 && t->sketches && !req->expected_groups && groups > COMPOSITE_SKETCH_MIN) {
        // correlated parts: the product overestimates; the key's own sketch
        // (+1/16 for the sketch's error) bounds it
        uint64_t nd = 0;
        tgpu_status st = composite_ndv(t, req->group_cols, req->n_group_cols, &nd);
        if (st != TGPU_OK) return st;
        if (nd) groups = std::min<uint64_t>(groups, nd + nd / 16 + 64);
    }
    groups = std::min<uint64_t>(groups, std::max<uint64_t>(1, sel_rows));
    if (req->expected_groups) groups = req->expected_groups;
    q->groups_est = groups;
    for (int d = 0; d < dq.n_dsets; ++d) {
        // pairs <= rows that reach the fold, and <= groups * distinct values
        int col = -1;
        for (uint32_t i = 0; i < req->n_aggs; ++i)
            if (dq.aggs[i].kind == AK_DISTINCT && dq.aggs[i].dset == d) col = req->aggs[i].column;
        uint64_t ndv = std::max<uint64_t>(1, t->cols[col].ndv);
        uint64_t pairs = groups > (1ULL << 40) / ndv ? (1ULL << 40) : groups * ndv;
        pairs = std::min<uint64_t>(pairs, std::max<uint64_t>(1, sel_rows));
        q->dset_need.push_back(pairs);
    }
    return TGPU_OK;
}

// Shared-memory cache size for a state width: the largest power of two that
// keeps two CTAs per SM (<= ~100 KB each).
int cache_slots_for(int state_words, size_t list_bytes) {
    size_t per = 12 + 8 * (size_t)state_words;
    int c = 4096;
    while (c >= 64 && (size_t)c * per + list_bytes + 16 > 110 * 1024) c >>= 1;
    return c;
}

tgpu_status size_workspace(tgpu_query *q, uint64_t cap) {
    DevQuery &dq = q->dq;
    DevFinal &df = q->df;
    cap = std::max<uint64_t>(cap, 64);
    if (cap > (1ULL << 31)) return fail(TGPU_ERR_MEMORY_BUDGET, "group table would exceed 2^31 slots");
    dq.cap = cap;
    df.cap = cap;

    // (equal digests are not equal keys: a hashed key folds lane by lane)
    dq.warp_combine = (q->flags & TGPU_FLAG_NO_WARP_COMBINE) || dq.hashed ? 0 : 1;
    dq.inline_fold = (q->flags & TGPU_FLAG_INLINE_FOLD) ? 1 : 0;
    // survivors are compacted and folded 32 at a time (gather) unless the
    // WHERE is estimated to keep most rows: folding in place runs a fold per
    // 32 scanned rows, however few of them survive
    // survivor gather for a WHERE (queue mode — dense coalesced loads,
    // survivors compacted into a per-warp shared-memory ring, full-batch
    // folds — on request: with the out-of-line fold its spills around each
    // call cost more than the gathers it saves)
    {
        const uint64_t rows = std::max<uint64_t>(1, q->rows_scanned);
        const bool dense_enough = q->sel_est * 10 >= rows * 6;  // >= 60%
        dq.gather = 0;
        if (dq.n_preds > 0 && !(q->flags & TGPU_FLAG_DENSE_SCAN)) {
            if (q->flags & TGPU_FLAG_GATHER_SCAN) dq.gather = 1;
            else if (dq.fast_id >= 0 && (q->flags & TGPU_FLAG_QUEUE_SCAN)) dq.gather = 2;
            else if (!dense_enough) dq.gather = 1;
        }
    }
    // the split scan runs a survivor gather whose row numbers fit 32 bits
    // (not with the staged, pipelined or inlined-fold scans, nor in batches)
    // (and the count sketch's filter pass: its select pass keeps the rows of
    // kept counters)
    q->split = !(q->flags & TGPU_FLAG_NO_SPLIT) &&
               !(q->flags & (TGPU_FLAG_STAGED_SCAN | TGPU_FLAG_PIPE_SCAN | TGPU_FLAG_INLINE_FOLD)) && !q->batched &&
               (dq.gather == 1 || q->sketch) && q->t->n_rows < (1ULL << 32);

    // chunking: about eight chunks per warp of a two-CTA-per-SM grid
    {
        DeviceCtx *dev;
        tgpu_status st = device_ctx(&dev);
        if (st != TGPU_OK) return st;
        uint64_t warps = (uint64_t)dev->sms * 2 * SCAN_WARPS;
        uint64_t chunk = q->chunk_req;
        if (!chunk) {
            chunk = std::max<uint64_t>(1, q->rows_scanned / (warps * 8));
            chunk = std::max<uint64_t>(CHUNK_ALIGN, chunk / CHUNK_ALIGN * CHUNK_ALIGN);
            chunk = std::min<uint64_t>(chunk, dq.gather == 1 ? 1024 : 4096);
        }
        dq.chunk_rows = (uint32_t)chunk;
    }
    const size_t list_bytes =
        dq.gather == 1 ? (size_t)SCAN_WARPS * dq.chunk_rows * 2
        : dq.gather == 2 ? (size_t)SCAN_WARPS * WQ_RING_ROWS * (24 + 8 * (size_t)std::max(1, dq.n_faggs)) + 16 : 0;

    // route: the shared-memory table holds every group (lowcard), keeps the
    // first-seen (hottest) keys of a larger key space (global route), or is off
    dq.cache_slots = 0;
    dq.cache_probe = 0;
    q->route = 2;
    if (dq.key_words == 1 && !(q->flags & TGPU_FLAG_FORCE_GLOBAL) && q->cache_req >= 0) {
        int C = cache_slots_for(dq.state_words, list_bytes);
        if (q->cache_req > 0) C = std::min(C, q->cache_req);
        if (C >= 64 && q->groups_est * 8 <= (uint64_t)C * 5) {
            dq.cache_slots = C;
            dq.cache_probe = C;  // resident: probe the whole table
            q->route = 1;
        } else if (C >= 64 && !dq.needs_gid) {
            dq.cache_slots = C;
            dq.cache_probe = 16;
        }
    }

    // ranking
    if (df.n_order == 0 && q->limit == TGPU_NO_LIMIT && q->offset == 0) {
        q->rank = RANK_NONE;
        q->out_rows_max = cap + 1;
    } else if (q->limit != TGPU_NO_LIMIT && q->offset + q->limit <= 32) {
        q->rank = RANK_TOPK;
        q->k = (uint32_t)(q->offset + q->limit);
        q->out_rows_max = q->limit;
    } else {
        q->rank = RANK_SORT;
        q->out_rows_max = q->limit == TGPU_NO_LIMIT ? cap + 1 : std::min<uint64_t>(q->limit, cap + 1);
    }

    // bytes
    const uint64_t slots = cap + 1;
    const size_t table_bytes = slots * (size_t)dq.slot_words * 8;
    const size_t occ_bytes = ((slots + 31) / 32) * 4;
    // COUNT(DISTINCT): partitioned (pairs to hash partitions, deduplicated
    // per partition in shared memory) for one distinct aggregate over many
    // rows, else a global (group, value) set
    dq.dpart_bits = 0;
    dq.dpart_cap = 0;
    q->dpart_word = -1;
    size_t dpart_bytes = 0;
    if (dq.n_dsets == 1 && !q->batched && !q->dpart_off && !(q->flags & TGPU_FLAG_NO_DISTINCT_PARTITION) &&
        ((q->flags & TGPU_FLAG_DISTINCT_PARTITION) || q->sel_est >= (2ULL << 20))) {
        // about three quarters of a partition's capacity expected
        const uint64_t per = DPART_CAP * 3 / 4, rows = std::max(q->sel_est, q->dpart_rows);
        int bits = 1;
        while (bits < DPART_MAX_BITS && ((uint64_t)1 << bits) * per < rows) ++bits;
        dq.dpart_bits = bits;
        dq.dpart_cap = DPART_CAP;
        for (int a = 0; a < dq.n_aggs; ++a)
            if (dq.aggs[a].kind == AK_DISTINCT) q->dpart_word = dq.aggs[a].word;
        dpart_bytes = ((size_t)4 << bits) + ((size_t)DPART_CAP * 16 << bits);
    }
    // the radix route: partitions of at most ~40% of a shared table's slots
    // in groups; the partitions' buffers sized from the rows expected to pass
    size_t radix_bytes = 0;
    if (q->radix) {
        RadixPlan &rp = q->rp;
        rp = RadixPlan{};
        const uint64_t per = RX_SLOTS * 2 / 5;
        uint32_t bits = 1;
        while (bits < RX_MAX_BITS && (q->groups_est >> bits) > per) ++bits;
        rp.bits = bits;
        if (dq.dpart_bits && dq.dpart_bits <= (int)bits) {
            dq.dpart_bits = (int)bits + 1;  // at least two pair sub-partitions per partition
            dpart_bytes = ((size_t)4 << dq.dpart_bits) + ((size_t)DPART_CAP * 16 << dq.dpart_bits);
        }
        rp.sub_bits = dq.dpart_bits ? (uint32_t)dq.dpart_bits - bits : 0u;
        const uint64_t rows = std::max<uint64_t>(1, q->sel_est);
        rp.cap = q->radix_cap_req ? q->radix_cap_req : ceil_div(rows * 5, (uint64_t)4 << bits) + RX_TILE;
        rp.tiles_per_rg = q->t->rg_rows / RX_TILE;
        rp.n_tiles = (uint32_t)q->rg_list.size() * rp.tiles_per_rg;
        const uint64_t words = 1 + (uint64_t)dq.n_faggs;
        radix_bytes = ((size_t)4 << bits) + ((size_t)rp.cap << bits) * words * 8;
        dq.cache_slots = (int32_t)RX_SLOTS;  // the aggregate kernel's per-partition table
        dq.cache_probe = (int32_t)RX_SLOTS;
        const uint32_t cache = RX_SLOTS * (12u + 8u * (uint32_t)dq.state_words);
        rp.dcur_off = (cache + 16 + 15) & ~15u;
        rp.agg_smem = rp.dcur_off + (4u << rp.sub_bits);
        rp.agg_per_sm = rp.agg_smem * 2 <= 227u * 1024 ? 2 : 1;
    }
    std::vector<uint64_t> dcap;
    size_t dset_bytes = 0;
    for (uint64_t need : q->dset_need) {
        if (dq.dpart_bits) break;
        uint64_t c = next_pow2(std::max<uint64_t>(64, need * 2));
        dcap.push_back(c);
        dset_bytes += c * 16;
    }
    q->n_cpt_blocks = compact_blocks(cap);
    {
        // enough CTAs to stream the group list, a few per SM at most
        DeviceCtx *dev;
        tgpu_status st = device_ctx(&dev);
        if (st != TGPU_OK) return st;
        const uint64_t want = (std::min<uint64_t>(q->groups_est, cap + 1) + 2047) / 2048;
        q->n_cand_blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)dev->sms * 2));
    }
    size_t row_bytes = 0;
    for (auto &oc : q->schema) row_bytes += oc.elem_bytes + 1;
    const size_t sw = (size_t)df.sort_words;
    size_t scratch = 0;
    auto add = [&](size_t b) {
        size_t o = scratch;
        scratch += (b + 255) & ~(size_t)255;
        return o;
    };
    size_t o_ctrl = add(16), o_counts = add(8 * 8), o_bc = add(4 * (size_t)q->n_cpt_blocks), o_gids = add(4 * slots);
    size_t o_ck = 0, o_cg = 0, o_sel = 0, o_sk0 = 0, o_sk1 = 0, o_si0 = 0, o_si1 = 0;
    if (q->rank == RANK_TOPK) {
        o_ck = add((size_t)q->n_cand_blocks * 32 * topk_width((int)sw) * 8);
        o_cg = add((size_t)q->n_cand_blocks * 32 * 4);
        o_sel = add(32 * 4);
    } else if (q->rank == RANK_SORT) {
        o_sk0 = add(slots * sw * 8);
        o_sk1 = add(slots * sw * 8);
        o_si0 = add(slots * 4);
        o_si1 = add(slots * 4);
    }
    size_t o_rg = add(4 * std::max<size_t>(1, q->rg_list.size()));
    std::vector<size_t> o_out, o_val;
    for (auto &oc : q->schema) {
        o_out.push_back(add(q->out_rows_max * oc.elem_bytes));
        o_val.push_back(add(q->out_rows_max));
    }
    size_t o_ptrs = add(q->schema.size() * 8), o_vptrs = add(q->schema.size() * 8);
    const size_t o_sketch = q->sketch ? add(((size_t)1 << SK_BITS) * 4 + ((size_t)1 << SK_BITS) / 8 + 64) : 0;
    (void)row_bytes;

    // the split scan's row list: every row of the kept row groups, at most
    const size_t split_bytes = q->split ? 256 + 4 * (size_t)q->rg_list.size() * q->t->rg_rows : 0;
    const size_t total = table_bytes + occ_bytes + dset_bytes + dpart_bytes + radix_bytes + split_bytes + scratch;
    if (q->budget && total > q->budget)
        return fail(TGPU_ERR_MEMORY_BUDGET, "query needs " + std::to_string(total) + " device bytes, budget " +
                                                std::to_string(q->budget));

    q->release_workspace();
    tgpu_status st;
    if ((st = g_pool.take(table_bytes, q->stream, &q->table_buf)) != TGPU_OK) return st;
    if ((st = g_pool.take(occ_bytes, q->stream, &q->occ_buf)) != TGPU_OK) return st;
    for (size_t d = 0; d < dcap.size(); ++d) {
        Buffer b;
        if ((st = g_set_pool.take(dcap[d] * 16, q->stream, &b)) != TGPU_OK) return st;
        q->dset_bufs.push_back(b);
        dq.dset[d] = (unsigned long long *)b.p;
        dq.dset_cap[d] = dcap[d];
    }
    if (dq.dpart_bits) {
        if ((st = g_scratch_pool.take((size_t)4 << dq.dpart_bits, q->stream, &q->dpart_cursor_buf)) != TGPU_OK)
            return st;
        if ((st = g_scratch_pool.take((size_t)DPART_CAP * 16 << dq.dpart_bits, q->stream, &q->dpart_pairs_buf)) !=
            TGPU_OK)
            return st;
        dq.dpart_cursor = (uint32_t *)q->dpart_cursor_buf.p;
        dq.dpart_buf = (ulonglong2 *)q->dpart_pairs_buf.p;
        dq.dset[0] = nullptr;
        dq.dset_cap[0] = 0;
    }
    if (q->split && (st = g_scratch_pool.take(split_bytes, q->stream, &q->split_buf)) != TGPU_OK) return st;
    if (q->radix) {
        if ((st = g_scratch_pool.take(radix_bytes, q->stream, &q->radix_buf)) != TGPU_OK) return st;
        q->rp.cursor = (uint32_t *)q->radix_buf.p;
        q->rp.buf = (unsigned long long *)((char *)q->radix_buf.p + ((size_t)4 << q->rp.bits));
    }
    if (scratch > q->scratch_bytes) {
        g_scratch_pool.give(q->scratch_buf);
        q->scratch_buf = Buffer();
        if ((st = g_scratch_pool.take(scratch, q->stream, &q->scratch_buf)) != TGPU_OK) return st;
        q->scratch = q->scratch_buf.p;
        q->scratch_bytes = q->scratch_buf.bytes;
    }
    char *base = (char *)q->scratch;
    q->d_ctrl = (unsigned int *)(base + o_ctrl);
    q->d_counts = (unsigned long long *)(base + o_counts);
    q->d_block_counts = (uint32_t *)(base + o_bc);
    q->d_gids = (uint32_t *)(base + o_gids);
    q->d_cand_keys = q->rank == RANK_TOPK ? (unsigned long long *)(base + o_ck) : nullptr;
    q->d_cand_gids = q->rank == RANK_TOPK ? (uint32_t *)(base + o_cg) : nullptr;
    q->d_sel = q->rank == RANK_TOPK ? (uint32_t *)(base + o_sel) : nullptr;
    if (q->rank == RANK_SORT) {
        q->d_sort_keys[0] = (unsigned long long *)(base + o_sk0);
        q->d_sort_keys[1] = (unsigned long long *)(base + o_sk1);
        q->d_sort_ids[0] = (uint32_t *)(base + o_si0);
        q->d_sort_ids[1] = (uint32_t *)(base + o_si1);
    }
    q->d_rg_list = (uint32_t *)(base + o_rg);
    q->d_out.clear();
    q->d_outvalid.clear();
    for (size_t c = 0; c < q->schema.size(); ++c) {
        q->d_out.push_back(base + o_out[c]);
        q->d_outvalid.push_back((uint8_t *)(base + o_val[c]));
    }
    q->d_sketch = q->sketch ? (uint32_t *)(base + o_sketch) : nullptr;
    q->d_out_ptrs = (void **)(base + o_ptrs);
    q->d_valid_ptrs = (uint8_t **)(base + o_vptrs);
    CU(cudaMemcpyAsync(q->d_out_ptrs, q->d_out.data(), q->schema.size() * 8, cudaMemcpyHostToDevice, q->stream));
    CU(cudaMemcpyAsync(q->d_valid_ptrs, q->d_outvalid.data(), q->schema.size() * 8, cudaMemcpyHostToDevice, q->stream));
    if (!q->rg_list.empty())
        CU(cudaMemcpyAsync(q->d_rg_list, q->rg_list.data(), 4 * q->rg_list.size(), cudaMemcpyHostToDevice, q->stream));
    // (pageable sources: each copy has staged its bytes when it returns, so
    // the vectors may change afterwards; no synchronisation needed)

    dq.table = (unsigned long long *)q->table_buf.p;
    dq.occ = (uint32_t *)q->occ_buf.p;
    df.table = dq.table;
    df.occ = dq.occ;
    dq.tile_counter = q->d_ctrl;
    dq.status = q->d_ctrl + 1;
    dq.selected_rows = q->d_counts + 4;
    dq.cancel = (const volatile int *)q->d_cancel;
    const tgpu_table *t = q->t;
    dq.n_rows = t->n_rows;
    dq.rg_rows = t->rg_rows;
    const bool pruned = q->rg_list.size() != t->n_rg;
    if (pruned) {
        dq.rg_list = q->d_rg_list;
        dq.n_rg = (uint32_t)q->rg_list.size();
        dq.chunks_per_rg = (t->rg_rows + dq.chunk_rows - 1) / dq.chunk_rows;
        dq.n_chunks = dq.n_rg * dq.chunks_per_rg;
    } else {
        dq.rg_list = nullptr;
        dq.n_rg = t->n_rg;
        dq.chunks_per_rg = 0;
        dq.n_chunks = (uint32_t)((t->n_rows + dq.chunk_rows - 1) / dq.chunk_rows);
    }

    // prefetching: group-table slots (and distinct entries on request) as
    // soon as a gathered row's key is known; each warp's next chunk of every
    // scanned column into L2 with one bulk prefetch per column
    dq.prefetch = ((q->flags & TGPU_FLAG_NO_PREFETCH) ? 0 : PF_SLOT) |
                  ((q->flags & TGPU_FLAG_NO_CHUNK_PREFETCH) ? 0 : PF_NEXT) |
                  ((q->flags & TGPU_FLAG_DISTINCT_PREFETCH) ? PF_DISTINCT : 0);
    dq.n_pf = 0;
    {
        auto add_pf = [&](int c) {
            if (c < 0 || dq.n_pf >= 8 || ((uintptr_t)dq.cols[c].data & 15)) return;
            for (int i = 0; i < dq.n_pf; ++i)
                if (dq.pf_cols[i] == c) return;
            dq.pf_cols[dq.n_pf++] = c;
        };
        for (int i = 0; i < dq.n_preds; ++i) add_pf(dq.preds[i].col);
        for (int i = 0; i < dq.n_parts; ++i) add_pf(dq.parts[i].col);
        for (int a = 0; a < dq.n_aggs; ++a) add_pf(dq.aggs[a].col);
    }

    // the staged scan (tiles of every column through a shared-memory ring of
    // bulk copies) for a compiled fold over NOT NULL columns, on request
    q->staged = false;
    const bool want_staged = !(q->flags & TGPU_FLAG_NO_STAGED) && (q->flags & TGPU_FLAG_STAGED_SCAN);
    if (want_staged && t->rg_rows % STAGE_TILE == 0) {
        DevQuery probe = dq;
        const uint64_t tiles = (uint64_t)dq.n_rg * (t->rg_rows / STAGE_TILE);
        DeviceCtx *dev;
        if (tiles > 0 && stage_plan(probe, tiles, &q->sp) && device_ctx(&dev) == TGPU_OK) {
            dq.cache_slots = probe.cache_slots;
            dq.cache_probe = probe.cache_probe;
            if (q->route == 1 && !(dq.cache_slots && dq.cache_probe == dq.cache_slots)) q->route = 2;
            q->stage_grid = (int)std::min<uint64_t>((uint64_t)dev->sms, tiles);
            q->staged = true;
        }
    }
    // the pipelined scan, on request
    q->piped = false;
    const bool want_pipe = !q->staged && !(q->flags & TGPU_FLAG_NO_PIPE) && (q->flags & TGPU_FLAG_PIPE_SCAN);
    if (want_pipe && t->rg_rows % PIPE_TILE == 0) {
        DevQuery probe = dq;
        const uint64_t tiles = (uint64_t)dq.n_rg * (t->rg_rows / PIPE_TILE);
        DeviceCtx *dev;
        if (tiles > 0 && tiles < (1ULL << 32) && pipe_plan(probe, tiles, &q->pp) && device_ctx(&dev) == TGPU_OK) {
            dq.cache_slots = probe.cache_slots;
            dq.cache_probe = probe.cache_probe;
            if (q->route == 1 && !(dq.cache_slots && dq.cache_probe == dq.cache_slots)) q->route = 2;
            q->pipe_grid = (int)std::min<uint64_t>((uint64_t)dev->sms, std::max<uint64_t>(1, tiles / PIPE_CWARPS));
            q->piped = true;
        }
    }
    return TGPU_OK;
}

// GROUP BY ... ORDER BY COUNT(*) DESC LIMIT k (k + OFFSET <= 1024, no
// HAVING, no COUNT(DISTINCT)): the count sketch runs first, as thinDB routes
// such a query to its two-pass top-K (v2_group_topn_engine.zig:1375,
// count_topk_sketch.zig MAX_NEED :64), unless the input is small.
// The radix-partitioned route, on request: a compiled fold over a key of at
// most 64 packed bits.
bool radix_eligible(const tgpu_query *q) {
    const DevQuery &dq = q->dq;
    if (q->batched || (q->flags & TGPU_FLAG_NO_RADIX) || q->staged || q->piped || q->global_agg) return false;
    if (dq.fast_id < 0 || dq.key_words != 1 || q->t->rg_rows % RX_TILE != 0) return false;
    return (q->flags & TGPU_FLAG_RADIX) != 0;
}

bool sketch_eligible(const tgpu_query *q, const tgpu_request *req) {
    if ((q->flags & TGPU_FLAG_NO_COUNT_SKETCH) || q->global_agg || req->n_order != 1 || req->n_having) return false;
    const tgpu_sort_spec &o = req->order[0];
    if (o.target != TGPU_SORT_AGG || !o.desc || q->limit == TGPU_NO_LIMIT || q->limit == 0 ||
        q->offset + q->limit > SK_MAX_NEED)
        return false;
    if (req->aggs[o.index].func != TGPU_AGG_COUNT || q->dq.aggs[o.index].kind != AK_COUNT_ROWS) return false;
    if (q->dq.needs_gid || q->dq.n_dsets || q->dq.hashed) return false;
    return q->rows_scanned >= SK_MIN_ROWS || (q->flags & TGPU_FLAG_COUNT_SKETCH);
}

tgpu_status enqueue(tgpu_query *q) {
    DevQuery &dq = q->dq;
    DevFinal &df = q->df;
    cudaStream_t s = q->stream;
    q->launches = 0;
    // epochs for the distinct sets
    uint32_t epoch = 0;
    for (auto &b : q->dset_bufs) epoch = std::max(epoch, b.epoch);
    ++epoch;
    if (epoch == 0xFFFFFFFFu) {
        for (auto &b : q->dset_bufs) {
            CU(cudaMemsetAsync(b.p, 0, b.bytes, s));
            b.epoch = 0;
        }
        epoch = 1;
    }
    for (auto &b : q->dset_bufs) b.epoch = epoch;
    dq.epoch = epoch;
    q->table_buf.dirty = true;  // until the clear kernel has run
    q->occ_buf.dirty = true;

    dq.wait_cycles = device_wait_limit();
    CU(cudaMemsetAsync(q->d_ctrl, 0, 16, s));
    CU(cudaMemsetAsync(q->d_counts, 0, 8 * 8, s));
    const bool timing = (q->flags & TGPU_FLAG_TIMING) != 0;
    if (timing && !q->ev[0])
        for (auto &e : q->ev) CU(cudaEventCreate(&e));
    if (timing) CU(cudaEventRecord(q->ev[0], s));
    if (dq.dpart_bits) CU(cudaMemsetAsync(dq.dpart_cursor, 0, (size_t)4 << dq.dpart_bits, s));
    uint32_t *sk_counts = q->d_sketch, *sk_keep = sk_counts ? sk_counts + (1u << SK_BITS) : nullptr;
    uint32_t *sk_ctl = sk_keep ? sk_keep + (1u << SK_BITS) / 32 : nullptr;
    if (q->sketch && !q->sketch_off) {
        DeviceCtx *dev;
        tgpu_status dst = device_ctx(&dev);
        if (dst != TGPU_OK) return dst;
        CU(launch_count_sketch(dq, (uint32_t)(q->offset + q->limit), sk_counts, sk_keep, sk_ctl, dev->sms, s));
        q->launches += 2;
        dq.sk_keep = sk_keep;
        dq.sk_on = sk_ctl;
    } else {
        dq.sk_keep = nullptr;
        dq.sk_on = nullptr;
    }
    if (q->radix) {
        DeviceCtx *dev;
        tgpu_status dst = device_ctx(&dev);
        if (dst != TGPU_OK) return dst;
        CU(launch_radix(dq, q->rp, dev->sms, s));
        q->launches += 2;
    } else if (q->staged) {
        CU(launch_staged_scan(dq, q->sp, q->stage_grid, s));
        q->launches++;
    } else if (q->piped) {
        CU(launch_pipe_scan(dq, q->pp, q->pipe_grid, s));
        q->launches++;
    } else if (q->split && (dq.gather == 1 || (q->sketch && !q->sketch_off)) && dq.n_chunks > 0) {
        DeviceCtx *dev;
        tgpu_status dst = device_ctx(&dev);
        if (dst != TGPU_OK) return dst;
        unsigned long long *n_sel = (unsigned long long *)q->split_buf.p;
        CU(launch_split_scan(dq, (uint32_t *)((char *)q->split_buf.p + 256), n_sel, dev->sms, s));
        q->launches += 2;
    } else if (dq.n_chunks > 0) {
        CU(launch_scan(dq, q->grid, s));
        q->launches++;
    }
    if (dq.dpart_bits) {
        CU(launch_distinct_partitions(dq, q->dpart_word, s));
        q->launches++;
    }
    if (timing) CU(cudaEventRecord(q->ev[1], s));
    if (q->rank != RANK_TOPK) {
        CU(launch_compact(df, q->d_block_counts, q->n_cpt_blocks, q->d_gids, q->d_counts, s));
        q->launches += 2;
    }
    const uint32_t *sel = q->d_gids;
    uint64_t gather_offset = 0, gather_rows = q->out_rows_max;
    if (q->rank == RANK_NONE) {
        CU(launch_sel_all(q->d_counts, s));
        q->launches++;
    } else if (q->rank == RANK_TOPK) {
        CU(launch_topk_scan(df, q->d_counts, q->k, q->d_cand_keys, q->d_cand_gids, q->n_cand_blocks, q->d_sel,
                            q->d_ctrl + 2, s));
        q->launches += 1;
        sel = q->d_sel;
        gather_offset = q->offset;
        gather_rows = q->limit;
    } else {
        uint32_t *sorted = nullptr;
        CU(launch_sort(df, q->d_gids, q->d_counts, dq.cap + 1, q->d_sort_keys[0], q->d_sort_keys[1], q->d_sort_ids[0],
                       q->d_sort_ids[1], &sorted, s));
        uint64_t passes = 0;
        for (uint64_t w = 1024; w < dq.cap + 1; w <<= 1) ++passes;
        q->launches += 3 + (uint32_t)passes;
        sel = sorted;
        gather_offset = q->offset;
        gather_rows = q->out_rows_max;
    }
    CU(launch_gather(df, sel, q->d_counts, gather_offset, gather_rows, q->d_out_ptrs, q->d_valid_ptrs, s));
    CU(launch_clear(dq.table, dq.cap, dq.slot_words, dq.occ, s));
    q->launches += 2;
    if (timing) CU(cudaEventRecord(q->ev[2], s));
    CU(cudaMemcpyAsync(q->h_counts, q->d_counts, 5 * 8, cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(q->h_counts + 5, q->d_ctrl + 1, 4, cudaMemcpyDeviceToHost, s));
    if (q->sketch && !q->sketch_off) {
        // [6] on | threshold << 32, [7] the COUNT of the page's last row,
        // [8] kept rows, [9] rows tallied (the exactness check in finish)
        CU(cudaMemcpyAsync(q->h_counts + 6, sk_ctl, 8, cudaMemcpyDeviceToHost, s));
        const size_t col = q->df.n_parts + (size_t)q->sketch_order_agg;
        CU(cudaMemcpyAsync(q->h_counts + 7, (const char *)q->d_out[col] + (q->limit - 1) * 8, 8,
                           cudaMemcpyDeviceToHost, s));
        CU(cudaMemcpyAsync(q->h_counts + 8, sk_ctl + 2, 16, cudaMemcpyDeviceToHost, s));
    }
    q->executed = true;
    q->synced = false;
    q->returned = 0;
    q->h_packed = nullptr;
    return TGPU_OK;
}

// A global aggregate whose WHERE kept no row still answers one row (COUNTs 0,
// the rest NULL), unless OFFSET or LIMIT 0 drops it.
void set_empty_global_row(tgpu_query *q, uint64_t groups) {
    q->synth_empty = q->global_agg && groups == 0 && q->offset == 0 && q->limit != 0;
    if (q->synth_empty) q->result_rows = 1;
}

tgpu_status finish(tgpu_query *q) {
    for (;;) {
        CU(cudaStreamSynchronize(q->stream));
        q->table_buf.dirty = false;
        q->occ_buf.dirty = false;
        const uint32_t status = (uint32_t)(q->h_counts[5] & 0xFFFFFFFFu);
        if (status & ST_CANCELLED) {
            q->synced = true;
            q->result_rows = 0;
            return fail(TGPU_ERR_CANCELLED, "query cancelled");
        }
        if (status & ST_WAIT_TIMEOUT) {
            // a bounded device wait on a bulk copy gave up; the kernel drained
            // its copies and returned, so the context and the query stay usable
            q->synced = true;
            q->result_rows = 0;
            return fail(TGPU_ERR_DEVICE_TIMEOUT, "a bulk column or pair copy did not complete within the "
                                                 "device wait limit");
        }
        if (status & ST_BAD_INDEX) {
            q->synced = true;
            q->result_rows = 0;
            return fail(TGPU_ERR_INTERNAL, "a device bounds check failed");
        }
        if (status & ST_PART_FULL) {
            // a radix partition held more rows than its buffer: the cursors
            // counted every row, so size the buffers for the largest
            if (++q->retries > 4) return fail(TGPU_ERR_INTERNAL, "radix partitions kept overflowing");
            std::vector<uint32_t> cur((size_t)1 << q->rp.bits);
            CU(cudaMemcpy(cur.data(), q->rp.cursor, cur.size() * 4, cudaMemcpyDeviceToHost));
            q->radix_cap_req = (uint64_t)*std::max_element(cur.begin(), cur.end()) + RX_TILE;
            tgpu_status st = size_workspace(q, q->dq.cap);
            if (st != TGPU_OK) return st;
            st = enqueue(q);
            if (st != TGPU_OK) return st;
            continue;
        }
        if (status & (ST_TABLE_FULL | ST_DISTINCT_FULL)) {
            if (++q->retries > 4) return fail(TGPU_ERR_INTERNAL, "group table kept overflowing");
            if (status & ST_TABLE_FULL) q->groups_est = std::max<uint64_t>(q->groups_est * 4, 1024);
            if (status & ST_DISTINCT_FULL) {
                if (q->dq.dpart_bits) {
                    // Partitions hold three quarters of their capacity on
                    // average, so with a uniform hash only more passing rows
                    // than planned overflow one: size for the rows that
                    // passed.  Otherwise one (group, value) pair repeated
                    // beyond a partition's capacity filled it (all its
                    // copies hash alike): deduplicate in the global set.
                    const uint64_t selected = q->h_counts[4];
                    const uint64_t room = ((uint64_t)DPART_CAP * 3 / 4) << q->dq.dpart_bits;
                    const uint64_t most = ((uint64_t)DPART_CAP * 3 / 4) << DPART_MAX_BITS;
                    if (selected > room && selected <= most) q->dpart_rows = selected;
                    else q->dpart_off = true;
                } else {
                    for (auto &n : q->dset_need) n *= 4;
                }
            }
            tgpu_status st = size_workspace(q, next_pow2(q->groups_est * 100 / q->load_pct));
            if (st != TGPU_OK) return st;
            st = enqueue(q);
            if (st != TGPU_OK) return st;
            continue;
        }
        if (q->sketch && !q->sketch_off && (q->h_counts[6] & 0xFFFFFFFFu)) {
            // CountSketch.exact (count_topk_sketch.zig:236-239): the kept
            // groups' top `need` is the answer once no dropped group (fewer
            // than `threshold` rows) can reach the need-th best.  thinDB
            // accepts a need-th best of threshold - 1 rows, leaving a tie at
            // the cut unordered; ties here break on the packed key, so a
            // dropped group may not even tie: the need-th best must hold
            // `threshold` rows.  Otherwise group every row.
            const uint64_t need = q->offset + q->limit, found = q->h_counts[0];
            const uint64_t thr = q->h_counts[6] >> 32, kth = q->h_counts[7];
            const bool all_kept = q->h_counts[8] == q->h_counts[9];
            if (!all_kept && !(found >= need && kth >= thr)) {
                q->sketch_off = true;
                q->sketch_reruns++;
                tgpu_status st = enqueue(q);
                if (st != TGPU_OK) return st;
                continue;
            }
        }
        break;
    }
    q->synced = true;
    q->result_rows = q->h_counts[2];
    set_empty_global_row(q, q->h_counts[0]);
    tgpu_query_stats &s = q->stats;
    s.rows_scanned = q->rows_scanned;
    s.rows_selected = q->h_counts[4];
    s.groups = q->h_counts[0];
    s.result_rows = q->h_counts[2];
    s.table_capacity = q->dq.cap;
    s.distinct_capacity = q->dq.dpart_bits ? ((uint64_t)q->dq.dpart_cap << q->dq.dpart_bits)
                                           : (q->dq.n_dsets ? q->dq.dset_cap[0] : 0);
    s.row_groups_total = q->rg_total;
    s.row_groups_pruned = q->rg_pruned;
    s.route = (uint32_t)q->route;
    s.retries = q->retries;
    s.kernel_launches = q->launches;
    s.flags = (q->tuned ? TGPU_STAT_TUNED : 0) |
              (q->dq.gather == 1 && !q->staged && !q->piped ? TGPU_STAT_GATHER : 0) |
              (q->dq.gather == 2 && !q->staged && !q->piped ? TGPU_STAT_QUEUE : 0) |
              (q->staged ? TGPU_STAT_STAGED : 0) | (q->piped ? TGPU_STAT_PIPE : 0) |
              (q->split && (q->dq.gather == 1 || (q->sketch && !q->sketch_off)) ? TGPU_STAT_SPLIT : 0) |
              (q->sketch && !q->sketch_off && (q->h_counts[6] & 0xFFFFFFFFu) ? TGPU_STAT_COUNT_SKETCH : 0) |
              (q->sketch_reruns ? TGPU_STAT_SKETCH_RERUN : 0) | (q->radix ? TGPU_STAT_RADIX : 0) |
              (q->dq.dpart_bits ? TGPU_STAT_DISTINCT_PARTITION : 0);
    s.device_bytes = q->table_buf.bytes + q->occ_buf.bytes + q->scratch_bytes;
    for (auto &b : q->dset_bufs) s.device_bytes += b.bytes;
    if (q->flags & TGPU_FLAG_TIMING) {
        float a = 0, b = 0, c = 0;
        CU(cudaEventElapsedTime(&a, q->ev[0], q->ev[1]));
        CU(cudaEventElapsedTime(&b, q->ev[1], q->ev[2]));
        CU(cudaEventElapsedTime(&c, q->ev[0], q->ev[2]));
        s.scan_ms = a;
        s.finalize_ms = b;
        s.total_ms = c;
    }
    return TGPU_OK;
}

// ---------------------------------------------------------------- tuning --

std::mutex g_tuning_mu;
std::vector<tgpu_tuning> g_tuning;

// The shape class of a planned query (the key of the tuning table).
tgpu_shape shape_of(const tgpu_query *q, const tgpu_request *req, int batched) {
    tgpu_shape s{};
    s.key_words = q->dq.key_words;
    s.fold = fast_fold_id(q->dq);
    s.n_aggs = (int32_t)req->n_aggs;
    s.distinct = q->dq.n_dsets > 0;
    s.filtered = req->n_where > 0;
    s.sel_log2 = 0;
    if (req->n_where > 0 && q->rows_scanned > 0) {
        const double f = (double)std::max<uint64_t>(1, q->sel_est) / (double)q->rows_scanned;
        s.sel_log2 = std::max(-30, std::min(0, (int)std::floor(std::log2(f))));
    }
    s.groups_log2 = (int32_t)std::ceil(std::log2((double)std::max<uint64_t>(1, q->groups_est)));
    s.batched = batched ? 1 : 0;
    return s;
}

// Take the tuned settings of the query's shape unless the request chose its own.
void apply_tuning(tgpu_query *q, const tgpu_request *req, int batched) {
    const int modes = TGPU_FLAG_DENSE_SCAN | TGPU_FLAG_GATHER_SCAN | TGPU_FLAG_NO_WARP_COMBINE |
                      TGPU_FLAG_STAGED_SCAN | TGPU_FLAG_NO_STAGED | TGPU_FLAG_NO_PREFETCH |
                      TGPU_FLAG_NO_CHUNK_PREFETCH | TGPU_FLAG_DISTINCT_PREFETCH | TGPU_FLAG_DISTINCT_PARTITION |
                      TGPU_FLAG_NO_DISTINCT_PARTITION | TGPU_FLAG_QUEUE_SCAN | TGPU_FLAG_PIPE_SCAN |
                      TGPU_FLAG_NO_PIPE | TGPU_FLAG_COUNT_SKETCH | TGPU_FLAG_NO_COUNT_SKETCH |
                      TGPU_FLAG_RADIX | TGPU_FLAG_NO_RADIX | TGPU_FLAG_INLINE_FOLD;
    const int own = modes | TGPU_FLAG_NO_TUNING;
    if (req->chunk_rows || req->cache_slots || req->table_load_pct || (req->flags & own)) return;
    const tgpu_shape s = shape_of(q, req, batched);
    std::lock_guard<std::mutex> lk(g_tuning_mu);
    for (const tgpu_tuning &t : g_tuning) {
        if (std::memcmp(&t.shape, &s, sizeof(s)) != 0) continue;
        q->chunk_req = (uint32_t)t.chunk_rows;
        q->cache_req = t.cache_slots;
        q->load_pct = t.table_load_pct ? t.table_load_pct : 50;
        q->flags |= t.flags & modes;
        if (t.groups_shift > 0 && !req->expected_groups)
            q->groups_est = std::max<uint64_t>(64, q->groups_est >> t.groups_shift);
        q->tuned = true;
        return;
    }
}

}  // namespace

tgpu_status query_create(tgpu_table *table, const tgpu_request *req, int batched, tgpu_query **out);

struct StatsLayout {
    size_t nrg, stat_bytes, reg_bytes;
};
StatsLayout stats_layout(uint32_t n_rg);
// Statistics a caller has computed in the stats_layout of every column
// (device), with which columns carry a sketch.
struct PreStats {
    const unsigned char *d_stats;
    const std::vector<bool> *sketch;
};
tgpu_status register_table(const tgpu_table_desc *desc, tgpu_table **out, const PreStats *pre);

// ================================================================ C ABI ====

extern "C" {

uint32_t tgpu_abi_version(void) { return TGPU_ABI_VERSION; }

tgpu_status tgpu_debug_set_wait_limit(uint64_t sm_cycles) {
    if (sm_cycles > (uint64_t)1 << 40) return fail(TGPU_ERR_INVALID_ARGUMENT, "wait limit above 2^40 SM clocks");
    g_wait_limit.store((long long)sm_cycles, std::memory_order_relaxed);
    return TGPU_OK;
}

tgpu_status tgpu_debug_set_digest_bits(uint32_t bits) {
    if (bits > 63) return fail(TGPU_ERR_INVALID_ARGUMENT, "digest bits above 63 (0 keeps all 64)");
    g_digest_bits.store(bits, std::memory_order_relaxed);
    return TGPU_OK;
}

const char *tgpu_build_info(void) {
    static char buf[128];
    std::snprintf(buf, sizeof(buf), "thindb_gpu sm_103a cuda %d.%d", CUDART_VERSION / 1000, (CUDART_VERSION % 1000) / 10);
    return buf;
}

const char *tgpu_last_error_message(void) { return g_err.c_str(); }

tgpu_status tgpu_table_register(const tgpu_table_desc *desc, tgpu_table **out) {
    return register_table(desc, out, nullptr);
}

tgpu_status tgpu_aggregate_register(const char *name) {
    const std::string k = udf_key(name);
    if (k.empty()) return fail(TGPU_ERR_INVALID_ARGUMENT, "aggregate name");
    if (udf_reserved(k)) return fail(TGPU_ERR_INVALID_ARGUMENT, "a built-in aggregate's name");
    std::lock_guard<std::mutex> lk(g_udf_mu);
    if (!g_udfs.insert(k).second) return fail(TGPU_ERR_INVALID_ARGUMENT, "aggregate already registered");
    return TGPU_OK;
}

tgpu_status tgpu_aggregate_unregister(const char *name) {
    const std::string k = udf_key(name);
    std::lock_guard<std::mutex> lk(g_udf_mu);
    if (k.empty() || !g_udfs.erase(k)) return fail(TGPU_ERR_INVALID_ARGUMENT, "aggregate not registered");
    return TGPU_OK;
}

int32_t tgpu_aggregate_registered(const char *name) {
    const std::string k = udf_key(name);
    std::lock_guard<std::mutex> lk(g_udf_mu);
    return !k.empty() && g_udfs.count(k) ? 1 : 0;
}

}  // extern "C"

// Per-column statistics slices: zone maps of every row group (min/max as i64
// and f64, NULL counts), rounded to 256 bytes so every column's slice and the
// 8-byte arrays inside it stay aligned whatever the row-group count, then an
// HLL register file.
StatsLayout stats_layout(uint32_t n_rg) {
    StatsLayout l;
    l.nrg = std::max<uint32_t>(1, n_rg);
    l.stat_bytes = round_up(l.nrg * (8 * 4 + 4), 256);
    l.reg_bytes = (size_t)(1u << HLL_P) * 4;
    return l;
}

tgpu_status register_table(const tgpu_table_desc *desc, tgpu_table **out, const PreStats *pre) {
    if (!desc || !out) return fail(TGPU_ERR_INVALID_ARGUMENT, "null argument");
    if (desc->n_columns == 0 || !desc->columns) return fail(TGPU_ERR_INVALID_ARGUMENT, "no columns");
    DeviceCtx *dev;
    tgpu_status st = device_ctx(&dev);
    if (st != TGPU_OK) return st;
    cudaStream_t s = desc->stream ? (cudaStream_t)desc->stream : dev->stream;
    std::unique_ptr<tgpu_table> t(new tgpu_table());
    t->n_rows = desc->n_rows;
    t->rg_rows = desc->row_group_rows ? desc->row_group_rows : 65536u;
    t->sketches = desc->compute_ndv != 0;
    t->n_rg = (uint32_t)((t->n_rows + t->rg_rows - 1) / t->rg_rows);
    t->stream = dev->stream;  // frees go on the library's stream (the caller's may be gone by then)
    const uint64_t n = t->n_rows;
    const uint64_t vwords = (n + 31) / 32 + 1;
    const uint32_t nc = desc->n_columns;
    for (uint32_t i = 0; i < nc; ++i) {
        const tgpu_column_desc &cd = desc->columns[i];
        if (cd.type < TGPU_BOOLEAN || cd.type > TGPU_VARCHAR || cd.type == TGPU_DECIMAL128)
            return fail(TGPU_ERR_UNSUPPORTED_TYPE, "column type");
        if (!cd.data && (n || cd.type == TGPU_VARCHAR)) return fail(TGPU_ERR_INVALID_ARGUMENT, "column without data");
        if (cd.type == TGPU_VARCHAR && !cd.dict_bytes) return fail(TGPU_ERR_INVALID_ARGUMENT, "string column without bytes");
        if (cd.type == TGPU_DICT32 && cd.dict_size && (!cd.dict_offsets || !cd.dict_bytes))
            return fail(TGPU_ERR_INVALID_ARGUMENT, "dictionary without offsets or bytes");
    }
    // Statistics scratch, one slice per column (stats_layout), then one HLL
    // scratch shared by the columns, whose statistics run in turn on one
    // stream; none when the caller computed them (pre).
    const StatsLayout lay = stats_layout(t->n_rg);
    const size_t nrg = lay.nrg, stat_bytes = lay.stat_bytes, reg_bytes = lay.reg_bytes;
    unsigned char *d_stats = nullptr;
    uint8_t *d_part = nullptr;
    if (!pre) {
        const size_t part_bytes = (size_t)STATS_GRID_MAX << HLL_P;
        CU(cudaMallocFromPoolAsync((void **)&d_stats, std::max<size_t>(1, nc) * (stat_bytes + reg_bytes) + part_bytes,
                                   dev->col_pool, s));
        d_part = d_stats + std::max<size_t>(1, nc) * (stat_bytes + reg_bytes);
    }
    struct StatsGuard {  // an error return leaves nothing allocated behind
        unsigned char *&p;
        cudaStream_t a, b;
        ~StatsGuard() {
            if (!p) return;
            cudaStreamSynchronize(b);
            cudaFreeAsync(p, a);
        }
    } stats_guard{d_stats, s, dev->stats_stream};
    std::vector<unsigned char> h_stats(std::max<size_t>(1, nc) * (stat_bytes + reg_bytes));
    // Column copies go back to back on s; each column's statistics run on the
    // statistics stream once its copy has landed, beside the next copy.
    std::vector<cudaEvent_t> landed(nc, nullptr);
    struct EvGuard {
        std::vector<cudaEvent_t> &v;
        ~EvGuard() {
            for (auto e : v)
                if (e) cudaEventDestroy(e);
        }
    } guard{landed};
    cudaStream_t ss = dev->stats_stream;
    std::vector<bool> sketch(nc, false);
    for (uint32_t i = 0; i < nc; ++i) {
        const tgpu_column_desc &cd = desc->columns[i];
        t->cols.emplace_back();
        Column &c = t->cols.back();
        c.name = cd.name ? cd.name : "";
        c.type = cd.type;
        c.precision = cd.decimal_precision;
        c.scale = cd.decimal_scale;
        c.nullable = cd.validity != nullptr;
        const size_t bytes = n * type_bytes(cd.type);
        if (cd.type == TGPU_VARCHAR) {
            // offsets and bytes: host copies (late materialisation) and device copies
            c.str_offs.resize(n + 1);
            const bool dev_src = desc->location == TGPU_LOC_DEVICE;
            CU(cudaMemcpyAsync(c.str_offs.data(), cd.data, (n + 1) * 4,
                               dev_src ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost, s));
            CU(cudaStreamSynchronize(s));
            for (uint64_t r = 0; r < n; ++r)
                if (c.str_offs[r + 1] < c.str_offs[r]) return fail(TGPU_ERR_INVALID_ARGUMENT, "string offsets decrease");
            const size_t nb = c.str_offs[n];
            c.str_bytes.resize(std::max<size_t>(nb, 1));
            if (nb) CU(cudaMemcpyAsync(c.str_bytes.data(), cd.dict_bytes, nb,
                                       dev_src ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost, s));
            CU(cudaMallocFromPoolAsync((void **)&c.d_offs, (n + 1) * 4, dev->col_pool, s));
            CU(cudaMemcpyAsync(c.d_offs, c.str_offs.data(), (n + 1) * 4, cudaMemcpyHostToDevice, s));
            CU(cudaMallocFromPoolAsync(&c.d_data, round_up(std::max<size_t>(nb, 16), 16), dev->col_pool, s));
            c.owned = true;
            CU(cudaStreamSynchronize(s));
            if (nb) CU(cudaMemcpyAsync(c.d_data, c.str_bytes.data(), nb, cudaMemcpyHostToDevice, s));
        } else if (desc->location == TGPU_LOC_DEVICE) {
            c.d_data = const_cast<void *>(cd.data);
            c.owned = false;
        } else {
            // a 16-byte multiple past the data: bulk copies of a last partial tile stay inside
            CU(cudaMallocFromPoolAsync(&c.d_data, round_up(std::max<size_t>(bytes, 16), 16), dev->col_pool, s));
            c.owned = true;
            if (bytes) CU(cudaMemcpyAsync(c.d_data, cd.data, bytes, cudaMemcpyHostToDevice, s));
        }
        if (cd.validity) {
            CU(cudaMallocFromPoolAsync((void **)&c.d_valid, vwords * 4, dev->col_pool, s));
            CU(cudaMemsetAsync(c.d_valid, 0, vwords * 4, s));
            CU(cudaMemcpyAsync(c.d_valid, cd.validity, (n + 7) / 8,
                               desc->location == TGPU_LOC_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
        }
        if (cd.type == TGPU_DICT32 && cd.dict_offsets && cd.dict_size) {
            c.dict_offsets.assign(cd.dict_offsets, cd.dict_offsets + cd.dict_size + 1);
            for (uint32_t j = 0; j < cd.dict_size; ++j)
                if (c.dict_offsets[j + 1] < c.dict_offsets[j])
                    return fail(TGPU_ERR_INVALID_ARGUMENT, "dictionary offsets decrease");
            c.dict_bytes.assign(cd.dict_bytes, cd.dict_bytes + cd.dict_offsets[cd.dict_size]);
            // each code's rank among the strings in bytewise order: ORDER BY a
            // string key ranks on it (its packed code only stands for the string)
            std::vector<uint32_t> ix(cd.dict_size);
            for (uint32_t j = 0; j < cd.dict_size; ++j) ix[j] = j;
            std::sort(ix.begin(), ix.end(), [&](uint32_t a, uint32_t b) { return dict_cmp(c, a, b) < 0; });
            c.h_rank.resize(cd.dict_size);
            for (uint32_t j = 0; j < cd.dict_size; ++j) {
                c.h_rank[ix[j]] = j;
                if (j && dict_cmp(c, ix[j - 1], ix[j]) == 0) c.dict_unique = false;
            }
            CU(cudaMallocFromPoolAsync((void **)&c.d_rank, (size_t)cd.dict_size * 4, dev->col_pool, s));
            CU(cudaMemcpyAsync(c.d_rank, c.h_rank.data(), (size_t)cd.dict_size * 4, cudaMemcpyHostToDevice, s));
        }
        CU(cudaEventCreateWithFlags(&landed[i], cudaEventDisableTiming));
        CU(cudaEventRecord(landed[i], s));
        CU(cudaStreamWaitEvent(ss, landed[i], 0));
        c.ndv = cd.ndv_hint;
        sketch[i] = !c.ndv && desc->compute_ndv && n;
        if (pre) {
            sketch[i] = (*pre->sketch)[i];
            continue;
        }
        unsigned char *st = d_stats + (size_t)i * (stat_bytes + reg_bytes);
        int64_t *imin = (int64_t *)st, *imax = imin + nrg;
        double *fmin = (double *)(imax + nrg), *fmax = fmin + nrg;
        uint32_t *nulls = (uint32_t *)(fmax + nrg);
        uint32_t *regs = (uint32_t *)(st + stat_bytes);
        if (c.type != TGPU_VARCHAR) {
            // zone maps and the sketch in one pass over the column
            CU(launch_column_stats(c.d_data, c.d_valid, c.type, n, t->rg_rows, 0, t->n_rg, imin, imax, fmin, fmax,
                                   nulls, sketch[i] ? regs : nullptr, d_part, 0, ss));
        } else if (sketch[i]) {  // strings: no zone maps (no WHERE on them here)
            CU(cudaMemsetAsync(regs, 0, reg_bytes, ss));
            CU(launch_hll(c.d_data, c.d_valid, c.type, n, regs, ss, c.d_offs));
        }
    }
    // one read-back of every column's statistics
    CU(cudaMemcpyAsync(h_stats.data(), pre ? pre->d_stats : d_stats, h_stats.size(), cudaMemcpyDeviceToHost, ss));
    CU(cudaStreamSynchronize(ss));
    if (d_stats) CU(cudaFreeAsync(d_stats, s));
    d_stats = nullptr;
    CU(cudaStreamSynchronize(s));
    for (uint32_t i = 0; i < nc; ++i) {
        Column &c = t->cols[i];
        const unsigned char *st = h_stats.data() + (size_t)i * (stat_bytes + reg_bytes);
        const int64_t *imin = (const int64_t *)st, *imax = imin + nrg;
        const double *fmin = (const double *)(imax + nrg), *fmax = fmin + nrg;
        const uint32_t *nulls = (const uint32_t *)(fmax + nrg);
        c.zmin.assign(imin, imin + t->n_rg);
        c.zmax.assign(imax, imax + t->n_rg);
        c.zfmin.assign(fmin, fmin + t->n_rg);
        c.zfmax.assign(fmax, fmax + t->n_rg);
        c.znull.assign(nulls, nulls + t->n_rg);
        if (sketch[i]) {
            const uint32_t *r = (const uint32_t *)(st + stat_bytes);
            c.ndv = (uint64_t)std::llround(hll_estimate(std::vector<uint32_t>(r, r + (1u << HLL_P))));
        }
        if (!c.ndv) {
            // without a sketch: bounded by the type's domain and the row count
            uint64_t dom = type_bits(c.type) && type_bits(c.type) < 40 ? (1ULL << type_bits(c.type)) : n;
            if (c.type == TGPU_DICT32 && c.dict_offsets.size() > 1) dom = c.dict_offsets.size() - 1;
            c.ndv = std::max<uint64_t>(1, std::min<uint64_t>(dom, n));
        }
    }
    *out = t.release();
    return TGPU_OK;
}

extern "C" {

tgpu_status tgpu_table_register_segment(const uint8_t *image, uint64_t bytes, const tgpu_segment_column *columns,
                                        uint32_t n_columns, int32_t compute_ndv, void *stream, tgpu_table **out) {
    if (!image || !columns || !n_columns || !out) return fail(TGPU_ERR_INVALID_ARGUMENT, "null argument");
    const auto t_call = std::chrono::steady_clock::now();
    auto u16 = [&](uint64_t o) { uint16_t v; std::memcpy(&v, image + o, 2); return v; };
    auto u32 = [&](uint64_t o) { uint32_t v; std::memcpy(&v, image + o, 4); return v; };
    auto u64 = [&](uint64_t o) { uint64_t v; std::memcpy(&v, image + o, 8); return v; };
    // header and trailer (format.zig:1-38)
    if (bytes < 32 + 8 || std::memcmp(image, "tDBS", 4) != 0 || std::memcmp(image + bytes - 4, "tDBS", 4) != 0)
        return fail(TGPU_ERR_INVALID_ARGUMENT, "not a segment image (magic)");
    const uint16_t version = u16(4);
    // segment_reader.zig:1388 reads the current version only
    if (version != 17) return fail(TGPU_ERR_UNSUPPORTED_TYPE, "segment version other than 17");
    const uint64_t n = u64(24);
    for (uint32_t c = 0; c < n_columns; ++c) {
        const int ty = columns[c].type;
        if (ty < TGPU_BOOLEAN || ty > TGPU_DOUBLE)
            return fail(TGPU_ERR_UNSUPPORTED_TYPE, "segment column type (string columns live in string tables)");
    }
    // the row groups' blocks
    std::vector<std::vector<SegBlock>> blocks(n_columns);
    std::vector<uint32_t> run_starts;
    std::vector<bool> nullable(n_columns, false);
    std::vector<uint64_t> rg_pos;  // each row group's header offset
    std::vector<uint32_t> rg_n;    // and its rows
    uint64_t pos = 32, done = 0;
    uint32_t rg_rows = 0;
    const uint64_t end = bytes - 8;
    while (done < n) {
        if (pos + 8 > end) return fail(TGPU_ERR_INVALID_ARGUMENT, "segment truncated in a row-group header");
        const uint32_t rows = u32(pos);
        rg_pos.push_back(pos);
        rg_n.push_back(rows);
        pos += 8;
        if (rows == 0 || done + rows > n) return fail(TGPU_ERR_INVALID_ARGUMENT, "row-group row count");
        if (!rg_rows) rg_rows = rows;
        for (uint32_t c = 0; c < n_columns; ++c) {
            if (pos + 12 > end) return fail(TGPU_ERR_INVALID_ARGUMENT, "segment truncated in a block header");
            const uint8_t comp = image[pos], flags = image[pos + 1], enc = image[pos + 2];
            const uint32_t usize = u32(pos + 4), ssize = u32(pos + 8);
            const uint64_t payload = pos + 12;
            if (comp != 0) return fail(TGPU_ERR_UNSUPPORTED_TYPE, "compressed column block (zstd/lz4)");
            if (flags & 2) return fail(TGPU_ERR_UNSUPPORTED_TYPE, "column block with integer-stream transforms");
            if (ssize != usize || payload + ssize > end) return fail(TGPU_ERR_INVALID_ARGUMENT, "column block size");
            const bool has_nulls = flags & 1;
            const uint32_t bm = has_nulls ? (rows + 7) / 8 : 0;
            const int ty = columns[c].type;
            const uint32_t elem = (uint32_t)type_bytes(ty);
            const bool integer = !is_float_t(ty);
            SegBlock b{};
            b.row0 = done;
            b.payload = payload;
            b.values = bm;
            b.rows = rows;
            b.encoding = enc;
            b.has_nulls = has_nulls;
            b.width = elem;
            b.elem = elem;
            if (enc == 0) {
                if ((uint64_t)bm + (uint64_t)rows * elem > usize) return fail(TGPU_ERR_INVALID_ARGUMENT, "raw block size");
            } else if (enc == 1) {
                if (!integer || (uint64_t)bm + 20 > usize) return fail(TGPU_ERR_INVALID_ARGUMENT, "FOR block");
                b.width = image[payload + bm + 16];
                if ((b.width != 1 && b.width != 2 && b.width != 4 && b.width != 8) ||
                    (uint64_t)bm + 20 + (uint64_t)rows * b.width > usize)
                    return fail(TGPU_ERR_INVALID_ARGUMENT, "FOR block width");
            } else if (enc == 3) {
                if (!integer || (uint64_t)bm + 8 > usize) return fail(TGPU_ERR_INVALID_ARGUMENT, "RLE block");
                b.runs = u32(payload + bm);
                b.width = image[payload + bm + 4];
                if ((b.width != 1 && b.width != 2 && b.width != 4 && b.width != 8) || b.width > elem ||
                    (uint64_t)bm + 8 + (uint64_t)b.runs * (b.width + 4) > usize || (b.runs == 0) != (rows == 0))
                    return fail(TGPU_ERR_INVALID_ARGUMENT, "RLE block size");
                b.run0 = (uint32_t)run_starts.size();
                const uint64_t lens = payload + bm + 8 + (uint64_t)b.runs * b.width;
                uint64_t at = 0;
                for (uint32_t r = 0; r < b.runs; ++r) {
                    run_starts.push_back((uint32_t)at);
                    at += u32(lens + 4ull * r);
                }
                if (at != rows) return fail(TGPU_ERR_INVALID_ARGUMENT, "RLE run lengths do not add up to the rows");
            } else {
                return fail(TGPU_ERR_UNSUPPORTED_TYPE, "column block encoding (dictionary / FSST)");
            }
            nullable[c] = nullable[c] || has_nulls;
            blocks[c].push_back(b);
            pos = payload + ssize;
        }
        done += rows;
    }
    DeviceCtx *dev;
    tgpu_status st = device_ctx(&dev);
    if (st != TGPU_OK) return st;
    cudaStream_t s = stream ? (cudaStream_t)stream : dev->stream;
    cudaStream_t cs = dev->stats_stream;  // the image copies (the registration's statistics stream is idle here)
    // The table's row groups are the segment's when every row group but the
    // last has the first one's rows: the image then goes to the device in
    // chunks of row groups, and each chunk is decoded and its statistics
    // taken while the next one is copied.  Otherwise one chunk, and the
    // statistics over the table's own row groups once it is decoded.
    const uint32_t n_seg_rg = (uint32_t)rg_pos.size();
    const uint32_t table_rg = rg_rows ? rg_rows : 65536u;
    const uint32_t n_rg = (uint32_t)((n + table_rg - 1) / table_rg);
    bool uniform = true;
    for (uint32_t g = 0; g < n_seg_rg; ++g) uniform = uniform && (g + 1 == n_seg_rg ? rg_n[g] <= table_rg : rg_n[g] == table_rg);
    const uint32_t per_chunk = uniform ? std::max<uint32_t>(1, (n_seg_rg + SEG_CHUNKS - 1) / SEG_CHUNKS)
                                       : std::max<uint32_t>(1, n_seg_rg);
    const uint32_t n_chunks = n_seg_rg ? (n_seg_rg + per_chunk - 1) / per_chunk : 0;
    uint8_t *d_image = nullptr;
    SegBlock *d_blocks = nullptr;
    uint32_t *d_runs = nullptr;
    unsigned char *d_stats = nullptr;
    std::vector<void *> data(n_columns, nullptr);
    std::vector<uint32_t *> valid(n_columns, nullptr);
    std::vector<cudaEvent_t> ev;
    auto release = [&](bool keep_data) {
        cudaStreamSynchronize(cs);
        cudaStreamSynchronize(s);
        if (d_image) cudaFreeAsync(d_image, s);
        if (d_blocks) cudaFreeAsync(d_blocks, s);
        if (d_runs) cudaFreeAsync(d_runs, s);
        if (d_stats) cudaFreeAsync(d_stats, s);
        for (uint32_t c = 0; c < n_columns; ++c) {
            if (valid[c]) cudaFreeAsync(valid[c], s);
            if (!keep_data && data[c]) cudaFreeAsync(data[c], s);
        }
        cudaStreamSynchronize(s);
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
    };
    cudaError_t e = cudaSuccess;
    auto event = [&]() {
        cudaEvent_t x = nullptr;
        if (e == cudaSuccess) e = cudaEventCreate(&x);
        if (e == cudaSuccess) ev.push_back(x);
        return x;
    };
    // columns and validity words (the blocks point into them)
    uint64_t decoded = 0;
    for (uint32_t c = 0; c < n_columns && e == cudaSuccess; ++c) {
        const size_t elem = (size_t)type_bytes(columns[c].type);
        e = cudaMallocFromPoolAsync(&data[c], round_up(std::max<size_t>(n * elem, 16), 16), dev->col_pool, s);
        decoded += n * elem;
        if (e == cudaSuccess && nullable[c]) {
            const size_t vw = ((n + 31) / 32 + 1) * 4;
            e = cudaMallocFromPoolAsync((void **)&valid[c], vw, dev->col_pool, s);
            if (e == cudaSuccess) e = cudaMemsetAsync(valid[c], 0, vw, s);
            decoded += (n + 7) / 8;
        }
    }
    // the block list, chunk by chunk, and in a chunk column by column; with
    // uniform row groups each block also takes its row group's zone map and
    // its rows' sketch registers (a scratch row per block of the chunk)
    const bool want_sketch = compute_ndv != 0 && n > 0;
    std::vector<SegBlock> all;
    std::vector<uint32_t> chunk_first(n_chunks + 1, 0);
    for (uint32_t k = 0; k < n_chunks; ++k) {
        chunk_first[k] = (uint32_t)all.size();
        const uint32_t g0 = k * per_chunk, g1 = std::min(n_seg_rg, g0 + per_chunk);
        for (uint32_t c = 0; c < n_columns; ++c)
            for (uint32_t g = g0; g < g1; ++g) {
                SegBlock b = blocks[c][g];
                b.out = data[c];
                b.valid = valid[c];
                b.col = c;
                b.rg = g;
                b.type = columns[c].type;
                b.flags = uniform ? SEG_ZONE | (want_sketch ? SEG_SKETCH : 0u) : 0u;
                b.part_row = c * per_chunk + (g - g0);
                all.push_back(b);
            }
    }
    chunk_first[n_chunks] = (uint32_t)all.size();
    // statistics slices as the registration lays them out, then the scratch:
    // a register row per block of a chunk, or the column-pass scratch
    const StatsLayout lay = stats_layout(n_rg);
    const size_t slice = lay.stat_bytes + lay.reg_bytes;
    std::vector<bool> sketch(n_columns, want_sketch);
    // (two register scratches: the chunks alternate between two streams)
    const size_t part_bytes = uniform ? ((size_t)n_columns * per_chunk << HLL_P) : ((size_t)STATS_GRID_MAX << HLL_P);
    if (e == cudaSuccess)
        e = cudaMallocFromPoolAsync((void **)&d_stats, n_columns * slice + 2 * part_bytes, dev->col_pool, s);
    uint8_t *d_part = d_stats ? d_stats + n_columns * slice : nullptr;
    const SegStats sst_pair[2] = {{d_stats, slice, lay.stat_bytes, lay.nrg, d_part},
                                  {d_stats, slice, lay.stat_bytes, lay.nrg, d_part ? d_part + part_bytes : nullptr}};
    for (uint32_t c = 0; c < n_columns && e == cudaSuccess; ++c)
        e = cudaMemsetAsync(d_stats + c * slice + lay.stat_bytes, 0, lay.reg_bytes, s);
    if (e == cudaSuccess) e = cudaMallocFromPoolAsync((void **)&d_image, bytes + SEG_IMAGE_PAD, dev->col_pool, s);
    if (e == cudaSuccess)
        e = cudaMallocFromPoolAsync((void **)&d_blocks, std::max<size_t>(1, all.size()) * sizeof(SegBlock), dev->col_pool, s);
    if (e == cudaSuccess && !all.empty())
        e = cudaMemcpyAsync(d_blocks, all.data(), all.size() * sizeof(SegBlock), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMallocFromPoolAsync((void **)&d_runs, std::max<size_t>(1, run_starts.size()) * 4, dev->col_pool, s);
    if (e == cudaSuccess && !run_starts.empty())
        e = cudaMemcpyAsync(d_runs, run_starts.data(), run_starts.size() * 4, cudaMemcpyHostToDevice, s);
    // Chunks alternate between two streams, each copying a chunk and then
    // decoding it, so one stream's copy runs beside the other's decode with
    // no wait between the streams.  (A copy stream feeding a decode stream
    // through events was observed to run every copy before the first decode
    // whenever the whole pipeline was queued at once.)  A chunk's copy covers
    // its row groups' bytes widened to 4 KiB boundaries, so every copy is
    // aligned; neighbouring copies overlap by less than 4 KiB and write the
    // same bytes there.
    cudaEvent_t ready = event(), copy0 = event(), copy1 = event();
    const cudaStream_t pair[2] = {s, cs};
    if (e == cudaSuccess) e = cudaEventRecord(ready, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, ready, 0);
    if (e == cudaSuccess) e = cudaEventRecord(copy0, s);
    std::vector<cudaEvent_t> landed(n_chunks), dec0(n_chunks), dec1(n_chunks), st1(n_chunks), done_ev(2);
    for (uint32_t k = 0; k < n_chunks; ++k) {
        landed[k] = event();
        dec0[k] = event();
        dec1[k] = event();
        st1[k] = event();
    }
    done_ev[0] = event();
    done_ev[1] = event();
    uint32_t launches = 0;
    for (uint32_t k = 0; k < n_chunks && e == cudaSuccess; ++k) {
        const cudaStream_t q = pair[k & 1];
        const SegStats &sst = sst_pair[k & 1];
        const uint32_t g0 = k * per_chunk, g1 = std::min(n_seg_rg, g0 + per_chunk);
        const uint64_t lo = k ? rg_pos[g0] / 4096 * 4096 : 0;
        const uint64_t hi = g1 < n_seg_rg ? std::min<uint64_t>(bytes, round_up(rg_pos[g1], 4096)) : bytes;
        e = cudaMemcpyAsync(d_image + lo, image + lo, hi - lo, cudaMemcpyHostToDevice, q);
        if (e == cudaSuccess) e = cudaEventRecord(landed[k], q);
        if (e == cudaSuccess) e = cudaEventRecord(dec0[k], q);
        if (e == cudaSuccess)
            e = launch_decode_blocks(d_image, d_blocks + chunk_first[k], chunk_first[k + 1] - chunk_first[k], d_runs,
                                     sst, q);
        launches += 1;
        if (e == cudaSuccess) e = cudaEventRecord(dec1[k], q);
        if (uniform && want_sketch && e == cudaSuccess) {
            // the chunk's register rows into the columns' registers, before this stream's next chunk reuses them
            e = launch_seg_hll_merge(sst, n_columns, g1 - g0, per_chunk, q);
            launches += 1;
        }
        if (e == cudaSuccess) e = cudaEventRecord(st1[k], q);
    }
    // not uniform: the table's own row groups, over the decoded columns
    for (uint32_t q = 0; q < 2 && e == cudaSuccess; ++q) {
        e = cudaEventRecord(done_ev[q], pair[q]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, done_ev[q], 0);
    }
    if (e == cudaSuccess && n_chunks) e = cudaEventRecord(copy1, s);
    if (!uniform) {
        for (uint32_t c = 0; c < n_columns && e == cudaSuccess; ++c) {
            unsigned char *sl = d_stats + c * slice;
            int64_t *imin = (int64_t *)sl, *imax = imin + lay.nrg;
            double *fmin = (double *)(imax + lay.nrg), *fmax = fmin + lay.nrg;
            uint32_t *nulls = (uint32_t *)(fmax + lay.nrg);
            uint32_t *regs = (uint32_t *)(sl + lay.stat_bytes);
            e = launch_column_stats(data[c], valid[c], columns[c].type, n, table_rg, 0, n_rg, imin, imax, fmin, fmax,
                                    nulls, sketch[c] ? regs : nullptr, d_part, 1, s);
            launches += sketch[c] ? 2 : 1;
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        release(false);
        return fail(TGPU_ERR_CUDA, std::string("segment decode: ") + cudaGetErrorString(e));
    }
    tgpu_load_stats ls{};
    ls.image_bytes = bytes;
    ls.decoded_bytes = decoded;
    ls.blocks = (uint32_t)all.size();
    ls.kernel_launches = launches;
    ls.chunks = n_chunks;
    float ms = 0;
    for (uint32_t k = 0; k < n_chunks; ++k) {
        if (cudaEventElapsedTime(&ms, copy0, landed[k]) == cudaSuccess) ls.h2d_ms = std::max<double>(ls.h2d_ms, ms);
        if (cudaEventElapsedTime(&ms, dec0[k], dec1[k]) == cudaSuccess) ls.decode_ms += ms;
        if (cudaEventElapsedTime(&ms, dec1[k], st1[k]) == cudaSuccess) ls.stats_ms += ms;
    }
    if (n_chunks && cudaEventElapsedTime(&ms, copy0, copy1) == cudaSuccess) ls.pipeline_ms = ms;
    if (n_chunks && cudaEventElapsedTime(&ms, copy0, dec0[0]) == cudaSuccess) ls.first_decode_ms = ms;
    // register the decoded columns in place, then hand them to the table
    std::vector<tgpu_column_desc> cd(n_columns);
    for (uint32_t c = 0; c < n_columns; ++c) {
        cd[c] = tgpu_column_desc{};
        cd[c].name = columns[c].name;
        cd[c].type = columns[c].type;
        cd[c].decimal_precision = columns[c].decimal_precision;
        cd[c].decimal_scale = columns[c].decimal_scale;
        cd[c].data = data[c];
        cd[c].validity = (const uint8_t *)valid[c];
    }
    tgpu_table_desc td{};
    td.columns = cd.data();
    td.n_columns = n_columns;
    td.row_group_rows = table_rg;
    td.n_rows = n;
    td.location = TGPU_LOC_DEVICE;
    td.compute_ndv = compute_ndv;
    td.stream = s;
    tgpu_table *t = nullptr;
    const PreStats pre{d_stats, &sketch};
    st = register_table(&td, &t, &pre);
    if (st != TGPU_OK) {
        const std::string msg = g_err;
        release(false);
        return fail(st, msg);
    }
    for (uint32_t c = 0; c < n_columns; ++c) t->cols[c].owned = true;  // freed with the table
    release(true);
    ls.total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_call).count();
    t->load = ls;
    *out = t;
    return TGPU_OK;
}

tgpu_status tgpu_table_read_column(const tgpu_table *t, uint32_t column, void *values, uint8_t *validity) {
    if (!t || !values || column >= t->cols.size()) return fail(TGPU_ERR_INVALID_ARGUMENT, "null table or bad column");
    const Column &c = t->cols[column];
    if (c.type == TGPU_VARCHAR) return fail(TGPU_ERR_UNSUPPORTED_TYPE, "VARCHAR columns read back by key strings");
    const size_t n = t->n_rows, bytes = n * type_bytes(c.type), vb = (n + 7) / 8;
    cudaError_t e = cudaSuccess;
    if (bytes) e = cudaMemcpyAsync(values, c.d_data, bytes, cudaMemcpyDeviceToHost, t->stream);
    if (e == cudaSuccess && validity && vb) {
        if (c.d_valid) e = cudaMemcpyAsync(validity, c.d_valid, vb, cudaMemcpyDeviceToHost, t->stream);
        else std::memset(validity, 0xFF, vb);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(t->stream);
    if (e != cudaSuccess) return fail(TGPU_ERR_CUDA, std::string("read column: ") + cudaGetErrorString(e));
    return TGPU_OK;
}

tgpu_status tgpu_table_load_stats(const tgpu_table *table, tgpu_load_stats *out) {
    if (!table || !out) return fail(TGPU_ERR_INVALID_ARGUMENT, "null argument");
    *out = table->load;
    return TGPU_OK;
}

tgpu_status tgpu_table_destroy(tgpu_table *table) {
    if (!table) return fail(TGPU_ERR_INVALID_ARGUMENT, "null table");
    delete table;
    return TGPU_OK;
}

tgpu_status tgpu_table_info(const tgpu_table *t, int32_t column, uint64_t *n_rows, uint32_t *n_rg, uint64_t *ndv) {
    if (!t) return fail(TGPU_ERR_INVALID_ARGUMENT, "null table");
    if (n_rows) *n_rows = t->n_rows;
    if (n_rg) *n_rg = t->n_rg;
    if (ndv) {
        if (column < 0 || (size_t)column >= t->cols.size()) *ndv = 0;
        else *ndv = t->cols[column].ndv;
    }
    return TGPU_OK;
}

tgpu_status tgpu_query_create(tgpu_table *table, const tgpu_request *req, tgpu_query **out) {
    return query_create(table, req, 0, out);
}

}  // extern "C"

tgpu_status query_create(tgpu_table *table, const tgpu_request *req, int batched, tgpu_query **out) {
    if (!table || !req || !out) return fail(TGPU_ERR_INVALID_ARGUMENT, "null argument");
    DeviceCtx *dev;
    tgpu_status st = device_ctx(&dev);
    if (st != TGPU_OK) return st;
    std::unique_ptr<tgpu_query> q(new tgpu_query());
    q->t = table;
    q->batched = batched != 0;
    q->stream = req->stream ? (cudaStream_t)req->stream : dev->stream;
    q->flags = req->flags;
    q->limit = req->limit;
    q->offset = req->offset;
    q->budget = req->memory_budget_bytes;
    if (req->chunk_rows < 0 || req->chunk_rows % CHUNK_ALIGN != 0 || req->chunk_rows > 65536)
        return fail(TGPU_ERR_INVALID_ARGUMENT, "chunk_rows must be a multiple of 256 up to 65536");
    if (req->cache_slots > 0 && (req->cache_slots & (req->cache_slots - 1)))
        return fail(TGPU_ERR_INVALID_ARGUMENT, "cache_slots must be a power of two");
    if (req->table_load_pct < 0 || req->table_load_pct > 90)
        return fail(TGPU_ERR_INVALID_ARGUMENT, "table_load_pct must be within 1..90");
    q->cache_req = req->cache_slots;
    q->chunk_req = (uint32_t)req->chunk_rows;
    q->load_pct = req->table_load_pct ? req->table_load_pct : 50;
    st = plan_query(q.get(), table, req);
    if (st != TGPU_OK) return st;
    apply_tuning(q.get(), req, batched);
    q->sketch = !batched && sketch_eligible(q.get(), req);
    q->radix = !q->sketch && radix_eligible(q.get());
    q->sketch_order_agg = q->sketch ? req->order[0].index : 0;
    st = g_slab.take(&q->h_block);
    if (st != TGPU_OK) return st;
    q->h_counts = (unsigned long long *)q->h_block;
    q->h_cancel = (int *)(q->h_block + 96);
    CU(cudaHostGetDevicePointer((void **)&q->d_cancel, q->h_cancel, 0));
    st = size_workspace(q.get(), next_pow2(std::max<uint64_t>(64, q->groups_est * 100 / q->load_pct)));
    if (st != TGPU_OK) return st;
    q->grid = scan_grid_size(q->dq, dev->sms);
    *out = q.release();
    return TGPU_OK;
}

extern "C" {

tgpu_status tgpu_query_output_schema(const tgpu_query *q, tgpu_output_column *cols, uint32_t cap, uint32_t *n) {
    if (!q) return fail(TGPU_ERR_INVALID_ARGUMENT, "null query");
    if (n) *n = (uint32_t)q->schema.size();
    for (uint32_t i = 0; cols && i < cap && i < q->schema.size(); ++i) cols[i] = q->schema[i];
    return TGPU_OK;
}

tgpu_status tgpu_query_execute(tgpu_query *q) {
    if (!q) return fail(TGPU_ERR_INVALID_ARGUMENT, "null query");
    if (*q->h_cancel) return fail(TGPU_ERR_CANCELLED, "query cancelled");
    return enqueue(q);
}

tgpu_status tgpu_query_synchronize(tgpu_query *q) {
    if (!q) return fail(TGPU_ERR_INVALID_ARGUMENT, "null query");
    if (!q->executed) return TGPU_OK;
    if (!q->synced) return finish(q);
    return TGPU_OK;
}

tgpu_status tgpu_query_next(tgpu_query *q, tgpu_batch *b, int32_t *done) {
    if (!q || !b || !done) return fail(TGPU_ERR_INVALID_ARGUMENT, "null argument");
    if (*q->h_cancel) return fail(TGPU_ERR_CANCELLED, "query cancelled");  // Query.next checks first (exec.zig:914)
    tgpu_status st;
    if (!q->executed && (st = enqueue(q)) != TGPU_OK) return st;
    if (!q->synced && (st = finish(q)) != TGPU_OK) return st;
    if (b->n_columns != q->schema.size()) return fail(TGPU_ERR_INVALID_ARGUMENT, "batch column count");
    const uint64_t n = std::min<uint64_t>(b->capacity_rows, q->result_rows - q->returned);
    const size_t nc = q->schema.size();
    std::vector<std::vector<uint8_t>> vbytes(nc);
    if (q->synth_empty) {
        // the global aggregate's row over no input: zero values, COUNTs valid
        for (size_t c = 0; c < nc; ++c) {
            if (n && b->values && b->values[c]) std::memset(b->values[c], 0, q->schema[c].elem_bytes);
            const int func = q->df.outs[c].func;
            vbytes[c].assign(n, (func == TGPU_AGG_COUNT || func == TGPU_AGG_COUNT_DISTINCT) ? 1 : 0);
        }
    } else if (q->h_packed) {
        // rows a batch already packed into host memory
        size_t off = 8;
        for (size_t c = 0; c < nc; ++c) {
            const size_t eb = q->schema[c].elem_bytes;
            if (n && b->values && b->values[c])
                std::memcpy(b->values[c], q->h_packed + off + q->returned * eb, n * eb);
            off += q->pack_rows * eb;
        }
        for (size_t c = 0; c < nc; ++c) {
            vbytes[c].assign(q->h_packed + off + q->returned, q->h_packed + off + q->returned + n);
            off += q->pack_rows;
        }
    } else {
        for (size_t c = 0; c < nc; ++c) {
            const size_t eb = q->schema[c].elem_bytes;
            if (n && b->values && b->values[c])
                CU(cudaMemcpyAsync(b->values[c], (char *)q->d_out[c] + q->returned * eb, n * eb,
                                   cudaMemcpyDeviceToHost, q->stream));
            if (n && b->validity && b->validity[c]) {
                vbytes[c].resize(n);
                CU(cudaMemcpyAsync(vbytes[c].data(), q->d_outvalid[c] + q->returned, n, cudaMemcpyDeviceToHost,
                                   q->stream));
            }
        }
        CU(cudaStreamSynchronize(q->stream));
    }
    for (size_t c = 0; c < nc; ++c) {
        if (!(n && b->validity && b->validity[c])) continue;
        uint8_t *bm = b->validity[c];
        std::memset(bm, 0, (n + 7) / 8);
        for (uint64_t r = 0; r < n; ++r)
            if (vbytes[c][r]) bm[r >> 3] |= (uint8_t)(1u << (r & 7));
    }
    q->returned += n;
    b->row_count = n;
    *done = q->returned >= q->result_rows ? 1 : 0;
    return TGPU_OK;
}

tgpu_status tgpu_query_key_strings(const tgpu_query *q, uint32_t column, const void *values, uint64_t n,
                                   uint64_t *offsets, uint8_t *bytes, uint64_t bytes_cap, uint64_t *bytes_needed) {
    if (!q || (n && (!values || !offsets)) || !bytes_needed) return fail(TGPU_ERR_INVALID_ARGUMENT, "null argument");
    if (column >= q->key_cols.size()) return fail(TGPU_ERR_INVALID_ARGUMENT, "not a group key column");
    const Column &c = q->t->cols[q->key_cols[column]];
    const bool dict = c.type == TGPU_DICT32 && c.dict_size();
    if (!dict && c.type != TGPU_VARCHAR)
        return fail(TGPU_ERR_INVALID_ARGUMENT, "not a string key (DICT32 with a dictionary, or VARCHAR)");
    uint64_t total = 0;
    offsets[0] = 0;
    for (uint64_t i = 0; i < n; ++i) {
        uint64_t b, len;
        if (dict) {
            const uint32_t code = (uint32_t)((const int32_t *)values)[i];
            if (code >= c.dict_size()) return fail(TGPU_ERR_INVALID_ARGUMENT, "code outside the dictionary");
            b = c.dict_offsets[code];
            len = c.dict_offsets[code + 1] - b;
        } else {
            const uint64_t row = (uint64_t)((const int64_t *)values)[i];
            if (row >= q->t->n_rows) return fail(TGPU_ERR_INVALID_ARGUMENT, "row index outside the table");
            b = c.str_offs[row];
            len = c.str_offs[row + 1] - b;
        }
        const uint8_t *src = dict ? c.dict_bytes.data() + b : c.str_bytes.data() + b;
        if (bytes && total + len <= bytes_cap) std::memcpy(bytes + total, src, len);
        total += len;
        offsets[i + 1] = total;
    }
    *bytes_needed = total;
    if (total > bytes_cap && bytes) return fail(TGPU_ERR_INVALID_ARGUMENT, "string buffer too small");
    return TGPU_OK;
}

tgpu_status tgpu_query_cancel(tgpu_query *q) {
    if (!q) return fail(TGPU_ERR_INVALID_ARGUMENT, "null query");
    __atomic_store_n(q->h_cancel, 1, __ATOMIC_SEQ_CST);
    return TGPU_OK;
}

tgpu_status tgpu_query_get_stats(const tgpu_query *q, tgpu_query_stats *out) {
    if (!q || !out) return fail(TGPU_ERR_INVALID_ARGUMENT, "null argument");
    *out = q->stats;
    return TGPU_OK;
}

tgpu_status tgpu_query_destroy(tgpu_query *q) {
    if (!q) return fail(TGPU_ERR_INVALID_ARGUMENT, "null query");
    delete q;
    return TGPU_OK;
}

}  // extern "C"

// ====================================================== batched execution ==

struct tgpu_query_batch {
    tgpu_table *t = nullptr;
    cudaStream_t stream = nullptr;
    int flags = 0;
    std::vector<tgpu_query *> qs;
    std::vector<DevQuery> h_qs;
    std::vector<DevFinal> h_fs;
    std::vector<DevFinalBufs> h_bs;
    std::vector<uint4> items;               // {query, first chunk, end chunk, 0}, by fold class, window major
    uint32_t class_off[BATCH_CLASSES + 1] = {0};  // items of fold class c: [class_off[c], class_off[c + 1])
    int class_grid[BATCH_CLASSES] = {0};
    Buffer dev_buf;                         // one pooled allocation for every array below
    void *dev = nullptr;
    DevQuery *d_qs = nullptr;
    DevFinal *d_fs = nullptr;
    DevFinalBufs *d_bs = nullptr;
    Buffer items_buf;                       // pooled
    uint4 *d_items = nullptr;
    unsigned int *d_ctrl = nullptr;         // [0] work counter, [1] status
    unsigned long long *d_counts = nullptr; // 8 per query
    unsigned int *d_qctrl = nullptr;        // 4 per query: tile counter, status
    unsigned long long *h_counts = nullptr; // pinned: 8 per query, then Q statuses + batch status
    size_t counts_bytes = 0;
    char *h_block = nullptr;                // slab block holding the cancel flag
    int *h_cancel = nullptr, *d_cancel = nullptr;
    uint8_t *h_stage = nullptr, *d_stage = nullptr;  // mapped pinned: packed result rows
    size_t stage_bytes = 0;
    std::vector<size_t> stage_off;
    std::vector<uint64_t> stage_rows;
    bool any_distinct = false, any_topk = false;
    int max_aggs = 0;
    uint32_t topk_widths = 0;  // TOPK_W* classes of the top-k queries
    size_t smem = 0;
    int grid = 0;
    uint32_t max_cpt_blocks = 1, max_cand_blocks = 1;
    uint64_t max_rows = 1, max_words = 1;
    uint32_t epoch = 0;
    bool descriptors_dirty = true;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool executed = false, synced = false;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    tgpu_batch_stats stats{};
    ~tgpu_query_batch() {
        if (stream) cudaStreamSynchronize(stream);
        for (auto *q : qs) delete q;
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        g_scratch_pool.give(dev_buf);
        g_scratch_pool.give(items_buf);
        g_pinned.give((char *)h_counts, counts_bytes);
        g_pinned.give((char *)h_stage, stage_bytes);
        g_slab.give(h_block);
        for (auto e : ev)
            if (e) cudaEventDestroy(e);
    }
};

namespace {

// Point every query's counters at the batch arrays and rebuild the device
// descriptors (after create, and after a query was regrown on its own).
tgpu_status batch_descriptors(tgpu_query_batch *b) {
    const uint32_t Q = (uint32_t)b->qs.size();
    b->h_qs.resize(Q);
    b->h_fs.resize(Q);
    b->h_bs.resize(Q);
    b->max_aggs = 0;
    b->topk_widths = 0;
    b->smem = 0;
    b->max_cpt_blocks = 1;
    b->max_cand_blocks = 1;
    b->max_rows = 1;
    b->max_words = 1;
    b->any_distinct = b->any_topk = false;
    // layout of the packed results (queries with at most 4,096 result rows)
    b->stage_off.assign(Q, 0);
    b->stage_rows.assign(Q, 0);
    size_t stage = 0;
    for (uint32_t i = 0; i < Q; ++i) {
        tgpu_query *q = b->qs[i];
        uint64_t rows = q->rank == RANK_TOPK ? q->limit : q->out_rows_max;
        if (rows > 4096) continue;
        size_t bytes = 8;
        for (auto &oc : q->schema) bytes += rows * (oc.elem_bytes + 1);
        b->stage_off[i] = stage;
        b->stage_rows[i] = rows;
        stage += (bytes + 15) & ~(size_t)15;
    }
    if (stage > b->stage_bytes) {
        g_pinned.give((char *)b->h_stage, b->stage_bytes);
        b->h_stage = nullptr;
        b->stage_bytes = 0;
        size_t got = 0;
        tgpu_status pst = g_pinned.take(stage, (char **)&b->h_stage, &got);
        if (pst != TGPU_OK) return pst;
        CU(cudaHostGetDevicePointer((void **)&b->d_stage, b->h_stage, 0));
        stage = got;
        b->stage_bytes = stage;
    }
    for (uint32_t i = 0; i < Q; ++i) {
        tgpu_query *q = b->qs[i];
        q->d_counts = b->d_counts + 8 * (size_t)i;
        q->d_ctrl = b->d_qctrl + 4 * (size_t)i;
        DevQuery dq = q->dq;
        if (dq.gather == 2) dq.gather = 1;  // the batched kernel gathers survivors per chunk
        // row-group aligned chunks: an item is the query's chunks of one row
        // group, split evenly over the CTA's warps
        dq.rg_list = q->d_rg_list;
        dq.n_rg = (uint32_t)q->rg_list.size();
        if (!dq.gather && !q->chunk_req)
            dq.chunk_rows = (uint32_t)std::min<uint64_t>(4096, round_up(ceil_div(b->t->rg_rows, SCAN_WARPS), CHUNK_ALIGN));
        dq.chunks_per_rg = (uint32_t)ceil_div(b->t->rg_rows, dq.chunk_rows);
        dq.n_chunks = dq.n_rg * dq.chunks_per_rg;
        dq.shared_scan = Q > 1;
        dq.tile_counter = q->d_ctrl;
        dq.status = q->d_ctrl + 1;
        dq.selected_rows = q->d_counts + 4;
        dq.cancel = (const volatile int *)b->d_cancel;
        dq.epoch = b->epoch;
        b->h_qs[i] = dq;
        b->h_fs[i] = q->df;
        DevFinalBufs &fb = b->h_bs[i];
        fb.block_counts = q->d_block_counts;
        fb.gids = q->d_gids;
        fb.counts = q->d_counts;
        fb.cand_keys = q->d_cand_keys;
        fb.cand_gids = q->d_cand_gids;
        fb.out_cols = q->d_out_ptrs;
        fb.out_valid = q->d_valid_ptrs;
        fb.n_cpt_blocks = q->n_cpt_blocks;
        fb.n_cand_blocks = q->n_cand_blocks;
        fb.k = q->k;
        fb.rank = q->rank == RANK_TOPK ? 1 : 0;
        fb.sel = q->rank == RANK_TOPK ? q->d_sel : q->d_gids;
        fb.offset = q->rank == RANK_TOPK ? q->offset : 0;
        fb.gather_rows = q->rank == RANK_TOPK ? q->limit : q->out_rows_max;
        fb.pack_rows = b->stage_rows[i];
        fb.pack_dst = fb.pack_rows ? b->d_stage + b->stage_off[i] : nullptr;
        fb.n_out = (uint32_t)q->schema.size();
        for (size_t c = 0; c < q->schema.size(); ++c) fb.out_bytes[c] = q->schema[c].elem_bytes;
        b->max_aggs = std::max(b->max_aggs, dq.n_aggs);
        if (fb.rank == 1) b->topk_widths |= topk_width_bit(q->df.sort_words);
        b->smem = std::max(b->smem, scan_smem_bytes(dq));
        b->max_cpt_blocks = std::max(b->max_cpt_blocks, q->n_cpt_blocks);
        b->max_cand_blocks = std::max(b->max_cand_blocks, q->n_cand_blocks);
        b->max_rows = std::max<uint64_t>(b->max_rows, fb.gather_rows);
        b->max_words = std::max<uint64_t>(b->max_words, (dq.cap + 1 + 31) / 32);
        b->any_distinct |= dq.n_dsets > 0;
        b->any_topk |= fb.rank == 1;
    }
    if (!b->d_items) {
        // per fold class, window major: the row groups go in windows of
        // about BATCH_WINDOW_ROWS rows, and an item is one query's kept row
        // groups of one window (one CTA, its shared table flushed once per
        // item); every query of the class for window w, then w + 1, ..., so
        // the CTAs running at any moment read the same window from L2
        const uint32_t win = std::max<uint32_t>(1, (uint32_t)(BATCH_WINDOW_ROWS / std::max<uint32_t>(1, b->t->rg_rows)));
        std::vector<size_t> pos(Q, 0);
        for (int cls = 0; cls < BATCH_CLASSES; ++cls) {
            b->class_off[cls] = (uint32_t)b->items.size();
            for (uint32_t g0 = 0; g0 < b->t->n_rg; g0 += win)
                for (uint32_t i = 0; i < Q; ++i) {
                    if (batch_fold_class(b->h_qs[i]) != cls) continue;
                    const std::vector<uint32_t> &rl = b->qs[i]->rg_list;
                    const size_t p0 = pos[i];
                    while (pos[i] < rl.size() && rl[pos[i]] < g0 + win) ++pos[i];
                    if (pos[i] > p0) {
                        const uint32_t cpr = b->h_qs[i].chunks_per_rg;
                        b->items.push_back(make_uint4(i, (uint32_t)(p0 * cpr),
                                                      std::min<uint32_t>((uint32_t)(pos[i] * cpr), b->h_qs[i].n_chunks), 0u));
                    }
                }
        }
        b->class_off[BATCH_CLASSES] = (uint32_t)b->items.size();
        tgpu_status ist = g_scratch_pool.take(sizeof(uint4) * std::max<size_t>(1, b->items.size()), b->stream,
                                              &b->items_buf);
        if (ist != TGPU_OK) return ist;
        b->d_items = (uint4 *)b->items_buf.p;
        if (!b->items.empty())
            CU(cudaMemcpyAsync(b->d_items, b->items.data(), sizeof(uint4) * b->items.size(), cudaMemcpyHostToDevice,
                               b->stream));
    }
    CU(cudaMemcpyAsync(b->d_qs, b->h_qs.data(), sizeof(DevQuery) * Q, cudaMemcpyHostToDevice, b->stream));
    CU(cudaMemcpyAsync(b->d_fs, b->h_fs.data(), sizeof(DevFinal) * Q, cudaMemcpyHostToDevice, b->stream));
    CU(cudaMemcpyAsync(b->d_bs, b->h_bs.data(), sizeof(DevFinalBufs) * Q, cudaMemcpyHostToDevice, b->stream));
    CU(cudaStreamSynchronize(b->stream));
    DeviceCtx *dev;
    tgpu_status st = device_ctx(&dev);
    if (st != TGPU_OK) return st;
    for (int cls = 0; cls < BATCH_CLASSES; ++cls)
        b->class_grid[cls] =
            b->class_off[cls + 1] > b->class_off[cls] ? batch_scan_grid(cls, b->smem, dev->sms) : 0;
    b->descriptors_dirty = false;
    b->stats.work_items = b->items.size();
    return TGPU_OK;
}

// The device work of one execute (also what a CUDA graph captures).
tgpu_status batch_enqueue_work(tgpu_query_batch *b, bool capturing) {
    const uint32_t Q = (uint32_t)b->qs.size();
    cudaStream_t s = b->stream;
    if (!capturing) CU(cudaEventRecord(b->ev[0], s));
    CU(cudaMemsetAsync(b->d_ctrl, 0, 8, s));
    CU(cudaMemsetAsync(b->d_counts, 0, 64 * (size_t)Q, s));
    CU(cudaMemsetAsync(b->d_qctrl, 0, 16 * (size_t)Q, s));
    uint32_t scans = 0;
    for (int cls = 0; cls < BATCH_CLASSES; ++cls) {
        const uint32_t n = b->class_off[cls + 1] - b->class_off[cls];
        if (!n) continue;
        CU(launch_batch_scan(cls, b->d_qs, b->d_items + b->class_off[cls], n, b->smem, b->class_grid[cls],
                             (const volatile int *)b->d_cancel, b->d_ctrl + 1, s));
        ++scans;
    }
    CU(launch_finalize_batch(b->d_fs, b->d_bs, Q, b->max_cpt_blocks, b->max_cand_blocks, b->topk_widths,
                             b->max_rows, b->max_words, s));
    CU(cudaMemcpyAsync(b->h_counts, b->d_counts, 64 * (size_t)Q, cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(b->h_counts + 8 * (size_t)Q, b->d_qctrl, 16 * (size_t)Q, cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(b->h_counts + 10 * (size_t)Q, b->d_ctrl, 8, cudaMemcpyDeviceToHost, s));
    if (!capturing) CU(cudaEventRecord(b->ev[1], s));
    b->stats.kernel_launches = scans + 5 + std::max(1, 2 * __builtin_popcount(b->topk_widths));
    return TGPU_OK;
}

}  // namespace

extern "C" {

tgpu_status tgpu_batch_create(tgpu_table *table, const tgpu_request *reqs, uint32_t n, int32_t flags, void *stream,
                              tgpu_query_batch **out) {
    if (!table || (!reqs && n) || !out) return fail(TGPU_ERR_INVALID_ARGUMENT, "null argument");
    if (n == 0) return fail(TGPU_ERR_INVALID_ARGUMENT, "empty batch");
    DeviceCtx *dev;
    tgpu_status st = device_ctx(&dev);
    if (st != TGPU_OK) return st;
    std::unique_ptr<tgpu_query_batch> b(new tgpu_query_batch());
    b->t = table;
    b->stream = stream ? (cudaStream_t)stream : dev->stream;
    b->flags = flags;
    for (uint32_t i = 0; i < n; ++i) {
        tgpu_request r = reqs[i];
        r.stream = b->stream;
        tgpu_query *q = nullptr;
        st = query_create(table, &r, 1, &q);
        if (st != TGPU_OK) return st;
        b->qs.push_back(q);
        if (q->rank == RANK_SORT) {
            return fail(TGPU_DECLINE, "batched queries return all groups or a top-k with offset + limit <= 32");
        }
    }
    const size_t Q = n;
    size_t off = 0;
    auto add = [&](size_t bytes) {
        size_t o = off;
        off += (bytes + 255) & ~(size_t)255;
        return o;
    };
    size_t o_qs = add(sizeof(DevQuery) * Q), o_fs = add(sizeof(DevFinal) * Q), o_bs = add(sizeof(DevFinalBufs) * Q),
           o_ctrl = add(16), o_counts = add(64 * Q), o_qctrl = add(16 * Q);
    st = g_scratch_pool.take(off, b->stream, &b->dev_buf);
    if (st != TGPU_OK) return st;
    b->dev = b->dev_buf.p;
    char *base = (char *)b->dev;
    b->d_qs = (DevQuery *)(base + o_qs);
    b->d_fs = (DevFinal *)(base + o_fs);
    b->d_bs = (DevFinalBufs *)(base + o_bs);
    b->d_ctrl = (unsigned int *)(base + o_ctrl);
    b->d_counts = (unsigned long long *)(base + o_counts);
    b->d_qctrl = (unsigned int *)(base + o_qctrl);
    st = g_pinned.take(8 * (11 * Q + 2), (char **)&b->h_counts, &b->counts_bytes);
    if (st != TGPU_OK) return st;
    std::memset(b->h_counts, 0, 8 * (11 * Q + 2));
    st = g_slab.take(&b->h_block);
    if (st != TGPU_OK) return st;
    b->h_cancel = (int *)b->h_block;
    CU(cudaHostGetDevicePointer((void **)&b->d_cancel, b->h_cancel, 0));
    for (auto &e : b->ev) CU(cudaEventCreate(&e));
    for (auto *q : b->qs)
        for (auto &buf : q->dset_bufs) b->epoch = std::max(b->epoch, buf.epoch);
    b->stats.n_queries = n;
    st = batch_descriptors(b.get());
    if (st != TGPU_OK) return st;
    *out = b.release();
    return TGPU_OK;
}

tgpu_status tgpu_batch_execute(tgpu_query_batch *b) {
    if (!b) return fail(TGPU_ERR_INVALID_ARGUMENT, "null batch");
    if (*b->h_cancel) return fail(TGPU_ERR_CANCELLED, "batch cancelled");
    tgpu_status st;
    if (b->any_distinct) {
        // distinct sets are reused across executes: a fresh epoch frees their entries
        ++b->epoch;
        if (b->epoch == 0xFFFFFFFFu) {
            for (auto *q : b->qs)
                for (auto &buf : q->dset_bufs) CU(cudaMemsetAsync(buf.p, 0, buf.bytes, b->stream));
            b->epoch = 1;
        }
        for (auto *q : b->qs)
            for (auto &buf : q->dset_bufs) buf.epoch = b->epoch;
        b->descriptors_dirty = true;
    }
    if (b->descriptors_dirty) {
        if ((st = batch_descriptors(b)) != TGPU_OK) return st;
    }
    for (auto *q : b->qs) {
        q->table_buf.dirty = true;
        q->occ_buf.dirty = true;
    }
    if (b->flags & TGPU_BATCH_GRAPH) {
        if (!b->exec) {
            CU(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            st = batch_enqueue_work(b, true);
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(b->stream, &g);
            if (st != TGPU_OK) {
                if (g) cudaGraphDestroy(g);
                return st;
            }
            CU(e);
            b->graph = g;
            CU(cudaGraphInstantiate(&b->exec, g, 0));
        }
        // events bracket the replay (an event recorded during capture is not a record node)
        CU(cudaEventRecord(b->ev[0], b->stream));
        CU(cudaGraphLaunch(b->exec, b->stream));
        CU(cudaEventRecord(b->ev[1], b->stream));
        b->stats.graph = 1;
    } else {
        if ((st = batch_enqueue_work(b, false)) != TGPU_OK) return st;
        b->stats.graph = 0;
    }
    b->executed = true;
    b->synced = false;
    return TGPU_OK;
}

tgpu_status tgpu_batch_synchronize(tgpu_query_batch *b) {
    if (!b) return fail(TGPU_ERR_INVALID_ARGUMENT, "null batch");
    if (!b->executed || b->synced) return TGPU_OK;
    CU(cudaStreamSynchronize(b->stream));
    const size_t Q = b->qs.size();
    const uint32_t *qctrl = (const uint32_t *)(b->h_counts + 8 * Q);
    const uint32_t bstatus = ((const uint32_t *)(b->h_counts + 10 * Q))[1];
    float ms = 0;
    CU(cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]));
    b->stats.total_ms = ms;
    b->stats.rerun_queries = 0;
    b->synced = true;
    if (bstatus & ST_CANCELLED) return fail(TGPU_ERR_CANCELLED, "batch cancelled");
    for (size_t i = 0; i < Q; ++i) {
        tgpu_query *q = b->qs[i];
        const uint32_t status = qctrl[4 * i + 1];
        q->table_buf.dirty = false;
        q->occ_buf.dirty = false;
        if (status & (ST_TABLE_FULL | ST_DISTINCT_FULL)) {
            // regrow this query and run it alone; its descriptors change
            if (status & ST_TABLE_FULL) q->groups_est = std::max<uint64_t>(q->groups_est * 4, 1024);
            if (status & ST_DISTINCT_FULL)
                for (auto &nd : q->dset_need) nd *= 4;
            tgpu_status st = size_workspace(q, next_pow2(q->groups_est * 100 / q->load_pct));
            if (st != TGPU_OK) return st;
            DeviceCtx *dev;
            if ((st = device_ctx(&dev)) != TGPU_OK) return st;
            q->grid = scan_grid_size(q->dq, dev->sms);
            if ((st = enqueue(q)) != TGPU_OK) return st;
            if ((st = finish(q)) != TGPU_OK) return st;
            b->stats.rerun_queries++;
            b->descriptors_dirty = true;
            if (b->exec) {
                cudaGraphExecDestroy(b->exec);
                cudaGraphDestroy(b->graph);
                b->exec = nullptr;
                b->graph = nullptr;
            }
            continue;
        }
        const unsigned long long *c = b->h_counts + 8 * i;
        q->executed = true;
        q->synced = true;
        q->returned = 0;
        q->result_rows = c[2];
        set_empty_global_row(q, c[0]);
        q->pack_rows = b->stage_rows[i];
        q->h_packed = q->pack_rows ? b->h_stage + b->stage_off[i] : nullptr;
        q->stats.rows_scanned = q->rows_scanned;
        q->stats.rows_selected = c[4];
        q->stats.groups = c[0];
        q->stats.result_rows = c[2];
        q->stats.table_capacity = q->dq.cap;
        q->stats.route = (uint32_t)q->route;
        q->stats.flags = (q->tuned ? TGPU_STAT_TUNED : 0) | (q->dq.gather ? TGPU_STAT_GATHER : 0);  // batched: gather
    }
    return TGPU_OK;
}

tgpu_status tgpu_batch_output_schema(const tgpu_query_batch *b, uint32_t i, tgpu_output_column *cols, uint32_t cap,
                                     uint32_t *n) {
    if (!b || i >= b->qs.size()) return fail(TGPU_ERR_INVALID_ARGUMENT, "query index");
    return tgpu_query_output_schema(b->qs[i], cols, cap, n);
}

tgpu_status tgpu_batch_next(tgpu_query_batch *b, uint32_t i, tgpu_batch *out, int32_t *done) {
    if (!b || i >= b->qs.size()) return fail(TGPU_ERR_INVALID_ARGUMENT, "query index");
    tgpu_status st = tgpu_batch_synchronize(b);
    if (st != TGPU_OK) return st;
    if (!b->qs[i]->executed) return fail(TGPU_ERR_INVALID_ARGUMENT, "batch not executed");
    return tgpu_query_next(b->qs[i], out, done);
}

tgpu_status tgpu_batch_cancel(tgpu_query_batch *b) {
    if (!b) return fail(TGPU_ERR_INVALID_ARGUMENT, "null batch");
    __atomic_store_n(b->h_cancel, 1, __ATOMIC_SEQ_CST);
    return TGPU_OK;
}

tgpu_status tgpu_batch_get_stats(const tgpu_query_batch *b, tgpu_batch_stats *out) {
    if (!b || !out) return fail(TGPU_ERR_INVALID_ARGUMENT, "null argument");
    *out = b->stats;
    return TGPU_OK;
}

tgpu_status tgpu_batch_destroy(tgpu_query_batch *b) {
    if (!b) return fail(TGPU_ERR_INVALID_ARGUMENT, "null batch");
    delete b;
    return TGPU_OK;
}

}  // extern "C"

// ================================================================ serving ==

namespace {

using Clock = std::chrono::steady_clock;

// A request with its own copies of every array it points to.
struct OwnedRequest {
    tgpu_request r{};
    std::vector<int32_t> group_cols;
    std::vector<tgpu_agg_spec> aggs;
    std::vector<std::string> names, udf_names;
    std::vector<tgpu_predicate> where;
    std::vector<tgpu_having> having;
    std::vector<tgpu_sort_spec> order;
    void set(const tgpu_request &in) {
        r = in;
        group_cols.assign(in.group_cols, in.group_cols + in.n_group_cols);
        aggs.assign(in.aggs, in.aggs + in.n_aggs);
        names.clear();
        udf_names.clear();
        for (auto &a : aggs) {
            names.push_back(a.as ? a.as : "");
            udf_names.push_back(a.udf_name ? a.udf_name : "");
        }
        for (size_t i = 0; i < aggs.size(); ++i) {
            aggs[i].as = names[i].c_str();
            if (aggs[i].udf_name) aggs[i].udf_name = udf_names[i].c_str();
        }
        where.assign(in.where, in.where + in.n_where);
        having.assign(in.having, in.having + in.n_having);
        order.assign(in.order, in.order + in.n_order);
        r.group_cols = group_cols.data();
        r.aggs = aggs.data();
        r.where = where.data();
        r.having = having.data();
        r.order = order.data();
        r.stream = nullptr;
    }
};

struct Ticket {
    uint64_t id = 0;
    uint32_t table = 0;
    OwnedRequest req;
    uint64_t est_bytes = 0;
    Clock::time_point submitted, done_at;
    int state = 0;  // 0 queued, 1 running, 2 done
    tgpu_status status = TGPU_OK;
    std::string error;
    std::vector<tgpu_output_column> schema;
    std::vector<std::vector<uint8_t>> data;
    std::vector<std::vector<uint8_t>> valid;  // one byte per row
    uint64_t rows = 0, returned = 0;
};

struct Wave {
    std::vector<Ticket *> tickets;
    tgpu_query_batch *batch = nullptr;
    tgpu_query *query = nullptr;
    int slot = 0;
    cudaEvent_t done = nullptr;
    uint64_t bytes = 0;
};

// Estimated device bytes of a request: group table + occupancy bitmap +
// distinct sets + id list and outputs (thinDB's accountant reserves before
// it allocates, src/memory.zig:841).
tgpu_status estimate_bytes(tgpu_table *t, const tgpu_request *req, uint64_t *out) {
    std::unique_ptr<tgpu_query> q(new tgpu_query());
    q->t = t;
    q->flags = req->flags;
    q->limit = req->limit;
    q->offset = req->offset;
    q->load_pct = req->table_load_pct ? req->table_load_pct : 50;
    tgpu_status st = plan_query(q.get(), t, req);
    if (st != TGPU_OK) return st;
    uint64_t cap = next_pow2(std::max<uint64_t>(64, q->groups_est * 100 / q->load_pct));
    uint64_t slots = cap + 1;
    uint64_t bytes = slots * (uint64_t)q->dq.slot_words * 8 + slots / 8 + slots * 4;
    for (uint64_t need : q->dset_need) bytes += next_pow2(std::max<uint64_t>(64, need * 2)) * 16;
    uint64_t rows = req->limit != TGPU_NO_LIMIT ? std::min<uint64_t>(req->limit, slots) : slots;
    for (auto &oc : q->schema) bytes += rows * (oc.elem_bytes + 1);
    *out = bytes;
    return TGPU_OK;
}

}  // namespace

struct tgpu_server {
    std::vector<tgpu_table *> tables;
    tgpu_server_options opt{};
    std::mutex mu;
    std::condition_variable cv_submit, cv_done;
    std::deque<Ticket *> pending;
    std::unordered_map<uint64_t, std::unique_ptr<Ticket>> tickets;
    uint64_t next_id = 1;
    uint64_t admitted_bytes = 0;
    bool stop = false;
    int device = 0;
    std::vector<cudaStream_t> streams;
    std::vector<bool> slot_busy;
    std::vector<Wave> inflight;   // dispatcher thread only
    tgpu_server_stats stats{};
    std::thread th;

    ~tgpu_server() {
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
        }
        cv_submit.notify_all();
        if (th.joinable()) th.join();
        for (auto s : streams) cudaStreamDestroy(s);
    }

    void finish_wave(Wave &w) {
        cudaEventSynchronize(w.done);
        cudaEventDestroy(w.done);
        std::vector<std::pair<Ticket *, tgpu_status>> results;
        for (size_t i = 0; i < w.tickets.size(); ++i) {
            Ticket *tk = w.tickets[i];
            tgpu_status st = TGPU_OK;
            tgpu_query *q = w.batch ? w.batch->qs[i] : w.query;
            if (w.batch) st = tgpu_batch_synchronize(w.batch);
            else st = tgpu_query_synchronize(q);
            if (st == TGPU_OK) {
                tk->schema = q->schema;
                const size_t nc = q->schema.size();
                std::vector<void *> vals(nc);
                std::vector<uint8_t *> bms(nc);
                uint64_t rows = q->result_rows;
                tk->data.assign(nc, {});
                tk->valid.assign(nc, {});
                std::vector<std::vector<uint8_t>> bits(nc);
                for (size_t c = 0; c < nc; ++c) {
                    tk->data[c].resize(std::max<uint64_t>(1, rows) * q->schema[c].elem_bytes);
                    bits[c].resize(std::max<uint64_t>(1, (rows + 7) / 8));
                    vals[c] = tk->data[c].data();
                    bms[c] = bits[c].data();
                }
                tgpu_batch ob{};
                ob.n_columns = (uint32_t)nc;
                ob.values = vals.data();
                ob.validity = bms.data();
                ob.capacity_rows = std::max<uint64_t>(1, rows);
                int32_t d = 0;
                st = tgpu_query_next(q, &ob, &d);
                tk->rows = ob.row_count;
                for (size_t c = 0; c < nc; ++c) {
                    tk->valid[c].resize(tk->rows);
                    for (uint64_t r = 0; r < tk->rows; ++r) tk->valid[c][r] = (bits[c][r >> 3] >> (r & 7)) & 1;
                }
            }
            results.push_back({tk, st});
        }
        std::string err = g_err;
        if (w.batch) tgpu_batch_destroy(w.batch);
        if (w.query) tgpu_query_destroy(w.query);
        auto now = Clock::now();
        {
            std::lock_guard<std::mutex> lk(mu);
            for (auto &pr : results) {
                pr.first->status = pr.second;
                if (pr.second != TGPU_OK) {
                    pr.first->error = err;
                    stats.failed++;
                }
                pr.first->state = 2;
                pr.first->done_at = now;
                stats.completed++;
            }
            admitted_bytes -= w.bytes;
            slot_busy[w.slot] = false;
        }
        cv_done.notify_all();
    }

    void fail_tickets(const std::vector<Ticket *> &tks, tgpu_status st, uint64_t bytes, int slot) {
        std::string err = g_err;
        auto now = Clock::now();
        {
            std::lock_guard<std::mutex> lk(mu);
            for (Ticket *tk : tks) {
                tk->status = st;
                tk->error = err;
                tk->state = 2;
                tk->done_at = now;
                stats.failed++;
                stats.completed++;
            }
            admitted_bytes -= bytes;
            if (slot >= 0) slot_busy[slot] = false;
        }
        cv_done.notify_all();
    }

    // Take the next wave: the oldest request's table, then every queued
    // request of that table that fits the budget (FIFO within the table).
    bool take_wave(std::vector<Ticket *> &out, uint32_t &table, uint64_t &bytes, int &slot) {
        std::lock_guard<std::mutex> lk(mu);
        if (pending.empty()) return false;
        slot = -1;
        for (size_t i = 0; i < slot_busy.size(); ++i)
            if (!slot_busy[i]) {
                slot = (int)i;
                break;
            }
        if (slot < 0) return false;
        uint32_t max_batch = opt.mode == TGPU_SERVE_PLAIN ? 1 : (opt.max_batch ? opt.max_batch : 256);
        table = pending.front()->table;
        if (max_batch > 1) {
            // separate executions overlapping on the wave streams, unless the
            // options ask for batched kernels from a backlog of batch_min
            // requests on one table
            uint32_t same = 0;
            for (Ticket *tk : pending) same += tk->table == table ? 1 : 0;
            if (opt.batch_min <= 0 || same < (uint32_t)opt.batch_min) max_batch = 1;
        }
        bytes = 0;
        for (auto it = pending.begin(); it != pending.end() && out.size() < max_batch;) {
            Ticket *tk = *it;
            if (tk->table != table) {
                ++it;
                continue;
            }
            if (admitted_bytes + bytes + tk->est_bytes > opt.memory_budget_bytes && !(out.empty() && admitted_bytes == 0))
                break;  // wait for memory to free up (a request larger than the budget runs alone)
            bytes += tk->est_bytes;
            tk->state = 1;
            out.push_back(tk);
            it = pending.erase(it);
        }
        if (out.empty()) return false;
        admitted_bytes += bytes;
        stats.peak_admitted_bytes = std::max(stats.peak_admitted_bytes, admitted_bytes);
        slot_busy[slot] = true;
        return true;
    }

    void launch(std::vector<Ticket *> &tks, uint32_t table, uint64_t bytes, int slot) {
        Wave w;
        w.tickets = tks;
        w.slot = slot;
        w.bytes = bytes;
        cudaStream_t s = streams[slot];
        tgpu_status st;
        if (opt.mode == TGPU_SERVE_PLAIN || tks.size() == 1) {
            tgpu_request r = tks[0]->req.r;
            r.stream = s;
            st = tgpu_query_create(tables[table], &r, &w.query);
            if (st == TGPU_OK) st = tgpu_query_execute(w.query);
        } else {
            std::vector<tgpu_request> reqs;
            for (Ticket *tk : tks) reqs.push_back(tk->req.r);
            st = tgpu_batch_create(tables[table], reqs.data(), (uint32_t)reqs.size(), 0, s, &w.batch);
            if (st == TGPU_DECLINE) {
                // a shape the batch does not run: run each request alone, in order
                for (Ticket *tk : tks) {
                    std::vector<Ticket *> one{tk};
                    launch_one_sync(one, table, s);
                }
                std::lock_guard<std::mutex> lk(mu);
                admitted_bytes -= bytes;
                slot_busy[slot] = false;
                return;
            }
            if (st == TGPU_OK) st = tgpu_batch_execute(w.batch);
        }
        if (st != TGPU_OK) {
            if (w.batch) tgpu_batch_destroy(w.batch);
            if (w.query) tgpu_query_destroy(w.query);
            fail_tickets(tks, st, bytes, slot);
            return;
        }
        cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming);
        cudaEventRecord(w.done, s);
        stats.waves++;
        inflight.push_back(w);
    }

    void launch_one_sync(std::vector<Ticket *> &one, uint32_t table, cudaStream_t s) {
        Wave w;
        w.tickets = one;
        w.slot = 0;
        w.bytes = 0;
        tgpu_request r = one[0]->req.r;
        r.stream = s;
        tgpu_status st = tgpu_query_create(tables[table], &r, &w.query);
        if (st == TGPU_OK) st = tgpu_query_execute(w.query);
        if (st != TGPU_OK) {
            if (w.query) tgpu_query_destroy(w.query);
            fail_tickets(one, st, 0, -1);
            return;
        }
        cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming);
        cudaEventRecord(w.done, s);
        stats.waves++;
        // completes before the dispatcher launches more on this stream
        bool busy = slot_busy[0];
        finish_wave(w);
        std::lock_guard<std::mutex> lk(mu);
        slot_busy[0] = busy;
    }

    void run() {
        cudaSetDevice(device);
        for (;;) {
            bool progressed = false;
            for (size_t i = 0; i < inflight.size();) {
                if (cudaEventQuery(inflight[i].done) == cudaSuccess) {
                    finish_wave(inflight[i]);
                    inflight.erase(inflight.begin() + i);
                    progressed = true;
                } else {
                    cudaGetLastError();
                    ++i;
                }
            }
            for (;;) {
                std::vector<Ticket *> tks;
                uint32_t table = 0;
                uint64_t bytes = 0;
                int slot = -1;
                if (!take_wave(tks, table, bytes, slot)) break;
                launch(tks, table, bytes, slot);
                progressed = true;
            }
            std::unique_lock<std::mutex> lk(mu);
            if (stop && pending.empty() && inflight.empty()) break;
            if (!progressed) {
                if (inflight.empty()) cv_submit.wait_for(lk, std::chrono::milliseconds(2));
                else {
                    lk.unlock();
                    std::this_thread::sleep_for(std::chrono::microseconds(20));
                }
            }
        }
    }
};

extern "C" {

tgpu_status tgpu_server_create(tgpu_table *const *tables, uint32_t n, const tgpu_server_options *opts,
                               tgpu_server **out) {
    if (!tables || !n || !out) return fail(TGPU_ERR_INVALID_ARGUMENT, "null argument");
    DeviceCtx *dev;
    tgpu_status st = device_ctx(&dev);
    if (st != TGPU_OK) return st;
    std::unique_ptr<tgpu_server> s(new tgpu_server());
    s->tables.assign(tables, tables + n);
    if (opts) s->opt = *opts;
    if (!s->opt.memory_budget_bytes) s->opt.memory_budget_bytes = 120ULL << 30;
    if (!s->opt.max_inflight) s->opt.max_inflight = 8;
    if (s->opt.mode == TGPU_SERVE_PLAIN) s->opt.max_inflight = 1;
    s->device = dev->id;
    for (uint32_t i = 0; i < s->opt.max_inflight; ++i) {
        cudaStream_t st2;
        CU(cudaStreamCreateWithFlags(&st2, cudaStreamNonBlocking));
        s->streams.push_back(st2);
        s->slot_busy.push_back(false);
    }
    tgpu_server *raw = s.get();
    s->th = std::thread([raw] { raw->run(); });
    *out = s.release();
    return TGPU_OK;
}

tgpu_status tgpu_server_submit(tgpu_server *s, uint32_t table, const tgpu_request *req, uint64_t *ticket) {
    if (!s || !req || !ticket) return fail(TGPU_ERR_INVALID_ARGUMENT, "null argument");
    if (table >= s->tables.size()) return fail(TGPU_ERR_INVALID_ARGUMENT, "table index");
    std::unique_ptr<Ticket> tk(new Ticket());
    tk->table = table;
    tk->req.set(*req);
    tgpu_status st = estimate_bytes(s->tables[table], &tk->req.r, &tk->est_bytes);
    if (st != TGPU_OK) return st;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        tk->id = s->next_id++;
        tk->submitted = Clock::now();
        *ticket = tk->id;
        s->pending.push_back(tk.get());
        s->stats.submitted++;
        s->stats.peak_queued = std::max<uint64_t>(s->stats.peak_queued, s->pending.size());
        s->tickets[tk->id] = std::move(tk);
    }
    s->cv_submit.notify_one();
    return TGPU_OK;
}

tgpu_status tgpu_server_wait(tgpu_server *s, uint64_t ticket, int32_t timeout_ms, int32_t *done) {
    if (!s || !done) return fail(TGPU_ERR_INVALID_ARGUMENT, "null argument");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return fail(TGPU_ERR_INVALID_ARGUMENT, "unknown ticket");
    Ticket *tk = it->second.get();
    if (timeout_ms < 0) s->cv_done.wait(lk, [&] { return tk->state == 2; });
    else s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return tk->state == 2; });
    *done = tk->state == 2 ? 1 : 0;
    return TGPU_OK;
}

tgpu_status tgpu_server_output_schema(tgpu_server *s, uint64_t ticket, tgpu_output_column *cols, uint32_t cap,
                                      uint32_t *n) {
    if (!s) return fail(TGPU_ERR_INVALID_ARGUMENT, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end() || it->second->state != 2) return fail(TGPU_ERR_INVALID_ARGUMENT, "ticket not done");
    Ticket *tk = it->second.get();
    if (tk->status != TGPU_OK) return fail(tk->status, tk->error);
    if (n) *n = (uint32_t)tk->schema.size();
    for (uint32_t i = 0; cols && i < cap && i < tk->schema.size(); ++i) cols[i] = tk->schema[i];
    return TGPU_OK;
}

tgpu_status tgpu_server_next(tgpu_server *s, uint64_t ticket, tgpu_batch *b, int32_t *done) {
    if (!s || !b || !done) return fail(TGPU_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end() || it->second->state != 2) return fail(TGPU_ERR_INVALID_ARGUMENT, "ticket not done");
    Ticket *tk = it->second.get();
    if (tk->status != TGPU_OK) return fail(tk->status, tk->error);
    if (b->n_columns != tk->schema.size()) return fail(TGPU_ERR_INVALID_ARGUMENT, "batch column count");
    const uint64_t n = std::min<uint64_t>(b->capacity_rows, tk->rows - tk->returned);
    for (size_t c = 0; c < tk->schema.size(); ++c) {
        const size_t eb = tk->schema[c].elem_bytes;
        if (n && b->values && b->values[c]) std::memcpy(b->values[c], tk->data[c].data() + tk->returned * eb, n * eb);
        if (n && b->validity && b->validity[c]) {
            std::memset(b->validity[c], 0, (n + 7) / 8);
            for (uint64_t r = 0; r < n; ++r)
                if (tk->valid[c][tk->returned + r]) b->validity[c][r >> 3] |= (uint8_t)(1u << (r & 7));
        }
    }
    tk->returned += n;
    b->row_count = n;
    *done = tk->returned >= tk->rows ? 1 : 0;
    return TGPU_OK;
}

tgpu_status tgpu_server_release(tgpu_server *s, uint64_t ticket) {
    if (!s) return fail(TGPU_ERR_INVALID_ARGUMENT, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return fail(TGPU_ERR_INVALID_ARGUMENT, "unknown ticket");
    if (it->second->state != 2) return fail(TGPU_ERR_INVALID_ARGUMENT, "ticket still running");
    s->tickets.erase(it);
    return TGPU_OK;
}

tgpu_status tgpu_server_get_stats(tgpu_server *s, tgpu_server_stats *out) {
    if (!s || !out) return fail(TGPU_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    return TGPU_OK;
}

tgpu_status tgpu_server_destroy(tgpu_server *s) {
    if (!s) return fail(TGPU_ERR_INVALID_ARGUMENT, "null server");
    delete s;
    return TGPU_OK;
}

tgpu_status tgpu_server_run_load(tgpu_server *s, const tgpu_load_spec *spec, tgpu_load_report *out) {
    if (!s || !spec || !out || !spec->n_requests || spec->rate_qps <= 0)
        return fail(TGPU_ERR_INVALID_ARGUMENT, "bad load spec");
    std::mt19937_64 rng(spec->seed);
    std::exponential_distribution<double> gap(spec->rate_qps);
    std::uniform_int_distribution<uint32_t> pick(0, spec->n_requests - 1);
    std::vector<uint64_t> ids;
    const auto t0 = Clock::now();
    auto next = t0;
    const auto end = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(spec->duration_s));
    while (next < end) {
        // open loop: each arrival is scheduled from the previous arrival time, not from completions
        while (Clock::now() < next) std::this_thread::yield();
        uint32_t j = pick(rng);
        uint64_t id = 0;
        tgpu_status st = tgpu_server_submit(s, spec->table_of ? spec->table_of[j] : 0, &spec->requests[j], &id);
        if (st != TGPU_OK) return st;
        ids.push_back(id);
        next += std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(gap(rng)));
    }
    std::vector<double> lat;
    lat.reserve(ids.size());
    uint64_t failed = 0;
    Clock::time_point first = Clock::time_point::max(), last = t0;
    for (uint64_t id : ids) {
        int32_t done = 0;
        tgpu_status st = tgpu_server_wait(s, id, 600000, &done);
        if (st != TGPU_OK) return st;
        if (!done) return fail(TGPU_ERR_DEVICE_TIMEOUT, "a request did not finish within 600 s");
        std::lock_guard<std::mutex> lk(s->mu);
        Ticket *tk = s->tickets[id].get();
        lat.push_back(std::chrono::duration<double, std::milli>(tk->done_at - tk->submitted).count());
        if (tk->status != TGPU_OK) ++failed;
        first = std::min(first, tk->submitted);
        last = std::max(last, tk->done_at);
    }
    for (uint64_t id : ids) tgpu_server_release(s, id);
    std::sort(lat.begin(), lat.end());
    auto pct = [&](double p) {
        if (lat.empty()) return 0.0;
        size_t i = (size_t)std::ceil(p * lat.size()) - 1;
        return lat[std::min(i, lat.size() - 1)];
    };
    std::memset(out, 0, sizeof(*out));
    out->submitted = ids.size();
    out->completed = lat.size();
    out->failed = failed;
    out->elapsed_s = lat.empty() ? 0 : std::chrono::duration<double>(last - first).count();
    out->achieved_qps = out->elapsed_s > 0 ? (double)lat.size() / out->elapsed_s : 0;
    out->p50_ms = pct(0.50);
    out->p99_ms = pct(0.99);
    out->p999_ms = pct(0.999);
    out->max_ms = lat.empty() ? 0 : lat.back();
    double sum = 0;
    for (double x : lat) sum += x;
    out->mean_ms = lat.empty() ? 0 : sum / lat.size();
    return TGPU_OK;
}

}  // extern "C"

// ================================================================ tuning ==

extern "C" {

tgpu_status tgpu_request_shape(tgpu_table *table, const tgpu_request *req, int32_t batched, tgpu_shape *out) {
    if (!table || !req || !out) return fail(TGPU_ERR_INVALID_ARGUMENT, "null argument");
    std::unique_ptr<tgpu_query> q(new tgpu_query());
    q->t = table;
    q->flags = req->flags;
    q->limit = req->limit;
    q->offset = req->offset;
    tgpu_status st = plan_query(q.get(), table, req);
    if (st != TGPU_OK) return st;
    *out = shape_of(q.get(), req, batched);
    return TGPU_OK;
}

tgpu_status tgpu_tuning_set(const tgpu_tuning *entries, uint32_t n) {
    if (n && !entries) return fail(TGPU_ERR_INVALID_ARGUMENT, "null entries");
    for (uint32_t i = 0; i < n; ++i) {
        const tgpu_tuning &t = entries[i];
        if (t.chunk_rows < 0 || t.chunk_rows % CHUNK_ALIGN != 0 || t.chunk_rows > 65536 ||
            (t.cache_slots > 0 && (t.cache_slots & (t.cache_slots - 1))) || t.cache_slots < -1 ||
            t.table_load_pct < 0 || t.table_load_pct > 90 || t.groups_shift < 0 || t.groups_shift > 8)
            return fail(TGPU_ERR_INVALID_ARGUMENT, "tuning entry out of range");
    }
    std::lock_guard<std::mutex> lk(g_tuning_mu);
    g_tuning.assign(entries, entries + n);
    return TGPU_OK;
}

uint32_t tgpu_tuning_get(tgpu_tuning *entries, uint32_t cap) {
    std::lock_guard<std::mutex> lk(g_tuning_mu);
    for (uint32_t i = 0; entries && i < cap && i < g_tuning.size(); ++i) entries[i] = g_tuning[i];
    return (uint32_t)g_tuning.size();
}

}  // extern "C"
