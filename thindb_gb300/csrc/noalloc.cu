// noalloc.cu — a GROUP BY entry point that allocates no memory.
//
// Some callers cannot let a library allocate device memory: an embedding
// host that hands the GPU to a fixed memory arena up front, a plugin running
// inside another runtime's pre-reserved pool, or a caller that must not block
// on cudaMalloc/cudaFree (which can synchronise the device) in a
// latency-critical loop.  tgpu_group_by_i64_noalloc runs the same fused scan
// + fold kernel and the same compaction / gather kernels as the regular
// operator, but its group table, occupancy bitmap, id list and bookkeeping
// live in one fixed file-scope device array below.  The caller passes its
// input columns and output buffers (device memory); the function calls no
// cudaMalloc, cudaFree or allocating library routine.
//
// The array is loaded with the library on every GPU that runs it and stays
// resident until the process exits.  All calls share it: calls that overlap
// on the GPU (different streams, or other threads) race and corrupt each
// other's results, so callers serialise them.
#include <mutex>

#include "common.cuh"

namespace tgpu {

namespace {

constexpr uint64_t NA_MAX_GROUPS = 65536;              // at most this many result groups
constexpr uint64_t NA_CAP = 131072;                    // table slots (load <= 0.5)
constexpr int NA_SLOT_WORDS = 8;                       // key, rows, sum lo/hi, min, max (+2 spare)
constexpr uint64_t NA_SLOTS = NA_CAP + 1;
constexpr uint64_t NA_TABLE_WORDS = NA_SLOTS * NA_SLOT_WORDS;
constexpr uint64_t NA_OCC_WORDS = ((NA_SLOTS + 31) / 32 + 1) / 2;      // u32 bitmap, counted in u64
constexpr uint64_t NA_GID_WORDS = (NA_SLOTS + 1) / 2;                  // u32 ids
constexpr uint64_t NA_BC_WORDS = 64;                                   // compaction block counts (u32)
constexpr uint64_t NA_MISC_WORDS = 64;                                 // counts, control, pointer arrays
constexpr uint64_t NA_VALID_WORDS = (5 * NA_SLOTS + 7) / 8;            // validity bytes of the 5 outputs
constexpr uint64_t NA_WORDS =
    NA_TABLE_WORDS + NA_OCC_WORDS + NA_GID_WORDS + NA_BC_WORDS + NA_MISC_WORDS + NA_VALID_WORDS;

// The scratch: about 9.6 MB.
static __device__ __align__(256) unsigned long long g_noalloc_scratch[NA_WORDS];

struct Layout {
    unsigned long long *table;
    uint32_t *occ;
    uint32_t *gids;
    uint32_t *block_counts;
    unsigned long long *counts;  // [0..4] as the regular operator's counts
    unsigned int *ctrl;          // [0] unused, [1] status
    void **out_ptrs;             // 5 output column pointers
    uint8_t **valid_ptrs;        // 5 validity buffers (in the scratch)
    uint8_t *valid;
};

Layout layout_of(unsigned long long *base) {
    Layout l;
    unsigned long long *p = base;
    l.table = p;
    p += NA_TABLE_WORDS;
    l.occ = (uint32_t *)p;
    p += NA_OCC_WORDS;
    l.gids = (uint32_t *)p;
    p += NA_GID_WORDS;
    l.block_counts = (uint32_t *)p;
    p += NA_BC_WORDS;
    l.counts = p;
    l.ctrl = (unsigned int *)(p + 8);
    l.out_ptrs = (void **)(p + 16);
    l.valid_ptrs = (uint8_t **)(p + 24);
    p += NA_MISC_WORDS;
    l.valid = (uint8_t *)p;
    return l;
}

// Device address of the scratch, per device (host code cannot use the
// array's name as a device address).
std::mutex g_na_mu;
unsigned long long *g_na_addr[64] = {nullptr};

}  // namespace

}  // namespace tgpu

using namespace tgpu;

extern "C" {

// No counterpart in thinDB: an allocation-free variant of the GROUP BY
// operator for callers that cannot allocate device memory.  See
// include/thindb_gpu.h for the contract.
tgpu_status tgpu_group_by_i64_noalloc(const int64_t *keys, const int64_t *values, uint64_t n_rows,
                                      int64_t *out_keys, int64_t *out_count, int64_t *out_sum, int64_t *out_min,
                                      int64_t *out_max, uint64_t *out_groups, void *stream) {
    if ((n_rows && (!keys || !values)) || !out_keys || !out_count || !out_sum || !out_min || !out_max ||
        !out_groups) {
        set_error("tgpu_group_by_i64_noalloc: null input or output pointer");
        return TGPU_ERR_INVALID_ARGUMENT;
    }
    if (n_rows > (uint64_t)0xFFFFFFFFu * 1024) {
        set_error("tgpu_group_by_i64_noalloc: more rows than the chunk index covers");
        return TGPU_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        set_error("tgpu_group_by_i64_noalloc: no usable CUDA device");
        return TGPU_ERR_NO_DEVICE;
    }
    unsigned long long *base;
    {
        // first call on this device: look up the scratch's device address.
        // Nothing is zeroed here: every call clears the table, bitmap and
        // counters it reads on its own stream below, and the rest of the
        // array is written before it is read.
        std::lock_guard<std::mutex> lk(g_na_mu);
        if (!g_na_addr[dev]) {
            unsigned long long *p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                cudaGetLastError();
                set_error(e != cudaSuccess ? cudaGetErrorString(e)
                                           : "tgpu_group_by_i64_noalloc: the scratch array has no device address");
                return TGPU_ERR_CUDA;
            }
            g_na_addr[dev] = p;
        }
        base = g_na_addr[dev];
    }
    const Layout L = layout_of(base);

    // the query: GROUP BY keys, COUNT(*), SUM(values) (BIGINT, wraps), MIN, MAX
    DevQuery q;
    memset(&q, 0, sizeof(q));
    q.n_rows = n_rows;
    q.rg_rows = 65536;
    q.n_rg = (uint32_t)((n_rows + 65535) / 65536);
    q.chunk_rows = 1024;
    q.n_chunks = (uint32_t)((n_rows + q.chunk_rows - 1) / q.chunk_rows);
    q.cols[0] = DevCol{keys, nullptr, nullptr, TGPU_BIGINT, 8};
    q.cols[1] = DevCol{values, nullptr, nullptr, TGPU_BIGINT, 8};
    q.n_cols = 2;
    q.parts[0] = DevKeyPart{0, 0, 64, 0};
    q.n_parts = 1;
    q.key_words = 1;
    q.aggs[0] = DevAgg{AK_COUNT_ROWS, -1, 0, -1, 0, 0, 1, 0};
    const int32_t sum_kind = n_rows < (1ULL << 32) ? AK_SUM_I128 : AK_SUM_I128C;  // carry-free below 2^32 rows
    q.aggs[1] = DevAgg{sum_kind, 1, 1, -1, 0, 0, 1, 1};
    q.aggs[2] = DevAgg{AK_MIN_I, 1, 3, -1, 0, 0, 1, 1};
    q.aggs[3] = DevAgg{AK_MAX_I, 1, 4, -1, 0, 0, 1, 1};
    q.n_aggs = 4;
    // the compiled fold the regular operator picks for this shape
    q.fast_km = 1;
    q.n_faggs = 3;
    q.faggs[0] = q.aggs[1];
    q.faggs[1] = q.aggs[2];
    q.faggs[2] = q.aggs[3];
    q.fast_id = fast_fold_id(q);
    q.state_words = 5;
    q.slot_words = NA_SLOT_WORDS;
    q.table = L.table;
    q.cap = NA_CAP;
    q.occ = L.occ;
    q.cache_slots = 2048;
    q.cache_probe = 16;
    q.warp_combine = 1;
    q.tile_counter = L.ctrl;
    q.status = L.ctrl + 1;
    q.selected_rows = L.counts + 4;

    DevFinal f;
    memset(&f, 0, sizeof(f));
    f.table = L.table;
    f.cap = NA_CAP;
    f.occ = L.occ;
    f.key_words = 1;
    f.slot_words = NA_SLOT_WORDS;
    f.n_parts = 1;
    f.n_aggs = 4;
    f.sort_words = 2;
    f.parts[0] = q.parts[0];
    f.part_types[0] = TGPU_BIGINT;
    f.outs[0] = DevOut{TGPU_AGG_COUNT, AK_COUNT_ROWS, 0, -1, TGPU_BIGINT, 0, 0, 0};
    f.outs[1] = DevOut{TGPU_AGG_SUM, sum_kind, 1, -1, TGPU_BIGINT, TGPU_BIGINT, 0, 0};
    f.outs[2] = DevOut{TGPU_AGG_MIN, AK_MIN_I, 3, -1, TGPU_BIGINT, TGPU_BIGINT, 0, 0};
    f.outs[3] = DevOut{TGPU_AGG_MAX, AK_MAX_I, 4, -1, TGPU_BIGINT, TGPU_BIGINT, 0, 0};

    void *outs[5] = {out_keys, out_count, out_sum, out_min, out_max};
    uint8_t *valid[5];
    for (int c = 0; c < 5; ++c) valid[c] = L.valid + (size_t)c * NA_SLOTS;

#define NA_TRY(call)                                                   \
    do {                                                               \
        cudaError_t e_ = (call);                                       \
        if (e_ != cudaSuccess) {                                       \
            cudaGetLastError();                                        \
            set_error(cudaGetErrorString(e_));                         \
            return TGPU_ERR_CUDA;                                      \
        }                                                              \
    } while (0)
    // every call starts from a zeroed table, bitmap and counters
    NA_TRY(cudaMemsetAsync(L.table, 0, NA_TABLE_WORDS * 8, s));
    NA_TRY(cudaMemsetAsync(L.occ, 0, NA_OCC_WORDS * 8, s));
    NA_TRY(cudaMemsetAsync(L.counts, 0, NA_MISC_WORDS * 8, s));
    NA_TRY(cudaMemcpyAsync(L.out_ptrs, outs, sizeof(outs), cudaMemcpyHostToDevice, s));
    NA_TRY(cudaMemcpyAsync(L.valid_ptrs, valid, sizeof(valid), cudaMemcpyHostToDevice, s));
    int sms = 0;
    NA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (q.n_chunks) NA_TRY(launch_scan(q, scan_grid_size(q, sms), s));
    const uint32_t nb = compact_blocks(NA_CAP);
    NA_TRY(launch_compact(f, L.block_counts, nb, L.gids, L.counts, s));
    NA_TRY(launch_sel_all(L.counts, s));
    NA_TRY(launch_gather(f, L.gids, L.counts, 0, NA_MAX_GROUPS, L.out_ptrs, L.valid_ptrs, s));
    NA_TRY(cudaMemcpyAsync(out_groups, L.counts + 2, 8, cudaMemcpyDeviceToDevice, s));
    // the status and group count decide the return value: read them back
    unsigned long long groups = 0;
    unsigned int status = 0;
    NA_TRY(cudaMemcpyAsync(&groups, L.counts, 8, cudaMemcpyDeviceToHost, s));
    NA_TRY(cudaMemcpyAsync(&status, L.ctrl + 1, 4, cudaMemcpyDeviceToHost, s));
    NA_TRY(cudaStreamSynchronize(s));
#undef NA_TRY
    if (groups > NA_MAX_GROUPS) {
        set_error("tgpu_group_by_i64_noalloc: more than 65,536 distinct keys; its fixed scratch holds at most "
                  "65,536 groups (use tgpu_query_create for larger results)");
        return TGPU_ERR_INVALID_ARGUMENT;
    }
    if (status & ST_TABLE_FULL) {
        // at most 65,536 groups, yet a bounded probe ran past its limit
        // (keys whose hashes cluster): not a size the caller chose
        set_error("tgpu_group_by_i64_noalloc: a group-table probe ran past its limit (clustered key hashes); "
                  "use tgpu_query_create, which regrows its table");
        return TGPU_ERR_INTERNAL;
    }
    if (status) {
        set_error("tgpu_group_by_i64_noalloc: a device bounds check failed");
        return TGPU_ERR_INTERNAL;
    }
    return TGPU_OK;
}

}  // extern "C"
