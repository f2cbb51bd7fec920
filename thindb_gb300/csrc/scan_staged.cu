// scan_staged.cu — the staged scan: every column the query reads streams
// through shared memory in tiles brought by bulk asynchronous copies
// (cp.async.bulk completing on an mbarrier), and the WHERE, the key packing
// and the fold all read from there.
//
// Why: with a selective WHERE the survivors still touch nearly every 128-byte
// line of the key and input columns, so late materialisation saves no DRAM
// bytes, while a warp that filters, then gathers, then folds waits on DRAM
// at every step.  Here one thread keeps S - 1 tiles of copies in flight per
// CTA whatever the warps are doing, so the column stream runs at the copy
// engine's pace and the warps only wait on the group table (L2).
//
// Per CTA (one per SM, 16 warps), for each of its tiles i (tile b + i * grid):
//   1. wait for stage i % S (bounded; ST_WAIT_TIMEOUT if it never lands);
//   2. every warp tests 32 rows at a time against the fast range predicate
//      and appends the survivors' packed key and inputs to the CTA's fold
//      queue (warp-aggregated shared atomic), prefetching each row's
//      group-table slot (and distinct-set entry) into L2;
//   3. barrier; thread 0 refills stage i % S with tile i + S;
//   4. once the queue holds STAGE_FOLD_AT rows, every warp folds full
//      32-row batches from it with the query's compiled fold (warp
//      pre-combine, shared-memory hot-key table, global table), and the
//      remainder (< 32 rows) moves to the queue's front.
// A partial last tile (the table's last rows) is copied with plain loads.
#include <algorithm>

#include "bulk.cuh"
#include "scan_impl.cuh"

namespace tgpu {

namespace {

constexpr int STAGE_WARPS = STAGE_THREADS / 32;

// First row and row count of tile t (0 rows: past the table's end).
__device__ __forceinline__ void tile_rows(const DevQuery &q, const StagePlan &sp, uint32_t t, uint64_t &row0,
                                          uint32_t &rows) {
    const uint32_t rgi = t / sp.tiles_per_rg, sub = t % sp.tiles_per_rg;
    const uint64_t rg = q.rg_list ? q.rg_list[rgi] : rgi;
    row0 = rg * q.rg_rows + (uint64_t)sub * STAGE_TILE;
    const uint64_t end = min(min(row0 + STAGE_TILE, (rg + 1) * (uint64_t)q.rg_rows), q.n_rows);
    rows = end > row0 ? (uint32_t)(end - row0) : 0;
}

// Thread 0: start tile t into stage buffer `stage`, completing on `bar`.
// A full tile is one bulk copy per staged column; a partial one completes
// the phase at once and the warps copy its rows themselves.
__device__ void issue_tile(const DevQuery &q, const StagePlan &sp, uint32_t t, unsigned char *stage, uint64_t *bar) {
    uint64_t row0;
    uint32_t rows;
    tile_rows(q, sp, t, row0, rows);
    if (rows != STAGE_TILE) {
        mbar_arrive_tx(bar, 0);
        return;
    }
    mbar_arrive_tx(bar, sp.stage_bytes);
    for (uint32_t i = 0; i < sp.n_cols; ++i) {
        const DevCol &c = q.cols[sp.col[i]];
        bulk_load(stage + sp.off[i], (const unsigned char *)c.data + row0 * (uint64_t)c.bytes,
                  STAGE_TILE * (uint32_t)c.bytes, bar);
    }
}

// Plain copy of a partial tile's rows into its stage (all threads).
__device__ void copy_partial(const DevQuery &q, const StagePlan &sp, uint64_t row0, uint32_t rows,
                             unsigned char *stage) {
    for (uint32_t i = 0; i < sp.n_cols; ++i) {
        const DevCol &c = q.cols[sp.col[i]];
        const uint32_t n = rows * (uint32_t)c.bytes;
        const unsigned char *src = (const unsigned char *)c.data + row0 * (uint64_t)c.bytes;
        for (uint32_t b = threadIdx.x; b < n; b += blockDim.x) stage[sp.off[i] + b] = src[b];
    }
}

// Sign-extended integer of staged column slot `si` at tile row r (BOOLEAN zero-extended).
__device__ __forceinline__ int64_t st_int(const DevCol &c, const unsigned char *p, uint32_t r) {
    switch (c.bytes) {
        case 1: return c.type == TGPU_BOOLEAN ? (int64_t)p[r] : (int64_t)(int8_t)p[r];
        case 2: return (int64_t)((const int16_t *)p)[r];
        case 4: return (int64_t)((const int32_t *)p)[r];
        default: return ((const int64_t *)p)[r];
    }
}

__device__ __forceinline__ double st_f64(const DevCol &c, const unsigned char *p, uint32_t r) {
    if (c.bytes == 4) return (double)((const float *)p)[r];
    return ((const double *)p)[r];
}

// Tile row r as the fold's row: packed key + inputs (FastFold::load over the stage).
template <class P>
__device__ __forceinline__ void stage_row(const DevQuery &q, const StagePlan &sp, const unsigned char *stage,
                                          uint32_t r, typename P::Row &rv) {
    rv = typename P::Row{};  // zero keys and inputs; a COUNT(DISTINCT) row unreserved
    rv.k0 = 0;
    rv.k1 = 0;
#pragma unroll
    for (int a = 0; a < P::NV; ++a) rv.val[a] = 0;
    if (P::KM_ == 1) {
        const DevKeyPart &kp = q.parts[0];
        const uint64_t raw = (uint64_t)st_int(q.cols[kp.col], stage + sp.off[sp.slot[kp.col]], r);
        rv.k0 = kp.payload < 64 ? (raw & ((1ULL << kp.payload) - 1)) : raw;
    } else {
        for (int i = 0; i < q.n_parts; ++i) {
            const DevKeyPart &kp = q.parts[i];
            uint64_t raw = (uint64_t)st_int(q.cols[kp.col], stage + sp.off[sp.slot[kp.col]], r);
            if (kp.payload < 64) raw &= (1ULL << kp.payload) - 1;
            const int off = kp.offset;
            if (off < 64) {
                rv.k0 |= raw << off;
                if (off > 0) rv.k1 |= raw >> (64 - off);
            } else {
                rv.k1 |= raw << (off - 64);
            }
        }
    }
#pragma unroll
    for (int a = 0; a < P::NA_; ++a) {
        const int col = q.faggs[a].col;
        const unsigned char *p = stage + sp.off[sp.slot[col]];
        rv.val[a] = P::is_f(a) ? f64_bits(st_f64(q.cols[col], p, r)) : (uint64_t)st_int(q.cols[col], p, r);
    }
}

// The fast range predicate on tile row r.
__device__ __forceinline__ bool stage_pass(const DevQuery &q, const unsigned char *p, uint32_t r) {
    int64_t x;
    switch (q.fp_bytes) {
        case 1: x = (int64_t)(int8_t)p[r]; break;
        case 2: x = (int64_t)((const int16_t *)p)[r]; break;
        case 4: x = (int64_t)((const int32_t *)p)[r]; break;
        default: x = ((const int64_t *)p)[r]; break;
    }
    return (x >= q.fp_lo && x <= q.fp_hi) != (q.fp_negate != 0);
}

// Fold rows [0, n) of the queue: batch b by warp b % 16.  Returns the rows
// left (n % 32 unless `all`).
template <class P>
__device__ __forceinline__ void fold_queue(const DevQuery &q, const ScanSmem &sm, typename P::Row *queue, uint32_t n,
                                           bool all) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t nb = all ? (n + 31) / 32 : n / 32;
    for (uint32_t b = warp; b < nb; b += STAGE_WARPS) {
        const uint32_t i = b * 32 + lane;
        const uint32_t left = n - b * 32;
        const unsigned act = left >= 32 ? 0xFFFFFFFFu : ((1u << left) - 1);
        typename P::Row rv = queue[i < n ? i : 0];
        P::fold(q, sm, rv, act);
    }
}

template <class P>
__global__ void __launch_bounds__(STAGE_THREADS, 1)
    staged_scan_kernel(const __grid_constant__ DevQuery q, const __grid_constant__ StagePlan sp) {
    extern __shared__ __align__(128) unsigned char smem[];
    using Row = typename P::Row;
    uint64_t *bars = (uint64_t *)smem;
    const ScanSmem sm = carve(q, smem + sp.cache_off);
    static_assert(sizeof(Row) <= 24 + 8 * P::NV, "fold-queue rows sized in stage_plan");
    Row *queue = (Row *)(smem + sp.queue_off);
    unsigned char *ring = smem + sp.ring_off;
    __shared__ uint32_t queue_n;
    __shared__ int stop;

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t G = gridDim.x;
    const uint32_t my_n = sp.n_tiles > blockIdx.x ? (sp.n_tiles - blockIdx.x + G - 1) / G : 0;
    const uint32_t S = sp.stages;

    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < S; ++s) mbar_init(&bars[s]);
        mbar_init_fence();
        queue_n = 0;
        stop = 0;
    }
    cache_init(q, sm);
    __syncthreads();
    uint32_t issued = 0;  // thread 0's count of tiles started
    if (threadIdx.x == 0) {
        for (; issued < S && issued < my_n; ++issued)
            issue_tile(q, sp, blockIdx.x + issued * G, ring + (size_t)issued * sp.stage_bytes, &bars[issued]);
    }

    unsigned long long selected = 0;
    uint32_t i = 0;
    for (; i < my_n; ++i) {
        const uint32_t s = i % S;
        unsigned char *stage = ring + (size_t)s * sp.stage_bytes;
        if (!mbar_wait(&bars[s], (i / S) & 1u, q.wait_cycles)) {
            atomicOr(q.status, ST_WAIT_TIMEOUT);
            stop = 1;
        }
        if (threadIdx.x == 0 && q.cancel && (i & 63) == 63 && *q.cancel) {
            atomicOr(q.status, ST_CANCELLED);
            stop = 1;
        }
        __syncthreads();
        if (stop) break;
        uint64_t row0;
        uint32_t rows;
        tile_rows(q, sp, blockIdx.x + i * G, row0, rows);
        if (rows != STAGE_TILE) {
            copy_partial(q, sp, row0, rows, stage);
            __syncthreads();
        }
        // filter + append survivors to the fold queue
        const unsigned char *pred = q.fp_bytes ? stage + sp.off[sp.slot[q.preds[0].col]] : nullptr;
        for (uint32_t base = warp * 32; base < rows; base += STAGE_THREADS) {
            const uint32_t r = base + lane;
            const bool pass = r < rows && (pred == nullptr || stage_pass(q, pred, r));
            const unsigned m = __ballot_sync(0xFFFFFFFFu, pass);
            if (m == 0) continue;
            Row rv{};
            if (pass) stage_row<P>(q, sp, stage, r, rv);
            const bool kp = P::prefetch(q, rv, pass);  // less any row the count sketch drops
            const unsigned mk = __ballot_sync(0xFFFFFFFFu, kp);
            uint32_t pos = 0;
            if (lane == 0) {
                pos = mk ? atomicAdd(&queue_n, (uint32_t)__popc(mk)) : 0u;
                selected += __popc(m);
            }
            pos = __shfl_sync(0xFFFFFFFFu, pos, 0);
            if (kp) {
                const uint32_t at = pos + __popc(mk & ((1u << lane) - 1));
                if (at < STAGE_QCAP) queue[at] = rv;
                else atomicOr(q.status, ST_BAD_INDEX);  // cannot happen: <= FOLD_AT - 1 + one tile
            }
        }
        __syncthreads();
        // the stage is consumed: refill it with tile i + S
        if (threadIdx.x == 0 && issued < my_n) {
            fence_proxy_async_smem();
            issue_tile(q, sp, blockIdx.x + issued * G, ring + (size_t)(issued % S) * sp.stage_bytes,
                       &bars[issued % S]);
            ++issued;
        }
        const uint32_t n = queue_n;
        if (n >= STAGE_FOLD_AT) {
            fold_queue<P>(q, sm, queue, n, false);
            __syncthreads();
            const uint32_t keep = n % 32, from = n - keep;
            if (threadIdx.x < keep) queue[threadIdx.x] = queue[from + threadIdx.x];
            if (threadIdx.x == 0) queue_n = keep;
            __syncthreads();
        }
    }
    if (stop) {
        // leave no copy in flight into this CTA's shared memory (bounded by
        // the built-in limit, whatever the query's: the copies are real and land)
        if (threadIdx.x == 0)
            for (uint32_t j = i; j < issued; ++j) (void)mbar_wait(&bars[j % S], (j / S) & 1u);
        __syncthreads();
    } else {
        fold_queue<P>(q, sm, queue, queue_n, true);
    }
    if (q.cache_slots) {
        __syncthreads();
        cache_flush(q, sm);
    }
    if (lane == 0 && selected) atomicAdd(q.selected_rows, selected);
}

using StagedFn = const void *;

template <class P>
StagedFn staged_of() {
    return (const void *)staged_scan_kernel<P>;
}

StagedFn pick_staged(const DevQuery &q) {
    switch (q.fast_id) {
#define TGPU_STAGED(I, KM, A, B, C2, D) \
    case I: return staged_of<FastFold<KM, A, B, C2, D>>();
        TGPU_FAST_FOLDS(TGPU_STAGED)
#undef TGPU_STAGED
        default: return nullptr;
    }
}

}  // namespace

bool stage_plan(DevQuery &q, uint64_t tile_count, StagePlan *sp) {
    if (q.fast_id < 0 || (q.n_preds > 0 && q.fp_bytes == 0) || q.rg_rows % STAGE_TILE != 0) return false;
    int cache_slots = q.cache_slots, cache_probe = q.cache_probe;
    StagePlan p{};
    for (int c = 0; c < MAX_QCOLS; ++c) p.slot[c] = -1;
    auto use = [&](int c) {
        if (c < 0 || p.slot[c] >= 0) return true;
        const DevCol &col = q.cols[c];
        if (col.valid || ((uintptr_t)col.data & 15)) return false;
        p.slot[c] = (int32_t)p.n_cols;
        p.col[p.n_cols] = c;
        p.off[p.n_cols] = p.stage_bytes;
        p.stage_bytes += STAGE_TILE * (uint32_t)col.bytes;
        ++p.n_cols;
        return true;
    };
    bool ok = q.n_preds == 0 || use(q.preds[0].col);
    for (int i = 0; ok && i < q.n_parts; ++i) ok = use(q.parts[i].col);
    for (int a = 0; ok && a < q.n_faggs; ++a) ok = use(q.faggs[a].col);
    if (!ok || p.n_cols == 0) return false;
    p.n_tiles = (uint32_t)tile_count;
    p.tiles_per_rg = q.rg_rows / STAGE_TILE;
    // two key words, one word per input, a COUNT(DISTINCT) row's reserved
    // pair place (FastFold::Row; 8 bytes, counted for every fold)
    p.row_bytes = 24 + 8 * (uint32_t)(q.n_faggs > 0 ? q.n_faggs : 1);
    // shared memory: barriers | hot-key cache | fold queue | ring of stages
    const uint32_t budget = 220 * 1024;
    const uint32_t queue_bytes = STAGE_QCAP * p.row_bytes;
    auto cache_bytes = [&](int c) { return (uint32_t)c * (12u + 8u * (uint32_t)q.state_words); };
    while (cache_slots > 0 && 128 + cache_bytes(cache_slots) + queue_bytes + 4 * p.stage_bytes > budget) {
        // a resident (every-group) table that no longer fits stops being resident
        const bool resident = cache_probe == cache_slots;
        cache_slots >>= 1;
        cache_probe = resident ? 16 : std::min(cache_probe, cache_slots);
        if (cache_slots < 64 || (resident && q.needs_gid)) cache_slots = cache_probe = 0;
    }
    p.cache_off = 128;
    p.queue_off = (p.cache_off + cache_bytes(cache_slots) + 127) & ~127u;
    p.ring_off = (p.queue_off + queue_bytes + 127) & ~127u;
    if (p.ring_off + 2 * p.stage_bytes > budget) return false;
    p.stages = std::min<uint32_t>(8, (budget - p.ring_off) / p.stage_bytes);
    p.smem_bytes = p.ring_off + p.stages * p.stage_bytes;
    q.cache_slots = cache_slots;
    q.cache_probe = cache_probe;
    *sp = p;
    return true;
}

cudaError_t launch_staged_scan(const DevQuery &q, const StagePlan &sp, int grid, cudaStream_t s) {
    const void *fn = pick_staged(q);
    if (!fn) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sp.smem_bytes);
    if (e != cudaSuccess) return e;
    void *args[] = {(void *)&q, (void *)&sp};
    return cudaLaunchKernel(fn, dim3(grid), dim3(STAGE_THREADS), args, sp.smem_bytes, s);
}

}  // namespace tgpu
