// scan_pipe.cu — the pipelined scan: warp-specialised producer and consumers
// over a shared-memory ring of bulk asynchronous copies.
//
// thinDB's grid scan (silo_group_core.zig runGridScanBurst :10705 ->
// appendBatchRawChunks :5364 -> groupChunkRowsDirectKeys :7456 ->
// foldKernel* :7832-8001) reads each row group's columns, evaluates the
// WHERE and folds the survivors.  On the GPU the cost of that loop is not the
// arithmetic but keeping enough column bytes in flight while warps also wait
// on the group table.  Here the two never share a warp:
//
//   * one producer warp per CTA keeps every consumer warp's next tiles of
//     PIPE_TILE rows of every scanned column in flight: one cp.async.bulk per
//     column per tile into a ring slot owned by that consumer, completing on
//     the slot's `full` mbarrier.  It polls the slots' `empty` mbarriers
//     without blocking, so a consumer busy folding never holds up the others'
//     refills (no head-of-line blocking, no CTA-wide barrier in the loop);
//   * PIPE_CWARPS consumer warps each own `depth` ring slots and take the
//     CTA's tiles round robin.  Per tile: wait for `full` (bounded), test the
//     WHERE 32 rows at a time from shared memory, append the survivors' packed
//     key and inputs to the warp's 64-row survivor ring (ballot + popc
//     positions) prefetching their group-table slots into L2, release the
//     slot (`empty` arrive), and fold every full 32-row batch with the
//     compiled fold (warp pre-combine, the CTA's shared-memory hot-key table,
//     the global table).  Without a WHERE every 32 rows fold as they come,
//     the next batch loaded and prefetched before the current one folds.
//
// Every wait is bounded (ST_WAIT_TIMEOUT); a consumer that gives up, a
// cancel, or a producer that sees no slot free up for the wait limit stops
// the CTA: consumers leave their loops, and the producer lets every copy it
// issued land (waiting with the built-in bound) before the CTA exits.
#include <algorithm>

#include "bulk.cuh"
#include "scan_impl.cuh"

namespace tgpu {

namespace {

constexpr int NCW = PIPE_CWARPS;
constexpr uint32_t PQ = 64;  // survivor ring rows per consumer warp (< 32 left + one 32-row step)
static_assert(PIPE_TILE <= 256, "survivor offsets of a tile are bytes");

struct PipeCtl {
    int stop;
    uint32_t consumed[NCW];  // tiles each consumer finished
    uint32_t issued[NCW];    // tiles the producer started for each consumer
};

// Rows [row0, row0 + rows) of tile t (rows = 0: past the table's end).
__device__ __forceinline__ void pipe_tile_rows(const DevQuery &q, const PipePlan &pp, uint32_t t, uint64_t &row0,
                                               uint32_t &rows) {
    const uint32_t rgi = t / pp.tiles_per_rg, sub = t % pp.tiles_per_rg;
    const uint64_t rg = q.rg_list ? q.rg_list[rgi] : rgi;
    row0 = rg * q.rg_rows + (uint64_t)sub * PIPE_TILE;
    const uint64_t end = min(min(row0 + PIPE_TILE, (rg + 1) * (uint64_t)q.rg_rows), q.n_rows);
    rows = end > row0 ? (uint32_t)(end - row0) : 0;
}

// One producer lane: start tile t into `stage`, completing on `bar`.  A
// full tile is one bulk copy per column (16-byte aligned and sized: the plan
// checks the column bases, and PIPE_TILE rows of any width are a multiple of
// 16 bytes).  A partial tile (the table's last rows) completes the phase at
// once and its consumer copies the rows itself.
__device__ __forceinline__ void pipe_issue(const DevQuery &q, const PipePlan &pp, uint32_t t, unsigned char *stage,
                                           uint64_t *bar) {
    uint64_t row0;
    uint32_t rows;
    pipe_tile_rows(q, pp, t, row0, rows);
    if (rows != PIPE_TILE) {
        mbar_arrive(bar);
        return;
    }
    fence_proxy_async_smem();  // the consumer's reads of this slot precede the copies into it
    mbar_arrive_tx(bar, pp.stage_bytes);
    for (uint32_t i = 0; i < pp.n_cols; ++i) {
        const DevCol &c = q.cols[pp.col[i]];
        bulk_load(stage + pp.off[i], (const unsigned char *)c.data + row0 * (uint64_t)c.bytes,
                  PIPE_TILE * (uint32_t)c.bytes, bar);
    }
}

// A consumer warp copies a partial tile's rows into its stage.
__device__ __noinline__ void pipe_copy_partial(const DevQuery &q, const PipePlan &pp, uint64_t row0, uint32_t rows,
                                               unsigned char *stage) {
    const int lane = threadIdx.x & 31;
    for (uint32_t i = 0; i < pp.n_cols; ++i) {
        const DevCol &c = q.cols[pp.col[i]];
        const uint32_t n = rows * (uint32_t)c.bytes;
        const unsigned char *src = (const unsigned char *)c.data + row0 * (uint64_t)c.bytes;
        unsigned char *dst = stage + pp.off[i];
        if ((n & 3) == 0 && ((uintptr_t)src & 3) == 0) {
            for (uint32_t b = lane; b < n / 4; b += 32) ((uint32_t *)dst)[b] = __ldg((const uint32_t *)src + b);
        } else {
            for (uint32_t b = lane; b < n; b += 32) dst[b] = __ldg(src + b);
        }
    }
    __syncwarp();
}

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

// Where a tile row's key and inputs sit in a stage (offsets and widths read
// once per kernel, not per row).
template <class P>
struct TileLayout {
    uint32_t key_off, key_bytes;
    uint64_t key_mask;
    uint32_t val_off[P::NV], val_bytes[P::NV];
};

template <class P>
__device__ __forceinline__ TileLayout<P> tile_layout(const DevQuery &q, const PipePlan &pp) {
    TileLayout<P> L;
    const DevKeyPart &kp = q.parts[0];
    L.key_off = pp.off[pp.slot[kp.col]];
    L.key_bytes = (uint32_t)q.cols[kp.col].bytes;
    L.key_mask = kp.payload < 64 ? (1ULL << kp.payload) - 1 : ~0ULL;
#pragma unroll
    for (int a = 0; a < P::NV; ++a) {
        L.val_off[a] = 0;
        L.val_bytes[a] = 8;
        if (a < P::NA_) {
            const int col = q.faggs[a].col;
            L.val_off[a] = pp.off[pp.slot[col]];
            L.val_bytes[a] = (uint32_t)q.cols[col].bytes;
        }
    }
    return L;
}

// Sign-extended integer of `bytes` width at index r of p (BOOLEAN columns
// never reach the compiled folds' inputs or one-part keys as signed: their
// payload mask keeps the low bit).
__device__ __forceinline__ int64_t ld_int(const unsigned char *p, uint32_t bytes, uint32_t r) {
    switch (bytes) {
        case 1: return (int64_t)(int8_t)p[r];
        case 2: return (int64_t)((const int16_t *)p)[r];
        case 4: return (int64_t)((const int32_t *)p)[r];
        default: return ((const int64_t *)p)[r];
    }
}

// Tile row r as the fold's row: packed key and inputs read from the stage.
template <class P>
__device__ __forceinline__ void pipe_row(const DevQuery &q, const PipePlan &pp, const TileLayout<P> &L,
                                         const unsigned char *stage, uint32_t r, typename P::Row &rv) {
    rv = typename P::Row{};
    rv.k0 = 0;
    rv.k1 = 0;
#pragma unroll
    for (int a = 0; a < P::NV; ++a) rv.val[a] = 0;
    if (P::KM_ == 1) {
        rv.k0 = (uint64_t)ld_int(stage + L.key_off, L.key_bytes, r) & L.key_mask;
    } else {
        for (int i = 0; i < q.n_parts; ++i) {
            const DevKeyPart &kp = q.parts[i];
            uint64_t raw = (uint64_t)st_int(q.cols[kp.col], stage + pp.off[pp.slot[kp.col]], r);
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
        const unsigned char *p = stage + L.val_off[a];
        if (P::is_f(a))
            rv.val[a] = L.val_bytes[a] == 4 ? f64_bits((double)((const float *)p)[r]) : ((const uint64_t *)p)[r];
        else
            rv.val[a] = (uint64_t)ld_int(p, L.val_bytes[a], r);
    }
}

// The fast range predicate on tile row r.
__device__ __forceinline__ bool pipe_pass(const DevQuery &q, const unsigned char *p, uint32_t r) {
    int64_t x;
    switch (q.fp_bytes) {
        case 1: x = (int64_t)(int8_t)p[r]; break;
        case 2: x = (int64_t)((const int16_t *)p)[r]; break;
        case 4: x = (int64_t)((const int32_t *)p)[r]; break;
        default: x = ((const int64_t *)p)[r]; break;
    }
    return (x >= q.fp_lo && x <= q.fp_hi) != (q.fp_negate != 0);
}

// Every lane waits for phase `parity` of `bar` (each lane's own acquire of
// the copied bytes); false after `limit` SM clocks or once the CTA stops.
__device__ __forceinline__ bool pipe_wait(uint64_t *bar, uint32_t parity, long long limit, const int *stop) {
    if (__all_sync(FULL, mbar_test(bar, parity))) return true;
    const long long t0 = clock64();
    for (uint32_t i = 1;; ++i) {
        if (__all_sync(FULL, mbar_test(bar, parity))) return true;
        if ((i & 15) == 0) {
            const bool give_up = *(volatile const int *)stop != 0 || clock64() - t0 > limit;
            if (__any_sync(FULL, give_up)) return false;
        }
    }
}

template <class P>
__global__ void __launch_bounds__(PIPE_THREADS, 1)
    pipe_scan_kernel(const __grid_constant__ DevQuery q, const __grid_constant__ PipePlan pp) {
    extern __shared__ __align__(128) unsigned char smem[];
    using Row = typename P::Row;
    static_assert(sizeof(Row) <= 24 + 8 * P::NV, "survivor rings sized in pipe_plan");
    const uint32_t D = 1u << pp.log_depth, DM = D - 1;
    uint64_t *full = (uint64_t *)(smem + pp.bar_off);
    uint64_t *empty = full + NCW * D;
    PipeCtl &ctl = *(PipeCtl *)(smem + pp.ctl_off);
    const ScanSmem sm = carve(q, smem + pp.cache_off);
    unsigned char *ring = smem + pp.ring_off;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t G = gridDim.x;
    const uint32_t my_n = pp.n_tiles > blockIdx.x ? (pp.n_tiles - blockIdx.x + G - 1) / G : 0;
    const long long limit = q.wait_cycles > 0 ? q.wait_cycles : WAIT_CYCLES;
    // consumer w takes the CTA's local tiles w, w + NCW, ...; its j-th tile
    // sits in slot w * D + j % D and completes phase (j / D) & 1 of `full`
    auto n_of = [&](int w) -> uint32_t { return my_n > (uint32_t)w ? (my_n - w + NCW - 1) / NCW : 0u; };

    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < NCW * D; ++s) {
            mbar_init_n(&full[s], 1);   // the producer lane's arrive(.expect_tx)
            mbar_init_n(&empty[s], 1);  // the consumer's lane 0
        }
        mbar_init_fence();
        ctl.stop = 0;
    }
    cache_init(q, sm);
    __syncthreads();

    unsigned long long selected = 0;
    if (warp == NCW) {
        // ---------------------------------------------------------- producer
        // lane w keeps consumer w's slots filled; the lanes poll their own
        // `empty` barriers side by side, so no consumer waits on another
        const int w = lane;
        const uint32_t nw = w < NCW ? n_of(w) : 0u;
        uint32_t j = 0;
        long long last = clock64();
        for (;;) {
            bool did = false;
            if (j < nw) {
                const uint32_t slot = w * D + (j & DM);
                if (j < D || mbar_test(&empty[slot], ((j >> pp.log_depth) - 1) & 1u)) {
                    pipe_issue(q, pp, blockIdx.x + (w + j * NCW) * G, ring + (size_t)slot * pp.stage_bytes,
                               &full[slot]);
                    ++j;
                    did = true;
                }
            }
            if (!__any_sync(FULL, j < nw)) break;
            if (__any_sync(FULL, did)) {
                last = clock64();
                continue;
            }
            const bool give_up = *(volatile int *)&ctl.stop != 0 || clock64() - last > limit;
            if (__any_sync(FULL, give_up)) {
                if (lane == 0 && !*(volatile int *)&ctl.stop) {
                    atomicOr(q.status, ST_WAIT_TIMEOUT);  // no consumer freed a slot within the limit
                    ctl.stop = 1;
                }
                break;
            }
        }
        if (w < NCW) ctl.issued[w] = j;
    } else {
        // --------------------------------------------------------- consumer
        const int w = warp;
        const uint32_t nw = n_of(w);
        const TileLayout<P> L = tile_layout<P>(q, pp);
        Row *queue = (Row *)(smem + pp.queue_off) + (size_t)w * PQ;
        uint8_t *list = smem + pp.list_off + (size_t)w * PIPE_TILE;  // survivor offsets of the current tile
        uint32_t qhead = 0, qcount = 0;
        const uint32_t pred_off = q.n_preds ? pp.off[pp.slot[q.preds[0].col]] : 0u;
        uint32_t j = 0;
        for (; j < nw; ++j) {
            const uint32_t slot = w * D + (j & DM);
            if (!pipe_wait(&full[slot], (j >> pp.log_depth) & 1u, limit, &ctl.stop)) {
                if (lane == 0 && !*(volatile int *)&ctl.stop) {
                    atomicOr(q.status, ST_WAIT_TIMEOUT);
                    ctl.stop = 1;
                }
                break;
            }
            if ((j & 63) == 63 && q.cancel) {
                const int c = lane == 0 ? *q.cancel : 0;
                if (__shfl_sync(FULL, c, 0)) {
                    if (lane == 0) {
                        atomicOr(q.status, ST_CANCELLED);
                        ctl.stop = 1;
                    }
                    break;
                }
            }
            unsigned char *stage = ring + (size_t)slot * pp.stage_bytes;
            uint64_t row0;
            uint32_t rows;
            pipe_tile_rows(q, pp, blockIdx.x + (w + j * NCW) * G, row0, rows);
            if (rows != PIPE_TILE) pipe_copy_partial(q, pp, row0, rows, stage);
            if (q.n_preds) {
                // the tile's survivors: their offsets first (ballot + popc),
                // then their rows built and queued 32 at a time (every lane
                // busy), folding each full batch of 32 queued rows
                const unsigned char *pred = stage + pred_off;
                uint32_t n = 0;
                for (uint32_t u = 0; u < rows; u += 32) {
                    const uint32_t r = u + lane;
                    const bool pass = r < rows && pipe_pass(q, pred, r);
                    const unsigned m = __ballot_sync(FULL, pass);
                    if (pass) list[n + __popc(m & ((1u << lane) - 1))] = (uint8_t)r;
                    n += __popc(m);
                }
                __syncwarp();
                selected += lane == 0 ? n : 0;
                for (uint32_t b = 0; b < n; b += 32) {
                    const uint32_t i = b + lane;
                    Row rv{};
                    if (i < n) pipe_row<P>(q, pp, L, stage, list[i], rv);
                    const bool kp = P::prefetch(q, rv, i < n);  // less any row the count sketch drops
                    const unsigned mk = __ballot_sync(FULL, kp);
                    if (kp) queue[(qhead + qcount + __popc(mk & ((1u << lane) - 1))) & (PQ - 1)] = rv;
                    qcount += __popc(mk);
                    if (qcount >= 32) {
                        __syncwarp();
                        Row rv = queue[(qhead + lane) & (PQ - 1)];
                        __syncwarp();
                        P::reserve(q, rv, true);
                        P::fold(q, sm, rv, FULL);
                        qhead = (qhead + 32) & (PQ - 1);
                        qcount -= 32;
                    }
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(&empty[slot]);  // the survivors live in the ring now
            } else {
                // every row folds: batch u + 32 is loaded and prefetched
                // before batch u folds; the slot is released after the last
                Row cur;
                bool me = lane < rows;
                if (me) pipe_row<P>(q, pp, L, stage, lane, cur);
                else cur = Row{};
                bool kp = P::prefetch(q, cur, me);  // less any row the count sketch drops
                for (uint32_t u = 0; u < rows; u += 32) {
                    const unsigned act = __ballot_sync(FULL, me), keep = __ballot_sync(FULL, kp);
                    Row nxt;
                    const uint32_t rn = u + 32 + lane;
                    const bool me_n = rn < rows;
                    if (me_n) pipe_row<P>(q, pp, L, stage, rn, nxt);
                    else nxt = Row{};
                    const bool kp_n = P::prefetch(q, nxt, me_n);
                    if (u + 32 >= rows) {
                        __syncwarp();
                        if (lane == 0) mbar_arrive(&empty[slot]);
                    }
                    selected += lane == 0 ? __popc(act) : 0;
                    P::reserve(q, cur, kp);
                    if (keep) P::fold(q, sm, cur, keep);
                    cur = nxt;
                    me = me_n;
                    kp = kp_n;
                }
                if (rows == 0) {
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&empty[slot]);
                }
            }
        }
        if (lane == 0) ctl.consumed[w] = j;
        if (qcount) {
            // the warp's last survivors: one partial batch
            __syncwarp();
            Row rv = queue[(qhead + lane) & (PQ - 1)];
            __syncwarp();
            const bool me = lane < (int)qcount;
            if (!me) rv = Row{};
            P::reserve(q, rv, me);
            P::fold(q, sm, rv, (1u << qcount) - 1);
        }
    }
    __syncthreads();
    if (ctl.stop && warp == NCW && lane == 0) {
        // leave no copy in flight into this CTA's shared memory (bounded by
        // the built-in limit, whatever the query's: the copies are real and land)
        for (int w = 0; w < NCW; ++w)
            for (uint32_t j = ctl.consumed[w]; j < ctl.issued[w]; ++j)
                (void)mbar_wait(&full[w * D + (j & DM)], (j >> pp.log_depth) & 1u);
    }
    if (q.cache_slots) {
        __syncthreads();
        cache_flush(q, sm);
    }
    if (lane == 0 && selected) atomicAdd(q.selected_rows, selected);
}

using PipeFn = const void *;

template <class P>
PipeFn pipe_of() {
    return (const void *)pipe_scan_kernel<P>;
}

PipeFn pick_pipe(const DevQuery &q) {
    switch (q.fast_id) {
#define TGPU_PIPE(I, KM, A, B, C2, D) \
    case I: return pipe_of<FastFold<KM, A, B, C2, D>>();
        TGPU_FAST_FOLDS(TGPU_PIPE)
#undef TGPU_PIPE
        default: return nullptr;
    }
}

}  // namespace

bool pipe_plan(DevQuery &q, uint64_t tile_count, PipePlan *pp) {
    if (q.fast_id < 0 || (q.n_preds > 0 && q.fp_bytes == 0) || q.n_preds > 1 || q.rg_rows % PIPE_TILE != 0)
        return false;
    int cache_slots = q.cache_slots, cache_probe = q.cache_probe;
    PipePlan p{};
    for (int c = 0; c < MAX_QCOLS; ++c) p.slot[c] = -1;
    auto use = [&](int c) {
        if (c < 0 || p.slot[c] >= 0) return true;
        const DevCol &col = q.cols[c];
        if (col.valid || ((uintptr_t)col.data & 15)) return false;
        p.slot[c] = (int32_t)p.n_cols;
        p.col[p.n_cols] = c;
        p.off[p.n_cols] = p.stage_bytes;
        p.stage_bytes += PIPE_TILE * (uint32_t)col.bytes;  // a multiple of 16 bytes: offsets stay aligned
        ++p.n_cols;
        return true;
    };
    bool ok = q.n_preds == 0 || use(q.preds[0].col);
    for (int i = 0; ok && i < q.n_parts; ++i) ok = use(q.parts[i].col);
    for (int a = 0; ok && a < q.n_faggs; ++a) ok = use(q.faggs[a].col);
    if (!ok || p.n_cols == 0 || p.n_cols > 8) return false;
    p.n_tiles = (uint32_t)tile_count;
    p.tiles_per_rg = q.rg_rows / PIPE_TILE;
    // shared memory: control | barriers | hot-key cache | survivor rings | ring of stages
    const uint32_t budget = 224 * 1024;
    const uint32_t row_bytes = 24 + 8 * (uint32_t)(q.n_faggs > 0 ? q.n_faggs : 1);  // FastFold::Row, widest
    const uint32_t queue_bytes = q.n_preds ? NCW * PQ * row_bytes : 0;
    auto cache_bytes = [&](int c) { return (uint32_t)c * (12u + 8u * (uint32_t)q.state_words); };
    const uint32_t fixed = 256 + 2 * NCW * 8 * 4;  // control + up to 4 slots per consumer
    const uint32_t list_bytes = q.n_preds ? NCW * PIPE_TILE : 0;
    while (cache_slots > 0 &&
           fixed + cache_bytes(cache_slots) + queue_bytes + list_bytes + 2 * NCW * p.stage_bytes + 256 > budget) {
        const bool resident = cache_probe == cache_slots;
        cache_slots >>= 1;
        cache_probe = resident ? 16 : std::min(cache_probe, cache_slots);
        if (cache_slots < 64 || (resident && q.needs_gid)) cache_slots = cache_probe = 0;
    }
    p.ctl_off = 0;
    p.bar_off = 256;
    p.cache_off = p.bar_off + 2 * NCW * 4 * 8;
    p.queue_off = (p.cache_off + cache_bytes(cache_slots) + 127) & ~127u;
    p.list_off = p.queue_off + queue_bytes;
    p.ring_off = (p.list_off + (q.n_preds ? NCW * PIPE_TILE : 0) + 127) & ~127u;
    if (p.ring_off + 2 * NCW * p.stage_bytes > budget) return false;
    p.log_depth = (budget - p.ring_off) / (NCW * p.stage_bytes) >= 4 ? 2 : 1;  // 4 or 2 slots per consumer
    p.smem_bytes = p.ring_off + (NCW << p.log_depth) * p.stage_bytes;
    static_assert(sizeof(PipeCtl) <= 256, "control block fits before the barriers");
    q.cache_slots = cache_slots;
    q.cache_probe = cache_probe;
    *pp = p;
    return true;
}

cudaError_t launch_pipe_scan(const DevQuery &q, const PipePlan &pp, int grid, cudaStream_t s) {
    const void *fn = pick_pipe(q);
    if (!fn) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pp.smem_bytes);
    if (e != cudaSuccess) return e;
    void *args[] = {(void *)&q, (void *)&pp};
    return cudaLaunchKernel(fn, dim3(grid), dim3(PIPE_THREADS), args, pp.smem_bytes, s);
}

}  // namespace tgpu
