// radix.cu — the radix-partitioned route for high-cardinality keys.
//
// thinDB stages each chunk's rows by a hash of their packed key into buckets
// (silo_group_core.zig stageBucketIds :9228, scatterStageLane :9348; bucket
// count from the expected groups, bucketCountForGroups :11475-11482), so each
// bucket's groups are folded by one worker in a table that stays in cache.
// Here the same idea keeps a partition's groups in one CTA's shared memory:
//
//   1. radix_scatter_kernel: per tile of RX_TILE rows, the rows that pass
//      the WHERE are packed (key + fold inputs), counted per partition
//      (top radix bits of the key hash) in a shared-memory histogram, given
//      their places by a block-wide exclusive scan and one global
//      reservation per (tile, partition), staged in shared memory in
//      partition order and written out as contiguous runs;
//   2. radix_aggregate_kernel: one CTA per partition folds the partition's
//      records with the query's compiled fold into a shared-memory table
//      that holds every group of the partition (a group lives in exactly one
//      partition), then flushes each group to the global table once.  A
//      COUNT(DISTINCT) pair's place is reserved in one of the partition's
//      2^sub_bits distinct sub-partitions by a shared-memory cursor (no
//      global atomic per row); the partition kernel of distinct.cu then
//      deduplicates every sub-partition.
// A partition whose groups overflow the shared table folds the excess in
// the global table (correct, slower); a partition buffer that overflows sets
// ST_PART_FULL and the host resizes and reruns.
#include <algorithm>

#include "scan_impl.cuh"

namespace tgpu {

namespace {

constexpr int RX_THREADS = 512;
constexpr int RX_WARPS = RX_THREADS / 32;

// Tile t: rows [row0, row_end) inside surviving row group t / tiles_per_rg.
__device__ __forceinline__ void rx_tile_rows(const DevQuery &q, const RadixPlan &rp, uint32_t t, uint64_t &row0,
                                             uint64_t &row_end) {
    const uint32_t rgi = t / rp.tiles_per_rg, sub = t % rp.tiles_per_rg;
    const uint64_t rg = q.rg_list ? q.rg_list[rgi] : rgi;
    row0 = rg * q.rg_rows + (uint64_t)sub * RX_TILE;
    row_end = min(min(row0 + RX_TILE, (rg + 1) * (uint64_t)q.rg_rows), q.n_rows);
}

__device__ __forceinline__ uint32_t rx_part(const RadixPlan &rp, uint64_t hk) {
    return rp.bits ? (uint32_t)(hk >> (64 - rp.bits)) : 0u;
}

// Block-wide exclusive scan of hist[0, n) into out (n <= 2 * RX_THREADS).
__device__ void rx_scan(const uint32_t *hist, uint32_t *out, uint32_t n, uint32_t *warp_sums) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t i0 = 2 * threadIdx.x, i1 = i0 + 1;
    const uint32_t a = i0 < n ? hist[i0] : 0u, b = i1 < n ? hist[i1] : 0u;
    uint32_t x = a + b;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < RX_WARPS ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, s, o);
            if (lane >= o) s += y;
        }
        if (lane < RX_WARPS) warp_sums[lane] = s;
    }
    __syncthreads();
    const uint32_t before = (warp ? warp_sums[warp - 1] : 0u) + x - (a + b);
    if (i0 < n) out[i0] = before;
    if (i1 < n) out[i1] = before + a;
    __syncthreads();
}

template <class P>
__global__ void __launch_bounds__(RX_THREADS, 1)
    radix_scatter_kernel(const __grid_constant__ DevQuery q, const __grid_constant__ RadixPlan rp) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int W = 1 + P::NA_;  // record words: packed key, then the fold's inputs
    constexpr int RPT = RX_TILE / RX_THREADS;
    const uint32_t NP = 1u << rp.bits;
    uint32_t *hist = (uint32_t *)smem;   // NP
    uint32_t *loc = hist + NP;           // NP: first staged index of the partition's run
    uint32_t *base = loc + NP;           // NP: the run's place in the partition buffer
    uint32_t *warp_sums = base + NP;     // RX_WARPS
    uint16_t *pid = (uint16_t *)(warp_sums + RX_WARPS);                              // RX_TILE
    unsigned long long *stage = (unsigned long long *)(((uintptr_t)(pid + RX_TILE) + 15) & ~(uintptr_t)15);
    unsigned long long selected = 0;
    const int lane = threadIdx.x & 31;

    for (uint32_t t = blockIdx.x; t < rp.n_tiles; t += gridDim.x) {
        if (q.cancel && (t & 63) == 63) {
            int c = threadIdx.x == 0 ? *q.cancel : 0;
            if (__syncthreads_or(c)) {
                if (threadIdx.x == 0) atomicOr(q.status, ST_CANCELLED);
                break;
            }
        }
        uint64_t row0, row_end;
        rx_tile_rows(q, rp, t, row0, row_end);
        for (uint32_t p = threadIdx.x; p < NP; p += RX_THREADS) hist[p] = 0;
        __syncthreads();
        // this thread's rows: row0 + threadIdx.x + k * RX_THREADS (coalesced)
        typename P::Row rows[RPT];
        uint32_t part[RPT], rank[RPT];
        bool keep[RPT];
#pragma unroll
        for (int k = 0; k < RPT; ++k) {
            const uint64_t r = row0 + threadIdx.x + (uint64_t)k * RX_THREADS;
            keep[k] = r < row_end && row_passes(q, r);
            P::load(q, r, keep[k], rows[k]);
        }
#pragma unroll
        for (int k = 0; k < RPT; ++k) {
            selected += __popc(__ballot_sync(FULL, keep[k])) * (lane == 0);
            part[k] = rx_part(rp, hash_key(rows[k].k0, rows[k].k1));
            rank[k] = keep[k] ? atomicAdd(&hist[part[k]], 1u) : 0u;
        }
        __syncthreads();
        rx_scan(hist, loc, NP, warp_sums);
        for (uint32_t p = threadIdx.x; p < NP; p += RX_THREADS)
            base[p] = hist[p] ? atomicAdd(rp.cursor + p, hist[p]) : 0u;
#pragma unroll
        for (int k = 0; k < RPT; ++k) {
            if (!keep[k]) continue;
            const uint32_t at = loc[part[k]] + rank[k];
            pid[at] = (uint16_t)part[k];
            unsigned long long *rec = stage + (size_t)at * W;
            rec[0] = rows[k].k0;
#pragma unroll
            for (int a = 0; a < P::NA_; ++a) rec[1 + a] = rows[k].val[a];
        }
        __syncthreads();
        // write the runs out: consecutive staged records of a partition go to
        // consecutive places of its buffer
        const uint32_t total = loc[NP - 1] + hist[NP - 1];
        for (uint32_t e = threadIdx.x; e < total * W; e += RX_THREADS) {
            const uint32_t i = e / W, w = e - i * W;
            const uint32_t p = pid[i];
            const uint64_t dst = (uint64_t)base[p] + (i - loc[p]);
            if (dst < rp.cap) rp.buf[((uint64_t)p * rp.cap + dst) * W + w] = stage[e];
            else if (w == 0) atomicOr(q.status, ST_PART_FULL);
        }
        __syncthreads();
    }
    if (lane == 0 && selected) atomicAdd(q.selected_rows, selected);
}

template <class P>
__global__ void __launch_bounds__(RX_THREADS, 1)
    radix_aggregate_kernel(const __grid_constant__ DevQuery q, const __grid_constant__ RadixPlan rp) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int W = 1 + P::NA_;
    const ScanSmem sm = carve(q, smem);
    uint32_t *dcur = (uint32_t *)(smem + rp.dcur_off);  // 2^sub_bits distinct sub-partition cursors
    const uint32_t NP = 1u << rp.bits, NS = 1u << rp.sub_bits;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t p = blockIdx.x; p < NP; p += gridDim.x) {
        cache_init(q, sm);
        for (uint32_t i = threadIdx.x; i < NS; i += RX_THREADS) dcur[i] = 0;
        __syncthreads();
        const uint32_t n = (uint32_t)min((uint64_t)__ldcg(rp.cursor + p), rp.cap);
        const unsigned long long *recs = rp.buf + (uint64_t)p * rp.cap * W;
        // each warp folds 32 records at a time; the next batch is loaded first
        for (uint32_t b = warp * 32; b < n; b += RX_THREADS) {
            const uint32_t i = b + lane;
            const bool me = i < n;
            typename P::Row rv{};
            if (me) {
                rv.k0 = __ldcs(recs + (size_t)i * W);
#pragma unroll
                for (int a = 0; a < P::NA_; ++a) rv.val[a] = __ldcs(recs + (size_t)i * W + 1 + a);
            }
            if constexpr (P::DISTINCT) {
                // the pair's place: sub-partition of (value, key hash), a
                // shared-memory cursor (this CTA owns the partition)
                if (me) {
#pragma unroll
                    for (int a = 0; a < P::NA_; ++a)
                        if (P::kind(a) == AK_DISTINCT) {
                            const uint64_t hk = hash_key(rv.k0, 0);
                            const uint32_t s = NS > 1 ? (uint32_t)(mix64(rv.val[a] ^ hk) >> (64 - rp.sub_bits)) : 0u;
                            rv.dp = (p << rp.sub_bits) | s;
                            rv.dpos = atomicAdd(&dcur[s], 1u);
                        }
                }
            }
            const unsigned act = __ballot_sync(FULL, me);
            if (act) P::fold(q, sm, rv, act);
        }
        __syncthreads();
        cache_flush(q, sm);
        if constexpr (P::DISTINCT) {
            if (q.dpart_bits)
                for (uint32_t i = threadIdx.x; i < NS; i += RX_THREADS) q.dpart_cursor[(p << rp.sub_bits) | i] = dcur[i];
        }
        __syncthreads();
    }
}

struct RadixFns {
    const void *scatter, *aggregate;
};

template <class P>
RadixFns radix_of() {
    return RadixFns{(const void *)radix_scatter_kernel<P>, (const void *)radix_aggregate_kernel<P>};
}

RadixFns pick_radix(const DevQuery &q) {
    switch (q.fast_id) {
#define TGPU_RX(I, KM, A, B, C2, D) \
    case I: return radix_of<FastFold<KM, A, B, C2, D>>();
        TGPU_FAST_FOLDS(TGPU_RX)
#undef TGPU_RX
        default: return RadixFns{nullptr, nullptr};
    }
}

}  // namespace

size_t radix_scatter_smem(const DevQuery &q, uint32_t bits) {
    const size_t np = (size_t)1 << bits;
    return np * 12 + RX_WARPS * 4 + RX_TILE * 2 + 16 + (size_t)RX_TILE * (1 + q.n_faggs) * 8;
}

cudaError_t launch_radix(const DevQuery &q, const RadixPlan &rp, int sms, cudaStream_t s) {
    const RadixFns f = pick_radix(q);
    if (!f.scatter) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(rp.cursor, 0, sizeof(uint32_t) << rp.bits, s);
    if (e != cudaSuccess) return e;
    const size_t s1 = radix_scatter_smem(q, rp.bits);
    if ((e = cudaFuncSetAttribute(f.scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s1)) != cudaSuccess)
        return e;
    if (rp.n_tiles) {
        const uint32_t g1 = std::min<uint32_t>(rp.n_tiles, (uint32_t)sms * 2);
        void *a1[] = {(void *)&q, (void *)&rp};
        if ((e = cudaLaunchKernel(f.scatter, dim3(g1), dim3(RX_THREADS), a1, s1, s)) != cudaSuccess) return e;
    }
    const size_t s2 = rp.agg_smem;
    if ((e = cudaFuncSetAttribute(f.aggregate, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s2)) != cudaSuccess)
        return e;
    const uint32_t g2 = std::min<uint32_t>(1u << rp.bits, (uint32_t)sms * rp.agg_per_sm);
    void *a2[] = {(void *)&q, (void *)&rp};
    return cudaLaunchKernel(f.aggregate, dim3(g2), dim3(RX_THREADS), a2, s2, s);
}

}  // namespace tgpu
