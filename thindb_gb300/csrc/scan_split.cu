// scan_split.cu — the split scan: the WHERE as its own streaming pass that
// writes the surviving row numbers, then a fold pass over that list.
//
// With the count sketch on, the select pass also drops the rows whose key's
// counter is not kept, so the fold pass sees only candidate rows.
//
// The fused gather-mode scan (scan_chunk) runs filter -> compaction ->
// gather -> fold per warp and chunk, so every warp waits on its own filter
// before its gathers can start.  Split, the select pass only streams the
// predicate column (one atomicAdd per chunk reserves the chunk's place in the
// list) and the fold pass reads the list densely: every batch of 32 rows is
// full, and a warp's LOOKAHEAD batches of gathers are in flight at once with
// their row numbers known up front.  The list costs 4 bytes per survivor
// written and read again.
#include <climits>
#include <type_traits>

#include "scan_impl.cuh"

namespace tgpu {

namespace {

constexpr uint32_t SELECT_SPAN = 2048;  // rows a warp filters before it writes their survivors out

// The range test over rows [row0, row_end) with 16-byte loads: lane l holds
// V = 16 / sizeof(T) consecutive rows of each 32 * V-row step, and the
// survivors' chunk offsets go to `list` in row order (V ballots place them).
// row0 and the column start on 16-byte boundaries; a vector that would run
// past the table's last row is read element by element.
template <typename T>
__device__ __forceinline__ uint32_t filter_vec(const DevQuery &q, uint64_t row0, uint64_t row_end, uint16_t *list) {
    // U steps' loads in flight.  The select kernel's occupancy matters more
    // than the depth per warp: at two CTAs an SM (64 registers) U = 2 and 4
    // measured within 1% of one another for 100M rows, at one CTA an SM (U = 4
    // took 128 registers unbounded) 4% slower, at three (40 registers, with
    // spills) 4% slower too
    constexpr int V = 16 / (int)sizeof(T), U = 2;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const T *col = (const T *)q.fp_data;
    const bool neg = q.fp_negate != 0;
    // the range as one unsigned compare, x - lo <= hi - lo, in the width the
    // values need (32 bits for elements of up to 4 bytes; an empty range
    // becomes lo = 1, hi = 0)
    using C = typename std::conditional<sizeof(T) == 8, long long, int>::type;
    using UC = typename std::conditional<sizeof(T) == 8, unsigned long long, unsigned>::type;
    int64_t lo64 = q.fp_lo, hi64 = q.fp_hi;
    if (sizeof(T) < 8) {
        lo64 = max(lo64, (int64_t)INT_MIN);
        hi64 = min(hi64, (int64_t)INT_MAX);
    }
    const bool empty = lo64 > hi64;
    const UC lo = (UC)(C)lo64;  // (unsigned arithmetic: x - lo wraps, as the compare wants)
    const UC span = empty ? (UC)0 : (UC)((uint64_t)hi64 - (uint64_t)lo64);
    uint32_t n = 0;
    for (uint64_t b = row0; b < row_end; b += (uint64_t)32 * V * U) {
        int4 raw[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t r = b + (uint64_t)u * 32 * V + (uint64_t)lane * V;
            raw[u] = make_int4(0, 0, 0, 0);
            if (r + V <= q.n_rows) {
                if (r < row_end) raw[u] = __ldcs((const int4 *)(col + r));
            } else {
                T t[V];
#pragma unroll
                for (int j = 0; j < V; ++j) t[j] = r + j < row_end ? col[r + j] : T(0);
                memcpy(&raw[u], t, 16);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t r = b + (uint64_t)u * 32 * V + (uint64_t)lane * V;
            T x[V];
            memcpy(x, &raw[u], 16);
            uint32_t own = 0;  // this lane's passing rows, bit j = row r + j
#pragma unroll
            for (int j = 0; j < V; ++j) {
                const bool in = !empty && (UC)((UC)(C)x[j] - lo) <= span;
                own |= (uint32_t)(r + j < row_end && in != neg) << j;
            }
            uint32_t before = 0, total = 0;
#pragma unroll
            for (int j = 0; j < V; ++j) {
                const unsigned m = __ballot_sync(FULL, (own >> j) & 1u);
                before += __popc(m & lt);
                total += __popc(m);
            }
            uint32_t at = n + before;
#pragma unroll
            for (int j = 0; j < V; ++j)
                if ((own >> j) & 1u) list[at++] = (uint16_t)(r + j - row0);
            n += total;
        }
    }
    return n;
}

// The count sketch's filter over rows [row0, row_end) of a table with no
// WHERE and one NOT NULL 8-byte key part: two keys a lane per 16-byte load,
// the kept rows' chunk offsets to `list` in row order.  (pack_key of such a
// key is key_or | the masked value, so the hash is the tally's.)
__device__ __forceinline__ uint32_t keep_vec(const DevQuery &q, uint64_t row0, uint64_t row_end, uint16_t *list) {
    constexpr int V = 2, U = 4;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const DevKeyPart &kp = q.parts[0];
    const unsigned long long *col = (const unsigned long long *)q.cols[kp.col].data;
    const uint64_t mask = kp.payload < 64 ? ((1ULL << kp.payload) - 1) : ~0ULL;
    uint32_t n = 0;
    for (uint64_t b = row0; b < row_end; b += (uint64_t)32 * V * U) {
        ulonglong2 raw[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t r = b + (uint64_t)u * 32 * V + (uint64_t)lane * V;
            raw[u] = make_ulonglong2(0, 0);
            if (r + V <= q.n_rows) {
                if (r < row_end) raw[u] = __ldcs((const ulonglong2 *)(col + r));
            } else if (r < row_end) {
                raw[u].x = col[r];
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t r = b + (uint64_t)u * 32 * V + (uint64_t)lane * V;
            const uint64_t k[V] = {raw[u].x, raw[u].y};
            uint32_t own = 0;
#pragma unroll
            for (int j = 0; j < V; ++j)
                own |= (uint32_t)(r + j < row_end && sketch_kept(q, hash_key(q.key_or | (k[j] & mask), 0))) << j;
            uint32_t before = 0, total = 0;
#pragma unroll
            for (int j = 0; j < V; ++j) {
                const unsigned m = __ballot_sync(FULL, (own >> j) & 1u);
                before += __popc(m & lt);
                total += __popc(m);
            }
            uint32_t at = n + before;
#pragma unroll
            for (int j = 0; j < V; ++j)
                if ((own >> j) & 1u) list[at++] = (uint16_t)(r + j - row0);
            n += total;
        }
    }
    return n;
}

__global__ void __launch_bounds__(SCAN_THREADS, 2) select_rows_kernel(const __grid_constant__ DevQuery q,
                                                                      uint32_t *rows, unsigned long long *n_rows) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint16_t *list = (uint16_t *)smem_raw + (size_t)warp * SELECT_SPAN;
    unsigned long long selected = 0;
    const uint32_t nw = gridDim.x * SCAN_WARPS;
    // one NOT NULL 8-byte key part at bit 0, not hashed, 16-byte aligned: keep_vec
    const bool fast_key = q.n_parts == 1 && !q.hashed && q.parts[0].offset == 0 && !q.parts[0].nullable &&
                          q.cols[q.parts[0].col].bytes == 8 && !q.cols[q.parts[0].col].valid &&
                          ((uintptr_t)q.cols[q.parts[0].col].data & 15u) == 0;
    uint32_t k = 0;
    for (uint32_t c = blockIdx.x * SCAN_WARPS + warp; c < q.n_chunks; c += nw, ++k) {
        if ((k & 31) == 31 && q.cancel) {
            int stop = 0;
            if (lane == 0) stop = *q.cancel;
            if (__shfl_sync(FULL, stop, 0)) {
                if (lane == 0) atomicOr(q.status, ST_CANCELLED);
                break;
            }
        }
        uint64_t c0, c1;
        chunk_rows(q, c, c0, c1);
        // the chunk in spans of at most SELECT_SPAN rows (the list's room)
        for (uint64_t row0 = c0; row0 < c1; row0 += SELECT_SPAN) {
            const uint64_t row_end = min(c1, row0 + SELECT_SPAN);
            uint32_t n;
            const bool vec = ((uintptr_t)q.fp_data & 15u) == 0 && ((row0 * (uint64_t)q.fp_bytes) & 15u) == 0;
            const bool sketch = q.sk_keep && __ldg(q.sk_on);
            bool kept_done = false;  // the sketch's keep test already applied
            if (q.n_preds == 0 && sketch && fast_key && (row0 & 1) == 0) {
                n = keep_vec(q, row0, row_end, list);
                kept_done = true;
            } else if (q.n_preds == 0) {  // no WHERE: every row (the count sketch below picks)
                n = (uint32_t)(row_end - row0);
                for (uint32_t i = lane; i < n; i += 32) list[i] = (uint16_t)i;
            } else {
                switch (vec ? q.fp_bytes : 0) {
                    case 1: n = filter_vec<signed char>(q, row0, row_end, list); break;
                    case 2: n = filter_vec<short>(q, row0, row_end, list); break;
                    case 4: n = filter_vec<int>(q, row0, row_end, list); break;
                    case 8: n = filter_vec<long long>(q, row0, row_end, list); break;
                    default: n = survivors(q, row0, row_end, list); break;
                }
            }
            __syncwarp();
            // the WHERE's rows, whatever the sketch keeps
            selected += lane == 0 ? (kept_done ? row_end - row0 : n) : 0;
            if (n && sketch && !kept_done) {
                // the count sketch's filter: keep the rows whose key's counter
                // is kept (the tally's pack_key + hash_key), compacted in place
                uint32_t m = 0;
                for (uint32_t g = 0; g < n; g += 32) {
                    const uint32_t i = g + lane;
                    const uint16_t off = i < n ? list[i] : 0;
                    bool kept = false;
                    if (i < n) {
                        uint64_t k0, k1;
                        pack_key(q, row0 + off, k0, k1);
                        kept = sketch_kept(q, hash_key(k0, k1));
                    }
                    const unsigned b = __ballot_sync(FULL, kept);
                    __syncwarp();
                    if (kept) list[m + __popc(b & ((1u << lane) - 1u))] = off;
                    m += __popc(b);
                }
                __syncwarp();
                n = m;
            }
            if (n) {
                unsigned long long at = 0;
                if (lane == 0) at = atomicAdd(n_rows, (unsigned long long)n);
                at = __shfl_sync(FULL, at, 0);
                for (uint32_t i = lane; i < n; i += 32) rows[at + i] = (uint32_t)(row0 + list[i]);
            }
            __syncwarp();
        }
    }
    if (lane == 0 && selected) atomicAdd(q.selected_rows, selected);
}

// Each warp folds LOOKAHEAD full batches of 32 listed rows per pass; the
// CTA's shared-memory hot table is the fused scan's.
template <class P, int MINB>
__global__ void __launch_bounds__(SCAN_THREADS, MINB)
    fold_rows_kernel(const __grid_constant__ DevQuery q, const uint32_t *__restrict__ rows,
                     const unsigned long long *__restrict__ n_rows) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const ScanSmem sm = carve(q, smem_raw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    cache_init(q, sm);
    __syncthreads();
    const uint64_t n = *n_rows;
    constexpr int L = P::LOOKAHEAD;
    const uint64_t span = 32ull * L, step = (uint64_t)gridDim.x * SCAN_WARPS * span;
    uint32_t k = 0;
    for (uint64_t i = ((uint64_t)blockIdx.x * SCAN_WARPS + warp) * span; i < n; i += step, ++k) {
        if ((k & 63) == 63 && q.cancel) {
            int stop = 0;
            if (lane == 0) stop = *q.cancel;
            if (__shfl_sync(FULL, stop, 0)) {
                if (lane == 0) atomicOr(q.status, ST_CANCELLED);
                break;
            }
        }
        uint32_t r[L];
#pragma unroll
        for (int j = 0; j < L; ++j) {
            const uint64_t s = i + 32 * j + lane;
            r[j] = s < n ? __ldcs(rows + s) : 0u;
        }
        typename P::Row rv[L];
#pragma unroll
        for (int j = 0; j < L; ++j) P::load(q, r[j], i + 32 * j + lane < n, rv[j]);
        unsigned keep[L];
#pragma unroll
        for (int j = 0; j < L; ++j) keep[j] = __ballot_sync(FULL, P::prefetch(q, rv[j], i + 32 * j + lane < n));
#pragma unroll
        for (int j = 0; j < L; ++j) P::reserve(q, rv[j], (keep[j] >> lane) & 1u);
#pragma unroll
        for (int j = 0; j < L; ++j)
            if (keep[j]) P::fold(q, sm, rv[j], keep[j]);
    }
    if (q.cache_slots) {
        __syncthreads();
        cache_flush(q, sm);
    }
}

// ---- the fold pass with its gathers staged by asynchronous copies ----
// For a compiled fold over one 8-byte key part and 8-byte inputs (the
// filtered DECIMAL shape): each warp owns a contiguous stretch of the row
// list and keeps stage_depth batches of 32 rows in flight as cp.async copies
// of the key and input values into its shared-memory slots, so the gathers
// need no registers while they wait; a batch folds once its copies have
// landed, and its slot takes the batch stage_depth ahead.
//
// HINT (the count sketch's fold pass): one batch ahead of its fold, each lane
// also loads the key its row's home slot in the group table holds, and a row
// whose key is already there skips the probe's load (global_slot_from).  The
// kept rows of a count sketch fall into few groups whose slots are claimed
// early: 2.73 -> 2.09 ms for 100M rows.  The filtered DECIMAL shape (1.1M
// groups, most of its rows folded in the shared table) measured 12% slower
// with it, so it runs without.

__host__ __device__ constexpr int stage_depth(bool hint) { return hint ? 3 : 2; }

__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <class P, bool HINT>
__global__ void __launch_bounds__(SCAN_THREADS, 2)
    fold_rows_staged_kernel(const __grid_constant__ DevQuery q, const uint32_t *__restrict__ rows,
                            const unsigned long long *__restrict__ n_rows, uint32_t stage_off) {
    static_assert(P::KM_ == 1, "one key part");
    constexpr int NA = P::NA_, W = 1 + NA;  // words a row stages: the key, then each input
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const ScanSmem sm = carve(q, smem_raw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int STAGE_DEPTH = stage_depth(HINT);
    // this warp's slots: STAGE_DEPTH x W x 32 words
    unsigned long long *slots =
        (unsigned long long *)(smem_raw + stage_off) + (size_t)warp * STAGE_DEPTH * W * 32;
    cache_init(q, sm);
    __syncthreads();
    const uint64_t n = *n_rows;
    const uint64_t warps = (uint64_t)gridDim.x * SCAN_WARPS, gw = (uint64_t)blockIdx.x * SCAN_WARPS + warp;
    const uint64_t per = (n + warps * 32 - 1) / (warps * 32) * 32;  // whole batches per warp
    const uint64_t begin = min(n, gw * per), end = min(n, begin + per);
    const uint64_t nb = (end - begin + 31) / 32;
    const DevKeyPart &kp = q.parts[0];
    const unsigned long long *kcol = (const unsigned long long *)q.cols[kp.col].data;
    const unsigned long long *vcol[NA > 0 ? NA : 1];
#pragma unroll
    for (int a = 0; a < NA; ++a) vcol[a] = (const unsigned long long *)q.cols[q.faggs[a].col].data;
    const uint64_t kmask = kp.payload < 64 ? ((1ULL << kp.payload) - 1) : ~0ULL;
    auto issue = [&](uint64_t b) {  // batch b's copies into its slot
        if (b < nb) {
            const uint64_t s = begin + b * 32 + lane;
            if (s < end) {
                const uint32_t r = __ldcs(rows + s);
                unsigned long long *dst = slots + (size_t)(b % STAGE_DEPTH) * W * 32 + lane;
                cp_async8(dst, kcol + r);
#pragma unroll
                for (int a = 0; a < NA; ++a) cp_async8(dst + (a + 1) * 32, vcol[a] + r);
            }
        }
        cp_async_commit();  // an empty group keeps the group count in step
    };
    // the key held by the home slot of this lane's row of batch b, whose
    // copies have landed (0: no row, or the zero key, which has its own slot)
    auto home_of = [&](uint64_t b) -> uint64_t {
        if (b >= nb || begin + b * 32 + lane >= end) return 0;
        const uint64_t k = slots[(size_t)(b % STAGE_DEPTH) * W * 32 + lane] & kmask;
        if (k == 0) return 0;
        return ld_relaxed(q.table + (hash_key(k, 0) & (q.cap - 1)) * (uint64_t)q.slot_words);
    };
#pragma unroll
    for (int d = 0; d < STAGE_DEPTH; ++d) issue(d);
    uint64_t home = 0;
    if constexpr (HINT) {
        cp_async_wait<STAGE_DEPTH - 1>();  // batch 0's group has landed
        home = home_of(0);
    }
    for (uint64_t b = 0; b < nb; ++b) {
        if (((b & 255) == 255) && q.cancel) {
            int stop = 0;
            if (lane == 0) stop = *q.cancel;
            if (__shfl_sync(FULL, stop, 0)) {
                if (lane == 0) atomicOr(q.status, ST_CANCELLED);
                break;
            }
        }
        // batch b's group has landed (HINT: and batch b + 1's)
        cp_async_wait<HINT ? STAGE_DEPTH - 2 : STAGE_DEPTH - 1>();
        const unsigned long long *src = slots + (size_t)(b % STAGE_DEPTH) * W * 32 + lane;
        const bool me = begin + b * 32 + lane < end;
        typename P::Row rv;
        rv.k0 = me ? (src[0] & kmask) : 0;
        rv.k1 = 0;
#pragma unroll
        for (int a = 0; a < P::NV; ++a) rv.val[a] = (me && a < NA) ? src[(a + 1) * 32] : 0;
        const uint64_t home_next = HINT ? home_of(b + 1) : 0;
        __syncwarp();
        issue(b + STAGE_DEPTH);  // the slot is free again
        const unsigned keep = __ballot_sync(FULL, P::prefetch(q, rv, me));
        P::reserve(q, rv, (keep >> lane) & 1u);
        if (keep) {
            if constexpr (HINT) P::fold_hinted(q, sm, rv, keep, home);
            else P::fold(q, sm, rv, keep);
        }
        home = home_next;
    }
    cp_async_wait<0>();
    if (q.cache_slots) {
        __syncthreads();
        cache_flush(q, sm);
    }
}

// The staged fold applies to a compiled fold whose one key part and every
// input are 8-byte NOT NULL columns.
bool staged_fold_ok(const DevQuery &q) {
    if (q.fast_km != 1 || q.n_parts != 1 || q.n_faggs > 3) return false;
    const DevCol &k = q.cols[q.parts[0].col];
    if (k.bytes != 8 || k.valid || k.offs) return false;
    for (int a = 0; a < q.n_faggs; ++a) {
        if (q.faggs[a].col < 0) return false;
        const DevCol &c = q.cols[q.faggs[a].col];
        if (c.bytes != 8 || c.valid || c.offs) return false;
    }
    return true;
}

template <int KM, int A, int B, int C2, int D>
const void *staged_kernel_of(bool hint) {
    if constexpr (KM == 1)
        return hint ? (const void *)fold_rows_staged_kernel<FastFold<KM, A, B, C2, D>, true>
                    : (const void *)fold_rows_staged_kernel<FastFold<KM, A, B, C2, D>, false>;
    else return nullptr;
}

// the count sketch's fold pass takes the home-slot hint
bool staged_hint(const DevQuery &q) { return q.sk_keep != nullptr; }

const void *fold_rows_staged_fn(const DevQuery &q) {
    const bool hint = staged_hint(q);
    switch (fast_fold_id(q)) {
#define TGPU_STAGED(I, KM, A, B, C2, D) \
    case I: return staged_kernel_of<KM, A, B, C2, D>(hint);
        TGPU_FAST_FOLDS(TGPU_STAGED)
#undef TGPU_STAGED
        default: return nullptr;
    }
}

const void *fold_rows_fn(const DevQuery &q) {
    switch (fast_fold_id(q)) {
#define TGPU_SPLIT(I, KM, A, B, C2, D) \
    case I: return (const void *)fold_rows_kernel<FastFold<KM, A, B, C2, D>, 2>;
        TGPU_FAST_FOLDS(TGPU_SPLIT)
#undef TGPU_SPLIT
        default: break;
    }
    if (q.n_aggs <= 4) return (const void *)fold_rows_kernel<GenericFold<4>, 2>;
    return (const void *)fold_rows_kernel<GenericFold<16>, 1>;
}

int per_sm(const void *fn, size_t smem) {
    int n = 1;
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, SCAN_THREADS, smem) != cudaSuccess || n < 1) {
        cudaGetLastError();
        n = 1;
    }
    return n;
}

}  // namespace

size_t split_select_smem(const DevQuery &) { return (size_t)SCAN_WARPS * SELECT_SPAN * 2; }

size_t split_fold_smem(const DevQuery &q) {
    DevQuery f = q;
    f.gather = 0;  // no survivor list in the fold pass
    return scan_smem_bytes(f);
}

cudaError_t launch_split_scan(const DevQuery &q, uint32_t *rows, unsigned long long *n_rows, int sms,
                              cudaStream_t s) {
    if (q.n_chunks == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(n_rows, 0, 8, s);
    if (e != cudaSuccess) return e;
    const size_t ss = split_select_smem(q);
    const void *sel = (const void *)select_rows_kernel;
    const int sgrid = sms * per_sm(sel, ss);
    e = cudaFuncSetAttribute(sel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ss);
    if (e != cudaSuccess) return e;
    select_rows_kernel<<<sgrid, SCAN_THREADS, ss, s>>>(q, rows, n_rows);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const unsigned long long *cn = n_rows;
    const void *staged = staged_fold_ok(q) ? fold_rows_staged_fn(q) : nullptr;
    if (staged) {
        const size_t base = (split_fold_smem(q) + 15) & ~(size_t)15;
        const uint32_t off = (uint32_t)base;
        const size_t fs = base + (size_t)SCAN_WARPS * stage_depth(staged_hint(q)) * (1 + q.n_faggs) * 32 * 8;
        const int fgrid = sms * per_sm(staged, fs);
        e = cudaFuncSetAttribute(staged, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fs);
        if (e != cudaSuccess) return e;
        void *args[] = {(void *)&q, (void *)&rows, (void *)&cn, (void *)&off};
        return cudaLaunchKernel(staged, dim3(fgrid), dim3(SCAN_THREADS), args, fs, s);
    }
    const size_t fs = split_fold_smem(q);
    const void *fn = fold_rows_fn(q);
    const int fgrid = sms * per_sm(fn, fs);
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fs);
    if (e != cudaSuccess) return e;
    void *args[] = {(void *)&q, (void *)&rows, (void *)&cn};
    return cudaLaunchKernel(fn, dim3(fgrid), dim3(SCAN_THREADS), args, fs, s);
}

}  // namespace tgpu
