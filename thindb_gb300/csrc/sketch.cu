// sketch.cu — the two-pass exact top-K for GROUP BY ... ORDER BY COUNT(*)
// DESC LIMIT k (thinDB's CountSketch, src/exec/count_topk_sketch.zig:1-30,
// :181-240; driven by runCountSketch, v2_group_topn_engine.zig:1375).
//
// Tally: every row that passes the WHERE adds one to counter
// hash(packed key) >> (64 - SK_BITS) — a CTA counts into its own
// shared-memory copy of the counters and adds them to the global ones once.
// A counter holds the summed row count of the groups hashing to it, so it
// bounds each of them from above.
// Settle (one CTA): the need-th largest counter (need = OFFSET + LIMIT) by
// radix selection; the sketch declines when that counter is within the
// collision noise of an even spread (collisionCeiling) or when more than an
// eighth of the counters reach the threshold (half the need-th largest);
// otherwise the keep bitmap marks those counters.  (thinDB declines when
// the kept counters hold more than a quarter of the rows,
// MAX_KEPT_FRACTION_DENOM: its filter pass costs per row.  Here the filter
// pass folds the rows of a few heavy groups in the shared-memory hot-key
// table, and what it saves is the groups it never creates: few kept
// counters, not few kept rows, make it pay.)
// Filter pass: the regular scan folds only rows whose counter is kept (the
// folds test the bitmap, FastFold::fold / fold_batch).  Every kept group is
// complete and every dropped group has fewer than `threshold` rows, so once
// the need-th best kept group holds threshold - 1 rows or more the kept
// groups' top need is the answer; the host checks that after the run and
// otherwise reruns without the sketch (CountSketch.exact, :236-239).
#include <cmath>

#include "scan_impl.cuh"

namespace tgpu {

namespace {

constexpr int SK_THREADS = 512;
constexpr uint32_t SK_N = 1u << SK_BITS;

__global__ void __launch_bounds__(SK_THREADS, 2)
    sketch_tally_kernel(const __grid_constant__ DevQuery q, uint32_t *__restrict__ counts) {
    extern __shared__ uint32_t sc[];  // SK_N counters
    for (uint32_t i = threadIdx.x; i < SK_N; i += blockDim.x) sc[i] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint32_t nw = gridDim.x * (SK_THREADS / 32);
    for (uint32_t c = blockIdx.x * (SK_THREADS / 32) + (threadIdx.x >> 5); c < q.n_chunks; c += nw) {
        uint64_t row0, row_end;
        chunk_rows(q, c, row0, row_end);
        for (uint64_t b = row0; b < row_end; b += 32) {
            const uint64_t r = b + lane;
            if (r < row_end && row_passes(q, r)) {
                uint64_t k0, k1;
                pack_key(q, r, k0, k1);
                atomicAdd(&sc[hash_key(k0, k1) >> (64 - SK_BITS)], 1u);
            }
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < SK_N; i += blockDim.x)
        if (sc[i]) atomicAdd(counts + i, sc[i]);
}

// ctl: [0] on, [1] threshold, [2..3] kept rows (u64), [4..5] rows (u64), [6] the need-th largest counter
__global__ void __launch_bounds__(1024, 1)
    sketch_settle_kernel(const uint32_t *__restrict__ counts, uint32_t need, uint32_t *__restrict__ keep,
                         uint32_t *__restrict__ ctl) {
    __shared__ uint32_t hist[256];
    __shared__ unsigned long long tot, kept;
    __shared__ uint32_t kept_counters;
    __shared__ uint32_t prefix_s, remaining_s, kth_s, thr_s;
    __shared__ int on_s;
    if (threadIdx.x == 0) {
        tot = 0;
        kept = 0;
        kept_counters = 0;
        prefix_s = 0;
        remaining_s = need;
    }
    __syncthreads();
    unsigned long long my = 0;
    for (uint32_t i = threadIdx.x; i < SK_N; i += blockDim.x) my += counts[i];
    atomicAdd(&tot, my);
    // the need-th largest counter, eight bits at a time from the top
    uint32_t mask = 0;
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0;
        __syncthreads();
        const uint32_t prefix = prefix_s;
        for (uint32_t i = threadIdx.x; i < SK_N; i += blockDim.x) {
            const uint32_t c = counts[i];
            if ((c & mask) == prefix) atomicAdd(&hist[(c >> shift) & 255u], 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t rem = remaining_s, cum = 0;
            int d = 255;
            for (; d > 0; --d) {
                if (cum + hist[d] >= rem) break;
                cum += hist[d];
            }
            remaining_s = rem - cum;
            prefix_s = prefix | ((uint32_t)d << shift);
        }
        mask |= 255u << shift;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        // (fewer than `need` counters holding rows make it 0: the sketch declines)
        kth_s = prefix_s;
        const double rows = (double)tot;
        const double n = (double)SK_N, mean = rows / n, ln = log(n);
        const double ceiling = mean + sqrt(2.0 * mean * ln) + ln;  // collisionCeiling, count_topk_sketch.zig:1281-1286
        on_s = (double)kth_s > ceiling ? 1 : 0;
        thr_s = kth_s / 2 > 1 ? kth_s / 2 : 1;
    }
    __syncthreads();
    const uint32_t thr = thr_s;
    unsigned long long k = 0;
    uint32_t kc = 0;
    for (uint32_t i = threadIdx.x; i < SK_N; i += blockDim.x) {
        k += counts[i] >= thr ? counts[i] : 0u;
        kc += counts[i] >= thr ? 1u : 0u;
    }
    atomicAdd(&kept, k);
    atomicAdd(&kept_counters, kc);
    __syncthreads();
    const int on = on_s && (uint64_t)kept_counters * 8 <= SK_N;
    for (uint32_t wd = threadIdx.x; wd < SK_N / 32; wd += blockDim.x) {
        uint32_t bits = 0;
        for (int b = 0; b < 32; ++b) bits |= (on && counts[wd * 32 + b] >= thr ? 1u : 0u) << b;
        keep[wd] = bits;
    }
    if (threadIdx.x == 0) {
        ctl[0] = (uint32_t)on;
        ctl[1] = thr;
        ctl[2] = (uint32_t)kept;
        ctl[3] = (uint32_t)(kept >> 32);
        ctl[4] = (uint32_t)tot;
        ctl[5] = (uint32_t)(tot >> 32);
        ctl[6] = kth_s;
    }
}

}  // namespace

cudaError_t launch_count_sketch(const DevQuery &q, uint32_t need, uint32_t *counts, uint32_t *keep, uint32_t *ctl,
                                int sms, cudaStream_t s) {
    const size_t smem = SK_N * sizeof(uint32_t);
    cudaError_t e = cudaFuncSetAttribute(sketch_tally_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(counts, 0, SK_N * sizeof(uint32_t), s)) != cudaSuccess) return e;
    if (q.n_chunks) {
        const uint32_t grid = (uint32_t)std::min<uint64_t>((uint64_t)sms * 2, (q.n_chunks + 15) / 16);
        sketch_tally_kernel<<<grid ? grid : 1, SK_THREADS, smem, s>>>(q, counts);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    sketch_settle_kernel<<<1, 1024, 0, s>>>(counts, need, keep, ctl);
    return cudaGetLastError();
}

}  // namespace tgpu
