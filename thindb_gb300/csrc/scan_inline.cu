// scan_inline.cu — the scan with one inlined fold call site.
//
// The regular scan (scan.cu) keeps LOOKAHEAD batches of gathered rows in
// registers and folds each through an out-of-line call: one copy of the fold
// per unrolled call site would overflow the instruction cache, but the call
// makes the compiler save every live register around it, and the saved
// registers go to local memory (the 20M-row filtered capture counts 406k
// local-memory spill requests; the count sketch's filter pass 1.8M).
// Here the loop over a chunk's 32-row batches is a rolling two-stage
// pipeline — batch i + 1 is loaded and its group-table slots prefetched,
// then batch i folds — so the loop body has exactly one fold call site and
// the fold's body (FastFold::fold_body) is inlined into it: no call, nothing
// saved around it.  The rows, the WHERE and the folds are the regular
// scan's (same helpers), so results are identical.
#include "scan_impl.cuh"

namespace tgpu {

namespace {

template <class P>
__device__ __forceinline__ void scan_chunk_inline(const DevQuery &q, const ScanSmem &sm, uint32_t c,
                                                  unsigned long long &selected) {
    using Row = typename P::Row;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t row0, row_end;
    chunk_rows(q, c, row0, row_end);
    if (row0 >= row_end) return;
    if (q.n_preds == 0 || !q.gather) {
        // every row (or every row in place under the WHERE): rolling batches
        // of 32 consecutive rows
        Row cur;
        uint64_t r = row0 + lane;
        P::load(q, r, r < row_end, cur);
        unsigned act = __ballot_sync(FULL, r < row_end && row_passes(q, r));
        unsigned keep = __ballot_sync(FULL, P::prefetch(q, cur, (act >> lane) & 1u));
        for (uint64_t base = row0; base < row_end; base += 32) {
            Row nxt;
            const uint64_t rn = base + 32 + lane;
            P::load(q, rn, rn < row_end, nxt);
            const unsigned act_n = __ballot_sync(FULL, rn < row_end && row_passes(q, rn));
            const unsigned keep_n = __ballot_sync(FULL, P::prefetch(q, nxt, (act_n >> lane) & 1u));
            selected += (lane == 0) ? __popc(act) : 0;
            P::reserve(q, cur, (keep >> lane) & 1u);
            if (keep) P::fold_body(q, sm, cur, keep);
            cur = nxt;
            act = act_n;
            keep = keep_n;
        }
        return;
    }
    // gather mode: the chunk's survivors first, then rolling batches of 32
    uint16_t *list = sm.wlist + (size_t)warp * q.chunk_rows;
    const uint32_t n = survivors(q, row0, row_end, list);
    __syncwarp();
    selected += (lane == 0) ? n : 0;
    if (n == 0) return;
    Row cur;
    P::load(q, row0 + list[lane < n ? lane : 0], lane < n, cur);
    unsigned keep = __ballot_sync(FULL, P::prefetch(q, cur, lane < n));
    for (uint32_t i = 0; i < n; i += 32) {
        Row nxt;
        const uint32_t s = i + 32 + lane;
        P::load(q, row0 + list[s < n ? s : 0], s < n, nxt);
        const unsigned keep_n = __ballot_sync(FULL, P::prefetch(q, nxt, s < n));
        P::reserve(q, cur, (keep >> lane) & 1u);
        if (keep) P::fold_body(q, sm, cur, keep);
        cur = nxt;
        keep = keep_n;
    }
}

template <class P>
__global__ void __launch_bounds__(SCAN_THREADS, 2) scan_inline_kernel(const __grid_constant__ DevQuery q) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const ScanSmem sm = carve(q, smem_raw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    cache_init(q, sm);
    __syncthreads();
    unsigned long long selected = 0;
    const uint32_t nw = gridDim.x * SCAN_WARPS;
    uint32_t k = 0;
    for (uint32_t c = blockIdx.x * SCAN_WARPS + warp; c < q.n_chunks; c += nw, ++k) {
        if ((k & 31) == 31 && q.cancel) {  // poll the host-mapped cancel flag now and then
            int stop = 0;
            if (lane == 0) stop = *q.cancel;
            if (__shfl_sync(FULL, stop, 0)) {
                if (lane == 0) atomicOr(q.status, ST_CANCELLED);
                break;
            }
        }
        prefetch_chunk(q, c + nw);  // this warp's next chunk
        scan_chunk_inline<P>(q, sm, c, selected);
    }
    if (q.cache_slots) {
        __syncthreads();
        cache_flush(q, sm);
    }
    if (lane == 0 && selected) atomicAdd(q.selected_rows, selected);
}

}  // namespace

const void *inline_scan_kernel(const DevQuery &q) {
    switch (q.fast_id) {
#define TGPU_INL(I, KM, A, B, C2, D) \
    case I: return (const void *)scan_inline_kernel<FastFold<KM, A, B, C2, D>>;
        TGPU_FAST_FOLDS(TGPU_INL)
#undef TGPU_INL
        default: return nullptr;
    }
}

cudaError_t launch_scan_inline(const DevQuery &q, int grid, size_t smem, cudaStream_t s) {
    const void *fn = inline_scan_kernel(q);
    if (!fn) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    void *args[] = {(void *)&q};
    return cudaLaunchKernel(fn, dim3(grid), dim3(SCAN_THREADS), args, smem, s);
}

}  // namespace tgpu
