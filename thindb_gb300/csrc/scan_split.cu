// scan_split.cu — the split scan: the WHERE as its own streaming pass that
// writes the surviving row numbers, then a fold pass over that list.
//
// The fused gather-mode scan (scan_chunk) runs filter -> compaction ->
// gather -> fold per warp and chunk, so every warp waits on its own filter
// before its gathers can start.  Split, the select pass only streams the
// predicate column (one atomicAdd per chunk reserves the chunk's place in the
// list) and the fold pass reads the list densely: every batch of 32 rows is
// full, and a warp's LOOKAHEAD batches of gathers are in flight at once with
// their row numbers known up front.  The list costs 4 bytes per survivor
// written and read again.
#include "scan_impl.cuh"

namespace tgpu {

namespace {

__global__ void __launch_bounds__(SCAN_THREADS) select_rows_kernel(const __grid_constant__ DevQuery q, uint32_t *rows,
                                                                   unsigned long long *n_rows) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint16_t *list = (uint16_t *)smem_raw + (size_t)warp * q.chunk_rows;
    unsigned long long selected = 0;
    const uint32_t nw = gridDim.x * SCAN_WARPS;
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
        uint64_t row0, row_end;
        chunk_rows(q, c, row0, row_end);
        if (row0 >= row_end) continue;
        const uint32_t n = survivors(q, row0, row_end, list);
        __syncwarp();
        if (n) {
            unsigned long long at = 0;
            if (lane == 0) at = atomicAdd(n_rows, (unsigned long long)n);
            at = __shfl_sync(FULL, at, 0);
            for (uint32_t i = lane; i < n; i += 32) rows[at + i] = (uint32_t)(row0 + list[i]);
            selected += lane == 0 ? n : 0;
        }
        __syncwarp();
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

size_t split_select_smem(const DevQuery &q) { return (size_t)SCAN_WARPS * q.chunk_rows * 2; }

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
    const size_t fs = split_fold_smem(q);
    const void *fn = fold_rows_fn(q);
    const int fgrid = sms * per_sm(fn, fs);
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fs);
    if (e != cudaSuccess) return e;
    const unsigned long long *cn = n_rows;
    void *args[] = {(void *)&q, (void *)&rows, (void *)&cn};
    return cudaLaunchKernel(fn, dim3(fgrid), dim3(SCAN_THREADS), args, fs, s);
}

}  // namespace tgpu
