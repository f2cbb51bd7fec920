// scan_batch.cu — the batched persistent scan kernels (many queries, one
// launch per fold class) and their launchers.
#include "scan_impl.cuh"

namespace tgpu {

namespace {

// Many queries of one fold class in one persistent kernel.  A work item is
// (query, that query's surviving row groups within a window of about
// BATCH_WINDOW_ROWS rows) as a chunk range; the host lists a class's items
// window by window, every query of a window in turn, so the CTAs running at
// any moment read the same window and all but the first query of it find
// its columns in L2.  CTA b takes items b, b + grid, ...; its 16 warps split
// the item's chunks, and the CTA's shared-memory table belongs to the item's
// query (flushed when the next item moves to another query: once per item,
// a few hundred times per query).  One kernel per fold class
// (rather than one kernel switching between every compiled fold) keeps each
// kernel's code as small as a single-query scan's.
template <class P, int MINB>
__global__ void __launch_bounds__(SCAN_THREADS, MINB)
    batch_scan_kernel(const DevQuery *__restrict__ qs, const uint4 *__restrict__ items, uint32_t n_items,
                      const volatile int *cancel, unsigned int *batch_status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int cur = -1;
    ScanSmem sm{};
    unsigned long long selected = 0;
    uint32_t k = 0;
    for (uint32_t item = blockIdx.x;; item += gridDim.x, ++k) {
        bool stop = item >= n_items;
        if (!stop && (k & 15) == 15 && cancel) {
            int c = 0;
            if (threadIdx.x == 0) c = *cancel;
            stop = __syncthreads_or(c) != 0;
            if (stop && threadIdx.x == 0) atomicOr(batch_status, ST_CANCELLED);
        }
        const uint4 it = stop ? make_uint4(0xFFFFFFFFu, 0u, 0u, 0u) : items[item];
        const int qn = stop ? -1 : (int)it.x;
        if (qn != cur) {
            if (cur >= 0) {
                const DevQuery &old = qs[cur];
                __syncthreads();
                if (old.cache_slots) cache_flush(old, sm);
                if (lane == 0 && selected) atomicAdd(old.selected_rows, selected);
                selected = 0;
            }
            if (qn < 0) break;
            __syncthreads();
            sm = carve(qs[qn], smem_raw);
            cache_init(qs[qn], sm);
            cur = qn;
            __syncthreads();
        }
        if (qn < 0) break;  // a CTA that got no item at all (cur == qn == -1)
        const DevQuery &q = qs[qn];
        const uint32_t end = min(it.z, q.n_chunks);
        for (uint32_t c = it.y + warp; c < end; c += SCAN_WARPS) scan_chunk<P>(q, sm, c, selected);
    }
}

// Kernel of fold class `cls` (batch_fold_class).
const void *batch_kernel(int cls) {
    switch (cls) {
#define TGPU_BK(I, KM, A, B, C2, D) \
    case I: return (const void *)batch_scan_kernel<FastFold<KM, A, B, C2, D>, 2>;
        TGPU_FAST_FOLDS(TGPU_BK)
#undef TGPU_BK
        case BATCH_GENERIC4: return (const void *)batch_scan_kernel<GenericFold<4>, 2>;
        default: return (const void *)batch_scan_kernel<GenericFold<16>, 1>;
    }
}

int blocks_per_sm(const void *kernel, size_t smem) {
    int per_sm = 1;
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, SCAN_THREADS, smem);
    if (e != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    return per_sm;
}

}  // namespace

int batch_fold_class(const DevQuery &q) {
    if (q.n_aggs > 4) return BATCH_GENERIC16;
    return q.fast_id >= 0 ? q.fast_id : BATCH_GENERIC4;
}

int batch_scan_grid(int cls, size_t smem, int sms) { return sms * blocks_per_sm(batch_kernel(cls), smem); }

cudaError_t launch_batch_scan(int cls, const DevQuery *qs, const uint4 *items, uint32_t n_items, size_t smem,
                              int grid, const volatile int *cancel, unsigned int *status, cudaStream_t s) {
    if (n_items == 0) return cudaSuccess;
    if ((uint32_t)grid > n_items) grid = (int)n_items;
    const void *fn = batch_kernel(cls);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    void *args[] = {(void *)&qs, (void *)&items, (void *)&n_items, (void *)&cancel, (void *)&status};
    return cudaLaunchKernel(fn, dim3(grid), dim3(SCAN_THREADS), args, smem, s);
}

}  // namespace tgpu
