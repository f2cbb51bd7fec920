// scan_batch.cu — the batched persistent scan kernel (many queries, one
// launch) and its launchers.
#include "scan_impl.cuh"

namespace tgpu {

namespace {

// Many queries in one persistent kernel: work items are (query, tile of
// SCAN_WARPS chunks) pairs, query-major.  CTA b takes items b, b + grid, ...;
// all warps of a CTA work on one query's tile at a time, so the CTA's
// shared-memory table belongs to that query until its next item moves on,
// when the table is flushed.
template <int NA>
__global__ void __launch_bounds__(SCAN_THREADS, NA <= 4 ? 2 : 1)
    batch_scan_kernel(const DevQuery *__restrict__ qs, const uint32_t *__restrict__ tile_start, uint32_t n_queries,
                      unsigned int *work_counter, const volatile int *cancel, unsigned int *batch_status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t total = tile_start[n_queries];
    (void)work_counter;
    int cur = -1;
    uint32_t qi = 0;
    ScanSmem sm{};
    unsigned long long selected = 0;
    uint32_t k = 0;
    for (uint32_t item = blockIdx.x;; item += gridDim.x, ++k) {
        bool stop = item >= total;
        if (!stop && (k & 15) == 15 && cancel) {
            int c = 0;
            if (threadIdx.x == 0) c = *cancel;
            stop = __syncthreads_or(c) != 0;
            if (stop && threadIdx.x == 0) atomicOr(batch_status, ST_CANCELLED);
        }
        int qn = -1;
        if (!stop) {
            while (qi + 1 < n_queries && tile_start[qi + 1] <= item) ++qi;  // items only grow
            qn = (int)qi;
        }
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
        if (qn < 0) break;
        const DevQuery &q = qs[qn];
        const uint32_t c = (item - tile_start[qn]) * SCAN_WARPS + warp;
        if (c < q.n_chunks) scan_chunk_dispatch<NA>(q, sm, c, selected);
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

int batch_scan_grid(int max_aggs, size_t smem, int sms) {
    return sms * (max_aggs <= 4 ? blocks_per_sm((const void *)batch_scan_kernel<4>, smem)
                                : blocks_per_sm((const void *)batch_scan_kernel<16>, smem));
}

cudaError_t launch_batch_scan(const DevQuery *qs, const uint32_t *tile_start, uint32_t n_queries, int max_aggs,
                              size_t smem, int grid, unsigned int *work_counter, const volatile int *cancel,
                              unsigned int *status, cudaStream_t s) {
    if (max_aggs <= 4) {
        cudaError_t e = cudaFuncSetAttribute(batch_scan_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        batch_scan_kernel<4><<<grid, SCAN_THREADS, smem, s>>>(qs, tile_start, n_queries, work_counter, cancel, status);
    } else {
        cudaError_t e = cudaFuncSetAttribute(batch_scan_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        batch_scan_kernel<16><<<grid, SCAN_THREADS, smem, s>>>(qs, tile_start, n_queries, work_counter, cancel, status);
    }
    return cudaGetLastError();
}

}  // namespace tgpu
