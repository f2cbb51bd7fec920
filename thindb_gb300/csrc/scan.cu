// scan.cu — single-query scan kernels: one instantiation per compiled fold
// signature plus the interpreter, and their launchers.
#include "scan_impl.cuh"

namespace tgpu {

namespace {

// ---------------------------------------------------------------- kernel --

template <class P, int MINB, bool QUEUE>
__global__ void __launch_bounds__(SCAN_THREADS, MINB) scan_group_kernel(const __grid_constant__ DevQuery q) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const ScanSmem sm = carve(q, smem_raw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    cache_init(q, sm);
    __syncthreads();
    unsigned long long selected = 0;
    const uint32_t nw = gridDim.x * SCAN_WARPS;
    WarpQueue<P> wq{(typename P::Row *)sm.wlist + (size_t)warp * WQ_ROWS, 0u, 0u};
    if constexpr (QUEUE)
        static_assert(sizeof(typename P::Row) <= 24 + 8 * P::NV, "queue ring rows sized in scan_smem_bytes");
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
        if constexpr (QUEUE) scan_chunk_queue<P>(q, sm, c, selected, wq);
        else scan_chunk<P>(q, sm, c, selected);
    }
    if constexpr (QUEUE) wq_flush<P>(q, sm, wq);
    if (q.cache_slots) {
        __syncthreads();
        cache_flush(q, sm);
    }
    if (lane == 0 && selected) atomicAdd(q.selected_rows, selected);
}

// The scan kernel a plan runs: a compiled fast fold when its signature is in
// the table above, else the interpreter.
struct ScanKernel {
    const void *fn;
};

template <class P, int MINB, bool QUEUE = false>
static ScanKernel kernel_of() {
    return ScanKernel{(const void *)scan_group_kernel<P, MINB, QUEUE>};
}

int fold_id_of(const DevQuery &q) {
    if (!q.fast_km) return -1;
    const int k[4] = {q.n_faggs > 0 ? q.faggs[0].kind : AK_NONE, q.n_faggs > 1 ? q.faggs[1].kind : AK_NONE,
                      q.n_faggs > 2 ? q.faggs[2].kind : AK_NONE, q.n_faggs > 3 ? q.faggs[3].kind : AK_NONE};
#define TGPU_MATCH(I, KM, A, B, C2, D) \
    if (q.fast_km == KM && k[0] == A && k[1] == B && k[2] == C2 && k[3] == D) return I;
    TGPU_FAST_FOLDS(TGPU_MATCH)
#undef TGPU_MATCH
    return -1;
}

ScanKernel pick_kernel(const DevQuery &q) {
    const bool queue = q.gather == 2;
    switch (fold_id_of(q)) {
#define TGPU_PICK(I, KM, A, B, C2, D)                                                       \
    case I:                                                                                  \
        return queue ? kernel_of<FastFold<KM, A, B, C2, D>, 2, true>() : kernel_of<FastFold<KM, A, B, C2, D>, 2>();
        TGPU_FAST_FOLDS(TGPU_PICK)
#undef TGPU_PICK
        default: break;
    }
    if (q.n_aggs <= 4) return kernel_of<GenericFold<4>, 2>();
    return kernel_of<GenericFold<16>, 1>();
}

}  // namespace

int fast_fold_id(const DevQuery &q) { return fold_id_of(q); }

size_t scan_smem_bytes(const DevQuery &q) {
    size_t list = 0;
    if (q.gather == 1) list = (size_t)SCAN_WARPS * q.chunk_rows * 2;
    // a fold row: two key words, one word per input, and a COUNT(DISTINCT)
    // row's reserved pair place (8 bytes, counted for every fold)
    if (q.gather == 2) list = (size_t)SCAN_WARPS * WQ_ROWS * (24 + 8 * (size_t)(q.n_faggs > 0 ? q.n_faggs : 1));
    return (size_t)q.cache_slots * (8 + 8 * (size_t)q.state_words + 4) + 16 + list + 16;
}

static int blocks_per_sm(const void *kernel, size_t smem) {
    int per_sm = 1;
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, SCAN_THREADS, smem);
    if (e != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    return per_sm;
}

bool scan_is_fast(const DevQuery &q) {
    const ScanKernel k = pick_kernel(q);
    return k.fn != kernel_of<GenericFold<4>, 2>().fn && k.fn != kernel_of<GenericFold<16>, 1>().fn;
}

// The inlined-fold loop serves compiled folds outside queue mode.
static bool use_inline(const DevQuery &q) { return q.inline_fold && q.gather != 2 && inline_scan_kernel(q); }

int scan_grid_size(const DevQuery &q, int sms) {
    // persistent grid: every CTA that fits on an SM at once
    const void *fn = use_inline(q) ? inline_scan_kernel(q) : pick_kernel(q).fn;
    return sms * blocks_per_sm(fn, scan_smem_bytes(q));
}

cudaError_t launch_scan(const DevQuery &q, int grid, cudaStream_t s) {
    const size_t smem = scan_smem_bytes(q);
    if (use_inline(q)) return launch_scan_inline(q, grid, smem, s);
    const ScanKernel k = pick_kernel(q);
    cudaError_t e = cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    void *args[] = {(void *)&q};
    return cudaLaunchKernel(k.fn, dim3(grid), dim3(SCAN_THREADS), args, smem, s);
}

}  // namespace tgpu
