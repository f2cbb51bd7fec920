// distinct.cu — the second phase of the partitioned COUNT(DISTINCT).
//
// thinDB counts distinct values per group with a (group, value) set per
// bucket (silo_group_core.zig DistinctSet :663-777, foldGroupDistinctTypedImpl
// :8125-8176).  Here the scan appends every (value, gid) pair to one of
// 2^dpart_bits hash partitions (scan_impl.cuh dpart_store); then this kernel
// deduplicates each partition in shared memory and adds one to the group's
// distinct-count word for every pair seen first.  No global set, no
// DRAM-random probes: the pairs stream in once.
//
// Persistent: one 1,024-thread CTA per SM walks partitions b, b + grid, ...
// A ring of S partition buffers (S = 3 where the device's shared memory per
// block allows, else 2) is filled by one bulk asynchronous copy per partition
// (its pairs are contiguous: 16-byte aligned, a multiple of 16 bytes),
// completing on the stage's mbarrier, so the next partitions' pairs arrive
// while the CTA deduplicates the current one.  Per partition: clear the
// 8,192-slot index table, wait for the stage (bounded), insert each pair's
// index (a slot holds the index of the first pair with that content;
// equality compares the full pair, so the count is exact), barrier, refill
// the stage with partition i + S.
#include <algorithm>
#include <mutex>

#include "bulk.cuh"
#include "common.cuh"

namespace tgpu {

namespace {

constexpr int DP_THREADS = 1024;
constexpr uint32_t DP_MAX_STAGES = 3;
constexpr uint32_t DP_EMPTY = 0xFFFFFFFFu;
constexpr size_t DP_HEADER = 64;  // mbarriers, pair counts, stop flag

struct DpHeader {
    uint64_t bars[DP_MAX_STAGES];
    uint32_t n[DP_MAX_STAGES];
    int stop;
};
static_assert(sizeof(DpHeader) <= DP_HEADER, "header fits");

// Thread 0: start the copy of partition p's pairs into `dst`.
__device__ __forceinline__ void dp_issue(const ulonglong2 *buf, const uint32_t *cursor, uint32_t cap, uint32_t p,
                                         ulonglong2 *dst, uint64_t *bar, uint32_t *n_out) {
    const uint32_t n = min(__ldcg(cursor + p), cap);  // a larger count set ST_DISTINCT_FULL already
    *n_out = n;
    mbar_arrive_tx(bar, n * (uint32_t)sizeof(ulonglong2));
    if (n) bulk_load(dst, buf + (size_t)p * cap, n * (uint32_t)sizeof(ulonglong2), bar);
}

__global__ void __launch_bounds__(DP_THREADS, 1)
    distinct_partition_kernel(const ulonglong2 *__restrict__ buf, const uint32_t *__restrict__ cursor, uint32_t cap,
                              uint32_t n_parts, uint32_t S, unsigned long long *table, uint64_t max_gid,
                              int32_t slot_words, int32_t key_words, int32_t word, unsigned int *status,
                              long long wait_cycles) {
    extern __shared__ __align__(16) unsigned char smem[];
    DpHeader &h = *(DpHeader *)smem;
    ulonglong2 *ring = (ulonglong2 *)(smem + DP_HEADER);
    uint32_t *slots = (uint32_t *)(smem + DP_HEADER + (size_t)S * cap * sizeof(ulonglong2));
    const uint32_t G = gridDim.x;
    const uint32_t my_n = n_parts > blockIdx.x ? (n_parts - blockIdx.x + G - 1) / G : 0;

    uint32_t issued = 0;  // thread 0's count of partitions started
    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < S; ++s) mbar_init(&h.bars[s]);
        mbar_init_fence();
        h.stop = 0;
        for (; issued < S && issued < my_n; ++issued)
            dp_issue(buf, cursor, cap, blockIdx.x + issued * G, ring + (size_t)issued * cap, &h.bars[issued],
                     &h.n[issued]);
    }
    __syncthreads();

    uint32_t i = 0;
    for (; i < my_n; ++i) {
        const uint32_t s = i % S;
        for (uint32_t j = threadIdx.x; j < DPART_SLOTS; j += DP_THREADS) slots[j] = DP_EMPTY;
        if (!mbar_wait(&h.bars[s], (i / S) & 1u, wait_cycles)) {
            atomicOr(status, ST_WAIT_TIMEOUT);
            h.stop = 1;
        }
        __syncthreads();
        if (h.stop) break;
        const uint32_t n = h.n[s];
        const ulonglong2 *pairs = ring + (size_t)s * cap;
        for (uint32_t j = threadIdx.x; j < n; j += DP_THREADS) {
            const ulonglong2 me = pairs[j];
            const uint32_t gid = (uint32_t)me.y;
            uint32_t at = (uint32_t)mix64(me.x ^ mix64(gid)) & (DPART_SLOTS - 1);
            bool fresh = false, done = false;
            for (uint32_t probe = 0; probe < DPART_SLOTS && !done; ++probe) {
                uint32_t cur = slots[at];
                if (cur == DP_EMPTY) {
                    cur = atomicCAS(&slots[at], DP_EMPTY, j);
                    if (cur == DP_EMPTY) {
                        fresh = true;
                        done = true;
                        break;
                    }
                }
                const ulonglong2 other = pairs[cur];
                if (other.x == me.x && other.y == me.y) {
                    done = true;
                    break;
                }
                at = (at + 1) & (DPART_SLOTS - 1);
            }
            if (!done) atomicOr(status, ST_BAD_INDEX);  // cannot happen: n <= cap < DPART_SLOTS
            // a pair stored with no group (NO_GID: the table filled up, the
            // host reruns) is deduplicated like any other and counted nowhere
            if (fresh && gid <= max_gid)
                asm volatile("red.global.add.u64 [%0], 1;" ::"l"(table + (uint64_t)gid * slot_words + key_words + word)
                             : "memory");
        }
        __syncthreads();  // stage s and the slots are free again
        if (threadIdx.x == 0 && issued < my_n) {
            fence_proxy_async_smem();
            const uint32_t r = issued % S;
            dp_issue(buf, cursor, cap, blockIdx.x + issued * G, ring + (size_t)r * cap, &h.bars[r], &h.n[r]);
            ++issued;
        }
    }
    if (h.stop && threadIdx.x == 0) {
        // leave no copy in flight into this CTA's shared memory (bounded by
        // the built-in limit: the copies are real and land)
        for (uint32_t j = i; j < issued; ++j) (void)mbar_wait(&h.bars[j % S], (j / S) & 1u);
    }
}

struct DpLaunch {
    int sms = 0;
    uint32_t stages = 0;
};

DpLaunch dp_launch_shape(uint32_t cap) {
    static std::mutex mu;
    static DpLaunch cached[64];  // per device ordinal
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    DpLaunch &d = cached[dev & 63];
    if (!d.sms) {
        int optin = 0, sms = 0;
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const size_t fixed = DP_HEADER + DPART_SLOTS * sizeof(uint32_t);
        const size_t per = (size_t)cap * sizeof(ulonglong2);
        uint32_t st = DP_MAX_STAGES;
        while (st > 2 && fixed + st * per > (size_t)optin) --st;
        d.stages = st;
        d.sms = sms > 0 ? sms : 1;
    }
    return d;
}

}  // namespace

cudaError_t launch_distinct_partitions(const DevQuery &q, int word, cudaStream_t s) {
    if (!q.dpart_bits) return cudaSuccess;
    const DpLaunch d = dp_launch_shape(q.dpart_cap);
    const size_t smem = DP_HEADER + (size_t)d.stages * q.dpart_cap * sizeof(ulonglong2) + DPART_SLOTS * sizeof(uint32_t);
    cudaError_t e = cudaFuncSetAttribute(distinct_partition_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    const uint32_t n_parts = 1u << q.dpart_bits;
    const uint32_t grid = std::min<uint32_t>(n_parts, (uint32_t)d.sms);
    distinct_partition_kernel<<<grid, DP_THREADS, smem, s>>>(q.dpart_buf, q.dpart_cursor, q.dpart_cap, n_parts,
                                                              d.stages, q.table, q.cap, q.slot_words, q.key_words,
                                                              word, q.status, q.wait_cycles);
    return cudaGetLastError();
}

}  // namespace tgpu
