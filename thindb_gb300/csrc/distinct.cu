// distinct.cu — the second phase of the partitioned COUNT(DISTINCT).
//
// thinDB counts distinct values per group with a (group, value) set per
// bucket (silo_group_core.zig DistinctSet :663-777, foldGroupDistinctTypedImpl
// :8125-8176).  Here the scan appends every (value, gid) pair to one of
// 2^dpart_bits hash partitions (scan_impl.cuh dpart_append); then one CTA per
// partition loads the partition's pairs into shared memory, inserts each
// pair's index into a shared-memory hash table (a slot holds the index of the
// first pair with that content; equality compares the full pairs, so the
// count is exact), and adds one to the group's distinct-count word for every
// pair that claimed a slot.  No global set, no DRAM-random probes: the pairs
// stream in and out once.
#include "common.cuh"

namespace tgpu {

namespace {

constexpr int DP_THREADS = 512;
constexpr uint32_t DP_EMPTY = 0xFFFFFFFFu;

__global__ void __launch_bounds__(DP_THREADS, 2)
    distinct_partition_kernel(const ulonglong2 *__restrict__ buf, const uint32_t *__restrict__ cursor, uint32_t cap,
                              unsigned long long *table, int32_t slot_words, int32_t key_words, int32_t word,
                              unsigned int *status) {
    extern __shared__ __align__(16) unsigned char smem[];
    ulonglong2 *pairs = (ulonglong2 *)smem;                         // cap pairs
    uint32_t *slots = (uint32_t *)(smem + (size_t)cap * sizeof(ulonglong2));  // DPART_SLOTS
    const uint32_t p = blockIdx.x;
    const uint32_t n = min(cursor[p], cap);  // a larger count set ST_DISTINCT_FULL already
    if (n == 0) return;
    const ulonglong2 *src = buf + (size_t)p * cap;
    // four 16-byte loads in flight per thread before the stores
    for (uint32_t i0 = threadIdx.x; i0 < n; i0 += 4 * blockDim.x) {
        ulonglong2 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t i = i0 + u * blockDim.x;
            if (i < n) v[u] = __ldcs(src + i);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t i = i0 + u * blockDim.x;
            if (i < n) pairs[i] = v[u];
        }
    }
    for (uint32_t i = threadIdx.x; i < DPART_SLOTS; i += blockDim.x) slots[i] = DP_EMPTY;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const ulonglong2 me = pairs[i];
        const uint32_t gid = (uint32_t)me.y;
        uint32_t s = (uint32_t)mix64(me.x ^ mix64(gid)) & (DPART_SLOTS - 1);
        bool fresh = false, done = false;
        for (uint32_t probe = 0; probe < DPART_SLOTS && !done; ++probe) {
            uint32_t cur = slots[s];
            if (cur == DP_EMPTY) {
                cur = atomicCAS(&slots[s], DP_EMPTY, i);
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
            s = (s + 1) & (DPART_SLOTS - 1);
        }
        if (!done) atomicOr(status, ST_BAD_INDEX);  // cannot happen: n <= cap < DPART_SLOTS
        if (fresh) atomicAdd(table + (uint64_t)gid * slot_words + key_words + word, 1ULL);
    }
}

}  // namespace

cudaError_t launch_distinct_partitions(const DevQuery &q, int word, cudaStream_t s) {
    if (!q.dpart_bits) return cudaSuccess;
    const size_t smem = (size_t)q.dpart_cap * sizeof(ulonglong2) + DPART_SLOTS * sizeof(uint32_t);
    cudaError_t e = cudaFuncSetAttribute(distinct_partition_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    distinct_partition_kernel<<<1u << q.dpart_bits, DP_THREADS, smem, s>>>(
        q.dpart_buf, q.dpart_cursor, q.dpart_cap, q.table, q.slot_words, q.key_words, word, q.status);
    return cudaGetLastError();
}

}  // namespace tgpu
