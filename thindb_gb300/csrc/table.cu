// table.cu — per-row-group zone maps and HyperLogLog NDV sketches, built
// once when a table is registered.
//
// thinDB keeps min/max per column per row group in the segment footer and
// prunes row groups with them before decoding (scan.zig rowGroupCanMatch
// :3539, predicate.zig statsOverlapPredicate :3380); its NDV estimates come
// from HLL sketches (src/util/hll.zig) and feed group-table sizing
// (silo_group_core.zig expectedTotalGroups :11398).  Here both are computed
// on the device from the resident columns.
#include <algorithm>
#include <cfloat>
#include <climits>

#include <math_constants.h>

#include "common.cuh"

namespace tgpu {

namespace {

__device__ __forceinline__ bool valid_at(const uint32_t *v, uint64_t r) {
    return v == nullptr || ((v[r >> 5] >> (r & 31)) & 1u);
}

__device__ __forceinline__ int64_t int_at(const void *d, int32_t type, uint64_t r) {
    switch (type) {
        case TGPU_BOOLEAN: return ((const uint8_t *)d)[r];
        case TGPU_TINYINT: return ((const int8_t *)d)[r];
        case TGPU_SMALLINT: return ((const int16_t *)d)[r];
        case TGPU_INT: case TGPU_DATE: case TGPU_DICT32: return ((const int32_t *)d)[r];
        default: return ((const long long *)d)[r];
    }
}

__device__ __forceinline__ double f_at(const void *d, int32_t type, uint64_t r) {
    return type == TGPU_FLOAT ? (double)((const float *)d)[r] : ((const double *)d)[r];
}

// One CTA per row group: min/max over the valid rows and the NULL count.
__global__ void zone_map_kernel(const void *data, const uint32_t *valid, int32_t type, uint64_t n_rows,
                                uint32_t rg_rows, int64_t *imin, int64_t *imax, double *zfmin, double *zfmax,
                                uint32_t *nulls) {
    __shared__ long long smin[32], smax[32];
    __shared__ double sfmin[32], sfmax[32];
    __shared__ unsigned snull[32];
    const uint64_t b = (uint64_t)blockIdx.x * rg_rows, e = min(b + rg_rows, n_rows);
    const bool is_f = type == TGPU_FLOAT || type == TGPU_DOUBLE;
    long long mn = LLONG_MAX, mx = LLONG_MIN;
    double fmn = DBL_MAX, fmx = -DBL_MAX;
    unsigned nn = 0;
    for (uint64_t r = b + threadIdx.x; r < e; r += blockDim.x) {
        if (!valid_at(valid, r)) {
            ++nn;
            continue;
        }
        if (is_f) {
            double x = f_at(data, type, r);
            if (x == x) {
                fmn = fmin(fmn, x);
                fmx = fmax(fmx, x);
            } else {
                fmx = CUDART_INF;  // a NaN row can satisfy only open ranges; keep the map conservative
            }
        } else {
            long long x = int_at(data, type, r);
            mn = min(mn, x);
            mx = max(mx, x);
        }
    }
    for (int o = 16; o; o >>= 1) {
        mn = min(mn, __shfl_down_sync(0xFFFFFFFFu, mn, o));
        mx = max(mx, __shfl_down_sync(0xFFFFFFFFu, mx, o));
        fmn = fmin(fmn, __shfl_down_sync(0xFFFFFFFFu, fmn, o));
        fmx = fmax(fmx, __shfl_down_sync(0xFFFFFFFFu, fmx, o));
        nn += __shfl_down_sync(0xFFFFFFFFu, nn, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        smin[warp] = mn;
        smax[warp] = mx;
        sfmin[warp] = fmn;
        sfmax[warp] = fmx;
        snull[warp] = nn;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            mn = min(mn, smin[w]);
            mx = max(mx, smax[w]);
            fmn = fmin(fmn, sfmin[w]);
            fmx = fmax(fmx, sfmax[w]);
            nn += snull[w];
        }
        imin[blockIdx.x] = mn;
        imax[blockIdx.x] = mx;
        zfmin[blockIdx.x] = fmn;
        zfmax[blockIdx.x] = fmx;
        nulls[blockIdx.x] = nn;
    }
}

constexpr int HLL_M = 1 << HLL_P;

// HyperLogLog registers: index = top HLL_P bits of mix64(value bits), rank =
// leading zeros of the rest + 1 (Flajolet et al. 2007).
__global__ void hll_kernel(const void *data, const uint32_t *valid, int32_t type, uint64_t n_rows, uint32_t *regs,
                           const uint32_t *offs) {
    extern __shared__ uint32_t sreg[];
    for (int i = threadIdx.x; i < HLL_M; i += blockDim.x) sreg[i] = 0;
    __syncthreads();
    const bool is_f = type == TGPU_FLOAT || type == TGPU_DOUBLE;
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n_rows; r += (uint64_t)gridDim.x * blockDim.x) {
        if (!valid_at(valid, r)) continue;
        uint64_t bits = offs ? str_hash((const uint8_t *)data + offs[r], offs[r + 1] - offs[r])
                             : is_f ? canon_f64_bits(f_at(data, type, r)) : (uint64_t)int_at(data, type, r);
        uint64_t h = mix64(bits ^ 0x6A09E667F3BCC909ULL);
        uint32_t idx = (uint32_t)(h >> (64 - HLL_P));
        uint64_t w = (h << HLL_P) | (1ULL << (HLL_P - 1));
        uint32_t rank = (uint32_t)__clzll((long long)w) + 1;
        if (rank > sreg[idx]) atomicMax(&sreg[idx], rank);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < HLL_M; i += blockDim.x)
        if (sreg[i]) atomicMax(&regs[i], sreg[i]);
}

// HyperLogLog of composite keys: each row's parts' value bits chained
// through mix64 (a NULL part hashes as a marker), registers as above.  The
// product of the parts' NDVs overestimates the groups of correlated parts
// (a url belongs to one region), and the group table sized from it would
// spread the groups over many times the memory they need.
__global__ void key_hll_kernel(const __grid_constant__ KeySketchCols k, uint64_t n_rows, uint32_t *regs) {
    extern __shared__ uint32_t sreg[];
    for (int i = threadIdx.x; i < HLL_M; i += blockDim.x) sreg[i] = 0;
    __syncthreads();
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n_rows; r += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t h = 0x6A09E667F3BCC909ULL;
        for (int i = 0; i < k.n; ++i) {
            const bool is_f = k.type[i] == TGPU_FLOAT || k.type[i] == TGPU_DOUBLE;
            uint64_t bits = 0x8000000000000001ULL;  // NULL
            if (valid_at(k.valid[i], r))
                bits = k.offs[i] ? str_hash((const uint8_t *)k.data[i] + k.offs[i][r], k.offs[i][r + 1] - k.offs[i][r])
                       : is_f ? canon_f64_bits(f_at(k.data[i], k.type[i], r)) : (uint64_t)int_at(k.data[i], k.type[i], r);
            h = mix64(h ^ bits);
        }
        uint32_t idx = (uint32_t)(h >> (64 - HLL_P));
        uint64_t w = (h << HLL_P) | (1ULL << (HLL_P - 1));
        uint32_t rank = (uint32_t)__clzll((long long)w) + 1;
        if (rank > sreg[idx]) atomicMax(&sreg[idx], rank);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < HLL_M; i += blockDim.x)
        if (sreg[i]) atomicMax(&regs[i], sreg[i]);
}

}  // namespace

cudaError_t launch_zone_maps(const void *data, const uint32_t *valid, int32_t type, uint64_t n_rows,
                             uint32_t rg_rows, uint32_t n_rg, int64_t *imin, int64_t *imax, double *fmin,
                             double *fmax, uint32_t *nulls, cudaStream_t s) {
    if (n_rg == 0) return cudaSuccess;
    zone_map_kernel<<<n_rg, 256, 0, s>>>(data, valid, type, n_rows, rg_rows, imin, imax, fmin, fmax, nulls);
    return cudaGetLastError();
}

cudaError_t launch_hll(const void *data, const uint32_t *valid, int32_t type, uint64_t n_rows, uint32_t *regs,
                       cudaStream_t s, const uint32_t *offs) {
    if (n_rows == 0) return cudaSuccess;
    int grid = (int)std::min<uint64_t>((n_rows + 1023) / 1024, 1024);
    size_t smem = HLL_M * sizeof(uint32_t);
    cudaError_t e = cudaFuncSetAttribute(hll_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    hll_kernel<<<grid, 512, smem, s>>>(data, valid, type, n_rows, regs, offs);
    return cudaGetLastError();
}

cudaError_t launch_key_hll(const KeySketchCols &k, uint64_t n_rows, uint32_t *regs, cudaStream_t s) {
    if (n_rows == 0) return cudaSuccess;
    int grid = (int)std::min<uint64_t>((n_rows + 1023) / 1024, 1024);
    size_t smem = HLL_M * sizeof(uint32_t);
    cudaError_t e = cudaFuncSetAttribute(key_hll_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    key_hll_kernel<<<grid, 512, smem, s>>>(k, n_rows, regs);
    return cudaGetLastError();
}

}  // namespace tgpu
