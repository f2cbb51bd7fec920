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
#include <type_traits>

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

namespace {

// Zone maps and the HyperLogLog registers of one fixed-width column in one
// pass: persistent CTAs stride over the row groups (min/max/NULL count of
// each, reduced in the CTA) and raise their own shared-memory registers;
// each CTA then stores its registers as bytes to `part` (a row of HLL_M per
// CTA) and hll_merge_kernel takes the maximum over the rows: one read of the
// column, no global atomics.
template <typename T>
__global__ void __launch_bounds__(512) column_stats_kernel(const T *__restrict__ data, const uint32_t *__restrict__ valid,
                                                           uint64_t n_rows, uint32_t rg_rows, uint32_t g0, uint32_t g1,
                                                           int64_t *imin, int64_t *imax, double *zfmin, double *zfmax,
                                                           uint32_t *nulls, uint8_t *part) {
    extern __shared__ uint32_t sreg[];
    __shared__ long long smin[16], smax[16];
    __shared__ double sfmin[16], sfmax[16];
    __shared__ unsigned snull[16];
    constexpr bool is_f = std::is_floating_point<T>::value;
    if (part) {
        for (int i = threadIdx.x; i < HLL_M; i += blockDim.x) sreg[i] = 0;
        __syncthreads();
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t g = g0 + blockIdx.x; g < g1; g += gridDim.x) {
        const uint64_t b = (uint64_t)g * rg_rows, e = min(b + rg_rows, n_rows);
        long long mn = LLONG_MAX, mx = LLONG_MIN;
        double fmn = DBL_MAX, fmx = -DBL_MAX;
        unsigned nn = 0;
#pragma unroll 4
        for (uint64_t r = b + threadIdx.x; r < e; r += blockDim.x) {
            const bool ok = valid_at(valid, r);
            const T x = data[r];
            nn += ok ? 0u : 1u;
            uint64_t bits;
            if constexpr (is_f) {
                const double d = (double)x;
                if (ok) {
                    if (d == d) {
                        fmn = fmin(fmn, d);
                        fmx = fmax(fmx, d);
                    } else {
                        fmx = CUDART_INF;  // a NaN row can satisfy only open ranges; keep the map conservative
                    }
                }
                bits = canon_f64_bits(d);
            } else {
                const long long v = (long long)x;
                if (ok) {
                    mn = min(mn, v);
                    mx = max(mx, v);
                }
                bits = (uint64_t)v;
            }
            if (part && ok) {
                const uint64_t h = mix64(bits ^ 0x6A09E667F3BCC909ULL);
                const uint32_t idx = (uint32_t)(h >> (64 - HLL_P));
                const uint64_t w = (h << HLL_P) | (1ULL << (HLL_P - 1));
                const uint32_t rank = (uint32_t)__clzll((long long)w) + 1;
                if (rank > sreg[idx]) atomicMax(&sreg[idx], rank);
            }
        }
        for (int o = 16; o; o >>= 1) {
            mn = min(mn, __shfl_down_sync(0xFFFFFFFFu, mn, o));
            mx = max(mx, __shfl_down_sync(0xFFFFFFFFu, mx, o));
            fmn = fmin(fmn, __shfl_down_sync(0xFFFFFFFFu, fmn, o));
            fmx = fmax(fmx, __shfl_down_sync(0xFFFFFFFFu, fmx, o));
            nn += __shfl_down_sync(0xFFFFFFFFu, nn, o);
        }
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
            imin[g] = mn;
            imax[g] = mx;
            zfmin[g] = fmn;
            zfmax[g] = fmx;
            nulls[g] = nn;
        }
        __syncthreads();
    }
    if (part) {
        __syncthreads();
        uint8_t *row = part + (size_t)blockIdx.x * HLL_M;
        for (int i = threadIdx.x; i < HLL_M; i += blockDim.x) row[i] = (uint8_t)sreg[i];
    }
}

// regs = max(regs, every part row): grid (HLL_M / 4 / 256, slices); a
// thread takes four registers over a slice of the rows and raises them with
// atomicMax (regs start zeroed, or hold earlier rows' maxima)
__global__ void hll_merge_kernel(const uint8_t *__restrict__ part, uint32_t rows, uint32_t *regs) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;  // registers 4i .. 4i + 3
    if (i >= (uint32_t)HLL_M / 4) return;
    const uint32_t per = (rows + gridDim.y - 1) / gridDim.y, r0 = blockIdx.y * per, r1 = min(rows, r0 + per);
    const uint32_t *p = (const uint32_t *)part + i;
    uint32_t m = 0;
    for (uint32_t r = r0; r < r1; ++r) m = __vmaxu4(m, __ldg(p + (size_t)r * (HLL_M / 4)));
    for (int k = 0; k < 4; ++k) {
        const uint32_t v = (m >> (8 * k)) & 0xFFu;
        if (v) atomicMax(regs + 4 * i + k, v);
    }
}

template <typename T>
cudaError_t launch_stats_t(const void *data, const uint32_t *valid, uint64_t n_rows, uint32_t rg_rows, uint32_t g0,
                           uint32_t g1, int64_t *imin, int64_t *imax, double *fmin, double *fmax, uint32_t *nulls,
                           uint32_t *regs, uint8_t *part, int accumulate, cudaStream_t s) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    const uint32_t grid = std::max<uint32_t>(1, std::min<uint32_t>({g1 - g0, 2u * (uint32_t)sms, STATS_GRID_MAX}));
    const size_t smem = regs ? HLL_M * sizeof(uint32_t) : 0;
    cudaError_t e = cudaFuncSetAttribute(column_stats_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         HLL_M * (int)sizeof(uint32_t));
    if (e != cudaSuccess) return e;
    column_stats_kernel<T><<<grid, 512, smem, s>>>((const T *)data, valid, n_rows, rg_rows, g0, g1, imin, imax, fmin,
                                                    fmax, nulls, regs ? part : nullptr);
    e = cudaGetLastError();
    if (e != cudaSuccess || !regs) return e;
    if (!accumulate) {
        e = cudaMemsetAsync(regs, 0, HLL_M * sizeof(uint32_t), s);
        if (e != cudaSuccess) return e;
    }
    hll_merge_kernel<<<dim3(HLL_M / 4 / 256, std::min<uint32_t>(grid, 16)), 256, 0, s>>>(part, grid, regs);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_column_stats(const void *data, const uint32_t *valid, int32_t type, uint64_t n_rows,
                                uint32_t rg_rows, uint32_t g0, uint32_t g1, int64_t *imin, int64_t *imax, double *fmin,
                                double *fmax, uint32_t *nulls, uint32_t *regs, uint8_t *part, int accumulate,
                                cudaStream_t s) {
    if (g1 <= g0 || n_rows == 0) return cudaSuccess;
    switch (type) {
        case TGPU_BOOLEAN: return launch_stats_t<uint8_t>(data, valid, n_rows, rg_rows, g0, g1, imin, imax, fmin, fmax, nulls, regs, part, accumulate, s);
        case TGPU_TINYINT: return launch_stats_t<int8_t>(data, valid, n_rows, rg_rows, g0, g1, imin, imax, fmin, fmax, nulls, regs, part, accumulate, s);
        case TGPU_SMALLINT: return launch_stats_t<int16_t>(data, valid, n_rows, rg_rows, g0, g1, imin, imax, fmin, fmax, nulls, regs, part, accumulate, s);
        case TGPU_INT: case TGPU_DATE: case TGPU_DICT32:
            return launch_stats_t<int32_t>(data, valid, n_rows, rg_rows, g0, g1, imin, imax, fmin, fmax, nulls, regs, part, accumulate, s);
        case TGPU_FLOAT: return launch_stats_t<float>(data, valid, n_rows, rg_rows, g0, g1, imin, imax, fmin, fmax, nulls, regs, part, accumulate, s);
        case TGPU_DOUBLE: return launch_stats_t<double>(data, valid, n_rows, rg_rows, g0, g1, imin, imax, fmin, fmax, nulls, regs, part, accumulate, s);
        default: return launch_stats_t<long long>(data, valid, n_rows, rg_rows, g0, g1, imin, imax, fmin, fmax, nulls, regs, part, accumulate, s);
    }
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
