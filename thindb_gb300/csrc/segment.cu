// segment.cu — registering a table from a thinDB segment image: the host
// walks the segment's layout, the device decodes its column blocks.
//
// Layout (src/storage/format.zig:1-38; version 17 at :85): a 32-byte header
// (magic "tDBS", u16 version, u16 flags, u64 schema fingerprint, u64 segment
// id, u64 row count), then the row groups in order — u32 row count, u32
// padding, and per column in schema order a 12-byte block header
// (column_block_header_size, :228: u8 compression, u8 flags (has_nulls,
// int_streams), u8 encoding, u8 reserved, u32 uncompressed size, u32 stored
// size) and the stored payload — then string tables and the footer, ending
// in u32 footer size and the magic again.
//
// A payload (segment_reader.zig decodeColumnPayload :1730) starts with the
// validity bitmap when has_nulls (bit 1 = valid, (rows + 7) / 8 bytes), then:
//   raw  : the native values;
//   FOR  : i128 base, u8 width (1/2/4/8), 3 pad, rows x width unsigned LE
//          deltas, value = base + delta (forBlockOf :1809, expandWidth);
//   RLE  : u32 runs, u8 value width, 3 pad, runs x value, runs x u32 length
//          (rleBlockOf, :2098).
// The host checks every header and bound, computes each RLE block's run
// starts, and copies the image to the device once; decode_blocks_kernel then
// expands every block of every column (one CTA per block, one launch) into
// the resident columns and their validity words.  Payloads sit at arbitrary
// byte offsets, so values are read as whole aligned 32-bit words and shifted
// into place (the image buffer is padded past its end for the last word).
// Blocks stored compressed (zstd, lz4) or with integer-stream transforms,
// string columns (whose blocks live in string tables) and dictionary / FSST
// encodings are not decoded here: the call returns TGPU_ERR_UNSUPPORTED_TYPE.
#include <algorithm>
#include <cfloat>
#include <climits>

#include <math_constants.h>

#include "common.cuh"

namespace tgpu {

namespace {

constexpr uint32_t ENC_RAW = 0, ENC_FOR = 1;
constexpr int DECODE_THREADS = 512;
constexpr int DECODE_UNROLL = 4;
constexpr uint32_t SMEM_RUNS = 4096;  // RLE run starts staged in shared memory up to this many runs
constexpr uint32_t HLL_BYTES = 1u << HLL_P;  // one byte register each (ranks stay below 64)

// Bytes p[0, w) (w = 1, 2, 4 or 8) as a little-endian integer, read as the
// aligned words around them.
__device__ __forceinline__ uint64_t ld_bytes(const uint8_t *p, uint32_t w) {
    const uint32_t a = (uint32_t)((uintptr_t)p & 3u);
    const uint32_t *q = (const uint32_t *)(p - a);
    const uint32_t w0 = __ldg(q), w1 = __ldg(q + 1);
    const uint32_t lo = __funnelshift_r(w0, w1, 8 * a);
    if (w == 8) return ((uint64_t)__funnelshift_r(w1, __ldg(q + 2), 8 * a) << 32) | lo;
    return w == 4 ? lo : lo & ((1u << (8 * w)) - 1u);
}

__device__ __forceinline__ void st_elem(void *out, uint32_t bytes, uint64_t row, uint64_t v) {
    switch (bytes) {
        case 1: ((uint8_t *)out)[row] = (uint8_t)v; break;
        case 2: ((uint16_t *)out)[row] = (uint16_t)v; break;
        case 4: ((uint32_t *)out)[row] = (uint32_t)v; break;
        default: ((uint64_t *)out)[row] = v; break;
    }
}

// Validity: the block's bitmap bits land at table rows row0 + i (all set
// for a block of a nullable column stored without a bitmap).  A word that
// lies wholly inside the block is stored; the (at most two) words it shares
// with neighbouring blocks are OR'ed in.
__device__ void decode_validity(const uint8_t *bm, const SegBlock &b) {
    const uint64_t first = b.row0 >> 5, last = (b.row0 + b.rows - 1) >> 5;
    for (uint64_t w = first + threadIdx.x; w <= last; w += blockDim.x) {
        // block-local bit of the word's row 0 (negative for a word starting before the block)
        const int64_t l0 = (int64_t)(w << 5) - (int64_t)b.row0;
        uint32_t word = 0;
        if (!b.has_nulls) {
            word = ~0u;
        } else {
            for (int byte = 0; byte < 5; ++byte) {
                const int64_t bit = l0 + 8 * byte - (l0 & 7);  // bitmap bytes covering the word's 32 rows
                if (bit + 8 <= 0 || bit >= (int64_t)b.rows) continue;
                const uint32_t v = bm[bit >> 3];
                const int64_t sh = bit - l0;                   // row of the word this byte's bit 0 lands on
                if (sh >= 0) word |= sh < 32 ? v << sh : 0u;
                else word |= v >> -sh;
            }
        }
        const uint64_t r0 = w << 5;
        const bool inner = r0 >= b.row0 && r0 + 32 <= b.row0 + b.rows;
        if (inner) {
            b.valid[w] = word;
        } else {
            // keep only the block's own rows
            const int64_t lo = (int64_t)b.row0 - (int64_t)r0, hi = (int64_t)(b.row0 + b.rows) - (int64_t)r0;
            uint32_t mask = ~0u;
            if (lo > 0) mask &= ~0u << lo;
            if (hi < 32) mask &= (1u << hi) - 1u;
            if (word & mask) atomicOr(b.valid + w, word & mask);
        }
    }
}

// Zone map and HyperLogLog state of one thread over its rows of the block:
// the same quantities column_stats_kernel takes from a resident column.
struct Stat {
    long long mn = LLONG_MAX, mx = LLONG_MIN;
    double fmn = DBL_MAX, fmx = -DBL_MAX;
    unsigned nn = 0;
};

// Raise byte register idx of the shared byte file to rank.
__device__ __forceinline__ void hll_raise(uint32_t *regs, uint32_t idx, uint32_t rank) {
    uint32_t *w = regs + (idx >> 2);
    const uint32_t sh = 8 * (idx & 3);
    uint32_t old = *w;
    while (((old >> sh) & 0xFFu) < rank) {
        const uint32_t prev = atomicCAS(w, old, (old & ~(0xFFu << sh)) | (rank << sh));
        if (prev == old) break;
        old = prev;
    }
}

__device__ __forceinline__ void stat_row(Stat &st, const SegBlock &b, uint64_t x, bool ok, uint32_t *regs) {
    if (!ok) {
        ++st.nn;
        return;
    }
    uint64_t bits;
    if (b.type == TGPU_FLOAT || b.type == TGPU_DOUBLE) {
        const double d = b.type == TGPU_FLOAT ? (double)__uint_as_float((uint32_t)x) : __longlong_as_double((long long)x);
        if (d == d) {
            st.fmn = fmin(st.fmn, d);
            st.fmx = fmax(st.fmx, d);
        } else {
            st.fmx = CUDART_INF;  // a NaN row can satisfy only open ranges; keep the map conservative
        }
        bits = canon_f64_bits(d);
    } else {
        // the typed value: sign-extended from the element, BOOLEAN unsigned
        long long v = (long long)x;
        if (b.elem < 8 && b.type != TGPU_BOOLEAN) v = (long long)(x << (64 - 8 * b.elem)) >> (64 - 8 * b.elem);
        else if (b.elem < 8) v = (long long)(x & ((1ULL << (8 * b.elem)) - 1));
        st.mn = min(st.mn, v);
        st.mx = max(st.mx, v);
        bits = (uint64_t)v;
    }
    if (regs) {
        const uint64_t h = mix64(bits ^ 0x6A09E667F3BCC909ULL);
        const uint32_t idx = (uint32_t)(h >> (64 - HLL_P));
        const uint64_t w = (h << HLL_P) | (1ULL << (HLL_P - 1));
        hll_raise(regs, idx, (uint32_t)__clzll((long long)w) + 1);
    }
}

__device__ __forceinline__ bool bit_at(const uint8_t *bm, bool has_nulls, uint32_t i) {
    return !has_nulls || ((bm[i >> 3] >> (i & 7)) & 1u);
}

__global__ void __launch_bounds__(DECODE_THREADS) decode_blocks_kernel(const uint8_t *__restrict__ image,
                                                                       const SegBlock *__restrict__ blocks,
                                                                       const uint32_t *__restrict__ run_starts,
                                                                       const SegStats st) {
    __shared__ uint32_t s_starts[SMEM_RUNS];
    __shared__ uint32_t s_regs[HLL_BYTES / 4];  // byte registers
    __shared__ long long s_mn[DECODE_THREADS / 32], s_mx[DECODE_THREADS / 32];
    __shared__ double s_fmn[DECODE_THREADS / 32], s_fmx[DECODE_THREADS / 32];
    __shared__ unsigned s_nn[DECODE_THREADS / 32];
    const SegBlock b = blocks[blockIdx.x];
    const uint8_t *p = image + b.payload;
    const bool zone = b.flags & SEG_ZONE;
    uint32_t *regs = (b.flags & SEG_SKETCH) ? s_regs : nullptr;
    if (regs) {
        for (uint32_t i = threadIdx.x; i < HLL_BYTES / 4; i += blockDim.x) s_regs[i] = 0;
        __syncthreads();
    }
    if (b.valid) decode_validity(p, b);
    const uint8_t *v = p + b.values;
    Stat stat;
    if (b.encoding == ENC_RAW || b.encoding == ENC_FOR) {
        // raw: base 0, codes of the element's width; FOR: the add wraps in the
        // element's width, as expandWidth's +%.  Four rows per thread per
        // pass, their loads issued before their stores.
        const bool raw = b.encoding == ENC_RAW;
        const uint64_t base = raw ? 0 : ld_bytes(v, 8);
        const uint8_t *codes = raw ? v : v + 20;
        const uint32_t w = raw ? b.elem : b.width, step = blockDim.x;
        for (uint32_t i0 = threadIdx.x; i0 < b.rows; i0 += DECODE_UNROLL * step) {
            uint64_t x[DECODE_UNROLL];
#pragma unroll
            for (int k = 0; k < DECODE_UNROLL; ++k) {
                const uint32_t i = i0 + k * step;
                x[k] = i < b.rows ? base + ld_bytes(codes + (size_t)i * w, w) : 0;
            }
#pragma unroll
            for (int k = 0; k < DECODE_UNROLL; ++k) {
                const uint32_t i = i0 + k * step;
                if (i < b.rows) {
                    st_elem(b.out, b.elem, b.row0 + i, x[k]);
                    if (zone) stat_row(stat, b, x[k], bit_at(p, b.has_nulls, i), regs);
                }
            }
        }
    } else {  // RLE: each row finds its run among the run starts
        const uint32_t *starts = run_starts + b.run0;
        if (b.runs <= SMEM_RUNS) {
            for (uint32_t r = threadIdx.x; r < b.runs; r += blockDim.x) s_starts[r] = starts[r];
            __syncthreads();
            starts = s_starts;
        }
        const uint8_t *vals = v + 8;
        for (uint32_t i = threadIdx.x; i < b.rows; i += blockDim.x) {
            uint32_t lo = 0, hi = b.runs;  // the last run starting at or before i
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) / 2;
                if (starts[mid] <= i) lo = mid;
                else hi = mid;
            }
            // a value narrower than the element sign-extends
            uint64_t x = ld_bytes(vals + (size_t)lo * b.width, b.width);
            if (b.width < 8 && ((x >> (8 * b.width - 1)) & 1u)) x |= ~0ULL << (8 * b.width);
            st_elem(b.out, b.elem, b.row0 + i, x);
            if (zone) stat_row(stat, b, x, bit_at(p, b.has_nulls, i), regs);
        }
    }
    if (!zone) return;
    // the block's zone map: warp, then CTA reduction
    for (int o = 16; o; o >>= 1) {
        stat.mn = min(stat.mn, __shfl_down_sync(0xFFFFFFFFu, stat.mn, o));
        stat.mx = max(stat.mx, __shfl_down_sync(0xFFFFFFFFu, stat.mx, o));
        stat.fmn = fmin(stat.fmn, __shfl_down_sync(0xFFFFFFFFu, stat.fmn, o));
        stat.fmx = fmax(stat.fmx, __shfl_down_sync(0xFFFFFFFFu, stat.fmx, o));
        stat.nn += __shfl_down_sync(0xFFFFFFFFu, stat.nn, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        s_mn[warp] = stat.mn;
        s_mx[warp] = stat.mx;
        s_fmn[warp] = stat.fmn;
        s_fmx[warp] = stat.fmx;
        s_nn[warp] = stat.nn;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            stat.mn = min(stat.mn, s_mn[w]);
            stat.mx = max(stat.mx, s_mx[w]);
            stat.fmn = fmin(stat.fmn, s_fmn[w]);
            stat.fmx = fmax(stat.fmx, s_fmx[w]);
            stat.nn += s_nn[w];
        }
        unsigned char *sl = st.stats + (size_t)b.col * st.slice;
        int64_t *imin = (int64_t *)sl, *imax = imin + st.nrg;
        double *fmin = (double *)(imax + st.nrg), *fmax = fmin + st.nrg;
        uint32_t *nulls = (uint32_t *)(fmax + st.nrg);
        imin[b.rg] = stat.mn;
        imax[b.rg] = stat.mx;
        fmin[b.rg] = stat.fmn;
        fmax[b.rg] = stat.fmx;
        nulls[b.rg] = stat.nn;
    }
    if (regs) {  // the block's registers, a row of the scratch
        uint32_t *row = (uint32_t *)(st.part + (size_t)b.part_row * HLL_BYTES);
        for (uint32_t i = threadIdx.x; i < HLL_BYTES / 4; i += blockDim.x) row[i] = s_regs[i];
    }
}

// grid (HLL_BYTES / 4 / 256, columns, slices): each thread takes four
// registers of one column over a slice of its part rows (column c's `rows`
// rows start at row c * stride) and raises the column's u32 registers with
// atomicMax.
__global__ void seg_hll_merge_kernel(const SegStats st, uint32_t rows, uint32_t stride) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;  // registers 4i .. 4i + 3
    if (i >= HLL_BYTES / 4) return;
    const uint32_t c = blockIdx.y;
    const uint32_t per = (rows + gridDim.z - 1) / gridDim.z, r0 = blockIdx.z * per, r1 = min(rows, r0 + per);
    const uint32_t *base = (const uint32_t *)(st.part + ((size_t)c * stride) * HLL_BYTES) + i;
    uint32_t m = 0;
    for (uint32_t r = r0; r < r1; ++r) m = __vmaxu4(m, __ldg(base + (size_t)r * (HLL_BYTES / 4)));
    if (!m) return;
    uint32_t *regs = (uint32_t *)(st.stats + (size_t)c * st.slice + st.reg_off);
    for (int k = 0; k < 4; ++k) {
        const uint32_t x = (m >> (8 * k)) & 0xFFu;
        if (x) atomicMax(regs + 4 * i + k, x);
    }
}

}  // namespace

cudaError_t launch_decode_blocks(const uint8_t *image, const SegBlock *blocks, uint32_t n_blocks,
                                 const uint32_t *run_starts, const SegStats &st, cudaStream_t s) {
    if (!n_blocks) return cudaSuccess;
    decode_blocks_kernel<<<n_blocks, DECODE_THREADS, 0, s>>>(image, blocks, run_starts, st);
    return cudaGetLastError();
}

cudaError_t launch_seg_hll_merge(const SegStats &st, uint32_t n_cols, uint32_t rows, uint32_t stride, cudaStream_t s) {
    if (!n_cols || !rows) return cudaSuccess;
    const uint32_t slices = std::min<uint32_t>(rows, 16);
    seg_hll_merge_kernel<<<dim3(HLL_BYTES / 4 / 256, n_cols, slices), 256, 0, s>>>(st, rows, stride);
    return cudaGetLastError();
}

}  // namespace tgpu
