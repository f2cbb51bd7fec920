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
#include <type_traits>

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

template <typename T> __device__ __forceinline__ T from_bits(uint64_t x) {
    if constexpr (std::is_same<T, float>::value) return __uint_as_float((uint32_t)x);
    else if constexpr (std::is_same<T, double>::value) return __longlong_as_double((long long)x);
    else return (T)x;  // the element's low bytes (a signed type sign-extends)
}

template <typename T> __device__ __forceinline__ uint64_t to_bits(T t) {
    if constexpr (std::is_same<T, float>::value) return __float_as_uint(t);
    else if constexpr (std::is_same<T, double>::value) return (uint64_t)__double_as_longlong(t);
    else return (uint64_t)t;
}

// One valid value into the thread's zone map and the block's registers.
template <typename T> __device__ __forceinline__ void stat_value(Stat &st, T t, uint32_t *regs) {
    uint64_t bits;
    if constexpr (std::is_floating_point<T>::value) {
        const double d = (double)t;
        if (d == d) {
            st.fmn = fmin(st.fmn, d);
            st.fmx = fmax(st.fmx, d);
        } else {
            st.fmx = CUDART_INF;  // a NaN row can satisfy only open ranges; keep the map conservative
        }
        bits = canon_f64_bits(d);
    } else {
        const long long v = (long long)t;
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

constexpr uint32_t DOM_WORDS = 65536 / 32;  // a bit per 16-bit code

struct Smem {
    uint32_t starts[SMEM_RUNS];    // RLE run starts
    uint32_t regs[HLL_BYTES / 4];  // byte registers
    uint32_t dom[DOM_WORDS];       // codes seen (raw 1-2 byte elements, FOR deltas of 1-2 bytes)
    uint8_t seen[SMEM_RUNS];       // RLE runs with a valid row
    long long mn[DECODE_THREADS / 32], mx[DECODE_THREADS / 32];
    double fmn[DECODE_THREADS / 32], fmx[DECODE_THREADS / 32];
    unsigned nn[DECODE_THREADS / 32];
};

// L bytes at p (unaligned) as (L + 3) / 4 little-endian words, read as the
// aligned words around them (the image is padded past its end).
template <int L> __device__ __forceinline__ void ld_stream(const uint8_t *p, uint32_t (&o)[(L + 3) / 4]) {
    constexpr int NW = (L + 3) / 4;
    const uint32_t a = (uint32_t)((uintptr_t)p & 3u);
    const uint32_t *q = (const uint32_t *)(p - a);
    uint32_t w[NW + 1];
#pragma unroll
    for (int j = 0; j <= NW; ++j) w[j] = __ldg(q + j);
#pragma unroll
    for (int j = 0; j < NW; ++j) o[j] = __funnelshift_r(w[j], w[j + 1], 8 * a);
}

// Code i (W bytes) of a word stream.
template <int W, int N> __device__ __forceinline__ uint64_t code_at(const uint32_t (&o)[N], int i) {
    if constexpr (W == 8) return (uint64_t)o[2 * i] | ((uint64_t)o[2 * i + 1] << 32);
    else if constexpr (W == 4) return o[i];
    else if constexpr (W == 2) return (o[i / 2] >> (16 * (i & 1))) & 0xFFFFu;
    else return (o[i / 4] >> (8 * (i & 3))) & 0xFFu;
}

// Bits of one element: 32 for elements of up to 4 bytes.
template <typename T> using bits_t = typename std::conditional<sizeof(T) == 8, uint64_t, uint32_t>::type;

// K elements of T (their low bytes in x) as 16 bytes.
template <typename T, int K> __device__ __forceinline__ uint4 pack16(const bits_t<T> (&x)[K]) {
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if constexpr (sizeof(T) == 8) w[j] = (uint32_t)(x[j / 2] >> (32 * (j & 1)));
        else if constexpr (sizeof(T) == 4) w[j] = (uint32_t)x[j];
        else if constexpr (sizeof(T) == 2) w[j] = ((uint32_t)x[2 * j] & 0xFFFFu) | ((uint32_t)x[2 * j + 1] << 16);
        else
            w[j] = ((uint32_t)x[4 * j] & 0xFFu) | (((uint32_t)x[4 * j + 1] & 0xFFu) << 8) |
                   (((uint32_t)x[4 * j + 2] & 0xFFu) << 16) | ((uint32_t)x[4 * j + 3] << 24);
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

// Validity bits of rows i .. i + K - 1 (bit j = row i + j).
template <int K> __device__ __forceinline__ uint32_t valid_bits(const uint8_t *bm, bool has_nulls, uint32_t i) {
    if (!has_nulls) return (K == 32) ? ~0u : (1u << K) - 1u;
    return (uint32_t)(ld_bytes(bm + (i >> 3), 4) >> (i & 7)) & ((1u << K) - 1u);
}

// One row's share of the statistics.
template <typename T>
__device__ __forceinline__ void stat_row(Stat &stat, bool ok, bool dom, uint32_t code, T t, Smem &sm, uint32_t *regs) {
    if (!ok) {
        ++stat.nn;
    } else if (dom) {
        const uint32_t bit = 1u << (code & 31);
        if (!(sm.dom[(code & 0xFFFFu) >> 5] & bit)) atomicOr(&sm.dom[(code & 0xFFFFu) >> 5], bit);
    } else {
        stat_value(stat, t, regs);
    }
}

// Raw / FOR rows with codes of W bytes, 16 output bytes per thread per pass
// (K = 16 / sizeof(T) consecutive rows: one 16-byte store, their codes read
// as a few aligned words).  The rows past the last whole pass go one by one.
template <typename T, int W>
__device__ void expand_vec(const SegBlock &b, const uint8_t *bm, const uint8_t *codes, uint64_t base, T *out,
                           bool zone, bool dom, Stat &stat, Smem &sm, uint32_t *regs) {
    constexpr int K = 16 / (int)sizeof(T), L = K * W;
    const uint32_t whole = b.rows / K * K;
    for (uint32_t e0 = threadIdx.x * K; e0 < whole; e0 += blockDim.x * K) {
        uint32_t o[(L + 3) / 4];
        ld_stream<L>(codes + (size_t)e0 * W, o);
        bits_t<T> x[K];
#pragma unroll
        for (int i = 0; i < K; ++i) x[i] = (bits_t<T>)(base + code_at<W>(o, i));
        *(uint4 *)(out + e0) = pack16<T, K>(x);
        if (!zone) continue;
        const uint32_t vb = valid_bits<K>(bm, b.has_nulls, e0);
#pragma unroll
        for (int i = 0; i < K; ++i)
            stat_row<T>(stat, (vb >> i) & 1u, dom, (uint32_t)code_at<W>(o, i), from_bits<T>(x[i]), sm, regs);
    }
    for (uint32_t e = whole + threadIdx.x; e < b.rows; e += blockDim.x) {
        const uint64_t c = ld_bytes(codes + (size_t)e * W, W);
        const T t = from_bits<T>(base + c);
        out[e] = t;
        if (zone) stat_row<T>(stat, bit_at(bm, b.has_nulls, e), dom, (uint32_t)c, t, sm, regs);
    }
}

// Decode one block of a column of element type T; with SEG_ZONE take the
// block's zone map and (SEG_SKETCH) its sketch registers.  A block whose
// codes span at most 2^16 values (1-2 byte raw elements, FOR deltas of 1-2
// bytes) marks the codes it sees and takes the statistics once per code; an
// RLE block marks its runs and takes them once per run; other blocks hash
// every valid row.
template <typename T>
__device__ void decode_block(const SegBlock &b, const uint8_t *p, const uint32_t *__restrict__ run_starts,
                             const SegStats &st, Smem &sm) {
    const bool zone = b.flags & SEG_ZONE;
    uint32_t *regs = (b.flags & SEG_SKETCH) ? sm.regs : nullptr;
    const bool hn = b.has_nulls;
    const uint8_t *v = p + b.values;
    T *out = (T *)b.out + b.row0;
    const bool rle = b.encoding != ENC_RAW && b.encoding != ENC_FOR;
    const bool staged = rle && b.runs <= SMEM_RUNS;
    const bool dom = zone && !rle && (b.encoding == ENC_RAW ? sizeof(T) <= 2 : b.width <= 2);
    if (regs)
        for (uint32_t i = threadIdx.x; i < HLL_BYTES / 4; i += blockDim.x) sm.regs[i] = 0;
    if (dom)
        for (uint32_t i = threadIdx.x; i < DOM_WORDS; i += blockDim.x) sm.dom[i] = 0;
    if (staged) {
        for (uint32_t r = threadIdx.x; r < b.runs; r += blockDim.x) {
            sm.starts[r] = run_starts[b.run0 + r];
            sm.seen[r] = 0;
        }
    }
    __syncthreads();
    if (b.valid) decode_validity(p, b);
    Stat stat;
    if (!rle) {
        // raw: base 0, codes of the element's width; FOR: the add wraps in the
        // element's width, as expandWidth's +%.  Four rows per thread per
        // pass, their loads issued before their stores.
        const bool raw = b.encoding == ENC_RAW;
        const uint64_t base = raw ? 0 : ld_bytes(v, 8);
        const uint8_t *codes = raw ? v : v + 20;
        const uint32_t w = raw ? b.elem : b.width, step = blockDim.x;
        // 16-byte stores need the block's first row on a 16-byte boundary;
        // codes wider than the element (never written by thinDB) go row by row
        const bool vec = ((uintptr_t)out & 15u) == 0 && w <= sizeof(T);
        if (vec) {
            if (w == 1) expand_vec<T, 1>(b, p, codes, base, out, zone, dom, stat, sm, regs);
            else if (w == 2) expand_vec<T, (sizeof(T) >= 2 ? 2 : 1)>(b, p, codes, base, out, zone, dom, stat, sm, regs);
            else if (w == 4) expand_vec<T, (sizeof(T) >= 4 ? 4 : 1)>(b, p, codes, base, out, zone, dom, stat, sm, regs);
            else expand_vec<T, (sizeof(T) >= 8 ? 8 : 1)>(b, p, codes, base, out, zone, dom, stat, sm, regs);
        }
        for (uint32_t i0 = vec ? b.rows : threadIdx.x; i0 < b.rows; i0 += DECODE_UNROLL * step) {
            uint64_t c[DECODE_UNROLL];
#pragma unroll
            for (int k = 0; k < DECODE_UNROLL; ++k) {
                const uint32_t i = i0 + k * step;
                c[k] = i < b.rows ? ld_bytes(codes + (size_t)i * w, w) : 0;
            }
#pragma unroll
            for (int k = 0; k < DECODE_UNROLL; ++k) {
                const uint32_t i = i0 + k * step;
                if (i >= b.rows) continue;
                const T t = from_bits<T>(base + c[k]);
                out[i] = t;
                if (!zone) continue;
                if (!bit_at(p, hn, i)) {
                    ++stat.nn;
                } else if (dom) {
                    const uint32_t code = (uint32_t)c[k] & 0xFFFFu, bit = 1u << (code & 31);
                    if (!(sm.dom[code >> 5] & bit)) atomicOr(&sm.dom[code >> 5], bit);
                } else {
                    stat_value(stat, t, regs);
                }
            }
        }
        if (dom) {
            __syncthreads();
            for (uint32_t wi = threadIdx.x; wi < DOM_WORDS; wi += blockDim.x)
                for (uint32_t word = sm.dom[wi]; word; word &= word - 1)
                    stat_value(stat, from_bits<T>(base + (wi * 32 + __ffs(word) - 1)), regs);
        }
    } else {  // RLE: each row finds its run among the run starts
        const uint32_t *starts = staged ? sm.starts : run_starts + b.run0;
        const uint8_t *vals = v + 8;
        const uint32_t vw = b.width;
        auto run_value = [&](uint32_t r) {
            // a value narrower than the element sign-extends
            uint64_t x = ld_bytes(vals + (size_t)r * vw, vw);
            if (vw < 8 && ((x >> (8 * vw - 1)) & 1u)) x |= ~0ULL << (8 * vw);
            return from_bits<T>(x);
        };
        uint32_t lo = 0;  // the thread's rows ascend: its run index only moves forward
        T t = run_value(0);
        // K consecutive rows per thread per pass and one 16-byte store (the
        // block's first row on a 16-byte boundary); then the rest row by row
        constexpr int K = 16 / (int)sizeof(T);
        const bool vec = ((uintptr_t)out & 15u) == 0;
        const uint32_t whole = vec ? b.rows / K * K : 0;
        for (uint32_t e0 = threadIdx.x * K; e0 < whole; e0 += blockDim.x * K) {
            if (lo + 1 < b.runs && starts[lo + 1] <= e0) {
                uint32_t hi = b.runs;  // the last run starting at or before e0
                ++lo;
                while (hi - lo > 1) {
                    const uint32_t mid = (lo + hi) / 2;
                    if (starts[mid] <= e0) lo = mid;
                    else hi = mid;
                }
                t = run_value(lo);
            }
            const uint32_t vb = zone ? valid_bits<K>(p, hn, e0) : 0u;
            bits_t<T> x[K];
#pragma unroll
            for (int i = 0; i < K; ++i) {
                while (lo + 1 < b.runs && starts[lo + 1] <= e0 + i) {
                    ++lo;
                    t = run_value(lo);
                }
                x[i] = (bits_t<T>)to_bits(t);
                if (!zone) continue;
                if (!((vb >> i) & 1u)) ++stat.nn;
                else if (staged) sm.seen[lo] = 1;
                else stat_value(stat, t, regs);
            }
            *(uint4 *)(out + e0) = pack16<T, K>(x);
        }
        for (uint32_t i = whole + threadIdx.x; i < b.rows; i += blockDim.x) {
            if (lo + 1 < b.runs && starts[lo + 1] <= i) {
                uint32_t hi = b.runs;  // the last run starting at or before i
                ++lo;
                while (hi - lo > 1) {
                    const uint32_t mid = (lo + hi) / 2;
                    if (starts[mid] <= i) lo = mid;
                    else hi = mid;
                }
                t = run_value(lo);
            }
            out[i] = t;
            if (!zone) continue;
            if (!bit_at(p, hn, i)) ++stat.nn;
            else if (staged) sm.seen[lo] = 1;
            else stat_value(stat, t, regs);
        }
        if (zone && staged) {
            __syncthreads();
            for (uint32_t r = threadIdx.x; r < b.runs; r += blockDim.x)
                if (sm.seen[r]) stat_value(stat, run_value(r), regs);
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
        sm.mn[warp] = stat.mn;
        sm.mx[warp] = stat.mx;
        sm.fmn[warp] = stat.fmn;
        sm.fmx[warp] = stat.fmx;
        sm.nn[warp] = stat.nn;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            stat.mn = min(stat.mn, sm.mn[w]);
            stat.mx = max(stat.mx, sm.mx[w]);
            stat.fmn = fmin(stat.fmn, sm.fmn[w]);
            stat.fmx = fmax(stat.fmx, sm.fmx[w]);
            stat.nn += sm.nn[w];
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
        for (uint32_t i = threadIdx.x; i < HLL_BYTES / 4; i += blockDim.x) row[i] = sm.regs[i];
    }
}

__global__ void __launch_bounds__(DECODE_THREADS, 2) decode_blocks_kernel(const uint8_t *__restrict__ image,
                                                                       const SegBlock *__restrict__ blocks,
                                                                       const uint32_t *__restrict__ run_starts,
                                                                       const SegStats st) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem &sm = *reinterpret_cast<Smem *>(smem_raw);
    const SegBlock b = blocks[blockIdx.x];
    const uint8_t *p = image + b.payload;
    switch (b.type) {
        case TGPU_BOOLEAN: decode_block<uint8_t>(b, p, run_starts, st, sm); break;
        case TGPU_TINYINT: decode_block<int8_t>(b, p, run_starts, st, sm); break;
        case TGPU_SMALLINT: decode_block<int16_t>(b, p, run_starts, st, sm); break;
        case TGPU_INT: case TGPU_DATE: decode_block<int32_t>(b, p, run_starts, st, sm); break;
        case TGPU_FLOAT: decode_block<float>(b, p, run_starts, st, sm); break;
        case TGPU_DOUBLE: decode_block<double>(b, p, run_starts, st, sm); break;
        default: decode_block<long long>(b, p, run_starts, st, sm); break;
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
    cudaError_t e = cudaFuncSetAttribute(decode_blocks_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(Smem));
    if (e != cudaSuccess) return e;
    decode_blocks_kernel<<<n_blocks, DECODE_THREADS, sizeof(Smem), s>>>(image, blocks, run_starts, st);
    return cudaGetLastError();
}

cudaError_t launch_seg_hll_merge(const SegStats &st, uint32_t n_cols, uint32_t rows, uint32_t stride, cudaStream_t s) {
    if (!n_cols || !rows) return cudaSuccess;
    const uint32_t slices = std::min<uint32_t>(rows, 16);
    seg_hll_merge_kernel<<<dim3(HLL_BYTES / 4 / 256, n_cols, slices), 256, 0, s>>>(st, rows, stride);
    return cudaGetLastError();
}

}  // namespace tgpu
