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
#include "common.cuh"

namespace tgpu {

namespace {

constexpr uint32_t ENC_RAW = 0, ENC_FOR = 1;
constexpr int DECODE_THREADS = 512;
constexpr int DECODE_UNROLL = 4;
constexpr uint32_t SMEM_RUNS = 4096;  // RLE run starts staged in shared memory up to this many runs

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

// Validity: the block's bitmap bits land at table rows row0 + i.  A word that
// lies wholly inside the block is stored; the (at most two) words it shares
// with neighbouring blocks are OR'ed in.
__device__ void decode_validity(const uint8_t *bm, const SegBlock &b) {
    const uint64_t first = b.row0 >> 5, last = (b.row0 + b.rows - 1) >> 5;
    for (uint64_t w = first + threadIdx.x; w <= last; w += blockDim.x) {
        // block-local bit of the word's row 0 (negative for a word starting before the block)
        const int64_t l0 = (int64_t)(w << 5) - (int64_t)b.row0;
        uint32_t word = 0;
        for (int byte = 0; byte < 5; ++byte) {
            const int64_t bit = l0 + 8 * byte - (l0 & 7);  // bitmap bytes covering the word's 32 rows
            if (bit + 8 <= 0 || bit >= (int64_t)b.rows) continue;
            const uint32_t v = bm[bit >> 3];
            const int64_t sh = bit - l0;                   // row of the word this byte's bit 0 lands on
            if (sh >= 0) word |= sh < 32 ? v << sh : 0u;
            else word |= v >> -sh;
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

__global__ void __launch_bounds__(DECODE_THREADS) decode_blocks_kernel(const uint8_t *__restrict__ image,
                                                                       const SegBlock *__restrict__ blocks,
                                                                       const uint32_t *__restrict__ run_starts) {
    __shared__ uint32_t s_starts[SMEM_RUNS];
    const SegBlock b = blocks[blockIdx.x];
    const uint8_t *p = image + b.payload;
    if (b.has_nulls && b.valid) decode_validity(p, b);
    const uint8_t *v = p + b.values;
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
                if (i < b.rows) st_elem(b.out, b.elem, b.row0 + i, x[k]);
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
        }
    }
}

}  // namespace

cudaError_t launch_decode_blocks(const uint8_t *image, const SegBlock *blocks, uint32_t n_blocks,
                                 const uint32_t *run_starts, cudaStream_t s) {
    if (!n_blocks) return cudaSuccess;
    decode_blocks_kernel<<<n_blocks, DECODE_THREADS, 0, s>>>(image, blocks, run_starts);
    return cudaGetLastError();
}

}  // namespace tgpu
