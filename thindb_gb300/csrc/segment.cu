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
//          (rleBlockOf, :2133).
// The host checks every header and bound, computes each RLE block's run
// starts, and copies the image to the device once; decode_blocks_kernel then
// expands every block of a column into the resident column (one CTA per
// block) and sets its validity bits.  Blocks stored compressed (zstd, lz4)
// or with integer-stream transforms, string columns (whose blocks live in
// string tables) and dictionary / FSST encodings are not decoded here: the
// call returns TGPU_ERR_UNSUPPORTED_TYPE.
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "common.cuh"

namespace tgpu {

namespace {

constexpr uint32_t ENC_RAW = 0, ENC_FOR = 1, ENC_RLE = 3;

__device__ __forceinline__ uint64_t ld_le(const uint8_t *p, uint32_t width) {
    uint64_t v = 0;
    for (uint32_t b = 0; b < width; ++b) v |= (uint64_t)p[b] << (8 * b);
    return v;
}

__device__ __forceinline__ void st_elem(void *out, uint32_t bytes, uint64_t row, uint64_t v) {
    switch (bytes) {
        case 1: ((uint8_t *)out)[row] = (uint8_t)v; break;
        case 2: ((uint16_t *)out)[row] = (uint16_t)v; break;
        case 4: ((uint32_t *)out)[row] = (uint32_t)v; break;
        default: ((uint64_t *)out)[row] = v; break;
    }
}

// One CTA per block: expand the block's values into out[row0, row0 + rows)
// (elements of `bytes` bytes) and OR its validity bits into `valid`.
__global__ void decode_blocks_kernel(const uint8_t *__restrict__ image, const SegBlock *__restrict__ blocks,
                                     const uint32_t *__restrict__ run_starts, void *out, uint32_t bytes,
                                     uint32_t *valid) {
    const SegBlock b = blocks[blockIdx.x];
    const uint8_t *p = image + b.payload;
    if (b.has_nulls && valid) {
        for (uint32_t i = threadIdx.x; i < b.rows; i += blockDim.x)
            if ((p[i >> 3] >> (i & 7)) & 1u) {
                const uint64_t r = b.row0 + i;
                atomicOr(valid + (r >> 5), 1u << (r & 31));
            }
    }
    const uint8_t *v = p + b.values;
    switch (b.encoding) {
        case ENC_RAW:
            for (uint32_t i = threadIdx.x; i < b.rows; i += blockDim.x)
                st_elem(out, bytes, b.row0 + i, ld_le(v + (size_t)i * bytes, bytes));
            break;
        case ENC_FOR: {
            // the add wraps in the element's width, as expandWidth's +%
            const uint64_t base = ld_le(v, 8);
            const uint8_t *codes = v + 20;
            for (uint32_t i = threadIdx.x; i < b.rows; i += blockDim.x)
                st_elem(out, bytes, b.row0 + i, base + ld_le(codes + (size_t)i * b.width, b.width));
            break;
        }
        default: {  // RLE: each row finds its run among the run starts
            const uint32_t *starts = run_starts + b.run0;
            const uint8_t *vals = v + 8;
            for (uint32_t i = threadIdx.x; i < b.rows; i += blockDim.x) {
                uint32_t lo = 0, hi = b.runs;  // the last run starting at or before i
                while (hi - lo > 1) {
                    const uint32_t mid = (lo + hi) / 2;
                    if (starts[mid] <= i) lo = mid;
                    else hi = mid;
                }
                // a value narrower than the element sign-extends as the writer truncated it
                uint64_t x = ld_le(vals + (size_t)lo * b.width, b.width);
                if (b.width < 8 && ((x >> (8 * b.width - 1)) & 1u)) x |= ~0ULL << (8 * b.width);
                st_elem(out, bytes, b.row0 + i, x);
            }
            break;
        }
    }
}

}  // namespace

cudaError_t launch_decode_blocks(const uint8_t *image, const SegBlock *blocks, uint32_t n_blocks,
                                 const uint32_t *run_starts, void *out, uint32_t bytes, uint32_t *valid,
                                 cudaStream_t s) {
    if (!n_blocks) return cudaSuccess;
    decode_blocks_kernel<<<n_blocks, 256, 0, s>>>(image, blocks, run_starts, out, bytes, valid);
    return cudaGetLastError();
}

}  // namespace tgpu
