// segment.cpp — CPU restatement of thinDB's segment block decoding.
//
// TEST INFRASTRUCTURE ONLY: the checker of the device decoder and the timed
// CPU baseline of segment ingest.  Nothing in the product links or calls it.
//
// Follows (paths in the thinDB tree):
//   layout: header, row groups, 12-byte block headers . src/storage/format.zig:1-38, :201-232
//   version check (current version only) .............. src/storage/segment_reader.zig:1388
//   payload: validity bitmap prefix, then the values .. segment_reader.zig decodeColumnPayload :1730
//   FOR: i128 base, u8 width, 3 pad, LE deltas,
//        value = base +% delta in the element type .... forBlockOf :1809, expandWidth :2058
//   RLE: u32 runs, u8 width, 3 pad, values, u32 lengths  rleBlockOf :2098, decodeRleColumn :2133
// Blocks are decoded on `threads` host threads, one (row group, column)
// block at a time, after a sequential walk that finds every block.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "oracle.h"

namespace {

struct Block {
    uint64_t row0;
    const uint8_t *payload;
    uint32_t rows, col, enc, has_nulls;
};

template <typename T> T rd(const uint8_t *p) {
    T v;
    std::memcpy(&v, p, sizeof(T));
    return v;
}

uint64_t rd_width(const uint8_t *p, uint32_t w) {
    uint64_t v = 0;
    std::memcpy(&v, p, w);  // little-endian host (x86-64 and aarch64)
    return v;
}

// value = base +% delta in T (expandWidth), deltas W-wide little-endian
template <typename T, typename W> void expand_for(T *out, uint64_t base, const uint8_t *codes, uint32_t rows) {
    for (uint32_t i = 0; i < rows; ++i) out[i] = (T)(base + (uint64_t)rd<W>(codes + (size_t)i * sizeof(W)));
}

template <typename T> void expand_for_w(T *out, uint64_t base, const uint8_t *codes, uint32_t w, uint32_t rows) {
    switch (w) {
        case 1: expand_for<T, uint8_t>(out, base, codes, rows); break;
        case 2: expand_for<T, uint16_t>(out, base, codes, rows); break;
        case 4: expand_for<T, uint32_t>(out, base, codes, rows); break;
        default: expand_for<T, uint64_t>(out, base, codes, rows); break;
    }
}

template <typename T> void fill_runs(T *out, const uint8_t *vals, const uint8_t *lens, uint32_t runs, uint32_t w) {
    for (uint32_t k = 0; k < runs; ++k) {
        uint64_t v = rd_width(vals + (size_t)k * w, w);
        if (w < 8 && ((v >> (8 * w - 1)) & 1)) v |= ~0ULL << (8 * w);
        const uint32_t len = rd<uint32_t>(lens + 4ull * k);
        std::fill_n(out, len, (T)v);
        out += len;
    }
}

void set_bits(uint8_t *dst, uint64_t row0, const uint8_t *bm, uint32_t rows) {
    if ((row0 & 7) == 0) {
        std::memcpy(dst + row0 / 8, bm, rows / 8);
        for (uint32_t i = rows & ~7u; i < rows; ++i)
            if ((bm[i >> 3] >> (i & 7)) & 1) dst[(row0 + i) >> 3] |= (uint8_t)(1u << ((row0 + i) & 7));
        return;
    }
    for (uint32_t i = 0; i < rows; ++i)
        if ((bm[i >> 3] >> (i & 7)) & 1) dst[(row0 + i) >> 3] |= (uint8_t)(1u << ((row0 + i) & 7));
}

int decode(const Block &b, uint32_t elem, uint8_t *out, uint8_t *valid) {
    const uint8_t *p = b.payload;
    if (b.has_nulls) {
        if (valid) set_bits(valid, b.row0, p, b.rows);
        p += (b.rows + 7) / 8;
    }
    uint8_t *dst = out + b.row0 * elem;
    if (b.enc == 0) {
        std::memcpy(dst, p, (size_t)b.rows * elem);
    } else if (b.enc == 1) {
        const uint64_t base = rd<uint64_t>(p);  // the low word of the i128: the sum wraps in the element
        const uint32_t w = p[16];
        const uint8_t *codes = p + 20;
        switch (elem) {
            case 1: expand_for_w((uint8_t *)dst, base, codes, w, b.rows); break;
            case 2: expand_for_w((uint16_t *)dst, base, codes, w, b.rows); break;
            case 4: expand_for_w((uint32_t *)dst, base, codes, w, b.rows); break;
            default: expand_for_w((uint64_t *)dst, base, codes, w, b.rows); break;
        }
    } else {
        const uint32_t runs = rd<uint32_t>(p);
        const uint32_t w = p[4];
        const uint8_t *vals = p + 8, *lens = vals + (size_t)runs * w;
        switch (elem) {
            case 1: fill_runs((uint8_t *)dst, vals, lens, runs, w); break;
            case 2: fill_runs((uint16_t *)dst, vals, lens, runs, w); break;
            case 4: fill_runs((uint32_t *)dst, vals, lens, runs, w); break;
            default: fill_runs((uint64_t *)dst, vals, lens, runs, w); break;
        }
    }
    return 0;
}

std::string g_seg_err;

int seg_fail(const char *m) {
    g_seg_err = m;
    return TGPU_ERR_INVALID_ARGUMENT;
}

}  // namespace

extern "C" {

// Decode a segment image into caller buffers: out[c] holds rows x elem[c]
// bytes, valid[c] (null for NOT NULL columns) (rows + 7) / 8 zeroed bytes.
// Returns TGPU_OK, TGPU_ERR_INVALID_ARGUMENT (malformed) or
// TGPU_ERR_UNSUPPORTED_TYPE (compressed, transformed or dictionary blocks).
int orc_segment_decode(const uint8_t *image, uint64_t bytes, const uint32_t *elem, uint32_t n_cols, void **out,
                       uint8_t **valid, int threads) {
    if (bytes < 40 || std::memcmp(image, "tDBS", 4) || std::memcmp(image + bytes - 4, "tDBS", 4))
        return seg_fail("magic");
    if (rd<uint16_t>(image + 4) != 17) {
        g_seg_err = "version";
        return TGPU_ERR_UNSUPPORTED_TYPE;
    }
    const uint64_t n = rd<uint64_t>(image + 24), end = bytes - 8;
    std::vector<Block> blocks;
    uint64_t pos = 32, done = 0;
    while (done < n) {
        if (pos + 8 > end) return seg_fail("truncated");
        const uint32_t rows = rd<uint32_t>(image + pos);
        pos += 8;
        if (!rows || done + rows > n) return seg_fail("row-group rows");
        for (uint32_t c = 0; c < n_cols; ++c) {
            if (pos + 12 > end) return seg_fail("truncated");
            const uint8_t comp = image[pos], flags = image[pos + 1], enc = image[pos + 2];
            const uint32_t usize = rd<uint32_t>(image + pos + 4), ssize = rd<uint32_t>(image + pos + 8);
            if (comp || (flags & 2) || (enc != 0 && enc != 1 && enc != 3)) {
                g_seg_err = "unsupported block";
                return TGPU_ERR_UNSUPPORTED_TYPE;
            }
            if (ssize != usize || pos + 12 + ssize > end) return seg_fail("block size");
            if ((flags & 1) && (rows + 7) / 8 > usize) return seg_fail("bitmap size");
            const uint8_t *v = image + pos + 12 + ((flags & 1) ? (rows + 7) / 8 : 0);
            const uint64_t room = usize - ((flags & 1) ? (rows + 7) / 8 : 0);
            if (enc == 0 && (uint64_t)rows * elem[c] > room) return seg_fail("raw size");
            if (enc == 1) {
                const uint32_t w = room >= 20 ? v[16] : 0;
                if ((w != 1 && w != 2 && w != 4 && w != 8) || 20 + (uint64_t)rows * w > room)
                    return seg_fail("FOR size");
            }
            if (enc == 3) {
                const uint32_t runs = room >= 8 ? rd<uint32_t>(v) : 0, w = room >= 8 ? v[4] : 0;
                if ((w != 1 && w != 2 && w != 4 && w != 8) || w > elem[c] || 8 + (uint64_t)runs * (w + 4) > room)
                    return seg_fail("RLE size");
                uint64_t sum = 0;
                for (uint32_t k = 0; k < runs; ++k) sum += rd<uint32_t>(v + 8 + (size_t)runs * w + 4ull * k);
                if (sum != rows) return seg_fail("RLE lengths");
            }
            blocks.push_back(Block{done, image + pos + 12, rows, c, enc, (uint32_t)(flags & 1)});
            pos += 12 + ssize;
        }
        done += rows;
    }
    threads = std::max(1, threads);
    std::atomic<size_t> next{0};
    auto work = [&] {
        for (size_t i; (i = next.fetch_add(1)) < blocks.size();) {
            const Block &b = blocks[i];
            decode(b, elem[b.col], (uint8_t *)out[b.col], valid ? valid[b.col] : nullptr);
        }
    };
    // validity bytes shared by two row groups are OR'ed from two blocks: when
    // row groups are not multiples of 8 rows one thread decodes everything
    bool aligned = true;
    for (const Block &b : blocks) aligned = aligned && (b.row0 & 7) == 0;
    if (!aligned) threads = 1;
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(work);
    work();
    for (auto &t : pool) t.join();
    return TGPU_OK;
}

const char *orc_segment_error(void) { return g_seg_err.c_str(); }

}  // extern "C"
