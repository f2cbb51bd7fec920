// finalize.cu — from the folded group table to the result rows.
//
// thinDB's emit stage (silo_group_core.zig emitAllGroupsNumeric :4802,
// emitRankedGroups :4856, TopSet :5083; v2_shape_group_topn.zig
// applyHaving :2586, rankedFinalRows :1137, rowOrderBefore :1327-1335,
// avgValue :1438-1446, integerAggValue :1448-1453, emitResultStage :1514):
//
//   compact   occupancy bitmap -> dense list of group slots passing HAVING
//             (two passes, block counts then ordered writes: deterministic)
//   rank      k <= 32: warp-register top-k per warp, merged per CTA, then by
//             one warp; otherwise a merge sort (bitonic 1024-runs + merge
//             passes).  Keys are encoded into unsigned words compared
//             lexicographically: each ORDER BY value (NULL first), then the
//             packed group key ascending.
//   gather    result rows -> typed output columns + validity bytes
//   clear     zero every used slot and the bitmap so the table is reusable
//             without a full memset.
#include <algorithm>

#include "common.cuh"

namespace tgpu {

namespace {

constexpr unsigned FULL = 0xFFFFFFFFu;

__device__ __constant__ double POW10[19] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8, 1e9,
                                            1e10, 1e11, 1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18};

struct EmitVal {
    bool null;
    bool is_f;
    uint64_t lo;   // i128 low word (integers)
    int64_t hi;    // i128 high word
    double f;
};

__device__ __forceinline__ const unsigned long long *slot_states(const DevFinal &f, uint32_t gid) {
    return f.table + (uint64_t)gid * f.slot_words + f.key_words;
}

// The emitted value of aggregate `a` (countValue / aggIsNull / avgValue /
// integerAggValue, v2_shape_group_topn.zig:1399-1453).
__device__ EmitVal emit_agg(const DevFinal &f, const unsigned long long *st, int a) {
    const DevOut &o = f.outs[a];
    EmitVal v{false, false, 0, 0, 0.0};
    const uint64_t rows = st[0];
    if (o.func == TGPU_AGG_COUNT) {
        v.lo = o.kind == AK_COUNT_VALID ? st[o.word] : rows;
        return v;
    }
    if (o.func == TGPU_AGG_COUNT_DISTINCT) {
        v.lo = st[o.word];
        return v;
    }
    const uint64_t den = o.vword >= 0 ? st[o.vword] : rows;
    if (o.nullable && den == 0) {
        v.null = true;
        return v;
    }
    switch (o.func) {
        case TGPU_AGG_SUM:
            if (o.kind == AK_SUM_F64) {
                v.is_f = true;
                v.f = bits_f64(st[o.word]);
            } else if (o.kind == AK_SUM_I64) {
                v.lo = st[o.word];
                v.hi = (int64_t)v.lo < 0 ? -1 : 0;
            } else {
                if (o.kind == AK_SUM_I128) {
                    i128_of_split(st[o.word], st[o.word + 1], v.lo, v.hi);
                } else {
                    v.lo = st[o.word];
                    v.hi = (int64_t)st[o.word + 1];
                }
                if (o.out_type == TGPU_BIGINT) v.hi = (int64_t)v.lo < 0 ? -1 : 0;  // wraps to BIGINT
            }
            return v;
        case TGPU_AGG_AVG: {
            v.is_f = true;
            if (den == 0) return v;
            if (o.kind == AK_SUM_F64) {
                v.f = bits_f64(st[o.word]) / (double)den;
            } else {
                uint64_t lo = st[o.word];
                int64_t hi = (int64_t)lo < 0 ? -1 : 0;
                if (o.kind == AK_SUM_I128) i128_of_split(st[o.word], st[o.word + 1], lo, hi);
                else if (o.kind == AK_SUM_I128C) hi = (int64_t)st[o.word + 1];
                // avgValue (v2_shape_group_topn.zig:1438-1446) divides by the
                // count, then by 10^scale; the global aggregate's emitRow
                // (v2_global_aggregate.zig:1872-1877) by count x 10^scale
                v.f = f.global_avg ? i128_to_f64(lo, hi) / ((double)den * POW10[o.scale])
                                   : i128_to_f64(lo, hi) / (double)den / POW10[o.scale];
            }
            return v;
        }
        default: {  // MIN / MAX
            uint64_t e = st[o.word];
            if (o.func == TGPU_AGG_MIN) e = ~e;
            if (o.kind == AK_MIN_F || o.kind == AK_MAX_F) {
                v.is_f = true;
                v.f = bits_f64(dec_f64_bits(e));
            } else {
                v.lo = (uint64_t)dec_i64(e);
                v.hi = (int64_t)v.lo < 0 ? -1 : 0;
            }
            return v;
        }
    }
}

__device__ __forceinline__ void slot_key(const DevFinal &f, uint32_t gid, uint64_t &k0, uint64_t &k1) {
    const unsigned long long *s = f.table + (uint64_t)gid * f.slot_words;
    k0 = s[0];
    k1 = f.key_words == 2 ? s[1] : 0;
}

// keyPartIsNull / keyPartValue (v2_shape_group_topn.zig:1426-1470).
__device__ EmitVal emit_key(const DevFinal &f, uint64_t k0, uint64_t k1, int p) {
    const DevKeyPart &kp = f.parts[p];
    EmitVal v{false, false, 0, 0, 0.0};
    if (f.hashed) {
        // a hashed key's parts are read at the group's representative row
        // (word 0 - 1); a string part emits that row (thinDB's rowref,
        // materialised on the host by tgpu_query_key_strings)
        const uint64_t row = k0 - 1;
        const DevCol &c = f.part_cols[p];
        if (c.valid && !((__ldg(c.valid + (row >> 5)) >> (row & 31)) & 1u)) {
            v.null = true;
            return v;
        }
        int64_t x;
        if (c.offs) x = (int64_t)row;
        else switch (c.bytes) {
                case 1: x = f.part_types[p] == TGPU_BOOLEAN ? (int64_t)__ldg((const uint8_t *)c.data + row)
                                                          : (int64_t)__ldg((const int8_t *)c.data + row);
                    break;
                case 2: x = __ldg((const int16_t *)c.data + row); break;
                case 4: x = __ldg((const int32_t *)c.data + row); break;
                default: x = (int64_t)__ldg((const long long *)c.data + row); break;
            }
        v.lo = (uint64_t)x;
        v.hi = x < 0 ? -1 : 0;
        return v;
    }
    auto bit = [&](int b) -> uint64_t { return b < 64 ? (k0 >> b) & 1 : (k1 >> (b - 64)) & 1; };
    if (kp.nullable && !bit(kp.offset + kp.payload)) {
        v.null = true;
        return v;
    }
    uint64_t raw;
    int off = kp.offset;
    if (off >= 64) raw = k1 >> (off - 64);
    else raw = (k0 >> off) | (off ? (k1 << (64 - off)) : 0);
    if (kp.payload < 64) raw &= (1ULL << kp.payload) - 1;
    int64_t s;
    switch (f.part_types[p]) {
        case TGPU_BOOLEAN: case TGPU_TINYINT: s = (int8_t)(uint8_t)raw; break;
        case TGPU_SMALLINT: s = (int16_t)(uint16_t)raw; break;
        case TGPU_INT: case TGPU_DATE: case TGPU_DICT32: s = (int32_t)(uint32_t)raw; break;
        default: s = (int64_t)raw; break;
    }
    v.lo = (uint64_t)s;
    v.hi = s < 0 ? -1 : 0;
    return v;
}

__device__ __forceinline__ int cmp_i128(uint64_t alo, int64_t ahi, uint64_t blo, int64_t bhi) {
    if (ahi != bhi) return ahi < bhi ? -1 : 1;
    if (alo != blo) return alo < blo ? -1 : 1;
    return 0;
}

__device__ bool having_pass(const DevFinal &f, const unsigned long long *st) {
    for (int i = 0; i < f.n_having; ++i) {
        const DevHaving &h = f.having[i];
        EmitVal v = emit_agg(f, st, h.agg);
        if (v.null) return false;
        int c;
        if (v.is_f) {
            if (v.f != v.f || h.fval != h.fval) {
                if (h.op != TGPU_PRED_NE) return false;
                continue;
            }
            c = v.f < h.fval ? -1 : (v.f > h.fval ? 1 : 0);
        } else {
            c = cmp_i128(v.lo, v.hi, (uint64_t)h.ival, h.ival < 0 ? -1 : 0);
        }
        bool ok;
        switch (h.op) {
            case TGPU_PRED_EQ: ok = c == 0; break;
            case TGPU_PRED_NE: ok = c != 0; break;
            case TGPU_PRED_LT: ok = c < 0; break;
            case TGPU_PRED_LE: ok = c <= 0; break;
            case TGPU_PRED_GT: ok = c > 0; break;
            default: ok = c >= 0; break;
        }
        if (!ok) return false;
    }
    return true;
}

// The two encoded words of ORDER BY entry `o` for a group: NULL = 0, a value
// = its order-preserving image + 1, complemented for DESC.  Smaller words =
// earlier row.
__device__ __forceinline__ void order_words(const DevFinal &f, const DevOrder &o, uint64_t k0, uint64_t k1,
                                            const unsigned long long *st, uint64_t &hi, uint64_t &lo) {
    EmitVal v = o.target == TGPU_SORT_KEY ? emit_key(f, k0, k1, o.index) : emit_agg(f, st, o.index);
    hi = 0;
    lo = 0;
    if (!v.null && o.target == TGPU_SORT_KEY && f.part_rank[o.index]) {
        // a string key: the code's rank among the dictionary's strings
        const uint32_t code = (uint32_t)v.lo, n = f.part_rank_n[o.index];
        v.lo = code < n ? (uint64_t)__ldg(f.part_rank[o.index] + code) : (uint64_t)n + code;
        v.hi = 0;
    }
    if (!v.null) {
        if (v.is_f) {
            double d = v.f;
            uint64_t b = (d != d) ? 0x7FF8000000000000ULL : (d == 0.0 ? 0ULL : f64_bits(d));
            lo = enc_f64_bits(b);
        } else {
            lo = v.lo;
            hi = (uint64_t)v.hi ^ 0x8000000000000000ULL;
        }
        lo += 1;
        if (lo == 0) hi += 1;
    }
    if (o.desc) {
        hi = ~hi;
        lo = ~lo;
    }
}

// Encoded sort key: the ORDER BY word pairs, then the packed key (ties break
// on the key ascending).  f.sort_words words.
__device__ void encode_sort_key(const DevFinal &f, uint32_t gid, uint64_t *w) {
    uint64_t k0, k1;
    slot_key(f, gid, k0, k1);
    const unsigned long long *st = slot_states(f, gid);
    int n = 0;
    for (int i = 0; i < f.n_order; ++i) {
        order_words(f, f.order[i], k0, k1, st, w[n], w[n + 1]);
        n += 2;
    }
    w[n++] = k1;
    w[n++] = k0;
}

template <typename A, typename B>
__device__ __forceinline__ bool key_less(const A *a, const B *b, int sw) {
#pragma unroll
    for (int i = 0; i < MAX_SORT_WORDS; ++i) {
        if (i >= sw) break;
        if (a[i] != b[i]) return a[i] < b[i];
    }
    return false;
}

// -------------------------------------------------------------- compact --

constexpr int CPT_THREADS = 256;
constexpr int CPT_WORDS_PER_THREAD = 8;
constexpr int CPT_WORDS_PER_BLOCK = CPT_THREADS * CPT_WORDS_PER_THREAD;

__device__ __forceinline__ int block_excl_scan(int v, int *sh, int &total) {
    // Kogge-Stone over warps
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int nw = blockDim.x >> 5;
        int s = lane < nw ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(FULL, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) sh[lane] = s;
    }
    __syncthreads();
    int before = warp ? sh[warp - 1] : 0;
    total = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before + x - v;
}

__device__ __forceinline__ void compact_count_body(const DevFinal &f, uint64_t n_words, uint32_t *block_counts,
                                                   unsigned long long *counts, uint32_t bid) {
    __shared__ int sh[32];
    uint64_t w0 = (uint64_t)bid * CPT_WORDS_PER_BLOCK + threadIdx.x * CPT_WORDS_PER_THREAD;
    int groups = 0, kept = 0;
    for (int i = 0; i < CPT_WORDS_PER_THREAD; ++i) {
        uint64_t w = w0 + i;
        if (w >= n_words) break;
        uint32_t bits = f.occ[w];
        while (bits) {
            int b = __ffs(bits) - 1;
            bits &= bits - 1;
            uint32_t gid = (uint32_t)(w * 32 + b);
            ++groups;
            if (f.n_having == 0 || having_pass(f, slot_states(f, gid))) ++kept;
        }
    }
    int tg, tk;
    block_excl_scan(groups, sh, tg);
    block_excl_scan(kept, sh, tk);
    if (threadIdx.x == 0) {
        block_counts[bid] = (uint32_t)tk;
        if (tg) atomicAdd(&counts[0], (unsigned long long)tg);
    }
}

__global__ void __launch_bounds__(CPT_THREADS) compact_count_kernel(const __grid_constant__ DevFinal f, uint64_t n_words,
                                                                    uint32_t *block_counts,
                                                                    unsigned long long *counts) {
    compact_count_body(f, n_words, block_counts, counts, blockIdx.x);
}

__device__ __forceinline__ void compact_write_body(const DevFinal &f, uint64_t n_words, const uint32_t *block_counts,
                                                   uint32_t n_blocks, uint32_t *gids_out, unsigned long long *counts,
                                                   uint32_t bid) {
    __shared__ int sh[32];
    __shared__ unsigned long long base_sh;
    // this block's output offset = sum of the previous blocks' counts
    unsigned long long part = 0;
    for (uint32_t b = threadIdx.x; b < bid; b += blockDim.x) part += block_counts[b];
    for (int o = 16; o; o >>= 1) part += __shfl_down_sync(FULL, part, o);
    if (threadIdx.x == 0) base_sh = 0;
    __syncthreads();
    if ((threadIdx.x & 31) == 0 && part) atomicAdd(&base_sh, part);
    __syncthreads();
    const unsigned long long base = base_sh;

    uint64_t w0 = (uint64_t)bid * CPT_WORDS_PER_BLOCK + threadIdx.x * CPT_WORDS_PER_THREAD;
    int kept = 0;
    for (int i = 0; i < CPT_WORDS_PER_THREAD; ++i) {
        uint64_t w = w0 + i;
        if (w >= n_words) break;
        uint32_t bits = f.occ[w];
        while (bits) {
            int b = __ffs(bits) - 1;
            bits &= bits - 1;
            uint32_t gid = (uint32_t)(w * 32 + b);
            if (f.n_having == 0 || having_pass(f, slot_states(f, gid))) ++kept;
        }
    }
    int total;
    int pos = block_excl_scan(kept, sh, total);
    for (int i = 0; i < CPT_WORDS_PER_THREAD; ++i) {
        uint64_t w = w0 + i;
        if (w >= n_words) break;
        uint32_t bits = f.occ[w];
        while (bits) {
            int b = __ffs(bits) - 1;
            bits &= bits - 1;
            uint32_t gid = (uint32_t)(w * 32 + b);
            if (f.n_having == 0 || having_pass(f, slot_states(f, gid))) gids_out[base + pos++] = gid;
        }
    }
    if (bid == n_blocks - 1 && threadIdx.x == 0) counts[1] = base + total;
}

__global__ void __launch_bounds__(CPT_THREADS) compact_write_kernel(const __grid_constant__ DevFinal f, uint64_t n_words,
                                                                    const uint32_t *block_counts,
                                                                    uint32_t n_blocks, uint32_t *gids_out,
                                                                    unsigned long long *counts) {
    compact_write_body(f, n_words, block_counts, n_blocks, gids_out, counts, blockIdx.x);
}

// ----------------------------------------------------------------- top-k --
//
// k <= 32.  The key width is a compile-time class SW (topk_width: 4, 6, 8 or
// 14 words) so the lists live in registers: the ORDER BY word pairs first,
// zero padding, then the packed key in the last two words — the same order
// as encode_sort_key's dense layout.

constexpr int TOPK_THREADS = 256;
constexpr int TOPK_LIST = 32 * 32;  // occupied slots of one warp's 32 bitmap words at most
constexpr int TOPK_WARPS = TOPK_THREADS / 32;
constexpr uint32_t NO_ID = 0xFFFFFFFFu;

template <int SW>
__device__ __forceinline__ bool lex_less(const uint64_t (&a)[SW], const uint64_t (&b)[SW]) {
#pragma unroll
    for (int i = 0; i < SW; ++i)
        if (a[i] != b[i]) return a[i] < b[i];
    return false;
}

template <int SW>
__device__ __forceinline__ void encode_top_key(const DevFinal &f, uint32_t gid, uint64_t (&w)[SW]) {
    uint64_t k0, k1;
    slot_key(f, gid, k0, k1);
    const unsigned long long *st = slot_states(f, gid);
#pragma unroll
    for (int i = 0; i < (SW - 2) / 2; ++i) {
        uint64_t hi = 0, lo = 0;
        if (i < f.n_order) order_words(f, f.order[i], k0, k1, st, hi, lo);
        w[2 * i] = hi;
        w[2 * i + 1] = lo;
    }
    w[SW - 2] = k1;
    w[SW - 1] = k0;
}

// A warp's sorted list of its best (up to k) entries, entry j in lane j.
template <int SW>
struct WarpList {
    uint64_t key[SW];
    uint64_t worst[SW];  // entry k-1 once the list is full (warp-uniform)
    uint32_t gid;
    int count;           // warp-uniform
};

template <int SW>
__device__ __forceinline__ void wl_init(WarpList<SW> &t) {
#pragma unroll
    for (int i = 0; i < SW; ++i) t.key[i] = t.worst[i] = ~0ULL;
    t.gid = NO_ID;
    t.count = 0;
}

// Offer each lane's candidate (if valid).  Once the list is full only
// candidates ahead of its k-th entry get past the first comparison, so the
// serial insertions are few after the first k.
template <int SW>
__device__ __forceinline__ void wl_offer(WarpList<SW> &t, const uint64_t (&cand)[SW], uint32_t cgid, bool valid,
                                         int k) {
    const int lane = threadIdx.x & 31;
    unsigned m = __ballot_sync(FULL, valid && (t.count < k || lex_less<SW>(cand, t.worst)));
    while (m) {
        const int src = __ffs(m) - 1;
        m &= m - 1;
        uint64_t c[SW];
#pragma unroll
        for (int i = 0; i < SW; ++i) c[i] = (uint64_t)__shfl_sync(FULL, (long long)cand[i], src);
        const uint32_t g = __shfl_sync(FULL, cgid, src);
        if (t.count == k && !lex_less<SW>(c, t.worst)) continue;  // an earlier insertion raised the bar
        const int pos = __popc(__ballot_sync(FULL, lane < t.count && lex_less<SW>(t.key, c)));
        uint64_t up[SW];
#pragma unroll
        for (int i = 0; i < SW; ++i) up[i] = (uint64_t)__shfl_up_sync(FULL, (long long)t.key[i], 1);
        const uint32_t upg = __shfl_up_sync(FULL, t.gid, 1);
        if (lane > pos && lane < k) {
#pragma unroll
            for (int i = 0; i < SW; ++i) t.key[i] = up[i];
            t.gid = upg;
        }
        if (lane == pos) {
#pragma unroll
            for (int i = 0; i < SW; ++i) t.key[i] = c[i];
            t.gid = g;
        }
        if (t.count < k) ++t.count;
        if (t.count == k) {
#pragma unroll
            for (int i = 0; i < SW; ++i) t.worst[i] = (uint64_t)__shfl_sync(FULL, (long long)t.key[i], k - 1);
        }
    }
}

// Every warp's list -> the CTA's best k, written to out_keys (if given) and
// out_gids (k entries, NO_ID pads), the count to *out_count (if given).  All
// threads return after the merge.
template <int SW>
__device__ __forceinline__ void block_merge(const WarpList<SW> &t, int k, unsigned long long *out_keys,
                                            uint32_t *out_gids, unsigned long long *out_count) {
    // Merge by rank: every thread owns one warp-list entry and counts the
    // valid entries ordered before it (ties, which distinct packed keys rule
    // out, fall back to the entry index), so the entry of rank r < k lands at
    // position r.  All threads at once, instead of one warp inserting the
    // lists one entry at a time.
    __shared__ unsigned long long s_keys[TOPK_WARPS * 32 * SW];
    __shared__ uint32_t s_ids[TOPK_WARPS * 32];
    __shared__ int s_cnt[TOPK_WARPS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < SW; ++i) s_keys[((size_t)warp * 32 + lane) * SW + i] = t.key[i];
    s_ids[warp * 32 + lane] = t.gid;
    if (lane == 0) s_cnt[warp] = t.count;
    __syncthreads();
    int total = 0;
    for (int w = 0; w < TOPK_WARPS; ++w) total += s_cnt[w];
    if (lane < t.count) {
        const int me = warp * 32 + lane;
        int rank = 0;
        for (int w = 0; w < TOPK_WARPS; ++w) {
            const int n = s_cnt[w];
            for (int j = 0; j < n; ++j) {
                const unsigned long long *o = s_keys + ((size_t)w * 32 + j) * SW;
                int cmp = 0;  // -1: o orders before mine, 1: after
#pragma unroll
                for (int i = 0; i < SW; ++i)
                    if (cmp == 0 && o[i] != t.key[i]) cmp = o[i] < t.key[i] ? -1 : 1;
                rank += (cmp < 0 || (cmp == 0 && w * 32 + j < me)) ? 1 : 0;
            }
        }
        if (rank < k) {
            if (out_keys) {
#pragma unroll
                for (int i = 0; i < SW; ++i) out_keys[(size_t)rank * SW + i] = t.key[i];
            }
            out_gids[rank] = t.gid;
        }
    }
    const int kept = total < k ? total : k;
    if ((int)threadIdx.x >= kept && (int)threadIdx.x < k) {
        if (out_keys) {
#pragma unroll
            for (int i = 0; i < SW; ++i) out_keys[(size_t)threadIdx.x * SW + i] = 0;
        }
        out_gids[threadIdx.x] = NO_ID;
    }
    if (out_count && threadIdx.x == 0) *out_count = (unsigned long long)kept;
    __syncthreads();
}

// Best k of the candidates i = first + warp*32 + lane (+ stride ...) < n, as
// produced by get(i, key, gid) -> valid.  Every warp keeps its own list, then
// block_merge writes the CTA's k entries (NO_ID pads) to out_keys (if given)
// and out_gids, and the kept count to *out_count (if given).
template <int SW, class Get>
__device__ __forceinline__ void block_topk(uint64_t n, uint64_t first, uint64_t stride, int k, Get get,
                                           unsigned long long *out_keys, uint32_t *out_gids,
                                           unsigned long long *out_count) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    WarpList<SW> t;
    wl_init(t);
    // U batches of 32 candidates are loaded (their gathers all in flight)
    // before any is offered
    constexpr int U = SW <= 6 ? 4 : 2;
    for (uint64_t base = first + (uint64_t)warp * 32; base < n; base += stride * U) {
        uint64_t c[U][SW];
        uint32_t g[U];
        bool valid[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t i = base + stride * u + lane;
            g[u] = NO_ID;
            valid[u] = false;
            if (i < n) {
                valid[u] = get(i, c[u], g[u]);
            } else {
#pragma unroll
                for (int j = 0; j < SW; ++j) c[u][j] = 0;
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) wl_offer<SW>(t, c[u], g[u], valid[u], k);
    }
    block_merge<SW>(t, k, out_keys, out_gids, out_count);
}

// Per-CTA top-k of the dense group list: k candidates per CTA, at
// cand_* + bid * 32.
template <int SW>
__device__ __forceinline__ void topk_partial_body(const DevFinal &f, const uint32_t *gids,
                                                  const unsigned long long *counts, int k,
                                                  unsigned long long *cand_keys, uint32_t *cand_gids, uint32_t bid,
                                                  uint32_t nblk) {
    const uint64_t n = counts[1];
    block_topk<SW>(
        n, (uint64_t)bid * TOPK_THREADS, (uint64_t)nblk * TOPK_THREADS, k,
        [&](uint64_t i, uint64_t(&c)[SW], uint32_t &g) {
            g = gids[i];
            encode_top_key<SW>(f, g, c);
            return true;
        },
        cand_keys + (size_t)bid * 32 * SW, cand_gids + (size_t)bid * 32, nullptr);
}

// The best k of all CTAs' candidates -> sel_out, counts[3] = rows in sel_out.
template <int SW>
__device__ __forceinline__ void topk_final_body(const unsigned long long *cand_keys, const uint32_t *cand_gids,
                                                uint32_t n_blocks, int k, uint32_t *sel_out,
                                                unsigned long long *counts) {
    block_topk<SW>(
        (uint64_t)n_blocks * k, 0, TOPK_THREADS, k,
        [&](uint64_t i, uint64_t(&c)[SW], uint32_t &g) {
            // every CTA's best first, then every CTA's second, ...: the
            // lists' heads set a high bar early, so few later entries insert
            const uint64_t e = (i % n_blocks) * 32 + (i / n_blocks);
            g = cand_gids[e];
#pragma unroll
            for (int j = 0; j < SW; ++j) c[j] = cand_keys[e * SW + j];
            return g != NO_ID;
        },
        nullptr, sel_out, counts + 3);
}

template <int SW>
__global__ void __launch_bounds__(TOPK_THREADS) topk_partial_kernel(const __grid_constant__ DevFinal f, const uint32_t *gids,
                                                                    const unsigned long long *counts, int k,
                                                                    unsigned long long *cand_keys,
                                                                    uint32_t *cand_gids) {
    topk_partial_body<SW>(f, gids, counts, k, cand_keys, cand_gids, blockIdx.x, gridDim.x);
}

template <int SW>
__global__ void __launch_bounds__(TOPK_THREADS) topk_final_kernel(const unsigned long long *cand_keys,
                                                                  const uint32_t *cand_gids, uint32_t n_blocks, int k,
                                                                  uint32_t *sel_out, unsigned long long *counts) {
    topk_final_body<SW>(cand_keys, cand_gids, n_blocks, k, sel_out, counts);
}

// Single-query top-k in one launch: CTA b walks bitmap words b*256 + ...,
// counts the groups and the HAVING survivors, offers each survivor's
// encoded key to its warp's list, merges them into the CTA's k candidates,
// and the last CTA to finish (a counter bumped after a threadfence; nobody
// waits) merges every CTA's candidates into sel_out / counts[3].
template <int SW>
__global__ void __launch_bounds__(TOPK_THREADS) topk_scan_kernel(const __grid_constant__ DevFinal f, uint64_t n_words,
                                                                 int k, unsigned long long *cand_keys,
                                                                 uint32_t *cand_gids, uint32_t *sel_out,
                                                                 unsigned long long *counts, unsigned int *done) {
    __shared__ unsigned long long s_sum[2][TOPK_WARPS];
    __shared__ int s_last;
    extern __shared__ uint32_t s_lists[];  // TOPK_WARPS lists of up to 32 x 32 occupied slots
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t *list = s_lists + (size_t)warp * TOPK_LIST;
    WarpList<SW> t;
    wl_init(t);
    unsigned long long groups = 0, kept = 0;
    const uint64_t stride = (uint64_t)gridDim.x * TOPK_THREADS;
    // U batches of 32 listed slots are loaded (all in flight) before any is offered
    constexpr int U = SW <= 6 ? 4 : 2;
    for (uint64_t base = (uint64_t)blockIdx.x * TOPK_THREADS + (uint64_t)warp * 32; base < n_words; base += stride) {
        // 32 bitmap words -> the warp's dense list of occupied slots, so the
        // candidates below keep every lane busy whatever the words' counts
        const uint64_t w = base + lane;
        uint32_t bits = w < n_words ? f.occ[w] : 0u;
        const int nb = __popc(bits);
        int end = nb;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL, end, o);
            if (lane >= o) end += y;
        }
        const int total = __shfl_sync(FULL, end, 31);
        groups += (unsigned)nb;
        for (int at = end - nb; bits; ++at) {
            list[at] = (uint32_t)(w * 32 + (__ffs(bits) - 1));
            bits &= bits - 1;
        }
        __syncwarp();
        for (int i0 = 0; i0 < total; i0 += 32 * U) {
            uint64_t c[U][SW];
            uint32_t g[U];
            bool valid[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int i = i0 + u * 32 + lane;
                g[u] = i < total ? list[i] : NO_ID;
                valid[u] = g[u] != NO_ID && (f.n_having == 0 || having_pass(f, slot_states(f, g[u])));
                if (valid[u]) {
                    encode_top_key<SW>(f, g[u], c[u]);
                    ++kept;
                } else {
#pragma unroll
                    for (int j = 0; j < SW; ++j) c[u][j] = 0;
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) wl_offer<SW>(t, c[u], g[u], valid[u], k);
        }
        __syncwarp();
    }
    for (int o = 16; o; o >>= 1) {
        groups += __shfl_down_sync(FULL, groups, o);
        kept += __shfl_down_sync(FULL, kept, o);
    }
    if (lane == 0) {
        s_sum[0][warp] = groups;
        s_sum[1][warp] = kept;
    }
    block_merge<SW>(t, k, cand_keys + (size_t)blockIdx.x * 32 * SW, cand_gids + (size_t)blockIdx.x * 32, nullptr);
    if (threadIdx.x == 0) {
        unsigned long long gsum = 0, ksum = 0;
        for (int i = 0; i < TOPK_WARPS; ++i) {
            gsum += s_sum[0][i];
            ksum += s_sum[1][i];
        }
        if (gsum) atomicAdd(&counts[0], gsum);
        if (ksum) atomicAdd(&counts[1], ksum);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const uint32_t nb = gridDim.x;
    block_topk<SW>(
        (uint64_t)nb * k, 0, TOPK_THREADS, k,
        [&](uint64_t i, uint64_t(&c)[SW], uint32_t &g) {
            // every CTA's best first, then every CTA's second, ...: the
            // lists' heads set a high bar early, so few later entries insert
            const uint64_t e = (i % nb) * 32 + (i / nb);
            g = __ldcg(cand_gids + e);
#pragma unroll
            for (int j = 0; j < SW; ++j) c[j] = __ldcg(cand_keys + e * SW + j);
            return g != NO_ID;
        },
        nullptr, sel_out, counts + 3);
}

// ------------------------------------------------------------ merge sort --

constexpr int SORT_TILE = 1024;
constexpr int SORT_THREADS = 512;

__global__ void sort_keys_kernel(const __grid_constant__ DevFinal f, const uint32_t *gids, const unsigned long long *counts,
                                 unsigned long long *keys, uint32_t *ids) {
    const uint64_t n = counts[1];
    const int sw = f.sort_words;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t w[MAX_SORT_WORDS];
        encode_sort_key(f, gids[i], w);
        for (int j = 0; j < sw; ++j) keys[i * sw + j] = w[j];
        ids[i] = gids[i];
    }
}

__global__ void __launch_bounds__(SORT_THREADS) sort_tile_kernel(int sw, const unsigned long long *counts,
                                                                 unsigned long long *keys, uint32_t *ids) {
    extern __shared__ unsigned long long st_sh[];
    unsigned long long *k = st_sh;                       // SORT_TILE * sw
    uint32_t *id = (uint32_t *)(k + (size_t)SORT_TILE * sw);
    const uint64_t n = counts[1];
    const uint64_t base = (uint64_t)blockIdx.x * SORT_TILE;
    if (base >= n) return;
    for (int i = threadIdx.x; i < SORT_TILE; i += blockDim.x) {
        uint64_t gi = base + i;
        for (int j = 0; j < sw; ++j) k[i * sw + j] = gi < n ? keys[gi * sw + j] : ~0ULL;
        id[i] = gi < n ? ids[gi] : 0xFFFFFFFFu;
    }
    __syncthreads();
    for (int size = 2; size <= SORT_TILE; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = threadIdx.x; t < SORT_TILE / 2; t += blockDim.x) {
                int lo = 2 * t - (t & (stride - 1));
                int hi = lo + stride;
                bool asc = ((lo & size) == 0);
                bool less = key_less(k + (size_t)hi * sw, k + (size_t)lo * sw, sw);
                if (less == asc) {
                    for (int j = 0; j < sw; ++j) {
                        unsigned long long x = k[lo * sw + j];
                        k[lo * sw + j] = k[hi * sw + j];
                        k[hi * sw + j] = x;
                    }
                    uint32_t x = id[lo];
                    id[lo] = id[hi];
                    id[hi] = x;
                }
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < SORT_TILE; i += blockDim.x) {
        uint64_t gi = base + i;
        if (gi >= n) break;
        for (int j = 0; j < sw; ++j) keys[gi * sw + j] = k[i * sw + j];
        ids[gi] = id[i];
    }
}

// Merge adjacent sorted runs of `width` (keys unique): each element's output
// position is its rank in its own run plus its rank in the partner run.
__global__ void merge_pass_kernel(int sw, const unsigned long long *counts, uint64_t width,
                                  const unsigned long long *kin, const uint32_t *iin, unsigned long long *kout,
                                  uint32_t *iout) {
    const uint64_t n = counts[1];
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t run = i / width;
        const uint64_t run_start = run * width;
        const uint64_t pair_start = (run & ~1ULL) * width;
        const uint64_t partner = run ^ 1ULL;
        const uint64_t p_start = partner * width;
        uint64_t out;
        if (p_start >= n) {
            out = i;
        } else {
            const uint64_t p_end = min(p_start + width, n);
            const unsigned long long *me = kin + i * sw;
            // first partner element that is not less than me
            uint64_t lo = p_start, hi = p_end;
            while (lo < hi) {
                uint64_t mid = (lo + hi) >> 1;
                if (key_less(kin + mid * sw, me, sw)) lo = mid + 1;
                else hi = mid;
            }
            out = pair_start + (i - run_start) + (lo - p_start);
        }
        for (int j = 0; j < sw; ++j) kout[out * sw + j] = kin[i * sw + j];
        iout[out] = iin[i];
    }
}

// Every kept group is a selection candidate: counts[3] = counts[1].
__global__ void sel_count_kernel(unsigned long long *counts) { counts[3] = counts[1]; }

// ---------------------------------------------------------------- gather --

__device__ __forceinline__ void gather_body(const DevFinal &f, const uint32_t *sel, uint64_t offset, uint64_t max_rows,
                                            void *const *out_cols, uint8_t *const *out_valid,
                                            unsigned long long *counts, uint32_t bid, uint32_t nblk) {
    const uint64_t ns = counts[3];
    const uint64_t avail = ns > offset ? ns - offset : 0;
    const uint64_t rows = avail < max_rows ? avail : max_rows;
    if (bid == 0 && threadIdx.x == 0) counts[2] = rows;
    for (uint64_t r = (uint64_t)bid * blockDim.x + threadIdx.x; r < rows; r += (uint64_t)nblk * blockDim.x) {
        const uint32_t gid = sel[offset + r];
        uint64_t k0, k1;
        slot_key(f, gid, k0, k1);
        for (int p = 0; p < f.n_parts; ++p) {
            EmitVal v = emit_key(f, k0, k1, p);
            out_valid[p][r] = v.null ? 0 : 1;
            void *col = out_cols[p];
            switch (f.part_types[p]) {
                case TGPU_BOOLEAN: case TGPU_TINYINT: ((int8_t *)col)[r] = (int8_t)v.lo; break;
                case TGPU_SMALLINT: ((int16_t *)col)[r] = (int16_t)v.lo; break;
                case TGPU_INT: case TGPU_DATE: case TGPU_DICT32: ((int32_t *)col)[r] = (int32_t)v.lo; break;
                default: ((int64_t *)col)[r] = (int64_t)v.lo; break;
            }
        }
        const unsigned long long *st = slot_states(f, gid);
        for (int a = 0; a < f.n_aggs; ++a) {
            const int c = f.n_parts + a;
            EmitVal v = emit_agg(f, st, a);
            out_valid[c][r] = v.null ? 0 : 1;
            void *col = out_cols[c];
            switch (f.outs[a].out_type) {
                case TGPU_DOUBLE: ((double *)col)[r] = v.null ? 0.0 : v.f; break;
                case TGPU_FLOAT: ((float *)col)[r] = v.null ? 0.0f : (float)v.f; break;
                case TGPU_DECIMAL128:
                    ((uint64_t *)col)[2 * r] = v.null ? 0 : v.lo;
                    ((int64_t *)col)[2 * r + 1] = v.null ? 0 : v.hi;
                    break;
                case TGPU_BOOLEAN: case TGPU_TINYINT: ((int8_t *)col)[r] = v.null ? 0 : (int8_t)v.lo; break;
                case TGPU_SMALLINT: ((int16_t *)col)[r] = v.null ? 0 : (int16_t)v.lo; break;
                case TGPU_INT: case TGPU_DATE: case TGPU_DICT32: ((int32_t *)col)[r] = v.null ? 0 : (int32_t)v.lo; break;
                default: ((int64_t *)col)[r] = v.null ? 0 : (int64_t)v.lo; break;
            }
        }
    }
}

__global__ void gather_kernel(const __grid_constant__ DevFinal f, const uint32_t *sel, uint64_t offset, uint64_t max_rows,
                              void *const *out_cols, uint8_t *const *out_valid, unsigned long long *counts) {
    gather_body(f, sel, offset, max_rows, out_cols, out_valid, counts, blockIdx.x, gridDim.x);
}

// ----------------------------------------------------------------- clear --

__device__ __forceinline__ void clear_body(unsigned long long *table, uint64_t n_words, int32_t slot_words, uint32_t *occ,
                                           uint32_t bid, uint32_t nblk) {
    for (uint64_t w = (uint64_t)bid * blockDim.x + threadIdx.x; w < n_words; w += (uint64_t)nblk * blockDim.x) {
        uint32_t bits = occ[w];
        if (!bits) continue;
        while (bits) {
            int b = __ffs(bits) - 1;
            bits &= bits - 1;
            unsigned long long *s = table + (w * 32 + b) * (uint64_t)slot_words;
            for (int i = 0; i < slot_words; ++i) s[i] = 0;
        }
        occ[w] = 0;
    }
}

__global__ void clear_kernel(unsigned long long *table, uint64_t n_words, int32_t slot_words, uint32_t *occ) {
    clear_body(table, n_words, slot_words, occ, blockIdx.x, gridDim.x);
}

__host__ __device__ inline uint64_t occ_words(uint64_t cap) { return (cap + 1 + 31) / 32; }

// ------------------------------------------------------ batched (y = query) --

__global__ void __launch_bounds__(CPT_THREADS) compact_count_batch(const DevFinal *fs, const DevFinalBufs *bs) {
    const DevFinal &f = fs[blockIdx.y];
    const DevFinalBufs &b = bs[blockIdx.y];
    if (blockIdx.x >= b.n_cpt_blocks) return;
    compact_count_body(f, occ_words(f.cap), b.block_counts, b.counts, blockIdx.x);
}

__global__ void __launch_bounds__(CPT_THREADS) compact_write_batch(const DevFinal *fs, const DevFinalBufs *bs) {
    const DevFinal &f = fs[blockIdx.y];
    const DevFinalBufs &b = bs[blockIdx.y];
    if (blockIdx.x >= b.n_cpt_blocks) return;
    compact_write_body(f, occ_words(f.cap), b.block_counts, b.n_cpt_blocks, b.gids, b.counts, blockIdx.x);
}

// One launch per key-width class present in the batch: a query runs in the
// launch of its own class (its candidate buffers are sized for that class).
template <int SW>
__global__ void __launch_bounds__(TOPK_THREADS) topk_partial_batch(const DevFinal *fs, const DevFinalBufs *bs) {
    const DevFinalBufs &b = bs[blockIdx.y];
    const DevFinal &f = fs[blockIdx.y];
    if (b.rank != 1 || topk_width(f.sort_words) != SW || blockIdx.x >= b.n_cand_blocks) return;
    topk_partial_body<SW>(f, b.gids, b.counts, (int)b.k, b.cand_keys, b.cand_gids, blockIdx.x, b.n_cand_blocks);
}

// do_all: this launch also sets the selection size of the all-groups queries.
template <int SW>
__global__ void __launch_bounds__(TOPK_THREADS) topk_final_batch(const DevFinal *fs, const DevFinalBufs *bs, int do_all) {
    const DevFinalBufs &b = bs[blockIdx.y];
    if (b.rank == 0) {
        if (do_all && threadIdx.x == 0) b.counts[3] = b.counts[1];
        return;
    }
    if (b.rank != 1 || topk_width(fs[blockIdx.y].sort_words) != SW) return;
    topk_final_body<SW>(b.cand_keys, b.cand_gids, b.n_cand_blocks, (int)b.k, b.sel, b.counts);
}

__global__ void gather_batch(const DevFinal *fs, const DevFinalBufs *bs) {
    const DevFinalBufs &b = bs[blockIdx.y];
    gather_body(fs[blockIdx.y], b.sel, b.offset, b.gather_rows, b.out_cols, b.out_valid, b.counts, blockIdx.x,
                gridDim.x);
}

// Every query's result rows into one mapped host buffer (no per-column copies).
__global__ void pack_batch(const DevFinalBufs *bs) {
    const DevFinalBufs &b = bs[blockIdx.y];
    if (b.pack_rows == 0) return;
    const uint64_t rows = min((uint64_t)b.counts[2], b.pack_rows);
    uint8_t *dst = b.pack_dst;
    if (threadIdx.x == 0) *(volatile unsigned long long *)dst = rows;
    uint64_t off = 8;
    for (uint32_t c = 0; c < b.n_out; ++c) {
        const uint8_t *src = (const uint8_t *)b.out_cols[c];
        const uint64_t n = rows * b.out_bytes[c];
        for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) dst[off + i] = src[i];
        off += b.pack_rows * b.out_bytes[c];
    }
    for (uint32_t c = 0; c < b.n_out; ++c) {
        const uint8_t *src = b.out_valid[c];
        for (uint64_t i = threadIdx.x; i < rows; i += blockDim.x) dst[off + i] = src[i];
        off += b.pack_rows;
    }
    __threadfence_system();
}

__global__ void clear_batch(const DevFinal *fs, const DevFinalBufs *bs) {
    const DevFinal &f = fs[blockIdx.y];
    clear_body(const_cast<unsigned long long *>(f.table), occ_words(f.cap), f.slot_words,
               const_cast<uint32_t *>(f.occ), blockIdx.x, gridDim.x);
}

}  // namespace

uint32_t compact_blocks(uint64_t cap) {
    return (uint32_t)((occ_words(cap) + CPT_WORDS_PER_BLOCK - 1) / CPT_WORDS_PER_BLOCK);
}

cudaError_t launch_compact(const DevFinal &f, uint32_t *block_counts, uint32_t n_blocks, uint32_t *gids_out,
                           unsigned long long *counts, cudaStream_t s) {
    const uint64_t nw = occ_words(f.cap);
    compact_count_kernel<<<n_blocks, CPT_THREADS, 0, s>>>(f, nw, block_counts, counts);
    compact_write_kernel<<<n_blocks, CPT_THREADS, 0, s>>>(f, nw, block_counts, n_blocks, gids_out, counts);
    return cudaGetLastError();
}

template <int SW>
static void launch_topk_w(const DevFinal &f, const uint32_t *gids, unsigned long long *counts, uint32_t k,
                          unsigned long long *cand_keys, uint32_t *cand_gids, uint32_t n_cand_blocks,
                          uint32_t *sel_out, cudaStream_t s) {
    topk_partial_kernel<SW><<<n_cand_blocks, TOPK_THREADS, 0, s>>>(f, gids, counts, (int)k, cand_keys, cand_gids);
    topk_final_kernel<SW><<<1, TOPK_THREADS, 0, s>>>(cand_keys, cand_gids, n_cand_blocks, (int)k, sel_out, counts);
}

cudaError_t launch_topk(const DevFinal &f, const uint32_t *gids, unsigned long long *counts, uint32_t k,
                        unsigned long long *cand_keys, uint32_t *cand_gids, uint32_t n_cand_blocks,
                        uint32_t *sel_out, cudaStream_t s) {
    switch (topk_width(f.sort_words)) {
        case 4: launch_topk_w<4>(f, gids, counts, k, cand_keys, cand_gids, n_cand_blocks, sel_out, s); break;
        case 6: launch_topk_w<6>(f, gids, counts, k, cand_keys, cand_gids, n_cand_blocks, sel_out, s); break;
        case 8: launch_topk_w<8>(f, gids, counts, k, cand_keys, cand_gids, n_cand_blocks, sel_out, s); break;
        default: launch_topk_w<14>(f, gids, counts, k, cand_keys, cand_gids, n_cand_blocks, sel_out, s); break;
    }
    return cudaGetLastError();
}

template <int SW>
static cudaError_t launch_topk_scan_w(const DevFinal &f, uint32_t k, unsigned long long *cand_keys, uint32_t *cand_gids,
                               uint32_t n_blocks, uint32_t *sel_out, unsigned long long *counts, unsigned int *done,
                               cudaStream_t s) {
    const size_t smem = (size_t)TOPK_WARPS * TOPK_LIST * sizeof(uint32_t);
    const cudaError_t e =
        cudaFuncSetAttribute(topk_scan_kernel<SW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    topk_scan_kernel<SW><<<n_blocks, TOPK_THREADS, smem, s>>>(f, occ_words(f.cap), (int)k, cand_keys, cand_gids,
                                                              sel_out, counts, done);
    return cudaGetLastError();
}

cudaError_t launch_topk_scan(const DevFinal &f, unsigned long long *counts, uint32_t k, unsigned long long *cand_keys,
                             uint32_t *cand_gids, uint32_t n_cand_blocks, uint32_t *sel_out, unsigned int *done,
                             cudaStream_t s) {
    switch (topk_width(f.sort_words)) {
        case 4: return launch_topk_scan_w<4>(f, k, cand_keys, cand_gids, n_cand_blocks, sel_out, counts, done, s);
        case 6: return launch_topk_scan_w<6>(f, k, cand_keys, cand_gids, n_cand_blocks, sel_out, counts, done, s);
        case 8: return launch_topk_scan_w<8>(f, k, cand_keys, cand_gids, n_cand_blocks, sel_out, counts, done, s);
        default: return launch_topk_scan_w<14>(f, k, cand_keys, cand_gids, n_cand_blocks, sel_out, counts, done, s);
    }
}

cudaError_t launch_sort(const DevFinal &f, const uint32_t *gids, unsigned long long *counts, uint64_t max_n,
                        unsigned long long *keys_a, unsigned long long *keys_b, uint32_t *ids_a, uint32_t *ids_b,
                        uint32_t **sorted_out, cudaStream_t s) {
    const int sw = f.sort_words;
    int grid = (int)std::min<uint64_t>((max_n + 255) / 256, 4096);
    if (grid < 1) grid = 1;
    sort_keys_kernel<<<grid, 256, 0, s>>>(f, gids, counts, keys_a, ids_a);
    uint64_t tiles = (max_n + SORT_TILE - 1) / SORT_TILE;
    if (tiles < 1) tiles = 1;
    size_t smem = (size_t)SORT_TILE * sw * 8 + SORT_TILE * 4;
    cudaError_t e = cudaFuncSetAttribute(sort_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    sort_tile_kernel<<<(unsigned)tiles, SORT_THREADS, smem, s>>>(sw, counts, keys_a, ids_a);
    unsigned long long *kin = keys_a, *kout = keys_b;
    uint32_t *iin = ids_a, *iout = ids_b;
    for (uint64_t width = SORT_TILE; width < max_n; width <<= 1) {
        merge_pass_kernel<<<grid, 256, 0, s>>>(sw, counts, width, kin, iin, kout, iout);
        std::swap(kin, kout);
        std::swap(iin, iout);
    }
    *sorted_out = iin;
    sel_count_kernel<<<1, 1, 0, s>>>(counts);
    return cudaGetLastError();
}

cudaError_t launch_sel_all(unsigned long long *counts, cudaStream_t s) {
    sel_count_kernel<<<1, 1, 0, s>>>(counts);
    return cudaGetLastError();
}

cudaError_t launch_gather(const DevFinal &f, const uint32_t *sel, unsigned long long *counts, uint64_t offset,
                          uint64_t max_rows, void *const *out_cols, uint8_t *const *out_valid, cudaStream_t s) {
    int grid = (int)std::min<uint64_t>((max_rows + 255) / 256, 2048);
    if (grid < 1) grid = 1;
    gather_kernel<<<grid, 256, 0, s>>>(f, sel, offset, max_rows, out_cols, out_valid, counts);
    return cudaGetLastError();
}

cudaError_t launch_clear(unsigned long long *table, uint64_t cap, int32_t slot_words, uint32_t *occ, cudaStream_t s) {
    uint64_t nw = occ_words(cap);
    int grid = (int)std::min<uint64_t>((nw + 255) / 256, 4096);
    if (grid < 1) grid = 1;
    clear_kernel<<<grid, 256, 0, s>>>(table, nw, slot_words, occ);
    return cudaGetLastError();
}

cudaError_t launch_finalize_batch(const DevFinal *fs, const DevFinalBufs *bs, uint32_t n_queries,
                                  uint32_t max_cpt_blocks, uint32_t max_cand_blocks, uint32_t topk_widths,
                                  uint64_t max_rows, uint64_t max_words, cudaStream_t s) {
    if (n_queries == 0) return cudaSuccess;
    dim3 gc(std::max<uint32_t>(1, max_cpt_blocks), n_queries);
    compact_count_batch<<<gc, CPT_THREADS, 0, s>>>(fs, bs);
    compact_write_batch<<<gc, CPT_THREADS, 0, s>>>(fs, bs);
    const dim3 gp(std::max<uint32_t>(1, max_cand_blocks), n_queries), gf(1, n_queries);
    int do_all = 1;
    if (topk_widths & TOPK_W4) {
        topk_partial_batch<4><<<gp, TOPK_THREADS, 0, s>>>(fs, bs);
        topk_final_batch<4><<<gf, TOPK_THREADS, 0, s>>>(fs, bs, do_all);
        do_all = 0;
    }
    if (topk_widths & TOPK_W6) {
        topk_partial_batch<6><<<gp, TOPK_THREADS, 0, s>>>(fs, bs);
        topk_final_batch<6><<<gf, TOPK_THREADS, 0, s>>>(fs, bs, do_all);
        do_all = 0;
    }
    if (topk_widths & TOPK_W8) {
        topk_partial_batch<8><<<gp, TOPK_THREADS, 0, s>>>(fs, bs);
        topk_final_batch<8><<<gf, TOPK_THREADS, 0, s>>>(fs, bs, do_all);
        do_all = 0;
    }
    if (topk_widths & TOPK_W14) {
        topk_partial_batch<14><<<gp, TOPK_THREADS, 0, s>>>(fs, bs);
        topk_final_batch<14><<<gf, TOPK_THREADS, 0, s>>>(fs, bs, do_all);
        do_all = 0;
    }
    if (do_all) topk_final_batch<4><<<gf, 32, 0, s>>>(fs, bs, 1);
    unsigned gx = (unsigned)std::min<uint64_t>(std::max<uint64_t>(1, (max_rows + 255) / 256), 64);
    gather_batch<<<dim3(gx, n_queries), 256, 0, s>>>(fs, bs);
    pack_batch<<<dim3(1, n_queries), 256, 0, s>>>(bs);
    unsigned cx = (unsigned)std::min<uint64_t>(std::max<uint64_t>(1, (max_words + 255) / 256), 512);
    clear_batch<<<dim3(cx, n_queries), 256, 0, s>>>(fs, bs);
    return cudaGetLastError();
}

}  // namespace tgpu
