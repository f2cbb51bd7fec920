// oracle.cpp — CPU restatement of thinDB's V2 GROUP BY semantics.
//
// TEST INFRASTRUCTURE ONLY: the parity checker and the timed CPU baseline.
// Nothing in the product (thindb_gb300/) links, loads or calls this file.
//
// What it restates, with the thinDB source it follows (paths in the thinDB
// tree):
//   shape validation / declines ....... src/exec/v2_shape_group_topn.zig:2051-2370
//   key packing (LSB-first parts, a nullable part adds a top validity bit,
//     NULL slice all-zero) ............ v2_shape_group_topn.zig:2076-2092, :105-119
//   state slots (i128 lo/hi for SUM/AVG over 64-bit ints, valid-count
//     companion for nullable inputs) .. v2_shape_group_topn.zig:2164-2184
//   folds ............................. src/exec/silo_group_core.zig:7832-8001
//   COUNT(DISTINCT) (gid, value bits)
//     with canonical float bits ....... silo_group_core.zig:8047-8057, :8125-8176
//   output types ...................... src/exec/aggregate.zig:3700-3742
//   AVG = f64(sum)/f64(n)/10^scale .... v2_shape_group_topn.zig:1438-1446
//   BIGINT SUM wraps (i128 -> i64) .... v2_shape_group_topn.zig:1448-1453
//   NULL results / nulls-first order .. v2_shape_group_topn.zig:1361-1424
//   result order: ORDER BY keys, then
//     the packed key ascending ........ v2_shape_group_topn.zig:1327-1335
//   ORDER BY a string key: the strings
//     compared bytewise, after the emit  v2_shape_group_topn.zig:302-325
//   hashed keys (a string part, or more
//     than 128 packed bits): grouped by
//     the parts' exact bytes / values,
//     ordered among exact ties by a digest
//     (thinDB: 128-bit Wyhash; here the
//     engine's str_hash chain) ........ v2_shape_group_topn.zig:2055-2070;
//                                       silo_group_core.zig:5284-5330, :6337
//     (finish_after_emit: a hashed key read by ORDER BY is ranked on the
//     emitted values; a packed id reads its string back)
//   silo grid shape (16-RG tiles, 256
//     buckets, bucket-owned folds) .... silo_group_core.zig:11493, :9228, :9348
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

typedef __int128 i128;
typedef unsigned __int128 u128;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

constexpr int MAX_GROUP_KEYS = 8;  // v2_shape_group_topn.zig:50
constexpr int MAX_AGGS = 16;       // v2_shape_group_topn.zig:54 (aggregates and numeric state slots)
constexpr int MAX_DISTINCT = 8;    // v2_shape_group_topn.zig:62

inline uint64_t mix64(uint64_t z) {  // group_table.zig:45-50
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
inline uint64_t hash_u128(u128 k) {  // group_table.zig:52-55
    return mix64((uint64_t)k ^ mix64((uint64_t)(k >> 64)));
}
inline uint64_t route_hash(u128 k) {  // silo_group_core.zig:5226-5230
    uint64_t x = (uint64_t)k ^ ((uint64_t)(uint32_t)(k >> 64) * 0x9e3779b97f4a7c15ULL);
    x ^= x >> 32;
    return x;
}

enum Phys { P_I8, P_I16, P_I32, P_I64, P_F32, P_F64 };

int type_bits(int t) {  // intTypeBits, v2_shape_group_topn.zig:2698-2706 (+ packed string ids)
    switch (t) {
        case TGPU_BOOLEAN: case TGPU_TINYINT: return 8;
        case TGPU_SMALLINT: return 16;
        case TGPU_INT: case TGPU_DATE: case TGPU_DICT32: return 32;
        case TGPU_BIGINT: case TGPU_DATETIME: case TGPU_DECIMAL64: return 64;
        default: return 0;
    }
}
Phys phys_of(int t) {  // physicalTypeFor, v2_shape_group_topn.zig:2682-2692
    switch (t) {
        case TGPU_BOOLEAN: case TGPU_TINYINT: return P_I8;
        case TGPU_SMALLINT: return P_I16;
        case TGPU_INT: case TGPU_DATE: case TGPU_DICT32: return P_I32;
        case TGPU_FLOAT: return P_F32;
        case TGPU_DOUBLE: return P_F64;
        default: return P_I64;
    }
}
int elem_bytes(int t) {
    switch (t) {
        case TGPU_BOOLEAN: case TGPU_TINYINT: return 1;
        case TGPU_SMALLINT: return 2;
        case TGPU_INT: case TGPU_DATE: case TGPU_DICT32: case TGPU_FLOAT: return 4;
        case TGPU_DECIMAL128: return 16;
        default: return 8;
    }
}
bool is_float(int t) { return t == TGPU_FLOAT || t == TGPU_DOUBLE; }
bool is_temporal(int t) { return t == TGPU_DATE || t == TGPU_DATETIME; }
bool valid_type(int t) { return t >= TGPU_BOOLEAN && t <= TGPU_VARCHAR && t != TGPU_DECIMAL128; }

struct Table {
    const tgpu_column_desc *cols;
    uint32_t ncols;
    uint64_t nrows;
    uint32_t rg_rows;
    bool valid(int c, uint64_t r) const {
        const uint8_t *v = cols[c].validity;
        return !v || ((v[r >> 3] >> (r & 7)) & 1);
    }
    int64_t ival(int c, uint64_t r) const {
        const void *p = cols[c].data;
        switch (cols[c].type) {
            case TGPU_BOOLEAN: return ((const uint8_t *)p)[r];
            case TGPU_TINYINT: return ((const int8_t *)p)[r];
            case TGPU_SMALLINT: return ((const int16_t *)p)[r];
            case TGPU_INT: case TGPU_DATE: case TGPU_DICT32: return ((const int32_t *)p)[r];
            default: return ((const int64_t *)p)[r];
        }
    }
    double fval(int c, uint64_t r) const {
        if (cols[c].type == TGPU_FLOAT) return (double)((const float *)cols[c].data)[r];
        return ((const double *)cols[c].data)[r];
    }
    // TGPU_VARCHAR: data holds n + 1 u32 offsets, dict_bytes the bytes
    const uint8_t *str(int c, uint64_t r, uint32_t &len) const {
        const uint32_t *o = (const uint32_t *)cols[c].data;
        len = o[r + 1] - o[r];
        return cols[c].dict_bytes + o[r];
    }
};

// The digest that orders exact ties among hashed keys — the engine's
// (common.cuh str_hash / digest_step), restated: a string's length and bytes
// as little-endian 8-byte words chained through mix64; an integer's value
// bits; a NULL marker.
uint64_t str_hash(const uint8_t *p, uint32_t n) {
    uint64_t h = mix64((uint64_t)n ^ 0x9E3779B97F4A7C15ULL), w = 0;
    uint32_t k = 0;
    for (uint32_t i = 0; i < n; ++i) {
        w |= (uint64_t)p[i] << (8 * k);
        if (++k == 8) {
            h = mix64(h ^ w);
            w = 0;
            k = 0;
        }
    }
    return k ? mix64(h ^ w) : h;
}

struct KeyPart { int col, type, offset, width; bool nullable; };

struct AggPlan {
    int func, col, in_type;
    bool fl = false, wide = false, nullable = false, distinct = false;
    int scale = 0;
    int state = 0;        // 1-based slot (0 = the group's row count)
    int valid_count = 0;  // 1-based companion slot, 0 = none
    int dslot = 0;        // distinct set index
    int out_type = 0;
};

struct Plan {
    std::vector<KeyPart> parts;
    bool hashed = false;                       // string part or > 128 packed bits
    const std::vector<uint64_t> *rep = nullptr;  // hashed: each passing row's group's first row
    std::vector<AggPlan> aggs;
    int n_slots = 0;
    int n_distinct = 0;
    bool global = false;  // no GROUP BY: v2_global_aggregate.zig, one output row
};

// Dictionary string i of a DICT32 column.
inline std::pair<const uint8_t *, uint32_t> dict_string(const tgpu_column_desc &c, uint32_t i) {
    return {c.dict_bytes + c.dict_offsets[i], c.dict_offsets[i + 1] - c.dict_offsets[i]};
}

// Bytewise order of two strings, a proper prefix first (std.mem.order on u8).
int cmp_bytes(std::pair<const uint8_t *, uint32_t> a, std::pair<const uint8_t *, uint32_t> b) {
    const uint32_t n = std::min(a.second, b.second);
    const int c = n ? std::memcmp(a.first, b.first, n) : 0;
    if (c) return c < 0 ? -1 : 1;
    return a.second == b.second ? 0 : (a.second < b.second ? -1 : 1);
}

bool dict_unique(const tgpu_column_desc &c) {
    if (!c.dict_size) return true;
    std::vector<uint32_t> ix(c.dict_size);
    for (uint32_t i = 0; i < c.dict_size; ++i) ix[i] = i;
    std::sort(ix.begin(), ix.end(),
              [&](uint32_t x, uint32_t y) { return cmp_bytes(dict_string(c, x), dict_string(c, y)) < 0; });
    for (uint32_t i = 1; i < c.dict_size; ++i)
        if (cmp_bytes(dict_string(c, ix[i - 1]), dict_string(c, ix[i])) == 0) return false;
    return true;
}

// validateShape restated (v2_shape_group_topn.zig:2051-2370) for the shapes
// this engine runs; wide decimals decline.
int build_plan(const Table &t, const tgpu_request *req, Plan &p) {
    if (req->n_group_cols > MAX_GROUP_KEYS) return fail(TGPU_DECLINE, "group key count");
    // No GROUP BY: the global aggregate (v2_global_aggregate.zig tryBuild
    // :1188-1191), which declines HAVING.
    p.global = req->n_group_cols == 0;
    if (p.global && req->n_having) return fail(TGPU_DECLINE, "HAVING on a global aggregate");
    if (req->n_aggs == 0 || req->n_aggs > MAX_AGGS) return fail(TGPU_DECLINE, "aggregate count");
    int off = 0;
    int total = 0;
    for (uint32_t i = 0; i < req->n_group_cols; ++i) {
        const int c = req->group_cols[i];
        if (c < 0 || (uint32_t)c >= t.ncols) return fail(TGPU_ERR_INVALID_ARGUMENT, "group column index");
        const int ty = t.cols[c].type;
        if (ty == TGPU_VARCHAR) p.hashed = true;
        else if (type_bits(ty) == 0) return fail(TGPU_DECLINE, "group key type");
        else total += type_bits(ty) + (t.cols[c].validity ? 1 : 0);
    }
    if (total > 128) p.hashed = true;  // validateShape :2067-2070
    for (uint32_t i = 0; i < req->n_group_cols; ++i) {
        int c = req->group_cols[i];
        int ty = t.cols[c].type;
        int w = ty == TGPU_VARCHAR ? 0 : type_bits(ty);
        bool nl = t.cols[c].validity != nullptr;
        // a packed id stands for its string only when no string has two ids
        // (thinDB's table ids are one per value)
        if (ty == TGPU_DICT32 && !dict_unique(t.cols[c])) return fail(TGPU_DECLINE, "dictionary repeats a string");
        KeyPart kp{c, ty, off, w + (nl ? 1 : 0), nl};
        off += kp.width;
        p.parts.push_back(kp);
    }

    int next = 1;
    for (uint32_t i = 0; i < req->n_aggs; ++i) {
        const tgpu_agg_spec &a = req->aggs[i];
        AggPlan ap;
        ap.func = a.func;
        ap.col = a.column;
        if (a.column >= 0) {
            if ((uint32_t)a.column >= t.ncols) return fail(TGPU_ERR_INVALID_ARGUMENT, "aggregate column index");
            ap.in_type = t.cols[a.column].type;
            ap.nullable = t.cols[a.column].validity != nullptr;
            ap.scale = ap.in_type == TGPU_DECIMAL64 ? t.cols[a.column].decimal_scale : 0;
            ap.fl = is_float(ap.in_type);
        }
        switch (a.func) {
            case TGPU_AGG_COUNT:
                if (ap.nullable) {
                    if (next > MAX_AGGS) return fail(TGPU_DECLINE, "aggregate state count");
                    ap.state = next++;
                }
                ap.out_type = TGPU_BIGINT;
                break;
            case TGPU_AGG_SUM: case TGPU_AGG_AVG: case TGPU_AGG_MIN: case TGPU_AGG_MAX: {
                if (a.column < 0) return fail(TGPU_ERR_INVALID_ARGUMENT, "aggregate column");
                if (ap.in_type == TGPU_DICT32 || ap.in_type == TGPU_VARCHAR) return fail(TGPU_DECLINE, "string aggregate");
                if ((a.func == TGPU_AGG_SUM || a.func == TGPU_AGG_AVG) && is_temporal(ap.in_type))
                    return fail(TGPU_DECLINE, "temporal read as a number");
                ap.wide = (a.func == TGPU_AGG_SUM || a.func == TGPU_AGG_AVG) && phys_of(ap.in_type) == P_I64;
                int width = (ap.wide ? 2 : 1) + (ap.nullable ? 1 : 0);
                if (next + width - 1 > MAX_AGGS) return fail(TGPU_DECLINE, "aggregate state count");
                ap.state = next;
                ap.valid_count = ap.nullable ? next + width - 1 : 0;
                next += width;
                if (a.func == TGPU_AGG_SUM)
                    ap.out_type = ap.in_type == TGPU_DECIMAL64 ? TGPU_DECIMAL128 : (ap.fl ? TGPU_DOUBLE : TGPU_BIGINT);
                else if (a.func == TGPU_AGG_AVG)
                    ap.out_type = TGPU_DOUBLE;
                else
                    ap.out_type = ap.in_type;
                break;
            }
            case TGPU_AGG_COUNT_DISTINCT:
                if (a.column < 0) return fail(TGPU_ERR_INVALID_ARGUMENT, "count distinct column");
                if (ap.in_type == TGPU_VARCHAR) return fail(TGPU_DECLINE, "COUNT(DISTINCT) over a string column");
                if (p.n_distinct >= MAX_DISTINCT) return fail(TGPU_DECLINE, "count distinct slot count");
                if (next > MAX_AGGS) return fail(TGPU_DECLINE, "aggregate state count");
                ap.distinct = true;
                ap.state = next++;
                ap.dslot = p.n_distinct++;
                ap.out_type = TGPU_BIGINT;
                break;
            default:
                return fail(TGPU_DECLINE, "aggregate func");
        }
        p.aggs.push_back(ap);
    }
    p.n_slots = next - 1;
    for (uint32_t i = 0; i < req->n_order; ++i) {
        const tgpu_sort_spec &s = req->order[i];
        if (s.target == TGPU_SORT_KEY && (s.index < 0 || (uint32_t)s.index >= req->n_group_cols))
            return fail(TGPU_DECLINE, "order key");
        if (s.target == TGPU_SORT_AGG && (s.index < 0 || (uint32_t)s.index >= req->n_aggs))
            return fail(TGPU_DECLINE, "order key");
        if (s.target != TGPU_SORT_KEY && s.target != TGPU_SORT_AGG) return fail(TGPU_DECLINE, "order key");
        if (s.target == TGPU_SORT_KEY && p.hashed) return fail(TGPU_DECLINE, "ORDER BY a hashed key");
        if (s.target == TGPU_SORT_KEY && p.parts[s.index].type == TGPU_DICT32 &&
            !t.cols[p.parts[s.index].col].dict_size)
            return fail(TGPU_DECLINE, "ORDER BY a string key without its dictionary");
    }
    for (uint32_t i = 0; i < req->n_having; ++i) {
        const tgpu_having &h = req->having[i];
        if (h.agg < 0 || (uint32_t)h.agg >= req->n_aggs || h.op < TGPU_PRED_EQ || h.op > TGPU_PRED_GE)
            return fail(TGPU_DECLINE, "having");
    }
    for (uint32_t i = 0; i < req->n_where; ++i) {
        const tgpu_predicate &w = req->where[i];
        if (w.column < 0 || (uint32_t)w.column >= t.ncols) return fail(TGPU_ERR_INVALID_ARGUMENT, "predicate column");
        if (w.op < TGPU_PRED_BETWEEN || w.op > TGPU_PRED_IS_NOT_NULL) return fail(TGPU_DECLINE, "predicate op");
        if (t.cols[w.column].type == TGPU_VARCHAR) return fail(TGPU_DECLINE, "predicate on a string column");
        if (t.cols[w.column].type == TGPU_DICT32 && !(w.op == TGPU_PRED_EQ || w.op == TGPU_PRED_NE ||
                                                      w.op == TGPU_PRED_IS_NULL || w.op == TGPU_PRED_IS_NOT_NULL))
            return fail(TGPU_DECLINE, "string range predicate");
    }
    return TGPU_OK;
}

// The fused WHERE: a conjunction of leaves; comparisons on NULL are not true.
bool row_passes(const Table &t, const tgpu_request *req, uint64_t r) {
    for (uint32_t i = 0; i < req->n_where; ++i) {
        const tgpu_predicate &w = req->where[i];
        bool v = t.valid(w.column, r);
        if (w.op == TGPU_PRED_IS_NULL) { if (v) return false; continue; }
        if (w.op == TGPU_PRED_IS_NOT_NULL) { if (!v) return false; continue; }
        if (!v) return false;
        bool ok;
        if (is_float(t.cols[w.column].type)) {
            double x = t.fval(w.column, r);
            switch (w.op) {
                case TGPU_PRED_BETWEEN: ok = x >= w.flo && x <= w.fhi; break;
                case TGPU_PRED_NOT_BETWEEN: ok = x < w.flo || x > w.fhi; break;
                case TGPU_PRED_EQ: ok = x == w.flo; break;
                case TGPU_PRED_NE: ok = x != w.flo; break;
                case TGPU_PRED_LT: ok = x < w.flo; break;
                case TGPU_PRED_LE: ok = x <= w.flo; break;
                case TGPU_PRED_GT: ok = x > w.flo; break;
                default: ok = x >= w.flo; break;
            }
        } else {
            int64_t x = t.ival(w.column, r);
            switch (w.op) {
                case TGPU_PRED_BETWEEN: ok = x >= w.lo && x <= w.hi; break;
                case TGPU_PRED_NOT_BETWEEN: ok = x < w.lo || x > w.hi; break;
                case TGPU_PRED_EQ: ok = x == w.lo; break;
                case TGPU_PRED_NE: ok = x != w.lo; break;
                case TGPU_PRED_LT: ok = x < w.lo; break;
                case TGPU_PRED_LE: ok = x <= w.lo; break;
                case TGPU_PRED_GT: ok = x > w.lo; break;
                default: ok = x >= w.lo; break;
            }
        }
        if (!ok) return false;
    }
    return true;
}

// A hashed key's digest over row r's parts.
uint64_t hashed_digest(const Table &t, const Plan &p, uint64_t r) {
    uint64_t d = 0x243F6A8885A308D3ULL;
    for (const KeyPart &kp : p.parts) {
        uint64_t ph;
        if (!t.valid(kp.col, r)) {
            ph = 0x8000000000000001ULL;
        } else if (kp.type == TGPU_VARCHAR) {
            uint32_t n;
            const uint8_t *s = t.str(kp.col, r, n);
            ph = str_hash(s, n);
        } else {
            ph = mix64((uint64_t)t.ival(kp.col, r) ^ 0x6A09E667F3BCC909ULL);
        }
        d = mix64(d ^ ph);
    }
    return d;
}

// A hashed key's exact identity: per part a validity byte, then an
// integer's 8 bytes or a string's u32 length and bytes.
std::string exact_key(const Table &t, const Plan &p, uint64_t r) {
    std::string k;
    for (const KeyPart &kp : p.parts) {
        const bool v = t.valid(kp.col, r);
        k.push_back(v ? 1 : 0);
        if (!v) continue;
        if (kp.type == TGPU_VARCHAR) {
            uint32_t n;
            const uint8_t *s = t.str(kp.col, r, n);
            k.append((const char *)&n, 4);
            k.append((const char *)s, n);
        } else {
            const int64_t x = t.ival(kp.col, r);
            k.append((const char *)&x, 8);
        }
    }
    return k;
}

u128 pack_key(const Table &t, const Plan &p, uint64_t r) {
    // a hashed key: the digest above the group's first passing row + 1
    if (p.hashed) return ((u128)hashed_digest(t, p, r) << 64) | (u128)((*p.rep)[r] + 1);
    u128 key = 0;
    for (const KeyPart &kp : p.parts) {
        u128 slice = 0;
        int payload = kp.width - (kp.nullable ? 1 : 0);
        if (!kp.nullable || t.valid(kp.col, r)) {
            uint64_t raw = (uint64_t)t.ival(kp.col, r);
            if (payload < 64) raw &= ((1ULL << payload) - 1);
            slice = raw;
            if (kp.nullable) slice |= (u128)1 << payload;
        }
        key |= slice << kp.offset;
    }
    return key;
}

// Canonical float bits: -0.0 and 0.0 are one value, every NaN is one value
// (types.zig:589-600, silo_group_core.zig:8047-8057).
uint64_t canon_bits(double v) {
    if (std::isnan(v)) return 0x7FF8000000000000ULL;
    if (v == 0) v = 0.0;
    uint64_t b;
    std::memcpy(&b, &v, 8);
    return b;
}

struct Group {
    u128 key;
    uint64_t count;
    int64_t slots[MAX_AGGS];
};

// Open-addressing u128 -> gid table (IntKeyMemsetTable, group_table.zig:737-890).
struct KeyTable {
    std::vector<u128> keys;
    std::vector<uint32_t> gids;
    size_t mask = 0, used = 0;
    static constexpr uint32_t EMPTY = 0xFFFFFFFFu;
    KeyTable() { resize(64); }
    void resize(size_t cap) {
        std::vector<u128> ok = std::move(keys);
        std::vector<uint32_t> og = std::move(gids);
        keys.assign(cap, 0);
        gids.assign(cap, EMPTY);
        mask = cap - 1;
        used = 0;
        for (size_t i = 0; i < og.size(); ++i)
            if (og[i] != EMPTY) insert_new(ok[i], og[i]);
    }
    void insert_new(u128 k, uint32_t g) {
        size_t h = hash_u128(k) & mask;
        while (gids[h] != EMPTY) h = (h + 1) & mask;
        keys[h] = k;
        gids[h] = g;
        ++used;
    }
    // Returns gid, sets is_new when the key was inserted with gid `next`.
    uint32_t get_or_put(u128 k, uint32_t next, bool &is_new) {
        if ((used + 1) * 4 > (mask + 1) * 3) resize((mask + 1) * 2);  // load <= 0.75
        size_t h = hash_u128(k) & mask;
        while (gids[h] != EMPTY) {
            if (keys[h] == k) { is_new = false; return gids[h]; }
            h = (h + 1) & mask;
        }
        keys[h] = k;
        gids[h] = next;
        ++used;
        is_new = true;
        return next;
    }
};

// Exact (gid, value-bits) membership set (DistinctSet u96 tier, silo_group_core.zig:663-777).
struct PairSet {
    std::vector<uint64_t> vals;
    std::vector<uint32_t> gids;
    size_t mask = 0, used = 0;
    static constexpr uint32_t EMPTY = 0xFFFFFFFFu;
    PairSet() { resize(64); }
    void resize(size_t cap) {
        std::vector<uint64_t> ov = std::move(vals);
        std::vector<uint32_t> og = std::move(gids);
        vals.assign(cap, 0);
        gids.assign(cap, EMPTY);
        mask = cap - 1;
        used = 0;
        for (size_t i = 0; i < og.size(); ++i)
            if (og[i] != EMPTY) insert(og[i], ov[i]);
    }
    bool insert(uint32_t g, uint64_t v) {
        if ((used + 1) * 4 > (mask + 1) * 3) resize((mask + 1) * 2);
        size_t h = mix64(v ^ mix64(g)) & mask;
        while (gids[h] != EMPTY) {
            if (gids[h] == g && vals[h] == v) return false;
            h = (h + 1) & mask;
        }
        gids[h] = g;
        vals[h] = v;
        ++used;
        return true;
    }
};

inline i128 wide_value(const int64_t *slots, int si) {  // wideStateValue: lo at si-1, hi at si
    return (i128)(((u128)(uint64_t)slots[si] << 64) | (u128)(uint64_t)slots[si - 1]);
}
inline void set_wide(int64_t *slots, int si, i128 v) {
    slots[si - 1] = (int64_t)(uint64_t)(u128)v;
    slots[si] = (int64_t)(uint64_t)((u128)v >> 64);
}
inline double slot_f64(const int64_t *slots, int si) {
    double d;
    std::memcpy(&d, &slots[si - 1], 8);
    return d;
}
inline void set_slot_f64(int64_t *slots, int si, double d) { std::memcpy(&slots[si - 1], &d, 8); }

// One bucket's (or the whole table's) fold state.
struct Folder {
    const Table &t;
    const Plan &p;
    KeyTable table;
    std::vector<Group> groups;
    std::vector<PairSet> dsets;
    Folder(const Table &t_, const Plan &p_) : t(t_), p(p_), dsets(p_.n_distinct) {}

    // Per-row fold: foldKernelSumInt/SumFloat/Extreme and the distinct insert
    // (silo_group_core.zig:7867-8001, :8125-8176) applied one row at a time.
    void fold(uint64_t r, u128 key) {
        bool is_new = false;
        uint32_t g = table.get_or_put(key, (uint32_t)groups.size(), is_new);
        if (is_new) {
            Group ng;
            ng.key = key;
            ng.count = 0;
            std::memset(ng.slots, 0, sizeof(ng.slots));
            groups.push_back(ng);
        }
        Group &G = groups[g];
        G.count += 1;
        for (const AggPlan &a : p.aggs) {
            if (a.func == TGPU_AGG_COUNT) {
                if (a.state && t.valid(a.col, r)) G.slots[a.state - 1] += 1;
                continue;
            }
            bool ok = !a.nullable || t.valid(a.col, r);
            if (a.distinct) {
                if (!ok) continue;
                uint64_t bits = a.fl ? canon_bits(t.fval(a.col, r)) : (uint64_t)t.ival(a.col, r);
                if (dsets[a.dslot].insert(g, bits)) G.slots[a.state - 1] += 1;
                continue;
            }
            if (!ok) continue;
            int64_t *s = G.slots;
            bool first = a.nullable ? s[a.valid_count - 1] == 0 : is_new;
            switch (a.func) {
                case TGPU_AGG_SUM: case TGPU_AGG_AVG:
                    if (a.fl) set_slot_f64(s, a.state, slot_f64(s, a.state) + t.fval(a.col, r));
                    else if (a.wide) set_wide(s, a.state, wide_value(s, a.state) + (i128)t.ival(a.col, r));
                    else s[a.state - 1] = (int64_t)((uint64_t)s[a.state - 1] + (uint64_t)t.ival(a.col, r));
                    break;
                case TGPU_AGG_MIN: case TGPU_AGG_MAX: {
                    bool mn = a.func == TGPU_AGG_MIN;
                    if (a.fl) {
                        double v = t.fval(a.col, r), cur = slot_f64(s, a.state);
                        if (first || (mn ? v < cur : v > cur)) set_slot_f64(s, a.state, v);
                    } else {
                        int64_t v = t.ival(a.col, r), cur = s[a.state - 1];
                        if (first || (mn ? v < cur : v > cur)) s[a.state - 1] = v;
                    }
                    break;
                }
            }
            if (a.valid_count) s[a.valid_count - 1] += 1;
        }
    }
};

// ------------------------------------------------------------ finalize --

struct Value {  // one emitted aggregate / key cell
    bool null = false;
    bool is_f = false;
    i128 i = 0;
    double f = 0;
};

const double POW10[] = {1e0, 1e1, 1e2, 1e3, 1e4, 1e5, 1e6, 1e7, 1e8, 1e9, 1e10,
                        1e11, 1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18};

uint64_t agg_denom(const Group &g, const AggPlan &a) {  // aggDenom, :1407-1411
    if (a.valid_count) return (uint64_t)g.slots[a.valid_count - 1];
    return g.count;
}

Value agg_value(const Group &g, const AggPlan &a, bool global) {
    Value v;
    switch (a.func) {
        case TGPU_AGG_COUNT:  // countValue, :1400-1404
            v.i = a.state ? (i128)g.slots[a.state - 1] : (i128)g.count;
            return v;
        case TGPU_AGG_COUNT_DISTINCT:
            v.i = (i128)g.slots[a.state - 1];
            return v;
        default: break;
    }
    uint64_t den = agg_denom(g, a);
    // aggIsNull, :1413-1424 (a group's non-nullable input always has rows);
    // the global aggregate's emitRow: NULL over zero non-NULL inputs
    // (v2_global_aggregate.zig:1853-1855)
    if (den == 0) { v.null = true; return v; }
    switch (a.func) {
        case TGPU_AGG_SUM:
            if (a.fl) { v.is_f = true; v.f = slot_f64(g.slots, a.state); }
            else {
                i128 s = a.wide ? wide_value(g.slots, a.state) : (i128)g.slots[a.state - 1];
                v.i = a.out_type == TGPU_BIGINT ? (i128)(int64_t)(uint64_t)(u128)s : s;  // integerAggValue
            }
            return v;
        case TGPU_AGG_AVG:
            v.is_f = true;
            if (den == 0) { v.f = 0.0; return v; }
            if (a.fl) v.f = slot_f64(g.slots, a.state) / (double)den;  // avgFloatValue, :1467-1470
            else {
                i128 s = a.wide ? wide_value(g.slots, a.state) : (i128)g.slots[a.state - 1];
                v.f = global ? (double)s / ((double)den * POW10[a.scale])  // emitRow, v2_global_aggregate.zig:1872-1877
                             : (double)s / (double)den / POW10[a.scale];   // avgValue, :1438-1446
            }
            return v;
        default:  // MIN / MAX
            if (a.fl) { v.is_f = true; v.f = slot_f64(g.slots, a.state); }
            else v.i = (i128)g.slots[a.state - 1];
            return v;
    }
}

Value key_value(const Table &t, const Plan &p, const Group &g, const KeyPart &kp) {  // keyPartValue / keyPartIsNull, :1426-1470
    Value v;
    if (p.hashed) {
        // read at the group's first row; a string part emits that row
        const uint64_t row = (uint64_t)g.key - 1;
        if (!t.valid(kp.col, row)) { v.null = true; return v; }
        v.i = kp.type == TGPU_VARCHAR ? (i128)row : (i128)t.ival(kp.col, row);
        return v;
    }
    int payload = kp.width - (kp.nullable ? 1 : 0);
    if (kp.nullable && !((g.key >> (kp.offset + kp.width - 1)) & 1)) { v.null = true; return v; }
    uint64_t raw = (uint64_t)(g.key >> kp.offset);
    if (payload < 64) raw &= (1ULL << payload) - 1;
    switch (kp.type) {
        case TGPU_BOOLEAN: case TGPU_TINYINT: v.i = (int8_t)(uint8_t)raw; break;
        case TGPU_SMALLINT: v.i = (int16_t)(uint16_t)raw; break;
        case TGPU_INT: case TGPU_DATE: case TGPU_DICT32: v.i = (int32_t)(uint32_t)raw; break;
        default: v.i = (int64_t)raw; break;
    }
    return v;
}

// compareF64 with NaN ordered largest (floatOrder, types.zig:579-587) so the
// sort is a strict weak order; -0.0 == 0.0 as in compareF64.
int cmp_f64(double a, double b) {
    bool an = std::isnan(a), bn = std::isnan(b);
    if (an || bn) return an && bn ? 0 : (an ? 1 : -1);
    return a < b ? -1 : (a > b ? 1 : 0);
}
int cmp_value(const Value &a, const Value &b) {  // NULLs first (compareAggregateValue, :1361-1369)
    if (a.null || b.null) return a.null && b.null ? 0 : (a.null ? -1 : 1);
    if (a.is_f) return cmp_f64(a.f, b.f);
    return a.i < b.i ? -1 : (a.i > b.i ? 1 : 0);
}

bool having_ok(const Value &v, const tgpu_having &h) {
    if (v.null) return false;
    int c = v.is_f ? cmp_f64(v.f, h.fval) : (v.i < (i128)h.ival ? -1 : (v.i > (i128)h.ival ? 1 : 0));
    if (v.is_f && (std::isnan(v.f) || std::isnan(h.fval))) return h.op == TGPU_PRED_NE;
    switch (h.op) {
        case TGPU_PRED_EQ: return c == 0;
        case TGPU_PRED_NE: return c != 0;
        case TGPU_PRED_LT: return c < 0;
        case TGPU_PRED_LE: return c <= 0;
        case TGPU_PRED_GT: return c > 0;
        default: return c >= 0;
    }
}

struct Result {
    std::vector<tgpu_output_column> schema;
    std::vector<std::vector<uint8_t>> data;
    std::vector<std::vector<uint8_t>> valid;
    uint64_t rows = 0, groups = 0, selected = 0;
};

void put_int(std::vector<uint8_t> &buf, int type, i128 v) {
    uint8_t tmp[16];
    int n = elem_bytes(type);
    u128 u = (u128)v;
    for (int i = 0; i < n; ++i) tmp[i] = (uint8_t)(u >> (8 * i));
    buf.insert(buf.end(), tmp, tmp + n);
}
void put_f(std::vector<uint8_t> &buf, int type, double v) {
    if (type == TGPU_FLOAT) {
        float f = (float)v;
        uint8_t *b = (uint8_t *)&f;
        buf.insert(buf.end(), b, b + 4);
    } else {
        uint8_t *b = (uint8_t *)&v;
        buf.insert(buf.end(), b, b + 8);
    }
}

int run(const Table &t, const tgpu_request *req, int threads, Result &res) {
    Plan p;
    int st = build_plan(t, req, p);
    if (st != TGPU_OK) return st;

    // hashed keys: every passing row's group's first passing row (exact
    // identity by bytes), the part of the packed key that tells groups apart
    std::vector<uint64_t> rep;
    if (p.hashed) {
        rep.assign(t.nrows, 0);
        std::unordered_map<std::string, uint64_t> first;
        for (uint64_t r = 0; r < t.nrows; ++r) {
            if (!row_passes(t, req, r)) continue;
            rep[r] = first.emplace(exact_key(t, p, r), r).first->second;
        }
        p.rep = &rep;
    }
    std::vector<Group> groups;
    uint64_t selected = 0;
    if (threads <= 1) {
        Folder f(t, p);
        for (uint64_t r = 0; r < t.nrows; ++r) {
            if (!row_passes(t, req, r)) continue;
            ++selected;
            f.fold(r, pack_key(t, p, r));
        }
        groups = std::move(f.groups);
    } else {
        // Silo shape: tiles of 16 row groups stage row ids into 256 buckets by
        // the route hash; each bucket is then folded by one worker, tiles in
        // order, so the result does not depend on the thread count.
        const uint32_t B = 256;
        const uint64_t tile_rows = (uint64_t)t.rg_rows * 16;
        const uint64_t n_tiles = (t.nrows + tile_rows - 1) / tile_rows;
        std::vector<std::vector<std::vector<uint32_t>>> staged(n_tiles, std::vector<std::vector<uint32_t>>(B));
        std::vector<uint64_t> sel(n_tiles, 0);
        std::atomic<uint64_t> next_tile{0};
        auto stage = [&]() {
            for (;;) {
                uint64_t ti = next_tile.fetch_add(1);
                if (ti >= n_tiles) return;
                uint64_t b = ti * tile_rows, e = std::min(t.nrows, b + tile_rows);
                for (uint64_t r = b; r < e; ++r) {
                    if (!row_passes(t, req, r)) continue;
                    ++sel[ti];
                    staged[ti][route_hash(pack_key(t, p, r)) & (B - 1)].push_back((uint32_t)(r - b));
                }
            }
        };
        std::vector<std::thread> ws;
        for (int i = 0; i < threads; ++i) ws.emplace_back(stage);
        for (auto &w : ws) w.join();
        ws.clear();
        for (uint64_t s : sel) selected += s;
        std::vector<std::vector<Group>> out(B);
        std::atomic<uint32_t> next_bucket{0};
        auto foldb = [&]() {
            for (;;) {
                uint32_t bi = next_bucket.fetch_add(1);
                if (bi >= B) return;
                Folder f(t, p);
                for (uint64_t ti = 0; ti < n_tiles; ++ti) {
                    uint64_t base = ti * tile_rows;
                    for (uint32_t off : staged[ti][bi]) f.fold(base + off, pack_key(t, p, base + off));
                    std::vector<uint32_t>().swap(staged[ti][bi]);
                }
                out[bi] = std::move(f.groups);
            }
        };
        for (int i = 0; i < threads; ++i) ws.emplace_back(foldb);
        for (auto &w : ws) w.join();
        for (auto &o : out) groups.insert(groups.end(), o.begin(), o.end());
    }
    res.groups = groups.size();
    res.selected = selected;
    // a global aggregate answers one row even when no row passed: COUNTs 0,
    // the other aggregates NULL (v2_global_aggregate.zig emitRow :1839-1905)
    if (p.global && groups.empty()) groups.push_back(Group{0, 0, {}});

    // HAVING (applyHaving, v2_shape_group_topn.zig:2586)
    std::vector<uint32_t> keep;
    keep.reserve(groups.size());
    for (uint32_t g = 0; g < groups.size(); ++g) {
        bool ok = true;
        for (uint32_t h = 0; h < req->n_having && ok; ++h)
            ok = having_ok(agg_value(groups[g], p.aggs[req->having[h].agg], p.global), req->having[h]);
        if (ok) keep.push_back(g);
    }
    // ORDER BY, then the packed key (rowOrderBefore, :1327-1335)
    if (req->n_order > 0) {
        auto order_val = [&](const Group &g, const tgpu_sort_spec &s) {
            return s.target == TGPU_SORT_KEY ? key_value(t, p, g, p.parts[s.index]) : agg_value(g, p.aggs[s.index], p.global);
        };
        // a DICT32 key orders by its strings; a code outside the dictionary
        // after every string, by code
        auto order_cmp = [&](const Group &a, const Group &b, const tgpu_sort_spec &s) {
            Value va = order_val(a, s), vb = order_val(b, s);
            if (s.target != TGPU_SORT_KEY || p.parts[s.index].type != TGPU_DICT32 || va.null || vb.null)
                return cmp_value(va, vb);
            const tgpu_column_desc &c = t.cols[p.parts[s.index].col];
            const uint32_t ca = (uint32_t)(int32_t)va.i, cb = (uint32_t)(int32_t)vb.i;
            const bool ia = ca < c.dict_size, ib = cb < c.dict_size;
            if (ia && ib) return cmp_bytes(dict_string(c, ca), dict_string(c, cb));
            if (ia != ib) return ia ? -1 : 1;
            return ca < cb ? -1 : (ca > cb ? 1 : 0);
        };
        std::sort(keep.begin(), keep.end(), [&](uint32_t x, uint32_t y) {
            const Group &a = groups[x], &b = groups[y];
            for (uint32_t i = 0; i < req->n_order; ++i) {
                int c = order_cmp(a, b, req->order[i]);
                if (c == 0) continue;
                return (c < 0) != (req->order[i].desc != 0);
            }
            return a.key < b.key;
        });
    }
    uint64_t begin = std::min<uint64_t>(req->offset, keep.size());
    uint64_t end = req->limit == TGPU_NO_LIMIT ? keep.size() : std::min<uint64_t>(keep.size(), begin + req->limit);
    if (req->n_order == 0 && (req->offset > 0 || req->limit != TGPU_NO_LIMIT)) {
        // Without ORDER BY the page is over the packed-key order so it is
        // deterministic (thinDB leaves it unspecified).
        std::sort(keep.begin(), keep.end(), [&](uint32_t x, uint32_t y) { return groups[x].key < groups[y].key; });
    }
    res.rows = end - begin;

    // schema + columns
    size_t ncols = p.parts.size() + p.aggs.size();
    res.data.assign(ncols, {});
    res.valid.assign(ncols, {});
    for (size_t i = 0; i < p.parts.size(); ++i) {
        tgpu_output_column oc{};
        const char *nm = t.cols[p.parts[i].col].name;
        std::snprintf(oc.name, sizeof(oc.name), "%s", nm ? nm : "");
        oc.type = p.parts[i].type;
        oc.nullable = p.parts[i].nullable;
        oc.decimal_precision = t.cols[p.parts[i].col].decimal_precision;
        oc.decimal_scale = t.cols[p.parts[i].col].decimal_scale;
        oc.elem_bytes = elem_bytes(oc.type);
        res.schema.push_back(oc);
    }
    for (size_t i = 0; i < p.aggs.size(); ++i) {
        tgpu_output_column oc{};
        const char *nm = req->aggs[i].as;
        std::snprintf(oc.name, sizeof(oc.name), "%s", nm ? nm : "");
        oc.type = p.aggs[i].out_type;
        oc.nullable = (p.aggs[i].nullable || p.global) && p.aggs[i].func != TGPU_AGG_COUNT && !p.aggs[i].distinct;
        if (oc.type == TGPU_DECIMAL128) { oc.decimal_precision = 38; oc.decimal_scale = (uint8_t)p.aggs[i].scale; }
        if (oc.type == TGPU_DECIMAL64) {
            oc.decimal_precision = t.cols[p.aggs[i].col].decimal_precision;
            oc.decimal_scale = t.cols[p.aggs[i].col].decimal_scale;
        }
        oc.elem_bytes = elem_bytes(oc.type);
        res.schema.push_back(oc);
    }
    for (uint64_t r = begin; r < end; ++r) {
        const Group &g = groups[keep[r]];
        for (size_t i = 0; i < p.parts.size(); ++i) {
            Value v = key_value(t, p, g, p.parts[i]);
            put_int(res.data[i], p.parts[i].type, v.null ? 0 : v.i);
            res.valid[i].push_back(v.null ? 0 : 1);
        }
        for (size_t i = 0; i < p.aggs.size(); ++i) {
            size_t c = p.parts.size() + i;
            Value v = agg_value(g, p.aggs[i], p.global);
            int ty = p.aggs[i].out_type;
            if (v.null) {
                std::vector<uint8_t> z(elem_bytes(ty), 0);
                res.data[c].insert(res.data[c].end(), z.begin(), z.end());
            } else if (ty == TGPU_DOUBLE || ty == TGPU_FLOAT) {
                put_f(res.data[c], ty, v.f);
            } else {
                put_int(res.data[c], ty, v.i);
            }
            res.valid[c].push_back(v.null ? 0 : 1);
        }
    }
    return TGPU_OK;
}

}  // namespace

extern "C" {

int orc_group_by(const tgpu_table_desc *td, const tgpu_request *req, int threads, void **out) {
    if (!td || !req || !out) return fail(TGPU_ERR_INVALID_ARGUMENT, "null argument");
    if (td->location != TGPU_LOC_HOST) return fail(TGPU_ERR_INVALID_ARGUMENT, "oracle reads host columns only");
    for (uint32_t c = 0; c < td->n_columns; ++c)
        if (!valid_type(td->columns[c].type)) return fail(TGPU_ERR_UNSUPPORTED_TYPE, "column type");
    Table t{td->columns, td->n_columns, td->n_rows, td->row_group_rows ? td->row_group_rows : 65536u};
    std::unique_ptr<Result> r(new Result());
    int st = run(t, req, threads, *r);
    if (st != TGPU_OK) return st;
    *out = r.release();
    return TGPU_OK;
}

uint64_t orc_result_rows(const void *r) { return ((const Result *)r)->rows; }
uint32_t orc_result_cols(const void *r) { return (uint32_t)((const Result *)r)->schema.size(); }
uint64_t orc_result_groups(const void *r) { return ((const Result *)r)->groups; }
uint64_t orc_result_selected(const void *r) { return ((const Result *)r)->selected; }
const void *orc_result_data(const void *r, uint32_t c) { return ((const Result *)r)->data[c].data(); }
const uint8_t *orc_result_valid(const void *r, uint32_t c) { return ((const Result *)r)->valid[c].data(); }
int orc_result_schema(const void *r, uint32_t c, tgpu_output_column *o) {
    const Result *res = (const Result *)r;
    if (c >= res->schema.size()) return TGPU_ERR_INVALID_ARGUMENT;
    *o = res->schema[c];
    return TGPU_OK;
}
void orc_result_free(void *r) { delete (Result *)r; }
const char *orc_last_error(void) { return g_err.c_str(); }

double orc_i128_to_f64(uint64_t lo, int64_t hi) {
    i128 v = (i128)(((u128)(uint64_t)hi << 64) | lo);
    return (double)v;
}
double orc_avg_decimal(uint64_t lo, int64_t hi, uint64_t count, int32_t scale) {
    i128 v = (i128)(((u128)(uint64_t)hi << 64) | lo);
    return (double)v / (double)count / POW10[scale];
}

}  // extern "C"
