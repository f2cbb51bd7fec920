// scan.cu — the fused scan + GROUP BY fold kernel.
//
// One persistent kernel does thinDB's whole per-row hot loop
// (silo_group_core.zig: runGridScanBurst :10705 -> appendBatchRawChunks :5364
// -> stageBucketIds :9228 / scatterStageLane :9348 -> groupChunkRowsDirectKeys
// :7456 -> foldKernel* :7832-8001 -> foldGroupDistinct :8003-8176):
//
//   1. CTAs claim tiles of q.tile_rows rows (inside the row groups that
//      survived the zone maps); each warp owns q.warp_rows consecutive rows.
//   2. The fused WHERE is evaluated 32 rows per warp step with coalesced loads;
//      a warp ballot gives the survivors, which are compacted into a per-warp
//      shared-memory ring (prefix = popc of the ballot below the lane).
//   3. Full batches of 32 survivors gather their key parts and aggregate
//      inputs (only survivor rows are read: late materialisation), pack the
//      key LSB-first exactly as thinDB (v2_shape_group_topn.zig:2076-2092).
//   4. __match_any_sync finds equal keys in the warp; their inputs are
//      pre-combined into the lowest lane with shuffles (i128 sums exact).
//   5. Leaders fold into a shared-memory table (key -> global slot + states,
//      shared atomics).  Misses (table full) and every flush go to the global
//      open-addressing table (atomicCAS claim, linear probing), whose slot
//      index is the group id used by COUNT(DISTINCT)'s (gid, value) set.
//
// No spin-waits: every probe loop is bounded by MAX_PROBE and reports
// ST_TABLE_FULL / ST_DISTINCT_FULL through the status word instead.
#include "common.cuh"

namespace tgpu {

namespace {

constexpr unsigned FULL = 0xFFFFFFFFu;
constexpr uint32_t NO_GID = 0xFFFFFFFFu;
constexpr int WBUF = 64;  // per-warp survivor ring

__device__ __forceinline__ bool col_valid(const DevCol &c, uint64_t r) {
    return c.valid == nullptr || ((__ldg(c.valid + (r >> 5)) >> (r & 31)) & 1u);
}

// Sign-extended integer value (BOOLEAN zero-extended).
__device__ __forceinline__ int64_t col_int(const DevCol &c, uint64_t r) {
    switch (c.bytes) {
        case 1:
            return c.type == TGPU_BOOLEAN ? (int64_t)__ldg((const uint8_t *)c.data + r)
                                          : (int64_t)(int8_t)__ldg((const int8_t *)c.data + r);
        case 2: return (int64_t)__ldg((const int16_t *)c.data + r);
        case 4: return (int64_t)__ldg((const int32_t *)c.data + r);
        default: return (int64_t)__ldg((const long long *)c.data + r);
    }
}

__device__ __forceinline__ double col_f64(const DevCol &c, uint64_t r) {
    if (c.bytes == 4) return (double)__ldg((const float *)c.data + r);
    return __ldg((const double *)c.data + r);
}

// Streaming (evict-first) loads for the predicate columns: read once.
__device__ __forceinline__ int64_t col_int_stream(const DevCol &c, uint64_t r) {
    switch (c.bytes) {
        case 1:
            return c.type == TGPU_BOOLEAN ? (int64_t)__ldcs((const unsigned char *)c.data + r)
                                          : (int64_t)(signed char)__ldcs((const signed char *)c.data + r);
        case 2: return (int64_t)__ldcs((const short *)c.data + r);
        case 4: return (int64_t)__ldcs((const int *)c.data + r);
        default: return (int64_t)__ldcs((const long long *)c.data + r);
    }
}

__device__ __forceinline__ bool cmp_int(int op, int64_t x, int64_t lo, int64_t hi) {
    switch (op) {
        case TGPU_PRED_BETWEEN: return x >= lo && x <= hi;
        case TGPU_PRED_NOT_BETWEEN: return x < lo || x > hi;
        case TGPU_PRED_EQ: return x == lo;
        case TGPU_PRED_NE: return x != lo;
        case TGPU_PRED_LT: return x < lo;
        case TGPU_PRED_LE: return x <= lo;
        case TGPU_PRED_GT: return x > lo;
        default: return x >= lo;
    }
}
__device__ __forceinline__ bool cmp_f(int op, double x, double lo, double hi) {
    switch (op) {
        case TGPU_PRED_BETWEEN: return x >= lo && x <= hi;
        case TGPU_PRED_NOT_BETWEEN: return x < lo || x > hi;
        case TGPU_PRED_EQ: return x == lo;
        case TGPU_PRED_NE: return x != lo;
        case TGPU_PRED_LT: return x < lo;
        case TGPU_PRED_LE: return x <= lo;
        case TGPU_PRED_GT: return x > lo;
        default: return x >= lo;
    }
}

__device__ __forceinline__ bool row_passes(const DevQuery &q, uint64_t r) {
    for (int i = 0; i < q.n_preds; ++i) {
        const DevPred &p = q.preds[i];
        const DevCol &c = q.cols[p.col];
        bool v = col_valid(c, r);
        if (p.op == TGPU_PRED_IS_NULL) {
            if (v) return false;
            continue;
        }
        if (p.op == TGPU_PRED_IS_NOT_NULL) {
            if (!v) return false;
            continue;
        }
        if (!v) return false;
        bool ok = p.is_float ? cmp_f(p.op, col_f64(c, r), p.flo, p.fhi)
                             : cmp_int(p.op, col_int_stream(c, r), p.lo, p.hi);
        if (!ok) return false;
    }
    return true;
}

// Packed key: parts LSB-first, a nullable part's slice is payload | valid-bit
// and all-zero for NULL (v2_shape_group_topn.zig:105-119, :2076-2092).
__device__ __forceinline__ void pack_key(const DevQuery &q, uint64_t r, uint64_t &k0, uint64_t &k1) {
    k0 = 0;
    k1 = 0;
    for (int i = 0; i < q.n_parts; ++i) {
        const DevKeyPart &kp = q.parts[i];
        const DevCol &c = q.cols[kp.col];
        uint64_t slice = 0;
        if (!kp.nullable || col_valid(c, r)) {
            uint64_t raw = (uint64_t)col_int(c, r);
            if (kp.payload < 64) raw &= (1ULL << kp.payload) - 1;
            slice = raw;
            if (kp.nullable) {
                // validity bit sits right above the payload (bit 64 of a 64-bit part)
                if (kp.payload < 64) {
                    slice |= 1ULL << kp.payload;
                } else {
                    int vb = kp.offset + 64;
                    if (vb < 64) k0 |= 1ULL << vb;
                    else k1 |= 1ULL << (vb - 64);
                }
            }
        }
        int off = kp.offset;
        if (off < 64) {
            k0 |= slice << off;
            if (off > 0) k1 |= slice >> (64 - off);
        } else {
            k1 |= slice << (off - 64);
        }
    }
}

__device__ __forceinline__ uint64_t shfl64(uint64_t v, int src) {
    return (uint64_t)__shfl_sync(FULL, (long long)v, src);
}

// ---------------------------------------------------------------- tables --

// Slot of `key` in the global table, inserting it if absent.  Slot `cap`
// holds the all-zero key (zero is the empty marker).
__device__ uint64_t global_slot(const DevQuery &q, uint64_t k0, uint64_t k1) {
    const uint64_t mask = q.cap - 1;
    if (k0 == 0 && k1 == 0) {
        uint32_t w = (uint32_t)(q.cap >> 5), b = 1u << (q.cap & 31);
        if (!(*((volatile uint32_t *)q.occ + w) & b)) atomicOr(q.occ + w, b);
        return q.cap;
    }
    uint64_t h = hash_key(k0, k1) & mask;
    if (q.key_words == 1) {
        for (unsigned p = 0; p < MAX_PROBE; ++p) {
            unsigned long long *sp = q.table + h * (uint64_t)q.slot_words;
            unsigned long long cur = ld_relaxed(sp);
            if (cur == k0) return h;
            if (cur == 0) {
                cur = atomicCAS(sp, 0ULL, (unsigned long long)k0);
                if (cur == 0) {
                    atomicOr(q.occ + (h >> 5), 1u << (h & 31));
                    return h;
                }
                if (cur == k0) return h;
            }
            h = (h + 1) & mask;
        }
    } else {
        const ulonglong2 want = make_ulonglong2(k0, k1);
        for (unsigned p = 0; p < MAX_PROBE; ++p) {
            unsigned long long *sp = q.table + h * (uint64_t)q.slot_words;
            // The CAS itself is the read: a plain 16-byte load may see the
            // halves of two different writes.
            ulonglong2 cur = cas128(sp, make_ulonglong2(0, 0), want);
            if (cur.x == 0 && cur.y == 0) {
                atomicOr(q.occ + (h >> 5), 1u << (h & 31));
                return h;
            }
            if (cur.x == k0 && cur.y == k1) return h;
            h = (h + 1) & mask;
        }
    }
    atomicOr(q.status, ST_TABLE_FULL);
    return NO_GID;
}

// Insert (gid, value bits) into a distinct set; true when the pair is new.
// Entries are {value, gid | epoch << 32}; an entry from an older epoch is free.
__device__ bool distinct_insert(const DevQuery &q, int d, uint32_t gid, uint64_t bits) {
    unsigned long long *set = q.dset[d];
    const uint64_t mask = q.dset_cap[d] - 1;
    const uint64_t tag = (uint64_t)gid | ((uint64_t)q.epoch << 32);
    uint64_t h = mix64(bits ^ mix64((uint64_t)gid)) & mask;
    for (unsigned p = 0; p < MAX_PROBE; ++p) {
        unsigned long long *sp = set + 2 * h;
        ulonglong2 cur = ld128(sp);  // a hint; every decision below is confirmed atomically
        bool next = false;
        for (int tries = 0; tries < 16 && !next; ++tries) {
            if ((uint32_t)(cur.y >> 32) == q.epoch) {
                ulonglong2 a = cas128(sp, cur, cur);
                if (a.x != cur.x || a.y != cur.y) {
                    cur = a;
                    continue;
                }
                if (cur.x == bits && cur.y == tag) return false;
                next = true;
            } else {
                ulonglong2 a = cas128(sp, cur, make_ulonglong2(bits, tag));
                if (a.x == cur.x && a.y == cur.y) return true;
                cur = a;
            }
        }
        h = (h + 1) & mask;
    }
    atomicOr(q.status, ST_DISTINCT_FULL);
    return false;
}

// ------------------------------------------------------- fold of states --

template <int NA>
struct Acc {
    uint64_t lo[NA];   // i64 sum / i128 lo / f64 bits / encoded extreme
    uint64_t hi[NA];   // i128 hi
    uint32_t vc[NA];   // valid inputs folded
    uint32_t rows;     // rows folded (COUNT(*))
};

// Apply a combined contribution to a slot's state words (shared or global:
// the atomics resolve to the address space of `st`).
template <int NA>
__device__ __forceinline__ void apply_states(const DevQuery &q, unsigned long long *st, const Acc<NA> &acc) {
    atomicAdd(st, (unsigned long long)acc.rows);
#pragma unroll
    for (int a = 0; a < NA; ++a) {
        if (a >= q.n_aggs) break;
        const DevAgg &g = q.aggs[a];
        const uint32_t vc = acc.vc[a];
        if (vc == 0) continue;
        unsigned long long *w = st + g.word;
        switch (g.kind) {
            case AK_COUNT_VALID: atomicAdd(w, (unsigned long long)vc); break;
            case AK_SUM_I64:
                if (acc.lo[a]) atomicAdd(w, (unsigned long long)acc.lo[a]);
                break;
            case AK_SUM_I128: {
                unsigned long long lo = acc.lo[a], hi = acc.hi[a];
                if (lo) {
                    unsigned long long old = atomicAdd(w, lo);
                    hi += (old + lo < old) ? 1ULL : 0ULL;
                }
                if (hi) atomicAdd(w + 1, hi);
                break;
            }
            case AK_SUM_F64: atomicAdd((double *)w, __longlong_as_double((long long)acc.lo[a])); break;
            case AK_MIN_I: case AK_MAX_I: case AK_MIN_F: case AK_MAX_F:
                atomicMax(w, (unsigned long long)acc.lo[a]);
                break;
            default: break;
        }
        if (g.vword >= 0) atomicAdd(st + g.vword, (unsigned long long)vc);
    }
}

// One lane's own contribution, already in folded form.
template <int NA>
__device__ __forceinline__ void acc_init(const DevQuery &q, Acc<NA> &acc, const uint64_t *val, unsigned ok) {
    acc.rows = 1;
#pragma unroll
    for (int a = 0; a < NA; ++a) {
        acc.lo[a] = 0;
        acc.hi[a] = 0;
        acc.vc[a] = 0;
        if (a >= q.n_aggs || !((ok >> a) & 1u)) continue;
        const int kind = q.aggs[a].kind;
        const uint64_t v = val[a];
        acc.vc[a] = 1;
        switch (kind) {
            case AK_SUM_I64: acc.lo[a] = v; break;
            case AK_SUM_I128: acc.lo[a] = v; acc.hi[a] = ((int64_t)v < 0) ? ~0ULL : 0ULL; break;
            case AK_SUM_F64: acc.lo[a] = v; break;
            case AK_MAX_I: acc.lo[a] = enc_i64((int64_t)v); break;
            case AK_MIN_I: acc.lo[a] = ~enc_i64((int64_t)v); break;
            case AK_MAX_F: acc.lo[a] = enc_f64_bits(v); break;
            case AK_MIN_F: acc.lo[a] = ~enc_f64_bits(v); break;
            default: break;
        }
    }
}

template <int NA>
__device__ __forceinline__ void acc_add(const DevQuery &q, Acc<NA> &acc, const uint64_t *x, unsigned ok) {
    acc.rows += 1;
#pragma unroll
    for (int a = 0; a < NA; ++a) {
        if (a >= q.n_aggs || !((ok >> a) & 1u)) continue;
        const int kind = q.aggs[a].kind;
        const uint64_t v = x[a];
        acc.vc[a] += 1;
        switch (kind) {
            case AK_SUM_I64: acc.lo[a] += v; break;
            case AK_SUM_I128: {
                uint64_t lo = acc.lo[a] + v;
                acc.hi[a] += (((int64_t)v < 0) ? ~0ULL : 0ULL) + (lo < acc.lo[a] ? 1ULL : 0ULL);
                acc.lo[a] = lo;
                break;
            }
            case AK_SUM_F64:
                acc.lo[a] = f64_bits(bits_f64(acc.lo[a]) + bits_f64(v));
                break;
            case AK_MAX_I: acc.lo[a] = max(acc.lo[a], (uint64_t)enc_i64((int64_t)v)); break;
            case AK_MIN_I: acc.lo[a] = max(acc.lo[a], ~enc_i64((int64_t)v)); break;
            case AK_MAX_F: acc.lo[a] = max(acc.lo[a], enc_f64_bits(v)); break;
            case AK_MIN_F: acc.lo[a] = max(acc.lo[a], ~enc_f64_bits(v)); break;
            default: break;
        }
    }
}

// ------------------------------------------------------ shared memory --

struct ScanSmem {
    unsigned long long *ckeys;   // cache_slots
    unsigned long long *cstate;  // cache_slots * state_words
    uint32_t *cgid;              // cache_slots
    uint32_t *wbuf;              // SCAN_WARPS * WBUF row offsets
    uint32_t *live;              // live cache entries
    uint32_t *tile;              // claimed tile
    uint32_t *flags;             // [0] flush now, [1] stop
};

__device__ __forceinline__ ScanSmem carve(const DevQuery &q, unsigned char *base) {
    ScanSmem s;
    const int C = q.cache_slots;
    s.ckeys = (unsigned long long *)base;
    s.cstate = s.ckeys + C;
    s.cgid = (uint32_t *)(s.cstate + (size_t)C * q.state_words);
    s.wbuf = s.cgid + C;
    s.live = s.wbuf + SCAN_WARPS * WBUF;
    s.tile = s.live + 1;
    s.flags = s.tile + 1;
    return s;
}

// Find or claim the cache entry of a non-zero one-word key; -1 when the
// bounded probe finds neither (the caller folds into the global table).
__device__ __forceinline__ int cache_find(const DevQuery &q, ScanSmem &sm, uint64_t k, bool &claimed) {
    const int C = q.cache_slots;
    const int limit = q.cache_flush_at >= C ? C : 16;  // a resident (lowcard) cache probes all
    uint32_t h = (uint32_t)hash_key(k, 0) & (C - 1);
    claimed = false;
    for (int p = 0; p < limit; ++p) {
        unsigned long long cur = sm.ckeys[h];
        if (cur == k) return (int)h;
        if (cur == 0) {
            cur = atomicCAS(&sm.ckeys[h], 0ULL, (unsigned long long)k);
            if (cur == 0) {
                claimed = true;
                atomicAdd(sm.live, 1u);
                return (int)h;
            }
            if (cur == k) return (int)h;
        }
        h = (h + 1) & (C - 1);
    }
    return -1;
}

// Fold every live cache entry into its global slot and clear the cache.
__device__ void cache_flush(const DevQuery &q, ScanSmem &sm) {
    const int C = q.cache_slots, S = q.state_words;
    for (int e = threadIdx.x; e < C; e += blockDim.x) {
        unsigned long long k = sm.ckeys[e];
        if (k == 0) continue;
        uint32_t gid = sm.cgid[e];
        unsigned long long *st = sm.cstate + (size_t)e * S;
        if (gid != NO_GID) {
            unsigned long long *gst = q.table + (uint64_t)gid * q.slot_words + q.key_words;
            atomicAdd(gst, st[0]);
            for (int a = 0; a < q.n_aggs; ++a) {
                const DevAgg &g = q.aggs[a];
                unsigned long long *w = gst + g.word;
                switch (g.kind) {
                    case AK_COUNT_VALID: case AK_SUM_I64:
                        if (st[g.word]) atomicAdd(w, st[g.word]);
                        break;
                    case AK_SUM_I128: {
                        unsigned long long lo = st[g.word], hi = st[g.word + 1];
                        if (lo) {
                            unsigned long long old = atomicAdd(w, lo);
                            hi += (old + lo < old) ? 1ULL : 0ULL;
                        }
                        if (hi) atomicAdd(w + 1, hi);
                        break;
                    }
                    case AK_SUM_F64: {
                        double v = __longlong_as_double((long long)st[g.word]);
                        if (v != 0.0 || (st[g.word] >> 63)) atomicAdd((double *)w, v);
                        break;
                    }
                    case AK_MIN_I: case AK_MAX_I: case AK_MIN_F: case AK_MAX_F:
                        if (st[g.word]) atomicMax(w, st[g.word]);
                        break;
                    default: break;  // distinct counts live only in the global slot
                }
                if (g.vword >= 0 && st[g.vword]) atomicAdd(gst + g.vword, st[g.vword]);
            }
        }
        sm.ckeys[e] = 0;
        sm.cgid[e] = NO_GID;
        for (int w = 0; w < S; ++w) st[w] = 0;
    }
}

// ------------------------------------------------------------- a batch --

// Fold up to 32 rows (lane i holds `row` when bit i of `active` is set).
template <int NA>
__device__ __forceinline__ void process_batch(const DevQuery &q, ScanSmem &sm, uint64_t row, unsigned active,
                                              int lane) {
    const bool me = (active >> lane) & 1u;
    uint64_t k0 = 0, k1 = 0;
    uint64_t val[NA];
    unsigned ok = 0;
#pragma unroll
    for (int a = 0; a < NA; ++a) val[a] = 0;
    if (me) {
        pack_key(q, row, k0, k1);
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            if (a >= q.n_aggs) break;
            const DevAgg &g = q.aggs[a];
            if (g.col < 0) continue;
            const DevCol &c = q.cols[g.col];
            if (!col_valid(c, row)) continue;
            ok |= 1u << a;
            if (g.kind == AK_COUNT_VALID) continue;
            if (g.is_float_in) val[a] = f64_bits(col_f64(c, row));
            else val[a] = (uint64_t)col_int(c, row);
            if (g.kind == AK_MIN_F || g.kind == AK_MAX_F) {
                double d = bits_f64(val[a]);
                if (d != d) val[a] = 0x7FF8000000000000ULL;  // one NaN, ordered largest
            }
        }
    }

    // Equal keys in the warp: the lowest lane of each group folds for all.
    unsigned grp;
    if (q.warp_combine) {
        grp = __match_any_sync(FULL, k0);
        if (q.key_words == 2) grp &= __match_any_sync(FULL, k1);
        grp &= active;
    } else {
        grp = 1u << lane;
    }
    const int leader_lane = me ? __ffs(grp) - 1 : lane;
    const bool leader = me && leader_lane == lane;

    Acc<NA> acc;
    acc_init<NA>(q, acc, val, ok);
    if (q.warp_combine) {
        unsigned rem = leader ? (grp & ~(1u << lane)) : 0u;
        while (__any_sync(FULL, rem != 0)) {
            const int src = rem ? __ffs(rem) - 1 : lane;
            const unsigned ob = __shfl_sync(FULL, ok, src);
            uint64_t x[NA];
#pragma unroll
            for (int a = 0; a < NA; ++a) x[a] = (a < q.n_aggs) ? shfl64(val[a], src) : 0;
            if (rem) {
                acc_add<NA>(q, acc, x, ob);
                rem &= rem - 1;
            }
        }
    }

    uint32_t gid = NO_GID;
    if (leader) {
        bool done = false;
        if (q.cache_slots && q.key_words == 1 && k0 != 0) {
            bool claimed;
            int e = cache_find(q, sm, k0, claimed);
            if (e >= 0) {
                if (claimed) {
                    gid = (uint32_t)global_slot(q, k0, 0);
                    sm.cgid[e] = gid;
                } else if (q.needs_gid) {
                    gid = *((volatile uint32_t *)sm.cgid + e);
                    if (gid == NO_GID) gid = (uint32_t)global_slot(q, k0, 0);
                }
                apply_states<NA>(q, sm.cstate + (size_t)e * q.state_words, acc);
                done = true;
            }
        }
        if (!done) {
            gid = (uint32_t)global_slot(q, k0, k1);
            if (gid != NO_GID) apply_states<NA>(q, q.table + (uint64_t)gid * q.slot_words + q.key_words, acc);
        }
    }

    if (q.needs_gid) {
        gid = __shfl_sync(FULL, gid, leader_lane);
        if (me && gid != NO_GID) {
            unsigned long long *gst = q.table + (uint64_t)gid * q.slot_words + q.key_words;
#pragma unroll
            for (int a = 0; a < NA; ++a) {
                if (a >= q.n_aggs) break;
                const DevAgg &g = q.aggs[a];
                if (g.kind != AK_DISTINCT || !((ok >> a) & 1u)) continue;
                uint64_t bits = g.is_float_in ? canon_f64_bits(bits_f64(val[a])) : val[a];
                if (distinct_insert(q, g.dset, gid, bits)) atomicAdd(gst + g.word, 1ULL);
            }
        }
    }
}

// ---------------------------------------------------------------- kernel --

__device__ __forceinline__ void cache_init(const DevQuery &q, ScanSmem &sm) {
    for (int e = threadIdx.x; e < q.cache_slots; e += blockDim.x) {
        sm.ckeys[e] = 0;
        sm.cgid[e] = NO_GID;
    }
    for (int e = threadIdx.x; e < q.cache_slots * q.state_words; e += blockDim.x) sm.cstate[e] = 0;
}

// Rows [row0, row_end) of scan tile t.
__device__ __forceinline__ void tile_rows(const DevQuery &q, uint32_t t, uint64_t &row0, uint64_t &row_end) {
    if (q.rg_list) {
        uint32_t rgi = t / q.tiles_per_rg, sub = t % q.tiles_per_rg;
        uint64_t rg = q.rg_list[rgi];
        row0 = rg * q.rg_rows + (uint64_t)sub * q.tile_rows;
        row_end = min(min(row0 + q.tile_rows, (rg + 1) * (uint64_t)q.rg_rows), q.n_rows);
    } else {
        row0 = (uint64_t)t * q.tile_rows;
        row_end = min(row0 + q.tile_rows, q.n_rows);
    }
}

// One warp's share of scan tile t: filter, compact, fold.
template <int NA>
__device__ __forceinline__ void scan_tile(const DevQuery &q, ScanSmem &sm, uint32_t t, unsigned long long &selected) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t *wb = sm.wbuf + warp * WBUF;
    uint64_t row0, row_end;
    tile_rows(q, t, row0, row_end);
    const uint64_t wbase = row0 + (uint64_t)warp * q.warp_rows;
    const uint64_t wend = min(wbase + q.warp_rows, row_end);
    if (wbase >= wend) return;
    if (q.n_preds == 0) {
        for (uint64_t b = wbase; b < wend; b += 32) {
            uint64_t r = b + lane;
            unsigned act = __ballot_sync(FULL, r < wend);
            selected += (lane == 0) ? __popc(act) : 0;
            process_batch<NA>(q, sm, r, act, lane);
        }
    } else if (!q.gather) {
        for (uint64_t b = wbase; b < wend; b += 32) {
            uint64_t r = b + lane;
            bool pass = r < wend && row_passes(q, r);
            unsigned act = __ballot_sync(FULL, pass);
            selected += (lane == 0) ? __popc(act) : 0;
            if (act) process_batch<NA>(q, sm, r, act, lane);
        }
    } else {
        int n = 0;  // survivors in this warp's ring
        for (uint64_t b = wbase; b < wend; b += 128) {
            bool pass[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                uint64_t r = b + u * 32 + lane;
                pass[u] = r < wend && row_passes(q, r);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                unsigned m = __ballot_sync(FULL, pass[u]);
                if (pass[u]) wb[n + __popc(m & ((1u << lane) - 1))] = (uint32_t)(b + u * 32 + lane - row0);
                n += __popc(m);
                selected += (lane == 0) ? __popc(m) : 0;
                __syncwarp();
                if (n >= 32) {
                    uint64_t r = row0 + wb[lane];
                    __syncwarp();
                    if (lane < n - 32) wb[lane] = wb[32 + lane];
                    n -= 32;
                    __syncwarp();
                    process_batch<NA>(q, sm, r, FULL, lane);
                }
            }
        }
        if (n > 0) {
            uint64_t r = row0 + wb[lane < n ? lane : 0];
            unsigned act = (n >= 32) ? FULL : ((1u << n) - 1);
            __syncwarp();
            process_batch<NA>(q, sm, r, act, lane);
        }
    }
}

template <int NA>
__global__ void __launch_bounds__(SCAN_THREADS, NA <= 4 ? 2 : 1) scan_group_kernel(const __grid_constant__ DevQuery q) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ScanSmem sm = carve(q, smem_raw);
    const int lane = threadIdx.x & 31;
    cache_init(q, sm);
    if (threadIdx.x == 0) {
        *sm.live = 0;
        sm.flags[0] = 0;
        sm.flags[1] = 0;
    }
    unsigned long long selected = 0;
    __syncthreads();

    for (;;) {
        if (threadIdx.x == 0) {
            uint32_t t = atomicAdd(q.tile_counter, 1u);
            *sm.tile = t;
            sm.flags[0] = (q.cache_slots && *sm.live >= (uint32_t)q.cache_flush_at) ? 1u : 0u;
            if (q.cancel && *q.cancel) {
                atomicOr(q.status, ST_CANCELLED);
                *sm.tile = 0xFFFFFFFFu;
            }
        }
        __syncthreads();
        const uint32_t t = *sm.tile;
        if (sm.flags[0]) {
            cache_flush(q, sm);
            if (threadIdx.x == 0) *sm.live = 0;
            __syncthreads();
        }
        if (t >= q.n_tiles) break;
        scan_tile<NA>(q, sm, t, selected);
        __syncthreads();
    }
    if (q.cache_slots) {
        __syncthreads();
        cache_flush(q, sm);
    }
    if (lane == 0 && selected) atomicAdd(q.selected_rows, selected);
}

// Many queries in one persistent kernel: work items are (query, tile) pairs,
// query-major (item i belongs to the query whose [tile_start[q],
// tile_start[q+1]) range holds it).  A CTA keeps one query's shared-memory
// table at a time and flushes it when its next item belongs to another query.
template <int NA>
__global__ void __launch_bounds__(SCAN_THREADS, NA <= 4 ? 2 : 1)
    batch_scan_kernel(const DevQuery *__restrict__ qs, const uint32_t *__restrict__ tile_start, uint32_t n_queries,
                      unsigned int *work_counter, const volatile int *cancel, unsigned int *batch_status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint32_t s_item, s_query;
    const int lane = threadIdx.x & 31;
    const uint32_t total = tile_start[n_queries];
    int cur = -1;
    ScanSmem sm{};
    unsigned long long selected = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            uint32_t item = atomicAdd(work_counter, 1u);
            if (cancel && *cancel) {
                atomicOr(batch_status, ST_CANCELLED);
                item = 0xFFFFFFFFu;
            }
            uint32_t qi = 0;
            if (item < total) {
                uint32_t lo = 0, hi = n_queries;  // last q with tile_start[q] <= item
                while (hi - lo > 1) {
                    uint32_t mid = (lo + hi) >> 1;
                    if (tile_start[mid] <= item) lo = mid;
                    else hi = mid;
                }
                qi = lo;
            }
            s_item = item;
            s_query = qi;
        }
        __syncthreads();
        const uint32_t item = s_item;
        const int qn = item < total ? (int)s_query : -1;
        if (qn != cur && cur >= 0) {
            const DevQuery &old = qs[cur];
            if (old.cache_slots) cache_flush(old, sm);
            if (lane == 0 && selected) atomicAdd(old.selected_rows, selected);
            selected = 0;
            __syncthreads();
        }
        if (qn < 0) break;
        const DevQuery &q = qs[qn];
        if (qn != cur) {
            sm = carve(q, smem_raw);
            cache_init(q, sm);
            if (threadIdx.x == 0) *sm.live = 0;
            cur = qn;
            __syncthreads();
        } else if (q.cache_slots && *sm.live >= (uint32_t)q.cache_flush_at) {
            __syncthreads();
            cache_flush(q, sm);
            if (threadIdx.x == 0) *sm.live = 0;
            __syncthreads();
        }
        scan_tile<NA>(q, sm, item - tile_start[qn], selected);
        __syncthreads();
    }
}

}  // namespace

size_t scan_smem_bytes(const DevQuery &q) {
    return (size_t)q.cache_slots * (8 + 8 * (size_t)q.state_words + 4) + SCAN_WARPS * WBUF * 4 + 16;
}

template <typename K>
static int blocks_per_sm(K kernel, size_t smem) {
    int per_sm = 1;
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, SCAN_THREADS, smem);
    if (e != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    return per_sm;
}

int scan_grid_size(const DevQuery &q, int sms) {
    // persistent grid: every CTA that fits on an SM at once
    size_t smem = scan_smem_bytes(q);
    return sms * (q.n_aggs <= 4 ? blocks_per_sm(scan_group_kernel<4>, smem) : blocks_per_sm(scan_group_kernel<16>, smem));
}

cudaError_t launch_scan(const DevQuery &q, int grid, cudaStream_t s) {
    size_t smem = scan_smem_bytes(q);
    if (q.n_aggs <= 4) {
        cudaError_t e = cudaFuncSetAttribute(scan_group_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        scan_group_kernel<4><<<grid, SCAN_THREADS, smem, s>>>(q);
    } else {
        cudaError_t e = cudaFuncSetAttribute(scan_group_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        scan_group_kernel<16><<<grid, SCAN_THREADS, smem, s>>>(q);
    }
    return cudaGetLastError();
}

int batch_scan_grid(int max_aggs, size_t smem, int sms) {
    return sms * (max_aggs <= 4 ? blocks_per_sm(batch_scan_kernel<4>, smem) : blocks_per_sm(batch_scan_kernel<16>, smem));
}

cudaError_t launch_batch_scan(const DevQuery *qs, const uint32_t *tile_start, uint32_t n_queries, int max_aggs,
                              size_t smem, int grid, unsigned int *work_counter, const volatile int *cancel,
                              unsigned int *status, cudaStream_t s) {
    if (max_aggs <= 4) {
        cudaError_t e = cudaFuncSetAttribute(batch_scan_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        batch_scan_kernel<4><<<grid, SCAN_THREADS, smem, s>>>(qs, tile_start, n_queries, work_counter, cancel, status);
    } else {
        cudaError_t e = cudaFuncSetAttribute(batch_scan_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        batch_scan_kernel<16><<<grid, SCAN_THREADS, smem, s>>>(qs, tile_start, n_queries, work_counter, cancel, status);
    }
    return cudaGetLastError();
}

}  // namespace tgpu
