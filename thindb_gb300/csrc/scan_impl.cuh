// scan_impl.cuh — device code of the fused scan + GROUP BY fold (shared by the
// single-query kernels in scan.cu and the batched kernel in scan_batch.cu).
//
// One persistent kernel does thinDB's whole per-row hot loop
// (silo_group_core.zig: runGridScanBurst :10705 -> appendBatchRawChunks :5364
// -> stageBucketIds :9228 / scatterStageLane :9348 -> groupChunkRowsDirectKeys
// :7456 -> foldKernel* :7832-8001 -> foldGroupDistinct :8003-8176):
//
//   1. Every warp owns a static, strided set of chunks of q.chunk_rows rows
//      (inside the row groups that survived the zone maps): no tile claims and
//      no block barriers in the main loop.
//   2. The fused WHERE is evaluated 32 rows per step with coalesced streaming
//      loads, sixteen steps in flight; a warp ballot gives the survivors, whose
//      chunk offsets are compacted into the warp's shared-memory list
//      (position = popc of the ballot below the lane).
//   3. Survivors are folded 32 at a time: their key parts and aggregate inputs
//      are gathered (only surviving rows are read: late materialisation; the
//      next batch's gathers are issued before the current batch folds), and the
//      key is packed LSB-first exactly as thinDB (v2_shape_group_topn.zig:2076-2092).
//   4. __match_any_sync finds equal keys in the warp; their inputs are
//      pre-combined into the lowest lane with shuffles (i128 sums exact).
//   5. Leaders fold into the CTA's shared-memory table (key -> global slot +
//      states, shared atomics; insert-if-free, so the hottest keys, which
//      arrive first, stay resident).  Misses fold into the global
//      open-addressing table (atomicCAS claim, linear probing), whose slot
//      index is the group id COUNT(DISTINCT)'s (gid, value) set keys on.  The
//      shared table is flushed into the global one once, when the CTA ends.
//
// No spin-waits: every probe loop is bounded by MAX_PROBE and reports
// ST_TABLE_FULL / ST_DISTINCT_FULL through the status word instead.
#pragma once

#include "common.cuh"

namespace tgpu {

namespace {

constexpr unsigned FULL = 0xFFFFFFFFu;
constexpr uint32_t NO_GID = 0xFFFFFFFFu;

// Pick<c, A, B>::type is A when c holds, else B.
template <bool C, typename A, typename B>
struct Pick {
    using type = A;
};
template <typename A, typename B>
struct Pick<false, A, B> {
    using type = B;
};
constexpr int FILTER_UNROLL = 16;  // 32-row filter steps in flight per warp

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

// Predicate-column loads: streaming (evict-first) when the rows are read
// once, default caching when other queries of a batch read them next.
template <typename T>
__device__ __forceinline__ T ld_pred(bool shared, const T *p) {
    return shared ? __ldg(p) : __ldcs(p);
}

__device__ __forceinline__ int64_t col_int_stream(const DevCol &c, uint64_t r, bool shared) {
    switch (c.bytes) {
        case 1:
            return c.type == TGPU_BOOLEAN ? (int64_t)ld_pred(shared, (const unsigned char *)c.data + r)
                                          : (int64_t)ld_pred(shared, (const signed char *)c.data + r);
        case 2: return (int64_t)ld_pred(shared, (const short *)c.data + r);
        case 4: return (int64_t)ld_pred(shared, (const int *)c.data + r);
        default: return (int64_t)ld_pred(shared, (const long long *)c.data + r);
    }
}

__device__ __forceinline__ double col_f64_stream(const DevCol &c, uint64_t r, bool shared) {
    if (c.bytes == 4) return (double)ld_pred(shared, (const float *)c.data + r);
    return ld_pred(shared, (const double *)c.data + r);
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

__device__ __forceinline__ bool pred_holds(const DevQuery &q, const DevPred &p, uint64_t r) {
    const DevCol &c = q.cols[p.col];
    bool v = col_valid(c, r);
    if (p.op == TGPU_PRED_IS_NULL) return !v;
    if (p.op == TGPU_PRED_IS_NOT_NULL) return v;
    if (!v) return false;
    return p.is_float ? cmp_f(p.op, col_f64(c, r), p.flo, p.fhi) : cmp_int(p.op, col_int_stream(c, r, q.shared_scan != 0), p.lo, p.hi);
}

// A hashed key's digest over row r's parts (a string's str_hash, an
// integer's value bits, a NULL marker), chained from HASHED_SEED.
__device__ uint64_t hashed_digest(const DevQuery &q, uint64_t r) {
    uint64_t d = HASHED_SEED;
    for (int i = 0; i < q.n_parts; ++i) {
        const DevCol &c = q.cols[q.parts[i].col];
        if (!col_valid(c, r)) {
            d = digest_step(d, HASHED_NULL);
            continue;
        }
        if (c.offs) {
            const uint32_t b = c.offs[r], e = c.offs[r + 1];
            d = digest_step(d, str_hash((const uint8_t *)c.data + b, e - b));
        } else {
            d = digest_step(d, int_part_hash(col_int(c, r)));
        }
    }
    return q.digest_bits ? d & ((1ULL << q.digest_bits) - 1) : d;
}

// Whether rows a and b hold the same key (every part: NULL alike, equal
// integers, strings of equal bytes) — the exact check behind a digest match
// (ExactKey, silo_group_core.zig:6337).
__device__ bool keys_equal(const DevQuery &q, uint64_t a, uint64_t b) {
    for (int i = 0; i < q.n_parts; ++i) {
        const DevCol &c = q.cols[q.parts[i].col];
        const bool va = col_valid(c, a), vb = col_valid(c, b);
        if (va != vb) return false;
        if (!va) continue;
        if (c.offs) {
            const uint32_t ab = c.offs[a], ae = c.offs[a + 1], bb = c.offs[b], be = c.offs[b + 1];
            if (ae - ab != be - bb) return false;
            const uint8_t *pa = (const uint8_t *)c.data + ab, *pb = (const uint8_t *)c.data + bb;
            for (uint32_t j = 0; j < ae - ab; ++j)
                if (pa[j] != pb[j]) return false;
        } else if (col_int(c, a) != col_int(c, b)) {
            return false;
        }
    }
    return true;
}

// Packed key: parts LSB-first, a nullable part's slice is payload | valid-bit
// and all-zero for NULL (v2_shape_group_topn.zig:105-119, :2076-2092).  A
// hashed key: word 1 the digest, word 0 the row + 1 (the group's
// representative row once it claims a slot).
__device__ __forceinline__ void pack_key(const DevQuery &q, uint64_t r, uint64_t &k0, uint64_t &k1) {
    if (q.hashed) {
        k1 = hashed_digest(q, r);
        k0 = r + 1;
        return;
    }
    k0 = q.key_or;
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
// (hk = hash_key(k0, k1), computed once by the caller)
__device__ uint64_t global_slot(const DevQuery &q, uint64_t k0, uint64_t k1, uint64_t hk) {
    const uint64_t mask = q.cap - 1;
    if (k0 == 0 && k1 == 0) {
        uint32_t w = (uint32_t)(q.cap >> 5), b = 1u << (q.cap & 31);
        if (!(*((volatile uint32_t *)q.occ + w) & b)) atomicOr(q.occ + w, b);
        return q.cap;
    }
    uint64_t h = hk & mask;
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

__device__ __forceinline__ uint64_t global_slot(const DevQuery &q, uint64_t k0, uint64_t k1) {
    return global_slot(q, k0, k1, hash_key(k0, k1));
}

// The slot of a one-word key when `home`, the key its home slot held at some
// earlier moment of this query, is the key itself (a claimed slot keeps its
// key), with no load; otherwise the probe.  home = 0 (no such load) always
// probes.
__device__ __forceinline__ uint64_t global_slot_from(const DevQuery &q, uint64_t k0, uint64_t k1, uint64_t hk,
                                                     uint64_t home) {
    if (q.key_words == 1 && k0 != 0 && home == k0) return hk & (q.cap - 1);
    return global_slot(q, k0, k1, hk);
}

// A hashed key's slot: probe by the digest (word 1); a slot holding the same
// digest is the group only if its representative row (word 0 - 1) holds the
// same key; claiming writes (row + 1, digest) in one 16-byte CAS.
__device__ uint64_t global_slot_hashed(const DevQuery &q, uint64_t row, uint64_t digest) {
    const uint64_t mask = q.cap - 1;
    uint64_t h = mix64(digest) & mask;
    const ulonglong2 mine = make_ulonglong2(row + 1, digest);
    for (unsigned p = 0; p < MAX_PROBE; ++p) {
        unsigned long long *sp = q.table + h * (uint64_t)q.slot_words;
        const ulonglong2 cur = cas128(sp, make_ulonglong2(0, 0), mine);
        if (cur.x == 0 && cur.y == 0) {
            atomicOr(q.occ + (h >> 5), 1u << (h & 31));
            return h;
        }
        if (cur.y == digest && keys_equal(q, row, cur.x - 1)) return h;
        h = (h + 1) & mask;
    }
    atomicOr(q.status, ST_TABLE_FULL);
    return NO_GID;
}

// A hash that every row of one group shares: the packed key's, or a hashed
// key's digest (its word 0 is the row).
__device__ __forceinline__ uint64_t group_hash(const DevQuery &q, uint64_t k0, uint64_t k1) {
    return q.hashed ? mix64(k1) : hash_key(k0, k1);
}

// Insert (gid, value bits) into a distinct set; true when the pair is new.
// Entries are {value, gid | epoch << 32}; an entry from an older epoch is free.
// Home slot of (group, value) in distinct set d.  It hashes the group's
// packed key (hk = hash_key of it) rather than its gid: key and gid are one
// to one within a query, and the key is known as soon as the row is loaded,
// so the entry can be prefetched before the group probe returns the gid.
__device__ __forceinline__ uint64_t distinct_home(const DevQuery &q, int d, uint64_t hk, uint64_t bits) {
    return mix64(bits ^ hk) & (q.dset_cap[d] - 1);
}

__device__ bool distinct_insert(const DevQuery &q, int d, uint32_t gid, uint64_t bits, uint64_t hk) {
    unsigned long long *set = q.dset[d];
    const uint64_t mask = q.dset_cap[d] - 1;
    const uint64_t tag = (uint64_t)gid | ((uint64_t)q.epoch << 32);
    uint64_t h = distinct_home(q, d, hk, bits);
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

// Partition of a (group, value) pair in the partitioned COUNT(DISTINCT): top
// bits of a hash of the value and the group key's hash (hash_key), so that a
// row can reserve its pair's place before its group id is known.
__device__ __forceinline__ uint32_t dpart_of(const DevQuery &q, uint64_t hk, uint64_t bits) {
    return (uint32_t)(mix64(bits ^ hk) >> (64 - q.dpart_bits));
}

// A reserved place: partition and position (DPOS_NONE = none reserved yet).
constexpr uint32_t DPOS_NONE = 0xFFFFFFFFu;

// Store (value, gid) at the place reserved for it.  Every reserved place is
// stored, a pair whose group found no slot (gid NO_GID: the table is full and
// the host reruns) too: the partition kernel skips it.  A full partition sets
// ST_DISTINCT_FULL (the host resizes or deduplicates in the global set).
__device__ __forceinline__ void dpart_store(const DevQuery &q, uint32_t p, uint32_t pos, uint32_t gid,
                                            uint64_t bits) {
    if (p >> q.dpart_bits) atomicOr(q.status, ST_BAD_INDEX);  // not a partition: report, never write
    else if (pos < q.dpart_cap) q.dpart_buf[(uint64_t)p * q.dpart_cap + pos] = make_ulonglong2(bits, gid);
    else atomicOr(q.status, ST_DISTINCT_FULL);
}

// Reserve a place and store (value, gid) in one go.
__device__ __forceinline__ void dpart_append(const DevQuery &q, uint64_t hk, uint32_t gid, uint64_t bits) {
    const uint32_t p = dpart_of(q, hk, bits);
    dpart_store(q, p, atomicAdd(q.dpart_cursor + p, 1u), gid, bits);
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
// the atomics resolve to the address space of `st`).  Aggregates that share a
// state word (SUM and AVG of one column) fold it once (g.owner).
// Fire-and-forget updates of a group's state words.  The folds reach a
// state through a pointer that may lead into the shared-memory table or the
// global one (and arrives as a parameter of an out-of-line fold), so the
// compiler sees a generic address; for a global state it then emits an
// atomic that returns the old value, a full round trip whose destination
// register the warp waits on, where red.global returns nothing.  Shared
// states keep the generic atomics (measured faster there than red.shared).
__device__ __forceinline__ void red_add(unsigned long long *p, unsigned long long v, bool smem) {
    if (smem) atomicAdd(p, v);
    else asm volatile("red.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void red_max(unsigned long long *p, unsigned long long v, bool smem) {
    if (smem) atomicMax(p, v);
    else asm volatile("red.global.max.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void red_add_f64(unsigned long long *p, double v, bool smem) {
    if (smem) atomicAdd((double *)p, v);
    else asm volatile("red.global.add.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}

template <int NA>
__device__ __forceinline__ void apply_states(const DevQuery &q, unsigned long long *st, bool smem,
                                             const Acc<NA> &acc) {
    red_add(st, (unsigned long long)acc.rows, smem);
#pragma unroll 1
    for (int a = 0; a < NA; ++a) {
        if (a >= q.n_aggs) break;
        const DevAgg &g = q.aggs[a];
        const uint32_t vc = acc.vc[a];
        if (vc == 0 || !g.owner) continue;
        unsigned long long *w = st + g.word;
        switch (g.kind) {
            case AK_COUNT_VALID: red_add(w, (unsigned long long)vc, smem); break;
            case AK_SUM_I64:
                if (acc.lo[a]) red_add(w, (unsigned long long)acc.lo[a], smem);
                break;
            case AK_SUM_I128:
                if (acc.lo[a]) red_add(w, (unsigned long long)acc.lo[a], smem);
                if (acc.hi[a]) red_add(w + 1, (unsigned long long)acc.hi[a], smem);
                break;
            case AK_SUM_I128C: {
                unsigned long long lo = acc.lo[a], hi = acc.hi[a];
                if (lo) {
                    unsigned long long old = atomicAdd(w, lo);
                    hi += (old + lo < old) ? 1ULL : 0ULL;
                }
                if (hi) red_add(w + 1, hi, smem);
                break;
            }
            case AK_SUM_F64: red_add_f64(w, __longlong_as_double((long long)acc.lo[a]), smem); break;
            case AK_MIN_I: case AK_MAX_I: case AK_MIN_F: case AK_MAX_F:
                red_max(w, (unsigned long long)acc.lo[a], smem);
                break;
            default: break;
        }
        if (g.vword >= 0) red_add(st + g.vword, (unsigned long long)vc, smem);
    }
}

// One lane's own contribution, already in folded form.
template <int NA>
__device__ __forceinline__ void acc_init(const DevQuery &q, Acc<NA> &acc, const uint64_t *val, unsigned ok) {
    acc.rows = 1;
#pragma unroll 1
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
            case AK_SUM_I128: acc.lo[a] = split_lo((int64_t)v); acc.hi[a] = split_hi((int64_t)v); break;
            case AK_SUM_I128C: acc.lo[a] = v; acc.hi[a] = ((int64_t)v < 0) ? ~0ULL : 0ULL; break;
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
#pragma unroll 1
    for (int a = 0; a < NA; ++a) {
        if (a >= q.n_aggs || !((ok >> a) & 1u)) continue;
        const int kind = q.aggs[a].kind;
        const uint64_t v = x[a];
        acc.vc[a] += 1;
        switch (kind) {
            case AK_SUM_I64: acc.lo[a] += v; break;
            case AK_SUM_I128:
                acc.lo[a] += split_lo((int64_t)v);
                acc.hi[a] += split_hi((int64_t)v);
                break;
            case AK_SUM_I128C: {
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
    uint16_t *wlist;             // gather mode: SCAN_WARPS * chunk_rows survivor offsets;
                                 // queue mode: SCAN_WARPS rings of WQ_ROWS fold rows (16-byte aligned)
};

__device__ __forceinline__ ScanSmem carve(const DevQuery &q, unsigned char *base) {
    ScanSmem s;
    const int C = q.cache_slots;
    s.ckeys = (unsigned long long *)base;
    s.cstate = s.ckeys + C;
    s.cgid = (uint32_t *)(s.cstate + (size_t)C * q.state_words);
    s.wlist = (uint16_t *)(((uintptr_t)(s.cgid + C) + 15) & ~(uintptr_t)15);
    return s;
}

__device__ __forceinline__ void cache_init(const DevQuery &q, const ScanSmem &sm) {
    for (int e = threadIdx.x; e < q.cache_slots; e += blockDim.x) {
        sm.ckeys[e] = 0;
        sm.cgid[e] = NO_GID;
    }
    for (int e = threadIdx.x; e < q.cache_slots * q.state_words; e += blockDim.x) sm.cstate[e] = 0;
}

// Find or claim the cache entry of a non-zero one-word key; -1 when the
// bounded probe finds neither (the caller folds into the global table).
// (hk = hash_key(k, 0), computed once by the caller)
__device__ __forceinline__ int cache_find(const DevQuery &q, const ScanSmem &sm, uint64_t k, uint64_t hk,
                                          bool &claimed) {
    const int C = q.cache_slots;
    const int limit = q.cache_probe;
    uint32_t h = (uint32_t)hk & (C - 1);
    claimed = false;
    for (int p = 0; p < limit; ++p) {
        unsigned long long cur = sm.ckeys[h];
        if (cur == k) return (int)h;
        if (cur == 0) {
            cur = atomicCAS(&sm.ckeys[h], 0ULL, (unsigned long long)k);
            if (cur == 0) {
                claimed = true;
                return (int)h;
            }
            if (cur == k) return (int)h;
        }
        h = (h + 1) & (C - 1);
    }
    return -1;
}

// Fold every live cache entry into its global slot.
__device__ void cache_flush(const DevQuery &q, const ScanSmem &sm) {
    const int C = q.cache_slots, S = q.state_words;
    for (int e = threadIdx.x; e < C; e += blockDim.x) {
        unsigned long long k = sm.ckeys[e];
        if (k == 0) continue;
        uint32_t gid = sm.cgid[e];
        const unsigned long long *st = sm.cstate + (size_t)e * S;
        if (gid == NO_GID) continue;  // only when the global table overflowed (rerun follows)
        unsigned long long *gst = q.table + (uint64_t)gid * q.slot_words + q.key_words;
        atomicAdd(gst, st[0]);
        for (int a = 0; a < q.n_aggs; ++a) {
            const DevAgg &g = q.aggs[a];
            if (!g.owner) continue;
            unsigned long long *w = gst + g.word;
            switch (g.kind) {
                case AK_COUNT_VALID: case AK_SUM_I64:
                    if (st[g.word]) atomicAdd(w, st[g.word]);
                    break;
                case AK_SUM_I128:
                    if (st[g.word]) atomicAdd(w, st[g.word]);
                    if (st[g.word + 1]) atomicAdd(w + 1, st[g.word + 1]);
                    break;
                case AK_SUM_I128C: {
                    unsigned long long lo = st[g.word], hi = st[g.word + 1];
                    if (lo) {
                        unsigned long long old = atomicAdd(w, lo);
                        hi += (old + lo < old) ? 1ULL : 0ULL;
                    }
                    if (hi) atomicAdd(w + 1, hi);
                    break;
                }
                case AK_SUM_F64:
                    if (st[g.word]) atomicAdd((double *)w, __longlong_as_double((long long)st[g.word]));
                    break;
                case AK_MIN_I: case AK_MAX_I: case AK_MIN_F: case AK_MAX_F:
                    if (st[g.word]) atomicMax(w, st[g.word]);
                    break;
                default: break;  // distinct counts live only in the global slot
            }
            if (g.vword >= 0 && st[g.vword]) atomicAdd(gst + g.vword, st[g.vword]);
        }
    }
}

// ------------------------------------------------------------ a batch --

// The gathered inputs of one row (one lane).
template <int NA>
struct RowVals {
    uint64_t k0, k1;
    uint64_t val[NA];
    unsigned ok;   // bit a: aggregate a's input is non-NULL
};

template <int NA>
__device__ __forceinline__ void load_row(const DevQuery &q, uint64_t row, bool me, RowVals<NA> &rv) {
    rv.k0 = 0;
    rv.k1 = 0;
    rv.ok = 0;
#pragma unroll 1
    for (int a = 0; a < NA; ++a) rv.val[a] = 0;
    if (!me) return;
    pack_key(q, row, rv.k0, rv.k1);
#pragma unroll 1
    for (int a = 0; a < NA; ++a) {
        if (a >= q.n_aggs) break;
        const DevAgg &g = q.aggs[a];
        if (g.col < 0) continue;
        const DevCol &c = q.cols[g.col];
        if (!col_valid(c, row)) continue;
        rv.ok |= 1u << a;
        if (g.kind == AK_COUNT_VALID || g.kind == AK_COUNT_ROWS || !g.needs_value) continue;
        rv.val[a] = g.is_float_in ? f64_bits(col_f64(c, row)) : (uint64_t)col_int(c, row);
    }
}

// Fold up to 32 gathered rows (bit i of `active` = lane i holds one).  One
// out-of-line copy keeps the instruction footprint small.
template <int NA>
__device__ __noinline__ void fold_batch(const DevQuery &q, const ScanSmem sm, const RowVals<NA> &in, unsigned active) {
    const int lane = threadIdx.x & 31;
    const bool me = (active >> lane) & 1u;
    uint64_t val[NA];
    const unsigned ok = in.ok;
#pragma unroll 1
    for (int a = 0; a < NA; ++a) {
        val[a] = in.val[a];
        if (a < q.n_aggs && (q.aggs[a].kind == AK_MIN_F || q.aggs[a].kind == AK_MAX_F)) {
            double d = bits_f64(val[a]);
            if (d != d) val[a] = 0x7FF8000000000000ULL;  // one NaN, ordered largest
        }
    }
    const uint64_t k0 = in.k0, k1 = in.k1;

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
#pragma unroll 1
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
            const uint64_t hk = hash_key(k0, 0);
            int e = cache_find(q, sm, k0, hk, claimed);
            if (e >= 0) {
                if (claimed) {
                    gid = (uint32_t)global_slot(q, k0, 0, hk);
                    sm.cgid[e] = gid;
                } else if (q.needs_gid) {
                    gid = *((volatile uint32_t *)sm.cgid + e);
                    if (gid == NO_GID) gid = (uint32_t)global_slot(q, k0, 0, hk);
                }
                apply_states<NA>(q, sm.cstate + (size_t)e * q.state_words, true, acc);
                done = true;
            }
        }
        if (!done) {
            gid = (uint32_t)(q.hashed ? global_slot_hashed(q, k0 - 1, k1) : global_slot(q, k0, k1));
            if (gid != NO_GID) apply_states<NA>(q, q.table + (uint64_t)gid * q.slot_words + q.key_words, false, acc);
        }
    }

    if (q.needs_gid) {
        gid = __shfl_sync(FULL, gid, leader_lane);
        if (me && gid != NO_GID) {
            unsigned long long *gst = q.table + (uint64_t)gid * q.slot_words + q.key_words;
#pragma unroll 1
            for (int a = 0; a < NA; ++a) {
                if (a >= q.n_aggs) break;
                const DevAgg &g = q.aggs[a];
                if (g.kind != AK_DISTINCT || !((ok >> a) & 1u)) continue;
                uint64_t bits = g.is_float_in ? canon_f64_bits(bits_f64(val[a])) : val[a];
                if (q.dpart_bits) dpart_append(q, group_hash(q, k0, k1), gid, bits);
                else if (distinct_insert(q, g.dset, gid, bits, group_hash(q, k0, k1))) red_add(gst + g.word, 1ULL, false);
            }
        }
    }
}

// Rows [row0, row_end) of chunk c.
__device__ __forceinline__ void chunk_rows(const DevQuery &q, uint32_t c, uint64_t &row0, uint64_t &row_end) {
    if (q.rg_list) {
        uint32_t rgi = c / q.chunks_per_rg, sub = c % q.chunks_per_rg;
        uint64_t rg = q.rg_list[rgi];
        row0 = rg * q.rg_rows + (uint64_t)sub * q.chunk_rows;
        row_end = min(min(row0 + q.chunk_rows, (rg + 1) * (uint64_t)q.rg_rows), q.n_rows);
    } else {
        row0 = (uint64_t)c * q.chunk_rows;
        row_end = min(row0 + q.chunk_rows, q.n_rows);
    }
}

// The fast WHERE: one range test on a NOT NULL integer column of type T,
// FILTER_UNROLL coalesced streaming loads in flight per lane.
template <typename T>
__device__ __forceinline__ uint32_t filter_range(const DevQuery &q, uint64_t row0, uint64_t row_end, uint16_t *list) {
    const int lane = threadIdx.x & 31;
    const T *col = (const T *)q.fp_data;
    const int64_t lo = q.fp_lo, hi = q.fp_hi;
    const bool neg = q.fp_negate != 0, shared = q.shared_scan != 0;
    uint32_t n = 0;
    for (uint64_t b = row0; b < row_end; b += 32 * FILTER_UNROLL) {
        T v[FILTER_UNROLL];
#pragma unroll
        for (int u = 0; u < FILTER_UNROLL; ++u) {
            const uint64_t r = b + u * 32 + lane;
            v[u] = r < row_end ? ld_pred(shared, col + r) : T(0);
        }
#pragma unroll
        for (int u = 0; u < FILTER_UNROLL; ++u) {
            const uint64_t r = b + u * 32 + lane;
            const int64_t x = (int64_t)v[u];
            const bool pass = r < row_end && ((x >= lo && x <= hi) != neg);
            const unsigned m = __ballot_sync(FULL, pass);
            if (pass) list[n + __popc(m & ((1u << lane) - 1))] = (uint16_t)(r - row0);
            n += __popc(m);
        }
    }
    return n;
}

// The whole WHERE for row r (the width-specialised range test when the plan
// has one).
__device__ __forceinline__ bool row_passes(const DevQuery &q, uint64_t r) {
    int64_t x;
    switch (q.fp_bytes) {
        case 0: {
            for (int i = 0; i < q.n_preds; ++i)
                if (!pred_holds(q, q.preds[i], r)) return false;
            return true;
        }
        case 1: x = ld_pred(q.shared_scan != 0, (const signed char *)q.fp_data + r); break;
        case 2: x = ld_pred(q.shared_scan != 0, (const short *)q.fp_data + r); break;
        case 4: x = ld_pred(q.shared_scan != 0, (const int *)q.fp_data + r); break;
        default: x = ld_pred(q.shared_scan != 0, (const long long *)q.fp_data + r); break;
    }
    return (x >= q.fp_lo && x <= q.fp_hi) != (q.fp_negate != 0);
}

// Pull a gathered row's global-table slot toward L2 as soon as its key is
// known, so the fold's probe of batch j + 1 .. j + LOOKAHEAD - 1 overlaps the
// fold of batch j instead of waiting on DRAM.  Not for the resident route,
// whose groups all live in shared memory.
__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// The count sketch's filter pass (sketch.cu): whether a row of key hash hk
// folds (always, without a sketch or when it declined).
__device__ __forceinline__ bool sketch_kept(const DevQuery &q, uint64_t hk) {
    if (!q.sk_keep || !__ldg(q.sk_on)) return true;
    const uint32_t c = (uint32_t)(hk >> (64 - SK_BITS));
    return (__ldg(q.sk_keep + (c >> 5)) >> (c & 31)) & 1u;
}

// Prefetch a row's slot (lane `me` holds a row); returns whether the row
// folds — false for a row the count sketch drops, whose slot is not touched.
// The key is hashed only when a prefetch or the sketch needs it.
__device__ __forceinline__ bool prefetch_slot(const DevQuery &q, uint64_t k0, uint64_t k1, bool me) {
    const bool pf = (q.prefetch & PF_SLOT) && !(q.cache_slots && q.cache_probe == q.cache_slots) && !q.hashed;
    if (!me || (!pf && !q.sk_keep)) return me;
    const uint64_t hk = hash_key(k0, k1);
    if (!sketch_kept(q, hk)) return false;
    if (pf) prefetch_l2(q.table + (hk & (q.cap - 1)) * (uint64_t)q.slot_words);
    return true;
}

// ------------------------------------------------------ fold policies --

// The interpreter: any plan, aggregate kinds read from the plan at run time.
template <int NA>
struct GenericFold {
    using Row = RowVals<NA>;
    static constexpr bool QUEUE_OK = false;  // rows too wide for the warp queue
    static constexpr int QLOOKAHEAD = 1;
    static constexpr int LOOKAHEAD = 1;  // batches gathered before folding
    __device__ __forceinline__ static void load(const DevQuery &q, uint64_t r, bool me, Row &rv) {
        load_row<NA>(q, r, me, rv);
    }
    __device__ __forceinline__ static void fold(const DevQuery &q, const ScanSmem &sm, const Row &rv, unsigned act) {
        fold_batch<NA>(q, sm, rv, act);
    }
    __device__ __forceinline__ static bool prefetch(const DevQuery &q, const Row &rv, bool me) {
        return prefetch_slot(q, rv.k0, rv.k1, me);
    }
    __device__ __forceinline__ static void reserve(const DevQuery &, Row &, bool) {}
};

// A plan whose NOT NULL inputs fold with the compile-time kinds K0..K3 (the
// owner aggregates of q.faggs, AK_NONE = none) and whose key is one NOT NULL
// integer part (KM = 1) or several NOT NULL parts (KM = 2): no per-row kind
// dispatch, no validity checks, the accumulators stay in registers.
constexpr int AK_NONE = -1;

template <int KM, int K0, int K1, int K2, int K3>
struct FastFold {
    static constexpr int NA = (K0 != AK_NONE) + (K1 != AK_NONE) + (K2 != AK_NONE) + (K3 != AK_NONE);
    static constexpr int NV = NA > 0 ? NA : 1;
    static constexpr int KM_ = KM, NA_ = NA;
    static constexpr bool QUEUE_OK = true;
    static constexpr int QLOOKAHEAD = 2;  // queue mode: 32-row steps loaded before any is compacted
    // batches whose gathers are all in flight before the first folds; the
    // rows stay in registers (64 per thread at two CTAs per SM), so the depth
    // shrinks as a row grows
    static constexpr int ROW_REGS = (KM == 1 ? 2 : 4) + 2 * NV;
    static constexpr int LOOKAHEAD = ROW_REGS <= 6 ? 4 : ROW_REGS <= 8 ? 2 : 1;
    __host__ __device__ static constexpr int kind(int a) { return a == 0 ? K0 : a == 1 ? K1 : a == 2 ? K2 : K3; }
    __host__ __device__ static constexpr bool is_f(int a) {
        return kind(a) == AK_SUM_F64 || kind(a) == AK_MIN_F || kind(a) == AK_MAX_F;
    }
    static constexpr bool DISTINCT = K0 == AK_DISTINCT || K1 == AK_DISTINCT || K2 == AK_DISTINCT || K3 == AK_DISTINCT;

    // a COUNT(DISTINCT) row also carries its pair's reserved place
    struct PlainRow {
        uint64_t k0, k1;
        uint64_t val[NV];
    };
    struct DistinctRow : PlainRow {
        uint32_t dp = 0, dpos = DPOS_NONE;  // a row built by any caller starts unreserved
    };
    using Row = typename Pick<DISTINCT, DistinctRow, PlainRow>::type;

    __device__ __forceinline__ static void load(const DevQuery &q, uint64_t r, bool me, Row &rv) {
        rv.k0 = 0;
        rv.k1 = 0;
#pragma unroll
        for (int a = 0; a < NV; ++a) rv.val[a] = 0;
        if constexpr (DISTINCT) rv.dpos = DPOS_NONE;
        if (!me) return;
        // gathered columns are read once unless other queries of a batch follow
        const bool shared = q.shared_scan != 0;
        if (KM == 1) {
            const DevKeyPart &kp = q.parts[0];
            uint64_t raw = (uint64_t)col_int_stream(q.cols[kp.col], r, shared);
            rv.k0 = kp.payload < 64 ? (raw & ((1ULL << kp.payload) - 1)) : raw;
        } else {
            for (int i = 0; i < q.n_parts; ++i) {
                const DevKeyPart &kp = q.parts[i];
                uint64_t raw = (uint64_t)col_int_stream(q.cols[kp.col], r, shared);
                if (kp.payload < 64) raw &= (1ULL << kp.payload) - 1;
                const int off = kp.offset;
                if (off < 64) {
                    rv.k0 |= raw << off;
                    if (off > 0) rv.k1 |= raw >> (64 - off);
                } else {
                    rv.k1 |= raw << (off - 64);
                }
            }
        }
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            const DevCol &c = q.cols[q.faggs[a].col];
            rv.val[a] = is_f(a) ? f64_bits(col_f64_stream(c, r, shared)) : (uint64_t)col_int_stream(c, r, shared);
        }
    }

    // returns whether the row folds (prefetch_slot)
    __device__ __forceinline__ static bool prefetch(const DevQuery &q, const Row &rv, bool me) {
        me = prefetch_slot(q, rv.k0, rv.k1, me);
        if (DISTINCT && me && (q.prefetch & PF_DISTINCT) && !q.dpart_bits) {
            const uint64_t hk = hash_key(rv.k0, rv.k1);
#pragma unroll
            for (int a = 0; a < NA; ++a)
                if (kind(a) == AK_DISTINCT) {
                    const int d = q.faggs[a].dset;
                    prefetch_l2(q.dset[d] + 2 * distinct_home(q, d, hk, rv.val[a]));
                }
        }
        return me;
    }

    // Partitioned COUNT(DISTINCT): reserve each row's pair place as soon as
    // the row is loaded (the partition needs the key, not the group id), so
    // the cursor atomics of all batches in flight overlap the folds' probes.
    // Every lane that reserves is active in the batch's fold, which stores.
    __device__ __forceinline__ static void reserve(const DevQuery &q, Row &rv, bool me) {
        if constexpr (DISTINCT) {
            if (!me || !q.dpart_bits) return;
#pragma unroll
            for (int a = 0; a < NA; ++a)
                if (kind(a) == AK_DISTINCT) {
                    rv.dp = dpart_of(q, hash_key(rv.k0, rv.k1), rv.val[a]);
                    rv.dpos = atomicAdd(q.dpart_cursor + rv.dp, 1u);
                }
        }
    }

    // The folded contribution of one group to its state words.
    template <bool SMEM>
    __device__ __forceinline__ static void apply(const DevQuery &q, unsigned long long *st, uint32_t rows,
                                                 const uint64_t (&lo)[NV], const uint64_t (&hi)[NV]) {
        red_add(st, (unsigned long long)rows, SMEM);
#pragma unroll
        for (int a = 0; a < NV; ++a) {
            if (a >= NA) continue;
            unsigned long long *w = st + q.faggs[a].word;
            switch (kind(a)) {
                case AK_SUM_I64:
                    if (lo[a]) red_add(w, (unsigned long long)lo[a], SMEM);
                    break;
                case AK_SUM_I128:
                    if (lo[a]) red_add(w, (unsigned long long)lo[a], SMEM);
                    if (hi[a]) red_add(w + 1, (unsigned long long)hi[a], SMEM);
                    break;
                case AK_SUM_F64: red_add_f64(w, bits_f64(lo[a]), SMEM); break;
                case AK_MIN_I: case AK_MAX_I: case AK_MIN_F: case AK_MAX_F:
                    red_max(w, (unsigned long long)lo[a], SMEM);
                    break;
                default: break;
            }
        }
    }

    // One out-of-line copy for the scan loops with several unrolled call
    // sites (an inlined copy per site overflows the instruction cache) ...
    __device__ __noinline__ static void fold(const DevQuery &q, const ScanSmem sm, const Row in, unsigned active) {
        fold_body(q, sm, in, active);
    }

    // ... one for a caller that loaded each row's home-slot key ahead (see
    // global_slot_from) ...
    __device__ __noinline__ static void fold_hinted(const DevQuery &q, const ScanSmem sm, const Row in,
                                                    unsigned active, uint64_t home) {
        fold_body(q, sm, in, active, home);
    }

    // ... and the body itself, inlined where a loop has one call site.
    __device__ __forceinline__ static void fold_body(const DevQuery &q, const ScanSmem &sm, const Row &in,
                                                     unsigned active, uint64_t home = 0) {
        const int lane = threadIdx.x & 31;
        const bool me = (active >> lane) & 1u;
        uint64_t val[NV];
#pragma unroll
        for (int a = 0; a < NV; ++a) {
            val[a] = in.val[a];
            if (a < NA && (kind(a) == AK_MIN_F || kind(a) == AK_MAX_F)) {
                const double d = bits_f64(val[a]);
                if (d != d) val[a] = 0x7FF8000000000000ULL;
            }
        }
        const uint64_t k0 = in.k0, k1 = in.k1;
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

        // own contribution in folded form
        uint32_t rows = 1;
        uint64_t lo[NV], hi[NV];
#pragma unroll
        for (int a = 0; a < NV; ++a) {
            lo[a] = 0;
            hi[a] = 0;
            if (a >= NA) continue;
            const uint64_t v = val[a];
            switch (kind(a)) {
                case AK_SUM_I64: case AK_SUM_F64: lo[a] = v; break;
                case AK_SUM_I128: lo[a] = split_lo((int64_t)v); hi[a] = split_hi((int64_t)v); break;
                case AK_MAX_I: lo[a] = enc_i64((int64_t)v); break;
                case AK_MIN_I: lo[a] = ~enc_i64((int64_t)v); break;
                case AK_MAX_F: lo[a] = enc_f64_bits(v); break;
                case AK_MIN_F: lo[a] = ~enc_f64_bits(v); break;
                default: break;
            }
        }
        if (q.warp_combine) {
            unsigned rem = leader ? (grp & ~(1u << lane)) : 0u;
            while (__any_sync(FULL, rem != 0)) {
                const int src = rem ? __ffs(rem) - 1 : lane;
                uint64_t x[NV];
#pragma unroll
                for (int a = 0; a < NV; ++a) x[a] = a < NA ? shfl64(val[a], src) : 0;
                if (rem) {
                    rows += 1;
#pragma unroll
                    for (int a = 0; a < NV; ++a) {
                        if (a >= NA) continue;
                        const uint64_t v = x[a];
                        switch (kind(a)) {
                            case AK_SUM_I64: lo[a] += v; break;
                            case AK_SUM_I128:
                                lo[a] += split_lo((int64_t)v);
                                hi[a] += split_hi((int64_t)v);
                                break;
                            case AK_SUM_F64: lo[a] = f64_bits(bits_f64(lo[a]) + bits_f64(v)); break;
                            case AK_MAX_I: lo[a] = max(lo[a], (uint64_t)enc_i64((int64_t)v)); break;
                            case AK_MIN_I: lo[a] = max(lo[a], ~enc_i64((int64_t)v)); break;
                            case AK_MAX_F: lo[a] = max(lo[a], enc_f64_bits(v)); break;
                            case AK_MIN_F: lo[a] = max(lo[a], ~enc_f64_bits(v)); break;
                            default: break;
                        }
                    }
                    rem &= rem - 1;
                }
            }
        }

        uint32_t gid = NO_GID;
        if (leader) {
            unsigned long long *st = nullptr;
            bool st_smem = false;
            const uint64_t hk = hash_key(k0, k1);  // once for the shared and the global probe
            if (q.cache_slots && q.key_words == 1 && k0 != 0) {
                bool claimed;
                const int e = cache_find(q, sm, k0, hk, claimed);
                if (e >= 0) {
                    if (claimed) {
                        gid = (uint32_t)global_slot_from(q, k0, 0, hk, home);
                        sm.cgid[e] = gid;
                    } else if (DISTINCT) {
                        gid = *((volatile uint32_t *)sm.cgid + e);
                        if (gid == NO_GID) gid = (uint32_t)global_slot(q, k0, 0, hk);
                    }
                    st = sm.cstate + (size_t)e * q.state_words;
                    st_smem = true;
                }
            }
            if (!st) {
                gid = (uint32_t)global_slot_from(q, k0, k1, hk, home);
                if (gid != NO_GID) st = q.table + (uint64_t)gid * q.slot_words + q.key_words;
            }
            if (st) {
                // one copy of the updates per state space, chosen once
                if (st_smem) apply<true>(q, st, rows, lo, hi);
                else apply<false>(q, st, rows, lo, hi);
            }
        }
        if constexpr (DISTINCT) {
            gid = __shfl_sync(FULL, gid, leader_lane);
            if (me) {
                const uint64_t hk = hash_key(k0, k1);
#pragma unroll
                for (int a = 0; a < NV; ++a) {
                    if (a >= NA || kind(a) != AK_DISTINCT) continue;
                    if (q.dpart_bits) {
                        uint32_t p = in.dp, pos = in.dpos;
                        if (pos == DPOS_NONE) {  // callers that do not reserve ahead
                            p = dpart_of(q, hk, val[a]);
                            pos = atomicAdd(q.dpart_cursor + p, 1u);
                        }
                        dpart_store(q, p, pos, gid, val[a]);
                    } else if (gid != NO_GID && distinct_insert(q, q.faggs[a].dset, gid, val[a], hk)) {
                        red_add(q.table + (uint64_t)gid * q.slot_words + q.key_words + q.faggs[a].word, 1ULL, false);
                    }
                }
            }
        }
    }
};

// Lanes 0 .. n_pf - 1 pull chunk c of one scanned column each into L2 (one
// bulk prefetch: 16-byte aligned start, size rounded down to 16 bytes), so
// the warp's filter and gathers of that chunk find it there.
__device__ __forceinline__ void prefetch_chunk(const DevQuery &q, uint32_t c) {
    const int lane = threadIdx.x & 31;
    if (!(q.prefetch & PF_NEXT) || lane >= q.n_pf || c >= q.n_chunks) return;
    uint64_t row0, row_end;
    chunk_rows(q, c, row0, row_end);
    if (row0 >= row_end) return;
    const DevCol &col = q.cols[q.pf_cols[lane]];
    // [begin, end) of the chunk's bytes, shrunk to whole 16-byte blocks
    const uintptr_t begin = (uintptr_t)col.data + row0 * (uint64_t)col.bytes;
    const uintptr_t end = (uintptr_t)col.data + row_end * (uint64_t)col.bytes;
    const uintptr_t b16 = (begin + 15) & ~(uintptr_t)15, e16 = end & ~(uintptr_t)15;
    if (e16 <= b16) return;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(b16), "r"((uint32_t)(e16 - b16)) : "memory");
}

// The WHERE over rows [row0, row_end): the survivors' chunk offsets into
// `list` (ballot + popc positions); returns their count.
__device__ __forceinline__ uint32_t survivors(const DevQuery &q, uint64_t row0, uint64_t row_end, uint16_t *list) {
    const int lane = threadIdx.x & 31;
    uint32_t n = 0;
    switch (q.fp_bytes) {
        case 1: n = filter_range<signed char>(q, row0, row_end, list); break;
        case 2: n = filter_range<short>(q, row0, row_end, list); break;
        case 4: n = filter_range<int>(q, row0, row_end, list); break;
        case 8: n = filter_range<long long>(q, row0, row_end, list); break;
        default: break;
    }
    for (uint64_t b = row0; q.fp_bytes == 0 && b < row_end; b += 32 * FILTER_UNROLL) {
        bool pass[FILTER_UNROLL];
        // first predicate for all steps (its loads are independent), then the rest
#pragma unroll
        for (int u = 0; u < FILTER_UNROLL; ++u) {
            const uint64_t r = b + u * 32 + lane;
            pass[u] = r < row_end && pred_holds(q, q.preds[0], r);
        }
        for (int i = 1; i < q.n_preds; ++i) {
#pragma unroll
            for (int u = 0; u < FILTER_UNROLL; ++u) {
                const uint64_t r = b + u * 32 + lane;
                if (pass[u]) pass[u] = pred_holds(q, q.preds[i], r);
            }
        }
#pragma unroll
        for (int u = 0; u < FILTER_UNROLL; ++u) {
            const unsigned m = __ballot_sync(FULL, pass[u]);
            if (pass[u]) list[n + __popc(m & ((1u << lane) - 1))] = (uint16_t)(b + u * 32 + lane - row0);
            n += __popc(m);
        }
    }
    return n;
}

// One warp folds chunk c: filter + compaction, then batches of 32 survivors
// (each batch's gathers issued before the previous batch folds).
template <class P>
__device__ __forceinline__ void scan_chunk(const DevQuery &q, const ScanSmem &sm, uint32_t c,
                                           unsigned long long &selected) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t row0, row_end;
    chunk_rows(q, c, row0, row_end);
    if (row0 >= row_end) return;
    if (q.n_preds == 0 || !q.gather) {
        // every row (or every filtered row in place): 32 consecutive rows per
        // batch, LOOKAHEAD batches loaded before any of them folds.  The key
        // and input loads do not wait for the WHERE: at the selectivities
        // that pick this mode the survivors touch nearly every line anyway,
        // so loading all rows costs no extra DRAM bytes and keeps every load
        // of the batch in flight at once.
        constexpr int L = P::LOOKAHEAD;
        for (uint64_t base = row0; base < row_end; base += 32 * L) {
            typename P::Row rows[L];
            unsigned act[L];
#pragma unroll
            for (int j = 0; j < L; ++j) {
                const uint64_t r = base + 32 * j + lane;
                P::load(q, r, r < row_end, rows[j]);
            }
#pragma unroll
            for (int j = 0; j < L; ++j) {
                const uint64_t r = base + 32 * j + lane;
                act[j] = __ballot_sync(FULL, r < row_end && row_passes(q, r));
            }
            unsigned keep[L];  // rows that fold (the WHERE's, less any the count sketch drops)
#pragma unroll
            for (int j = 0; j < L; ++j) keep[j] = __ballot_sync(FULL, P::prefetch(q, rows[j], (act[j] >> lane) & 1u));
#pragma unroll
            for (int j = 0; j < L; ++j) P::reserve(q, rows[j], (keep[j] >> lane) & 1u);
#pragma unroll
            for (int j = 0; j < L; ++j) {
                selected += (lane == 0) ? __popc(act[j]) : 0;
                if (keep[j]) P::fold(q, sm, rows[j], keep[j]);
            }
        }
        return;
    }
    // gather mode: the chunk's survivors first, then folds
    uint16_t *list = sm.wlist + (size_t)warp * q.chunk_rows;
    const uint32_t n = survivors(q, row0, row_end, list);
    __syncwarp();
    selected += (lane == 0) ? n : 0;
    if (n == 0) return;
    constexpr int L = P::LOOKAHEAD;
    for (uint32_t i = 0; i < n; i += 32 * L) {
        typename P::Row rows[L];
#pragma unroll
        for (int j = 0; j < L; ++j) {
            const uint32_t s = i + 32 * j + lane;
            P::load(q, row0 + list[s < n ? s : 0], s < n, rows[j]);
        }
        unsigned keep[L];  // survivors that fold (less any the count sketch drops)
#pragma unroll
        for (int j = 0; j < L; ++j) keep[j] = __ballot_sync(FULL, P::prefetch(q, rows[j], i + 32 * j + lane < n));
#pragma unroll
        for (int j = 0; j < L; ++j) P::reserve(q, rows[j], (keep[j] >> lane) & 1u);
#pragma unroll
        for (int j = 0; j < L; ++j)
            if (keep[j]) P::fold(q, sm, rows[j], keep[j]);
    }
}

// ------------------------------------------------------------ queue mode --
// (q.gather == 2) Every row's key and inputs are loaded densely — coalesced,
// with the predicate's, LOOKAHEAD steps of 32 rows in flight — and the
// WHERE's survivors are appended to the warp's ring of WQ_ROWS fold rows in
// shared memory; every time the ring holds 32 rows the warp folds them as
// one full batch.  The ring persists across the warp's chunks (a row carries
// its key and inputs, not a chunk offset), so only the warp's last batch is
// partial.  At the selectivities that pick this mode the survivors touch
// nearly every line of the key and input columns, so loading them densely
// costs no extra DRAM bytes and removes the filter -> gather dependency.

constexpr uint32_t WQ_ROWS = WQ_RING_ROWS;

template <class P>
struct WarpQueue {
    typename P::Row *ring;  // this warp's WQ_ROWS rows
    uint32_t head, count;   // warp-uniform; count < 32 between steps
};

template <class P>
__device__ __forceinline__ void wq_fold_full(const DevQuery &q, const ScanSmem &sm, WarpQueue<P> &wq) {
    const int lane = threadIdx.x & 31;
    while (wq.count >= 32) {
        __syncwarp();
        const typename P::Row rv = wq.ring[(wq.head + lane) & (WQ_ROWS - 1)];
        __syncwarp();
        P::fold(q, sm, rv, FULL);
        wq.head = (wq.head + 32) & (WQ_ROWS - 1);
        wq.count -= 32;
    }
}

template <class P>
__device__ __forceinline__ void wq_flush(const DevQuery &q, const ScanSmem &sm, WarpQueue<P> &wq) {
    const int lane = threadIdx.x & 31;
    if (wq.count == 0) return;
    __syncwarp();
    const typename P::Row rv = wq.ring[(wq.head + lane) & (WQ_ROWS - 1)];
    __syncwarp();
    P::fold(q, sm, rv, (1u << wq.count) - 1);
    wq.head = 0;
    wq.count = 0;
}

template <class P>
__device__ __forceinline__ void scan_chunk_queue(const DevQuery &q, const ScanSmem &sm, uint32_t c,
                                                 unsigned long long &selected, WarpQueue<P> &wq) {
    const int lane = threadIdx.x & 31;
    uint64_t row0, row_end;
    chunk_rows(q, c, row0, row_end);
    if (row0 >= row_end) return;
    constexpr int L = P::QLOOKAHEAD;
    for (uint64_t base = row0; base < row_end; base += 32 * L) {
        typename P::Row rows[L];
        bool pass[L];
#pragma unroll
        for (int j = 0; j < L; ++j) {
            const uint64_t r = base + 32 * j + lane;
            P::load(q, r, r < row_end, rows[j]);
        }
#pragma unroll
        for (int j = 0; j < L; ++j) {
            const uint64_t r = base + 32 * j + lane;
            pass[j] = r < row_end && row_passes(q, r);
        }
#pragma unroll
        for (int j = 0; j < L; ++j) {
            const unsigned m = __ballot_sync(FULL, pass[j]);
            if (m == 0) continue;
            selected += (lane == 0) ? __popc(m) : 0;
            const bool kp = P::prefetch(q, rows[j], pass[j]);
            const unsigned mk = __ballot_sync(FULL, kp);
            if (kp) wq.ring[(wq.head + wq.count + __popc(mk & ((1u << lane) - 1))) & (WQ_ROWS - 1)] = rows[j];
            wq.count += __popc(mk);
            wq_fold_full<P>(q, sm, wq);
        }
    }
}

// The compiled fast-fold signatures: (index, key mode, owner aggregate kinds).
#define TGPU_FAST_FOLDS(X)                                             \
    X(0, 1, AK_SUM_I64, AK_MIN_I, AK_MAX_I, AK_NONE)                   \
    X(1, 1, AK_SUM_I128, AK_NONE, AK_NONE, AK_NONE)                    \
    X(2, 1, AK_SUM_I128, AK_MIN_I, AK_MAX_I, AK_NONE)                  \
    X(3, 1, AK_SUM_I128, AK_MIN_I, AK_NONE, AK_NONE)                   \
    X(4, 1, AK_SUM_I128, AK_MAX_I, AK_NONE, AK_NONE)                   \
    X(5, 1, AK_MIN_I, AK_MAX_I, AK_NONE, AK_NONE)                      \
    X(6, 1, AK_MIN_I, AK_NONE, AK_NONE, AK_NONE)                       \
    X(7, 1, AK_MAX_I, AK_NONE, AK_NONE, AK_NONE)                       \
    X(8, 1, AK_NONE, AK_NONE, AK_NONE, AK_NONE)                        \
    X(9, 1, AK_SUM_I64, AK_NONE, AK_NONE, AK_NONE)                     \
    X(10, 2, AK_DISTINCT, AK_SUM_F64, AK_NONE, AK_NONE)                \
    X(11, 2, AK_NONE, AK_NONE, AK_NONE, AK_NONE)

}  // namespace

}  // namespace tgpu
