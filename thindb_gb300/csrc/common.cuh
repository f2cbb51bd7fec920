// common.cuh — device helpers shared by the grouped-aggregation kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "engine.h"

namespace tgpu {

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
    // splitmix64 finalizer, thinDB's group-key mixer (src/exec/group_table.zig:45-50)
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// Carry-free exact sums of 64-bit integers: w0 accumulates the unsigned low
// 32-bit halves, w1 the signed high halves, so every update is a plain
// add (an atomic whose result nobody waits for).  The sum is w1 * 2^32 + w0,
// exact while fewer than 2^32 values are added (|w1| < 2^63, w0 < 2^64).
__host__ __device__ __forceinline__ uint64_t split_lo(int64_t v) { return (uint64_t)(uint32_t)(uint64_t)v; }
__host__ __device__ __forceinline__ uint64_t split_hi(int64_t v) { return (uint64_t)(v >> 32); }
__host__ __device__ __forceinline__ void i128_of_split(uint64_t w0, uint64_t w1, uint64_t &lo, int64_t &hi) {
    lo = w0 + (w1 << 32);
    hi = ((int64_t)w1 >> 32) + (lo < w0 ? 1 : 0);
}

// Digest of a string's bytes for the hashed-key layout: the length, then the
// bytes as little-endian 8-byte words (the last one zero-padded), chained
// through mix64.  (thinDB digests string keys with a 128-bit Wyhash,
// stringKeyDigest; the digest only places a group and orders exact ties —
// equality is always decided on the bytes.)
__host__ __device__ inline uint64_t str_hash(const uint8_t *p, uint32_t n) {
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

// One key part's contribution to a hashed key's digest: a NULL marker, a
// string's str_hash, or an integer's value bits; chained from HASHED_SEED.
constexpr uint64_t HASHED_SEED = 0x243F6A8885A308D3ULL;
constexpr uint64_t HASHED_NULL = 0x8000000000000001ULL;
__host__ __device__ __forceinline__ uint64_t digest_step(uint64_t d, uint64_t part) { return mix64(d ^ part); }
__host__ __device__ __forceinline__ uint64_t int_part_hash(int64_t v) {
    return mix64((uint64_t)v ^ 0x6A09E667F3BCC909ULL);
}

__host__ __device__ __forceinline__ uint64_t hash_key(uint64_t lo, uint64_t hi) {
    // hashU128 (group_table.zig:52-55): mix64(lo ^ mix64(hi))
    return mix64(lo ^ mix64(hi));
}

// 128-bit compare-and-swap on global memory (sm_90+ `atom.cas.b128`).
// Returns the value found at `p` (== cmp on success).
__device__ __forceinline__ ulonglong2 cas128(unsigned long long *p, ulonglong2 cmp, ulonglong2 val) {
    ulonglong2 out;
    asm volatile(
        "{\n\t"
        ".reg .b128 d, c, s;\n\t"
        "mov.b128 c, {%2, %3};\n\t"
        "mov.b128 s, {%4, %5};\n\t"
        "atom.global.cas.b128 d, [%6], c, s;\n\t"
        "mov.b128 {%0, %1}, d;\n\t"
        "}"
        : "=l"(out.x), "=l"(out.y)
        : "l"(cmp.x), "l"(cmp.y), "l"(val.x), "l"(val.y), "l"(p)
        : "memory");
    return out;
}

// 16-byte relaxed load (may observe the two halves from different writes;
// callers confirm a match with cas128).
__device__ __forceinline__ ulonglong2 ld128(const unsigned long long *p) {
    ulonglong2 v;
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Order-preserving maps to u64 so MIN/MAX fold with an unsigned atomicMax on a
// zero-initialised word: MAX stores enc(x), MIN stores ~enc(x); 0 is the
// identity of both and decodes to the type's extreme.
__host__ __device__ __forceinline__ uint64_t enc_i64(int64_t x) { return (uint64_t)x ^ 0x8000000000000000ULL; }
__host__ __device__ __forceinline__ int64_t dec_i64(uint64_t u) { return (int64_t)(u ^ 0x8000000000000000ULL); }
__host__ __device__ __forceinline__ uint64_t enc_f64_bits(uint64_t b) {
    return (b & 0x8000000000000000ULL) ? ~b : (b | 0x8000000000000000ULL);
}
__host__ __device__ __forceinline__ uint64_t dec_f64_bits(uint64_t u) {
    return (u & 0x8000000000000000ULL) ? (u & 0x7FFFFFFFFFFFFFFFULL) : ~u;
}

// f64 of a signed 128-bit integer, rounded to nearest with ties to even —
// the IEEE conversion Zig's @floatFromInt performs.  Written from the
// definition: take the top 53 significant bits, round on the next bit with the
// OR of all lower bits as sticky.  Exact when |v| < 2^53.
__host__ __device__ inline double i128_to_f64(uint64_t lo, int64_t hi) {
    bool neg = hi < 0;
    uint64_t mlo = lo, mhi = (uint64_t)hi;
    if (neg) {  // magnitude = -v (two's complement)
        mlo = ~mlo + 1;
        mhi = ~mhi + (mlo == 0 ? 1 : 0);
    }
    if (mhi == 0 && mlo < (1ULL << 53)) {
        double d = (double)mlo;
        return neg ? -d : d;
    }
    // bit length
    int len;
    if (mhi) {
#ifdef __CUDA_ARCH__
        len = 128 - __clzll((long long)mhi);
#else
        len = 128 - __builtin_clzll(mhi);
#endif
    } else {
#ifdef __CUDA_ARCH__
        len = 64 - __clzll((long long)mlo);
#else
        len = 64 - __builtin_clzll(mlo);
#endif
    }
    int shift = len - 53;  // > 0 here
    // mantissa = magnitude >> shift (53 bits), round bit, sticky
    uint64_t mant, round_bit, sticky;
    if (shift >= 64) {
        int s = shift - 64;
        mant = mhi >> s;
        round_bit = s ? (mhi >> (s - 1)) & 1 : (mlo >> 63) & 1;
        uint64_t below_hi = s >= 2 ? (mhi & ((1ULL << (s - 1)) - 1)) : 0;
        uint64_t below_lo = s ? mlo : (mlo & 0x7FFFFFFFFFFFFFFFULL);
        sticky = (below_hi | below_lo) != 0;
    } else {
        mant = (mlo >> shift) | (shift ? (mhi << (64 - shift)) : 0);
        round_bit = (mlo >> (shift - 1)) & 1;
        sticky = shift >= 2 ? ((mlo & ((1ULL << (shift - 1)) - 1)) != 0) : 0;
    }
    if (round_bit && (sticky || (mant & 1))) {
        mant += 1;
        if (mant == (1ULL << 53)) {
            mant >>= 1;
            shift += 1;
        }
    }
    // value = mant * 2^shift ; mant < 2^53 so the product below is exact
    double d = (double)mant;
    // scale by 2^shift exactly (shift <= 75)
    uint64_t ebits = (uint64_t)(1023 + shift) << 52;
    double scale;
#ifdef __CUDA_ARCH__
    scale = __longlong_as_double((long long)ebits);
#else
    __builtin_memcpy(&scale, &ebits, 8);
#endif
    d *= scale;
    return neg ? -d : d;
}

__device__ __forceinline__ uint64_t f64_bits(double d) { return (uint64_t)__double_as_longlong(d); }
__device__ __forceinline__ double bits_f64(uint64_t b) { return __longlong_as_double((long long)b); }

// Canonical distinct bits of a float value: -0.0 == 0.0, every NaN is one value
// (thinDB types.canonicalFloatBits, src/types.zig:589-600).
__device__ __forceinline__ uint64_t canon_f64_bits(double v) {
    if (v != v) return 0x7FF8000000000000ULL;
    if (v == 0.0) return 0;
    return f64_bits(v);
}

}  // namespace tgpu
