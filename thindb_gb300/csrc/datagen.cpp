// Seeded synthetic inputs for the grouped-aggregation workloads.
//
// Every column is a pure function of (seed, column stream, row index): row i
// of a stream with seed s is mix64(s + (i + 1) * GOLDEN), the i-th output of
// splitmix64 seeded with s.  So generation is embarrassingly parallel and the
// same on any thread count.  mix64 is the splitmix64 finalizer, the same
// mixer thinDB hashes group keys with (src/exec/group_table.zig:45-50).
//
// Workloads (all NOT NULL, row groups of 65,536 rows):
//   plain      16,777,216 rows: k BIGINT = one of 1,024 values (the first 1,024
//              outputs of splitmix64 seeded with 1), v INT uniform in [-1e6, 1e6].
//   filtered   100M rows: k BIGINT = Zipf(s=1.1) rank over 10M values mapped
//              through mix64 (a bijection, so distinct ranks stay distinct);
//              amount DECIMAL(18,2) cents = clip(round(exp(8 + 1.5 z)), 1, 1e12)
//              with z from Box-Muller; d DATE = 2026-01-01 + U[0,365) days.
//   distinct   200M rows: region SMALLINT U[0,64); url DICT32 code =
//              (region * 781 + U[0,6250)) mod 50,000 (about 400k (region, url)
//              pairs); user_id BIGINT = Zipf(s=0.9) rank over 5M through mix64;
//              latency DOUBLE exponential with mean 120.
//   batched    the filtered table plus k10/k1k/k1m INT uniform over 10, 1,000
//              and 1,000,000 values.
// Host-only C++ (no intrinsics), so x86 and Arm builds produce the same
// integer columns; the libm-derived columns (amount, latency) may differ in
// the last ulp between machines, which is why committed fixtures never
// depend on them.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

constexpr uint64_t GOLDEN = 0x9E3779B97F4A7C15ULL;

inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// i-th output (0-based) of splitmix64 seeded with s.
inline uint64_t sm_at(uint64_t s, uint64_t i) { return mix64(s + (i + 1) * GOLDEN); }

// Independent stream seed per (config seed, column id).
inline uint64_t stream_seed(uint64_t seed, uint64_t col) {
    return mix64(seed * 0xD1B54A32D192ED03ULL + col * 0xABCDEF0123456789ULL + 0x5851F42D4C957F2DULL);
}

// Uniform double in [0, 1) from the top 53 bits.
inline double unit(uint64_t x) { return (double)(x >> 11) * (1.0 / 9007199254740992.0); }

template <typename F>
void parallel_rows(uint64_t n, int threads, F f) {
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    if (n < (1u << 16) || threads == 1) {
        f(0, n);
        return;
    }
    std::vector<std::thread> ts;
    uint64_t per = (n + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        uint64_t b = (uint64_t)t * per, e = std::min(n, b + per);
        if (b >= e) break;
        ts.emplace_back([=] { f(b, e); });
    }
    for (auto &t : ts) t.join();
}

// Inverse-CDF sampler for Zipf(s) over ranks 1..m with a guide table so each
// draw searches a short range.
struct Zipf {
    std::vector<double> cdf;       // cdf[k-1] = P(rank <= k) * total (unnormalised)
    std::vector<uint32_t> guide;   // guide[b] = first index with cdf > b/G * total
    double total = 0;
    static constexpr uint32_t G = 1u << 20;
    Zipf(uint64_t m, double s) : cdf(m), guide(G + 1) {
        double acc = 0;
        for (uint64_t k = 1; k <= m; ++k) {
            acc += std::pow((double)k, -s);
            cdf[k - 1] = acc;
        }
        total = acc;
        uint64_t idx = 0;
        for (uint32_t b = 0; b <= G; ++b) {
            double thr = total * ((double)b / (double)G);
            while (idx < m - 1 && cdf[idx] <= thr) ++idx;
            guide[b] = (uint32_t)idx;
        }
    }
    // Rank in [1, m] for a uniform u in [0, 1).
    uint64_t rank(double u) const {
        double x = u * total;
        uint32_t b = (uint32_t)(u * G);
        if (b >= G) b = G - 1;
        uint64_t lo = guide[b], hi = guide[b + 1];
        if (hi < lo) hi = lo;
        // first index in [lo, hi] with cdf > x; widen if the guide is loose
        while (lo > 0 && cdf[lo - 1] > x) lo = lo > 64 ? lo - 64 : 0;
        while (hi < cdf.size() - 1 && cdf[hi] <= x) hi = std::min<uint64_t>(cdf.size() - 1, hi + 64);
        auto it = std::upper_bound(cdf.begin() + lo, cdf.begin() + hi + 1, x);
        uint64_t i = (uint64_t)(it - cdf.begin());
        if (i >= cdf.size()) i = cdf.size() - 1;
        return i + 1;
    }
};

constexpr uint64_t PERM_K2 = 0x2545F4914F6CDD1DULL;
constexpr uint64_t PERM_USER = 0x9FB21C651E98DF25ULL;

}  // namespace

extern "C" {

// 0-based i-th output of splitmix64 seeded with s (exported for tests).
uint64_t tdg_splitmix_at(uint64_t s, uint64_t i) { return sm_at(s, i); }
uint64_t tdg_mix64(uint64_t x) { return mix64(x); }

// plain: 1,024 BIGINT keys, INT values in [-1e6, 1e6].
void tdg_plain(uint64_t n, uint64_t seed, int64_t *k, int32_t *v, int threads) {
    int64_t keys[1024];
    for (uint64_t j = 0; j < 1024; ++j) keys[j] = (int64_t)sm_at(1, j);
    uint64_t sk = stream_seed(seed, 1), sv = stream_seed(seed, 2);
    parallel_rows(n, threads, [&](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; ++i) {
            k[i] = keys[sm_at(sk, i) % 1024];
            v[i] = (int32_t)((int64_t)(sm_at(sv, i) % 2000001ULL) - 1000000);
        }
    });
}

// filtered: Zipf(1.1) BIGINT key over `n_keys` values, DECIMAL(18,2) cents
// amount (log-normal mu=8 sigma=1.5, clipped to [1, 1e12]), DATE over 365 days
// from 2026-01-01 (20454 days since the epoch).
void tdg_filtered(uint64_t n, uint64_t seed, uint64_t n_keys, int64_t *k, int64_t *amount,
                  int32_t *d, int threads) {
    Zipf z(n_keys, 1.1);
    uint64_t sk = stream_seed(seed, 11), sa = stream_seed(seed, 12), sb = stream_seed(seed, 13),
             sd = stream_seed(seed, 14);
    parallel_rows(n, threads, [&](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; ++i) {
            uint64_t r = z.rank(unit(sm_at(sk, i)));
            k[i] = (int64_t)mix64(r ^ PERM_K2);
            double u1 = unit(sm_at(sa, i)), u2 = unit(sm_at(sb, i));
            if (u1 < 1e-300) u1 = 1e-300;
            double g = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
            double a = std::exp(8.0 + 1.5 * g);
            long long c = std::llround(a);
            if (c < 1) c = 1;
            if (a > 1e12 || c > 1000000000000LL) c = 1000000000000LL;
            amount[i] = c;
            d[i] = 20454 + (int32_t)(sm_at(sd, i) % 365);
        }
    });
}

// batched extra keys: INT uniform over 10, 1,000 and 1,000,000 values.
void tdg_extra_keys(uint64_t n, uint64_t seed, int32_t *k10, int32_t *k1k, int32_t *k1m, int threads) {
    uint64_t s1 = stream_seed(seed, 21), s2 = stream_seed(seed, 22), s3 = stream_seed(seed, 23);
    parallel_rows(n, threads, [&](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; ++i) {
            k10[i] = (int32_t)(sm_at(s1, i) % 10);
            k1k[i] = (int32_t)(sm_at(s2, i) % 1000);
            k1m[i] = (int32_t)(sm_at(s3, i) % 1000000);
        }
    });
}

// distinct: region SMALLINT, url DICT32 code, user_id BIGINT Zipf(0.9) over
// `n_users`, latency DOUBLE exponential(mean 120).
void tdg_distinct(uint64_t n, uint64_t seed, uint64_t n_users, int16_t *region, int32_t *url,
                  int64_t *user, double *latency, int threads) {
    Zipf z(n_users, 0.9);
    uint64_t sr = stream_seed(seed, 31), su = stream_seed(seed, 32), sz = stream_seed(seed, 33),
             sl = stream_seed(seed, 34);
    parallel_rows(n, threads, [&](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; ++i) {
            int32_t r = (int32_t)(sm_at(sr, i) % 64);
            region[i] = (int16_t)r;
            url[i] = (int32_t)(((uint64_t)r * 781ULL + sm_at(su, i) % 6250ULL) % 50000ULL);
            user[i] = (int64_t)mix64(z.rank(unit(sm_at(sz, i))) ^ PERM_USER);
            latency[i] = -120.0 * std::log1p(-unit(sm_at(sl, i)));
        }
    });
}

// The url dictionary: `count` strings of length U[8, 64] over [a-z0-9/.].
// offsets has count+1 entries; returns the bytes needed (writes only when
// bytes != nullptr and cap suffices).
uint64_t tdg_url_dictionary(uint64_t seed, uint32_t count, uint32_t *offsets, uint8_t *bytes, uint64_t cap) {
    static const char ALPHA[] = "abcdefghijklmnopqrstuvwxyz0123456789/.";
    uint64_t s = stream_seed(seed, 41);
    uint64_t pos = 0;
    for (uint32_t i = 0; i < count; ++i) {
        uint64_t h = sm_at(s, i);
        uint32_t len = 8 + (uint32_t)(h % 57);
        if (offsets) offsets[i] = (uint32_t)pos;
        for (uint32_t j = 0; j < len; ++j) {
            uint64_t c = mix64(h + j * GOLDEN) % 38;
            if (bytes && pos + j < cap) bytes[pos + j] = (uint8_t)ALPHA[c];
        }
        pos += len;
    }
    if (offsets) offsets[count] = (uint32_t)pos;
    return pos;
}

}  // extern "C"
