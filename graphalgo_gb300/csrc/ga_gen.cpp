// Seeded synthetic graph generators (host side): R-MAT, Erdos-Renyi G(n, m)
// and Gaussian k-nearest-neighbour graphs. Output: sorted, duplicate-free,
// loop-free, symmetric int32 CSR in malloc'd arrays.
//
// Random numbers: splitmix64 seeding and xoshiro256** streams, one stream per
// fixed-size chunk of edges, so results do not depend on the thread count.
// R-MAT and Erdos-Renyi use integer and uniform arithmetic only and are
// bit-identical on every platform; the Gaussian points use the C library's
// log/cos (Box-Muller).
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <thread>
#include <unordered_set>
#include <vector>

#include "../../include/graphalgo_gb300.h"

namespace {

inline uint64_t splitmix64(uint64_t& x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct Xoshiro {
    uint64_t s[4];
    explicit Xoshiro(uint64_t seed) {
        uint64_t x = seed;
        for (int i = 0; i < 4; ++i) s[i] = splitmix64(x);
    }
    static inline uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
    inline uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    inline double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    // unbiased integer in [0, n)
    inline uint64_t below(uint64_t n) {
        uint64_t lim = (~0ull) - ((~0ull) % n);
        uint64_t r;
        do { r = next(); } while (r >= lim);
        return r % n;
    }
};

uint64_t stream_seed(uint64_t seed, uint64_t chunk) {
    uint64_t x = seed ^ (0xD1B54A32D192ED03ull * (chunk + 1));
    return splitmix64(x);
}

unsigned worker_count() {
    unsigned t = std::thread::hardware_concurrency();
    return t == 0 ? 1 : (t > 32 ? 32 : t);
}

template <typename F>
void parallel_chunks(int64_t nchunks, F f) {
    unsigned T = worker_count();
    std::vector<std::thread> th;
    for (unsigned w = 0; w < T; ++w)
        th.emplace_back([&, w]() {
            for (int64_t c = w; c < nchunks; c += T) f(c);
        });
    for (auto& t : th) t.join();
}

// LSD radix sort of 64-bit keys on their low `bits` bits.
void radix_sort(std::vector<uint64_t>& keys, int bits) {
    std::vector<uint64_t> tmp(keys.size());
    const int D = 11;
    for (int shift = 0; shift < bits; shift += D) {
        std::vector<size_t> cnt((1u << D) + 1, 0);
        const uint64_t mask = (1ull << D) - 1;
        for (uint64_t k : keys) ++cnt[((k >> shift) & mask) + 1];
        for (size_t i = 1; i < cnt.size(); ++i) cnt[i] += cnt[i - 1];
        for (uint64_t k : keys) tmp[cnt[(k >> shift) & mask]++] = k;
        keys.swap(tmp);
    }
}

// Symmetrise (u,v) pairs, drop loops and duplicates, build CSR.
int build_csr(int64_t n, std::vector<uint64_t>& pairs, int64_t* m, int64_t* nnz, int32_t** rst, int32_t** col) {
    int bits = 1;
    while ((1ll << bits) < n) ++bits;
    radix_sort(pairs, 2 * bits);
    size_t w = 0;
    for (size_t i = 0; i < pairs.size(); ++i)
        if (i == 0 || pairs[i] != pairs[i - 1]) pairs[w++] = pairs[i];
    pairs.resize(w);
    if ((int64_t)w > INT32_MAX) return GA_ERR_UNSUPPORTED;
    int32_t* r = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n + 1));
    int32_t* c = (int32_t*)malloc(sizeof(int32_t) * (w ? w : 1));
    if (!r || !c) { free(r); free(c); return GA_ERR_OOM; }
    std::memset(r, 0, sizeof(int32_t) * (size_t)(n + 1));
    for (size_t i = 0; i < w; ++i) {
        ++r[(pairs[i] >> bits) + 1];
        c[i] = (int32_t)(pairs[i] & ((1ull << bits) - 1));
    }
    for (int64_t i = 0; i < n; ++i) r[i + 1] += r[i];
    *m = n; *nnz = (int64_t)w; *rst = r; *col = c;
    return GA_OK;
}

}  // namespace

extern "C" {

void ga_host_free(void* p) { free(p); }

int ga_gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed, int64_t* m, int64_t* nnz,
                int32_t** rst, int32_t** col) {
    if (scale < 1 || scale > 30 || edge_factor < 1 || !m || !nnz || !rst || !col) return GA_ERR_INVALID_ARG;
    if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return GA_ERR_INVALID_ARG;
    try {
        const int64_t n = 1ll << scale;
        const int64_t edges = n * edge_factor;
        const int64_t chunk = 1 << 16;
        const int64_t nchunks = (edges + chunk - 1) / chunk;
        std::vector<uint64_t> pairs((size_t)(2 * edges));
        std::vector<uint8_t> keep((size_t)edges, 1);
        const double ab = a + b, abc = a + b + c;
        parallel_chunks(nchunks, [&](int64_t ch) {
            Xoshiro rng(stream_seed(seed, (uint64_t)ch));
            int64_t e0 = ch * chunk, e1 = std::min(edges, e0 + chunk);
            for (int64_t e = e0; e < e1; ++e) {
                uint64_t u = 0, v = 0;
                for (int l = 0; l < scale; ++l) {
                    double r = rng.uniform();
                    int bu = 0, bv = 0;
                    if (r < a) { }
                    else if (r < ab) { bv = 1; }
                    else if (r < abc) { bu = 1; }
                    else { bu = 1; bv = 1; }
                    u = (u << 1) | (uint64_t)bu;
                    v = (v << 1) | (uint64_t)bv;
                }
                pairs[(size_t)(2 * e)] = (u << scale) | v;
                pairs[(size_t)(2 * e + 1)] = (v << scale) | u;
                if (u == v) keep[(size_t)e] = 0;
            }
        });
        size_t w = 0;
        for (int64_t e = 0; e < edges; ++e)
            if (keep[(size_t)e]) {
                pairs[w++] = pairs[(size_t)(2 * e)];
                pairs[w++] = pairs[(size_t)(2 * e + 1)];
            }
        pairs.resize(w);
        return build_csr(n, pairs, m, nnz, rst, col);
    } catch (const std::bad_alloc&) {
        return GA_ERR_OOM;
    }
}

int ga_gen_er(int64_t n, int64_t edges, uint64_t seed, int64_t* m, int64_t* nnz, int32_t** rst, int32_t** col) {
    if (n < 1 || edges < 0 || !m || !nnz || !rst || !col) return GA_ERR_INVALID_ARG;
    if ((double)edges > (double)n * (double)(n - 1) / 2.0) return GA_ERR_INVALID_ARG;
    try {
        int bits = 1;
        while ((1ll << bits) < n) ++bits;
        Xoshiro rng(stream_seed(seed, 0));
        std::unordered_set<uint64_t> seen;
        seen.reserve((size_t)edges * 2);
        std::vector<uint64_t> pairs;
        pairs.reserve((size_t)edges * 2);
        while ((int64_t)seen.size() < edges) {
            uint64_t u = rng.below((uint64_t)n), v = rng.below((uint64_t)n);
            if (u == v) continue;
            if (u > v) std::swap(u, v);
            uint64_t key = (u << bits) | v;
            if (seen.insert(key).second) {
                pairs.push_back(key);
                pairs.push_back((v << bits) | u);
            }
        }
        return build_csr(n, pairs, m, nnz, rst, col);
    } catch (const std::bad_alloc&) {
        return GA_ERR_OOM;
    }
}

int ga_gen_knn(int64_t n, int dim, int k, uint64_t seed, int64_t* m, int64_t* nnz, int32_t** rst, int32_t** col) {
    if (n < 2 || dim < 1 || k < 1 || !m || !nnz || !rst || !col) return GA_ERR_INVALID_ARG;
    try {
        const int kk = (int)std::min<int64_t>(k, n - 1);
        std::vector<double> pts((size_t)(n * dim));
        {
            Xoshiro rng(stream_seed(seed, 0));
            for (size_t i = 0; i < pts.size(); i += 2) {
                double u1 = rng.uniform(), u2 = rng.uniform();
                if (u1 < 1e-300) u1 = 1e-300;
                double rad = std::sqrt(-2.0 * std::log(u1));
                double th = 6.283185307179586 * u2;
                pts[i] = rad * std::cos(th);
                if (i + 1 < pts.size()) pts[i + 1] = rad * std::sin(th);
            }
        }
        int bits = 1;
        while ((1ll << bits) < n) ++bits;
        std::vector<uint64_t> pairs((size_t)(2 * n * kk));
        const int64_t chunk = 64;
        const int64_t nchunks = (n + chunk - 1) / chunk;
        parallel_chunks(nchunks, [&](int64_t ch) {
            std::vector<std::pair<double, int64_t>> cand((size_t)(n - 1));
            for (int64_t i = ch * chunk; i < std::min(n, (ch + 1) * chunk); ++i) {
                const double* pi = &pts[(size_t)(i * dim)];
                size_t w = 0;
                for (int64_t j = 0; j < n; ++j) {
                    if (j == i) continue;
                    const double* pj = &pts[(size_t)(j * dim)];
                    double d2 = 0.0;
                    for (int t = 0; t < dim; ++t) {
                        double df = pi[t] - pj[t];
                        d2 += df * df;
                    }
                    cand[w++] = {d2, j};
                }
                std::partial_sort(cand.begin(), cand.begin() + kk, cand.end());
                for (int t = 0; t < kk; ++t) {
                    uint64_t u = (uint64_t)i, v = (uint64_t)cand[(size_t)t].second;
                    pairs[(size_t)(2 * (i * kk + t))] = (u << bits) | v;
                    pairs[(size_t)(2 * (i * kk + t) + 1)] = (v << bits) | u;
                }
            }
        });
        return build_csr(n, pairs, m, nnz, rst, col);
    } catch (const std::bad_alloc&) {
        return GA_ERR_OOM;
    }
}

}  // extern "C"
