/*
 * Seeded R-MAT input generator for the oracle side (TEST INFRASTRUCTURE
 * ONLY: the reference arm of bench.py and the fixture scripts make their
 * inputs with it, so they never load the product's library).
 *
 * It restates the product's host generator (graphalgo_gb300/csrc/ga_gen.cpp,
 * ga_gen_rmat) so that both give the same graph bit for bit
 * (tests/test_host_logic.py checks this): edges in chunks of 2^16, each chunk
 * drawing from its own xoshiro256** stream seeded by splitmix64 of
 * (seed, chunk); per edge `scale` uniform draws pick the quadrant
 * (a / b / c / d); loops dropped; both directions of every edge kept;
 * duplicates merged; rows sorted. The reference has no R-MAT generator
 * (its include/matrix_utils.h generators are unseeded), so this is not a
 * restatement of reference code.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static uint64_t sm64(uint64_t* x) {
    uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

typedef struct {
    uint64_t s[4];
} xo256;

static uint64_t rotl64(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }

static uint64_t xo_next(xo256* g) {
    const uint64_t r = rotl64(g->s[1] * 5, 7) * 9;
    const uint64_t t = g->s[1] << 17;
    g->s[2] ^= g->s[0];
    g->s[3] ^= g->s[1];
    g->s[1] ^= g->s[2];
    g->s[0] ^= g->s[3];
    g->s[2] ^= t;
    g->s[3] = rotl64(g->s[3], 45);
    return r;
}

static double xo_uniform(xo256* g) { return (double)(xo_next(g) >> 11) * (1.0 / 9007199254740992.0); }

static void xo_seed(xo256* g, uint64_t seed, uint64_t chunk) {
    uint64_t x = seed ^ (0xD1B54A32D192ED03ull * (chunk + 1));
    uint64_t s0 = sm64(&x);
    for (int i = 0; i < 4; ++i) g->s[i] = sm64(&s0);
}

/* LSD radix sort of keys on their low `bits` bits, 11 bits per pass. */
static int radix_sort_u64(uint64_t* keys, size_t n, int bits) {
    uint64_t* tmp = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
    size_t* cnt = (size_t*)malloc(sizeof(size_t) * ((1u << 11) + 1));
    if (!tmp || !cnt) {
        free(tmp);
        free(cnt);
        return -1;
    }
    uint64_t *src = keys, *dst = tmp;
    for (int shift = 0; shift < bits; shift += 11) {
        memset(cnt, 0, sizeof(size_t) * ((1u << 11) + 1));
        for (size_t i = 0; i < n; ++i) ++cnt[((src[i] >> shift) & 2047u) + 1];
        for (size_t i = 1; i <= 2048; ++i) cnt[i] += cnt[i - 1];
        for (size_t i = 0; i < n; ++i) dst[cnt[(src[i] >> shift) & 2047u]++] = src[i];
        uint64_t* t = src;
        src = dst;
        dst = t;
    }
    if (src != keys) memcpy(keys, src, sizeof(uint64_t) * n);
    free(tmp);
    free(cnt);
    return 0;
}

int or_gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed, int64_t* m_out,
                int64_t* nnz_out, int** rst_out, int** col_out) {
    if (scale < 1 || scale > 30 || edge_factor < 1) return -1;
    const int64_t n = (int64_t)1 << scale;
    const int64_t edges = n * edge_factor;
    const int64_t chunk = 1 << 16;
    const int64_t nchunks = (edges + chunk - 1) / chunk;
    uint64_t* pairs = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(2 * edges));
    unsigned char* keep = (unsigned char*)malloc((size_t)edges);
    if (!pairs || !keep) {
        free(pairs);
        free(keep);
        return -2;
    }
    const double ab = a + b, abc = a + b + c;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t ch = 0; ch < nchunks; ++ch) {
        xo256 g;
        xo_seed(&g, seed, (uint64_t)ch);
        const int64_t e0 = ch * chunk, e1 = e0 + chunk < edges ? e0 + chunk : edges;
        for (int64_t e = e0; e < e1; ++e) {
            uint64_t u = 0, v = 0;
            for (int l = 0; l < scale; ++l) {
                const double r = xo_uniform(&g);
                int bu = 0, bv = 0;
                if (r < a) {
                } else if (r < ab) {
                    bv = 1;
                } else if (r < abc) {
                    bu = 1;
                } else {
                    bu = 1;
                    bv = 1;
                }
                u = (u << 1) | (uint64_t)bu;
                v = (v << 1) | (uint64_t)bv;
            }
            pairs[2 * e] = (u << scale) | v;
            pairs[2 * e + 1] = (v << scale) | u;
            keep[e] = u != v;
        }
    }
    size_t w = 0;
    for (int64_t e = 0; e < edges; ++e)
        if (keep[e]) {
            pairs[w++] = pairs[2 * e];
            pairs[w++] = pairs[2 * e + 1];
        }
    free(keep);
    int bits = 1;
    while (((int64_t)1 << bits) < n) ++bits;
    if (radix_sort_u64(pairs, w, 2 * bits) != 0) {
        free(pairs);
        return -2;
    }
    size_t u = 0;
    for (size_t i = 0; i < w; ++i)
        if (i == 0 || pairs[i] != pairs[i - 1]) pairs[u++] = pairs[i];
    int* rst = (int*)calloc((size_t)n + 1, sizeof(int));
    int* col = (int*)malloc(sizeof(int) * (u ? u : 1));
    if (!rst || !col) {
        free(pairs);
        free(rst);
        free(col);
        return -2;
    }
    for (size_t i = 0; i < u; ++i) {
        ++rst[(pairs[i] >> bits) + 1];
        col[i] = (int)(pairs[i] & (((uint64_t)1 << bits) - 1));
    }
    for (int64_t i = 0; i < n; ++i) rst[i + 1] += rst[i];
    free(pairs);
    *m_out = n;
    *nnz_out = (int64_t)u;
    *rst_out = rst;
    *col_out = col;
    return 0;
}
