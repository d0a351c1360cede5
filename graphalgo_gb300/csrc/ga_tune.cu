// Autotuner for the masked products: times candidate schedules (variant,
// bin thresholds, persistent grid size, inner-product chunk) on the caller's
// own problem, with the L2 flushed before each run, and keeps the fastest per
// problem signature (device, kind, half-octave buckets of the sizes,
// symmetry) in a process-wide cache. Calls with GA_AUTO resolve to the cached
// choice, tuning on first use. Every candidate computes the same values, so
// tuning changes only speed. The context's work counters are restored
// afterwards: tuning launches are not counted as work.
#include "ga_internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <functional>
#include <mutex>
#include <tuple>

namespace ga {

namespace {

struct Cand {
    ga_algo algo;
    MxmTune t;
};

struct TuneEntry {
    ga_algo algo = GA_MSA;
    MxmTune t;
    double ms = 0.0, default_ms = 0.0;
    int candidates = 0;
};

using TuneKey = std::tuple<int, int, int, int, int, int, int, int, int>;

std::mutex g_tune_mu;
std::map<TuneKey, TuneEntry> g_tune_cache;

int bucket(int64_t x) { return x <= 0 ? 0 : 1 + (int)std::floor(2.0 * std::log2((double)x)); }

MxmTune tune_of(int64_t warp_max, int ctas, int chunk, int64_t ratio = 16) {
    MxmTune t;
    t.warp_max_flops = warp_max;
    t.ctas_per_sm = ctas;
    t.dot_chunk = chunk;
    t.hybrid_ratio = ratio;
    return t;
}

// Candidates, the default MSA schedule first; `only` >= 0 keeps one variant
// (its schedules only). tri_ok: the operands are one symmetric 0/1 matrix.
std::vector<Cand> product_candidates(bool dot_ok, int only, bool tri_ok = false) {
    std::vector<Cand> c;
    if (only < 0 || only == GA_MSA) {
        c.push_back({GA_MSA, MxmTune()});
        c.push_back({GA_MSA, tune_of(8192, 0, 8)});
        c.push_back({GA_MSA, tune_of(131072, 0, 8)});
        c.push_back({GA_MSA, tune_of(32768, 1, 8)});
        c.push_back({GA_MSA, tune_of(131072, 1, 8)});
    }
    if (only < 0 || only == GA_MCA) {
        c.push_back({GA_MCA, MxmTune()});
        if (only == GA_MCA) c.push_back({GA_MCA, tune_of(131072, 0, 8)});
    }
    if (dot_ok && (only < 0 || only == GA_DOT))
        for (int chunk : {4, 8, 16}) c.push_back({GA_DOT, tune_of(32768, 0, chunk)});
    if (dot_ok && (only < 0 || only == GA_HYBRID))
        for (int64_t ratio : {4, 16, 64}) c.push_back({GA_HYBRID, tune_of(32768, 0, 8, ratio)});
    if (tri_ok && (only < 0 || only == GA_TRI))
        for (int order : {0, 1}) {
            MxmTune t;
            t.tri_order = order;
            c.push_back({GA_TRI, t});
        }
    return c;
}

// Saves the context's work counters and puts them back on scope exit.
struct CounterGuard {
    ga_ctx ctx;
    unsigned long long saved[GA_CTR_COUNT];
    explicit CounterGuard(ga_ctx c) : ctx(c) {
        GA_CUDA(cudaMemcpyAsync(saved, ctx->d_counters, sizeof(saved), cudaMemcpyDeviceToHost, ctx->stream));
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    ~CounterGuard() {
        cudaMemcpyAsync(ctx->d_counters, saved, sizeof(saved), cudaMemcpyHostToDevice, ctx->stream);
        cudaStreamSynchronize(ctx->stream);
    }
};

double time_once(ga_ctx ctx, const std::function<void()>& f) {
    if (ga_ctx_flush_l2(ctx) != GA_OK) fail(GA_ERR_CUDA, ctx->last_error);
    cudaEvent_t a, b;
    GA_CUDA(cudaEventCreate(&a));
    GA_CUDA(cudaEventCreate(&b));
    float ms = 0.f;
    try {
        GA_CUDA(cudaEventRecord(a, ctx->stream));
        f();
        GA_CUDA(cudaEventRecord(b, ctx->stream));
        GA_CUDA(cudaEventSynchronize(b));
        GA_CUDA(cudaEventElapsedTime(&ms, a, b));
    } catch (...) {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        throw;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms;
}

// Runs every candidate once after one untimed warm-up of the first, times
// the three fastest and the default once more (each keeps its better run),
// and returns the fastest.
TuneEntry pick(ga_ctx ctx, const std::vector<Cand>& cands, const std::function<void(const Cand&)>& run) {
    CounterGuard cg(ctx);
    const MxmTune saved = ctx->tune;
    TuneEntry best;
    try {
        ctx->tune = cands[0].t;
        run(cands[0]);
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
        std::vector<double> ms(cands.size());
        for (size_t i = 0; i < cands.size(); ++i) {
            ctx->tune = cands[i].t;
            ms[i] = time_once(ctx, [&] { run(cands[i]); });
        }
        std::vector<size_t> order(cands.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = i;
        std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return ms[a] < ms[b]; });
        std::vector<size_t> again(order.begin(), order.begin() + std::min<size_t>(3, order.size()));
        if (std::find(again.begin(), again.end(), (size_t)0) == again.end()) again.push_back(0);
        for (size_t i : again) {
            ctx->tune = cands[i].t;
            ms[i] = std::min(ms[i], time_once(ctx, [&] { run(cands[i]); }));
        }
        best.ms = INFINITY;
        for (size_t i = 0; i < cands.size(); ++i)
            if (ms[i] < best.ms) {
                best.ms = ms[i];
                best.algo = cands[i].algo;
                best.t = cands[i].t;
            }
        best.default_ms = ms[0];
    } catch (...) {
        ctx->tune = saved;
        throw;
    }
    ctx->tune = saved;
    best.candidates = (int)cands.size();
    return best;
}

TuneEntry tune_support(ga_ctx ctx, ga_csr A, int only) {
    const int64_t m = A->m, nnz = A->nnz;
    const bool sym = csr_is_symmetric(ctx, A);
    const bool unit = csr_unit_values(ctx, A);
    DBuf<int32_t> sup(ctx, (size_t)nnz + 1), ust(ctx, (size_t)m + 1);
    DBuf<unsigned char> scr(ctx, mxm_scratch_bytes(m, m, nnz));
    ga_csr_s Au = *A;
    if (sym) {
        upper_starts(ctx, A, ust.p);
        Au.rst = ust.p;
    }
    ga_csr M = sym ? &Au : A;
    const int32_t* mre = sym ? A->rst + 1 : nullptr;
    // triangle listing: the k-truss loop's buffers (rows, mirrors, positions)
    const bool tri_ok = sym && unit && A->dtype == GA_INT32 && (only < 0 || only == GA_TRI);
    const size_t aux = tri_ok ? (size_t)nnz + 1 : 1;
    DBuf<int32_t> row_of(ctx, aux), mir(ctx, aux), pos(ctx, aux);
    DBuf<unsigned char> tscr(ctx, tri_ok ? tri_scratch_bytes(m, nnz) : 1);
    if (tri_ok) {
        expand_rows(ctx, A, row_of.p);
        mirror_index(ctx, A, row_of.p, mir.p);
    }
    auto support = [&](const Cand& c) {
        if (c.algo == GA_TRI) {
            tri_prepare(ctx, A, tscr.p, nnz);  // ranks of the candidate's order (ctx->tune)
            tri_support_launch(ctx, A, row_of.p, mir.p, pos.p, sup.p, tscr.p, nnz, true);
        } else if (c.algo == GA_DOT) mxm_dot_launch(ctx, A, A, A, M, sup.p, unit, mre);
        else mxm_masked_launch(ctx, c.algo, A, A, M, sup.p, scr.p, nnz, unit, mre, unit,
                               c.algo == GA_HYBRID ? A : nullptr);
    };
    const std::vector<Cand> cands = product_candidates(sym, only, tri_ok);
    if (!tri_ok || !ctx->kt_frontier) return pick(ctx, cands, support);
    // With the frontier loop GA_TRI lists the triangles once per call, while
    // the other forms compute the support in every iteration: whole 4-truss
    // calls are compared. A candidate whose single support product already
    // takes longer than the fastest GA_TRI 4-truss cannot win and is not run.
    auto whole = [&](const Cand& c) { csr_destroy(ctx, ktruss_impl(ctx, c.algo, A, 4, nullptr, nullptr)); };
    std::vector<Cand> finalists;
    {
        CounterGuard cg(ctx);
        const MxmTune saved = ctx->tune;
        double t_tri = INFINITY;
        try {
            for (const Cand& c : cands)
                if (c.algo == GA_TRI) {
                    ctx->tune = c.t;
                    whole(c);
                    t_tri = std::min(t_tri, time_once(ctx, [&] { whole(c); }));
                    finalists.push_back(c);
                }
            for (const Cand& c : cands)
                if (c.algo != GA_TRI) {
                    ctx->tune = c.t;
                    if (time_once(ctx, [&] { support(c); }) < t_tri) finalists.push_back(c);
                }
        } catch (...) {
            ctx->tune = saved;
            throw;
        }
        ctx->tune = saved;
    }
    TuneEntry e = pick(ctx, finalists, whole);
    e.candidates = (int)cands.size();
    return e;
}

TuneEntry tune_product(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr M, int only) {
    DBuf<unsigned char> cv(ctx, (size_t)(M->nnz + 1) * dtype_size(A->dtype));
    return pick(ctx, product_candidates(true, only, tri_applies(ctx, A, B, M)),
                [&](const Cand& c) { mxm_masked_into(ctx, c.algo, A, B, M, cv.p); });
}

TuneEntry tune_tc(ga_ctx ctx, ga_csr A, int only) {
    DBuf<int64_t> tot(ctx, 1);
    std::vector<Cand> all = {{GA_MSA, MxmTune()}, {GA_DOT, MxmTune()}, {GA_MCA, MxmTune()},
                             {GA_MSA, tune_of(8192, 0, 8)}, {GA_MSA, tune_of(131072, 0, 8)}};
    if (csr_is_symmetric(ctx, A))
        for (int order : {0, 1}) {
            MxmTune t;
            t.tri_order = order;
            all.push_back({GA_TRI, t});
        }
    std::vector<Cand> c;
    for (const Cand& x : all)
        if (only < 0 || x.algo == only) c.push_back(x);
    return pick(ctx, c, [&](const Cand& x) {
        const int rc = ga_tc_device(ctx, x.algo, A, tot.p, nullptr);
        if (rc != GA_OK) fail(rc, ctx->last_error);
    });
}

TuneEntry lookup_or_tune(ga_ctx ctx, int kind, ga_csr A, ga_csr B, ga_csr M, bool force, bool* cached,
                         int only = -1) {
    // the candidate set depends on symmetry and, for triangle listing, unit values
    const bool sym = csr_is_symmetric(ctx, A);
    const int shape = sym ? (csr_unit_values(ctx, A) ? 2 : 1) : 0;
    const TuneKey key{ctx->device, kind, bucket(A->m), bucket(A->n), bucket(A->nnz), bucket(B ? B->nnz : 0),
                      bucket(M ? M->nnz : 0), shape, only};
    if (!force) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            if (cached) *cached = true;
            return it->second;
        }
    }
    TuneEntry e = kind == GA_TUNE_KTRUSS ? tune_support(ctx, A, only)
                  : kind == GA_TUNE_TC   ? tune_tc(ctx, A, only)
                                         : tune_product(ctx, A, B, M, only);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = e;
    }
    if (cached) *cached = false;
    return e;
}

}  // namespace

ga_algo resolve_ktruss_algo(ga_ctx ctx, ga_algo algo, ga_csr A) {
    if (algo != GA_AUTO) return algo;
    if (A->m == 0 || A->nnz == 0) return GA_MSA;
    const TuneEntry e = lookup_or_tune(ctx, GA_TUNE_KTRUSS, A, nullptr, nullptr, false, nullptr);
    ctx->tune = e.t;
    return e.algo;
}

ga_algo resolve_tc_algo(ga_ctx ctx, ga_algo algo, ga_csr A) {
    if (algo != GA_AUTO) return algo;
    if (A->m == 0 || A->nnz == 0) return GA_DOT;
    const TuneEntry e = lookup_or_tune(ctx, GA_TUNE_TC, A, nullptr, nullptr, false, nullptr);
    ctx->tune = e.t;
    return e.algo;
}

ga_algo resolve_mxm_algo(ga_ctx ctx, ga_algo algo, ga_csr A, ga_csr B, ga_csr M) {
    if (algo != GA_AUTO) return algo;
    if (M->nnz == 0 || A->nnz == 0 || B->nnz == 0) return GA_MSA;
    const TuneEntry e = lookup_or_tune(ctx, GA_TUNE_PRODUCT, A, B, M, false, nullptr);
    ctx->tune = e.t;
    return e.algo;
}

}  // namespace ga

using namespace ga;

extern "C" {

int ga_autotune(ga_ctx ctx, int kind, ga_csr A, ga_csr B, ga_csr M, int force, ga_tune_result* out) {
    return ga_autotune_variant(ctx, kind, -1, A, B, M, force, out);
}

int ga_autotune_variant(ga_ctx ctx, int kind, int algo, ga_csr A, ga_csr B, ga_csr M, int force,
                        ga_tune_result* out) {
    if (!ctx || !A || !out) return GA_ERR_INVALID_ARG;
    if (algo != -1 && algo != GA_MSA && algo != GA_MCA && algo != GA_DOT && algo != GA_HYBRID && algo != GA_TRI)
        return GA_ERR_INVALID_ARG;
    if (kind != GA_TUNE_KTRUSS && kind != GA_TUNE_TC && kind != GA_TUNE_PRODUCT) return GA_ERR_INVALID_ARG;
    if (kind == GA_TUNE_PRODUCT && (!B || !M)) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        GA_REQUIRE(kind == GA_TUNE_PRODUCT || A->m == A->n, GA_ERR_SHAPE, "autotune: square matrix expected");
        GA_REQUIRE(A->nnz > 0, GA_ERR_INVALID_ARG, "autotune: empty matrix");
        bool cached = false;
        if ((algo == GA_DOT || algo == GA_HYBRID) && kind == GA_TUNE_KTRUSS)
            GA_REQUIRE(csr_is_symmetric(ctx, A), GA_ERR_UNSUPPORTED,
                       "autotune: GA_DOT / GA_HYBRID k-truss needs a symmetric matrix");
        const TuneEntry e = lookup_or_tune(ctx, kind, A, B, M, force != 0, &cached, algo);
        out->algo = e.algo;
        out->warp_max_flops = e.t.warp_max_flops;
        out->heavy_flops = e.t.heavy_flops;
        out->ctas_per_sm = e.t.ctas_per_sm;
        out->dot_chunk = e.t.dot_chunk;
        out->hybrid_ratio = e.t.hybrid_ratio;
        out->ms = e.ms;
        out->default_ms = e.default_ms;
        out->candidates = e.candidates;
        out->cached = cached ? 1 : 0;
        out->tri_order = e.t.tri_order;
    });
}

// Cache file: one line per entry, "ga_tune 1" then the key's nine fields
// (device, kind, size buckets of m, n, nnz(A), nnz(B), nnz(M), shape,
// restriction) and the entry (variant, warp threshold, heavy threshold, CTAs
// per SM, inner-product chunk, hybrid ratio, vertex order, its time, the
// default's time, candidates).
int ga_tune_save(const char* path, int64_t* entries) {
    if (!path) return GA_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    FILE* f = fopen(path, "w");
    if (!f) return GA_ERR_INVALID_ARG;
    int64_t n = 0;
    for (const auto& kv : g_tune_cache) {
        const TuneKey& k = kv.first;
        const TuneEntry& e = kv.second;
        fprintf(f, "ga_tune 1 %d %d %d %d %d %d %d %d %d  %d %lld %lld %d %d %lld %d %.9g %.9g %d\n",
                std::get<0>(k), std::get<1>(k), std::get<2>(k), std::get<3>(k), std::get<4>(k), std::get<5>(k),
                std::get<6>(k), std::get<7>(k), std::get<8>(k), (int)e.algo, (long long)e.t.warp_max_flops,
                (long long)e.t.heavy_flops, e.t.ctas_per_sm, e.t.dot_chunk, (long long)e.t.hybrid_ratio,
                e.t.tri_order, e.ms, e.default_ms, e.candidates);
        ++n;
    }
    const bool ok = fclose(f) == 0;
    if (entries) *entries = n;
    return ok ? GA_OK : GA_ERR_INVALID_ARG;
}

int ga_tune_load(const char* path, int64_t* entries) {
    if (!path) return GA_ERR_INVALID_ARG;
    FILE* f = fopen(path, "r");
    if (!f) return GA_ERR_INVALID_ARG;
    std::vector<std::pair<TuneKey, TuneEntry>> got;
    char line[512];
    int rc = GA_OK;
    while (fgets(line, sizeof(line), f)) {
        int ver = 0, k[9], algo = 0, ctas = 0, chunk = 0, order = 0, cands = 0;
        long long warp = 0, heavy = 0, ratio = 0;
        double ms = 0, dms = 0;
        const int got_fields = sscanf(line, "ga_tune %d %d %d %d %d %d %d %d %d %d %d %lld %lld %d %d %lld %d %lg %lg %d",
                                      &ver, &k[0], &k[1], &k[2], &k[3], &k[4], &k[5], &k[6], &k[7], &k[8], &algo,
                                      &warp, &heavy, &ctas, &chunk, &ratio, &order, &ms, &dms, &cands);
        if (got_fields != 20 || ver != 1 || algo < GA_MSA || algo > GA_TRI || algo == GA_AUTO || ctas < 0 ||
            chunk < 1 || chunk > 4096 || ratio < 0 || (order != 0 && order != 1)) {
            rc = GA_ERR_INVALID_ARG;  // a malformed file loads nothing
            break;
        }
        TuneEntry e;
        e.algo = (ga_algo)algo;
        e.t.warp_max_flops = warp;
        e.t.heavy_flops = heavy;
        e.t.ctas_per_sm = ctas;
        e.t.dot_chunk = chunk;
        e.t.hybrid_ratio = ratio;
        e.t.tri_order = order;
        e.ms = ms;
        e.default_ms = dms;
        e.candidates = cands;
        got.emplace_back(TuneKey{k[0], k[1], k[2], k[3], k[4], k[5], k[6], k[7], k[8]}, e);
    }
    fclose(f);
    if (rc != GA_OK) return rc;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (const auto& kv : got) g_tune_cache[kv.first] = kv.second;
    if (entries) *entries = (int64_t)got.size();
    return GA_OK;
}

int ga_tune_clear(void) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache.clear();
    return GA_OK;
}

}  // extern "C"
