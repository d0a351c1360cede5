// Drop-in test: the reference's call shapes (mxmOp plugins, k_truss,
// triangle_counting_*, betweenness_centrality_batch) compiled against
// include/graphalgo_gb300.hpp, checked against the CPU oracle.
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <vector>

#include "graphalgo_gb300.hpp"
#include "../../oracle/oracle.h"

using namespace ga;

static int failures = 0;
#define EXPECT(cond, ...)                                   \
    do {                                                    \
        if (!(cond)) {                                      \
            ++failures;                                     \
            std::fprintf(stderr, "FAIL %s:%d: ", __FILE__, __LINE__); \
            std::fprintf(stderr, __VA_ARGS__);              \
            std::fprintf(stderr, "\n");                     \
        }                                                   \
    } while (0)

static spMtx<int> graph_er(int64_t n, int64_t edges, uint64_t seed) {
    int64_t m, nnz;
    int32_t *rst, *col;
    check(ga_gen_er(n, edges, seed, &m, &nnz, &rst, &col));
    spMtx<int> A((size_t)m, (size_t)m, (size_t)nnz);
    std::memcpy(A.Rst, rst, sizeof(int) * (m + 1));
    std::memcpy(A.Col, col, sizeof(int) * nnz);
    for (int64_t j = 0; j < nnz; ++j) A.Val[j] = 1;
    ga_host_free(rst);
    ga_host_free(col);
    return A;
}

int main() {
    spMtx<int> A = graph_er(1000, 9990, 7);
    // the CLI's preparation (src/main.cpp:221-222)
    spMtx<int> S = build_symm_from_lower(extract_lower_triangle(A));
    EXPECT(S == A, "symmetrise(lower(A)) != A for a symmetric A");

    // triangle counting through each plugin (src/main.cpp:206-218 shapes)
    const int64_t expect_tc = or_tc_sandia((int64_t)A.m, A.Rst, A.Col, nullptr);
    mxmOp<int> ops[] = {mxmm_msa<int>, mxmm_mca<int>, mxmm_heap<int>, mxmm_naive<int>, mxmm_hybrid<int>,
                        mxmm_tri<int>};
    for (mxmOp<int> op : ops) {
        int64_t t = triangle_counting_masked_sandia(A, op, true);
        EXPECT(t == expect_tc, "sandia %lld != %lld", (long long)t, (long long)expect_tc);
        EXPECT(triangle_counting_masked_lu(A, op, true) == expect_tc, "lu form");
    }
    std::vector<int64_t> rows;
    EXPECT(triangle_counting_dot(A, &rows) == expect_tc, "dot form");
    std::vector<int64_t> ref_rows(A.m);
    or_tc_sandia((int64_t)A.m, A.Rst, A.Col, ref_rows.data());
    EXPECT(rows == ref_rows, "per-row counts");
    int* pv = triangle_counting_vertex(A, mxmm_msa<int>, true);
    int64_t sum = 0;
    for (size_t i = 0; i < A.m; ++i) sum += pv[i];
    EXPECT(sum == 3 * expect_tc, "per-vertex counts sum %lld", (long long)sum);
    delete[] pv;

    // masked product with an explicit C, as mxm in the CLI (src/main.cpp:235-240)
    spMtx<int> C;
    mxmm_msa<int>(true, A, A, A, C);
    std::vector<int> ref(A.nz);
    or_mxm_masked_i32((int64_t)A.m, (int64_t)A.n, A.Rst, A.Col, A.Val, A.Rst, A.Col, A.Val, A.Rst, A.Col, ref.data());
    bool same = C.nz == A.nz;
    for (size_t j = 0; same && j < C.nz; ++j) same = C.Val[j] == ref[j] && C.Col[j] == A.Col[j];
    EXPECT(same, "mxmm_msa values");
    spMtx<int> Ct;
    mxmm_tri<int>(true, A, A, A, Ct);
    same = Ct.nz == A.nz;
    for (size_t j = 0; same && j < Ct.nz; ++j) same = Ct.Val[j] == ref[j] && Ct.Col[j] == A.Col[j];
    EXPECT(same, "mxmm_tri values");

    // k-truss for several k with every plugin
    for (int k : {3, 4, 5}) {
        int *cr, *cc, *cv, it_ref;
        int64_t cnz;
        or_ktruss((int64_t)A.m, A.Rst, A.Col, A.Val, k, &cr, &cc, &cv, &cnz, &it_ref);
        for (mxmOp<int> op : {ops[0], ops[1], ops[2], ops[4], ops[5]}) {
            int it = -1;
            spMtx<int> T = k_truss(A, k, op, true, &it);
            bool eq = (int64_t)T.nz == cnz && it == it_ref;
            for (size_t i = 0; eq && i <= T.m; ++i) eq = T.Rst[i] == cr[i];
            for (int64_t j = 0; eq && j < cnz; ++j) eq = T.Col[j] == cc[j] && T.Val[j] == cv[j];
            EXPECT(eq, "k_truss k=%d", k);
        }
        or_free(cr); or_free(cc); or_free(cv);
    }

    // batched BC, sources 0..batch-1 (include/betweenness_centrality.h:125)
    std::vector<float> bcf = betweenness_centrality_batch(true, A, 32);
    std::vector<int> src(32);
    for (int j = 0; j < 32; ++j) src[j] = j;
    std::vector<double> bref(A.m);
    or_bc_batch((int64_t)A.m, A.Rst, A.Col, A.Val, 32, src.data(), bref.data());
    std::vector<double> bcd = betweenness_centrality_sources(A, src);
    for (size_t v = 0; v < A.m; ++v) {
        EXPECT(std::fabs(bcd[v] - bref[v]) <= 1e-9 * std::fmax(1.0, std::fabs(bref[v])), "bc[%zu]", v);
        EXPECT(std::fabs((double)bcf[v] - bref[v]) <= 1e-5 * std::fmax(1.0, std::fabs(bref[v])), "bc float[%zu]", v);
    }

    // all-source BC in blocks (include/betweenness_centrality.h:5), a ragged
    // last block; the reference's float result from FP64 device sums
    bool threw = false;
    std::vector<float> ball = betweenness_centrality(true, A, 48);
    std::vector<double> aref(A.m);
    or_bc_all((int64_t)A.m, A.Rst, A.Col, A.Val, 48, aref.data());
    for (size_t v = 0; v < A.m; ++v)
        EXPECT(std::fabs((double)ball[v] - aref[v]) <= 1e-5 * std::fmax(1.0, std::fabs(aref[v])), "bc all[%zu]", v);
    threw = false;
    try {
        betweenness_centrality(true, A, 0);  // the reference would never finish
    } catch (const ga::error&) {
        threw = true;
    }
    EXPECT(threw, "blockSize 0 must throw");

    // unknown plugins are rejected, not run on the host
    threw = false;
    try {
        triangle_counting_masked_sandia(A, [](bool, const spMtx<int>&, const spMtx<int>&, const spMtx<int>&,
                                              spMtx<int>&) {}, true);
    } catch (const ga::error&) {
        threw = true;
    }
    EXPECT(threw, "an unknown mxmOp must throw");

    if (failures) {
        std::fprintf(stderr, "%d failure(s)\n", failures);
        return 1;
    }
    std::printf("drop-in ok: %lld triangles\n", (long long)expect_tc);
    return 0;
}
