// Test-only harness around the UNMODIFIED reference (UAlex322/GraphAlgo).
//
// This file is compiled by oracle/build_ref.sh against the reference's own
// headers and sources where they lie (include/matrix.h, include/matrix_la.h,
// include/betweenness_centrality.h, src/main.cpp, src/mmio.cpp). It is never
// part of the product: only the golden-fixture script and the CPU tests load
// the resulting oracle/_ref/libref.so, to pin the C restatement in
// oracle/oracle.c against the reference's real output.
//
// Known reference bugs are routed around here, never patched in the sources:
//  * mxmm_heap never zero-fills C.Val (matrix_la.h:1016-1017 with +=, 1069):
//    C is pre-sized with zeroed values so resizeVals keeps that storage.
//  * _mxmm_msa_sequential reads stale accumulator values (matrix_la.h:781-784):
//    MSA and MCA are always called with isParallel = true.
//  * mxmm_naive's parallel branch never sizes C (matrix_la.h:1155-1172):
//    naive is always called with isParallel = false.
#include <sstream>
#include <vector>
#include <string>
#include <cstdint>
#include <cstdlib>
#include <cstring>

#define main ref_cli_main
#include "main.cpp"   // src/main.cpp: k_truss, triangle_counting_* (and includes)
#undef main

namespace {

template <typename T>
spMtx<T> make_csr(int64_t m, int64_t n, int64_t nnz, const int* rst,
                  const int* col, const T* val) {
    spMtx<T> A((size_t)m, (size_t)n, (size_t)nnz);
    std::memcpy(A.Rst, rst, sizeof(int) * (m + 1));
    if (nnz) {
        std::memcpy(A.Col, col, sizeof(int) * nnz);
        if (val) std::memcpy(A.Val, val, sizeof(T) * nnz);
        else for (int64_t i = 0; i < nnz; ++i) A.Val[i] = (T)1;
    }
    A.matcode[0] = 'M'; A.matcode[1] = 'C'; A.matcode[2] = 'I'; A.matcode[3] = 'G';
    return A;
}

template <typename T>
void export_csr(const spMtx<T>& C, int64_t* m, int64_t* n, int64_t* nnz,
                int** rst, int** col, T** val) {
    *m = (int64_t)C.m; *n = (int64_t)C.n;
    int64_t z = C.Rst ? (int64_t)C.Rst[C.m] : 0;
    *nnz = z;
    *rst = (int*)std::malloc(sizeof(int) * (C.m + 1));
    std::memcpy(*rst, C.Rst, sizeof(int) * (C.m + 1));
    *col = (int*)std::malloc(sizeof(int) * (z ? z : 1));
    *val = (T*)std::malloc(sizeof(T) * (z ? z : 1));
    if (z) {
        std::memcpy(*col, C.Col, sizeof(int) * z);
        std::memcpy(*val, C.Val, sizeof(T) * z);
    }
}

template <typename T>
using op_t = void (*)(bool, const spMtx<T>&, const spMtx<T>&, const spMtx<T>&, spMtx<T>&);

template <typename T>
int run_mxm(int algo, const spMtx<T>& A, const spMtx<T>& B, const spMtx<T>& M, spMtx<T>& C) {
    switch (algo) {
    case 0: mxmm_msa<T, T>(true, A, B, M, C); return 0;
    case 1: mxmm_mca<T, T>(true, A, B, M, C); return 0;
    case 2: {
        // pre-size C with zeroed values; mxmm_heap's resizeVals keeps them.
        spMtx<T> Z(M.m, M.n, M.nz);
        C = std::move(Z);
        mxmm_heap<T>(true, A, B, M, C);
        return 0;
    }
    case 3: mxmm_naive<T>(false, A, B, M, C); return 0;
    default: return 1;
    }
}

op_t<int> int_op(int algo) {
    switch (algo) {
    case 0: return mxmm_msa<int, int>;
    case 1: return mxmm_mca<int, int>;
    case 3: return mxmm_naive<int>;
    default: return nullptr;
    }
}

// mxmm_heap with C zero-filled on entry (see header comment).
void heap_zeroed(bool par, const spMtx<int>& A, const spMtx<int>& B,
                 const spMtx<int>& M, spMtx<int>& C) {
    spMtx<int> Z(M.m, M.n, M.nz);
    C = std::move(Z);
    mxmm_heap<int>(par, A, B, M, C);
}

// Naive must run its sequential branch; the CLI's isParallel is ignored.
void naive_seq(bool, const spMtx<int>& A, const spMtx<int>& B,
               const spMtx<int>& M, spMtx<int>& C) {
    mxmm_naive<int>(false, A, B, M, C);
}

op_t<int> ktruss_op(int algo) {
    switch (algo) {
    case 0: return mxmm_msa<int, int>;
    case 1: return mxmm_mca<int, int>;
    case 2: return heap_zeroed;
    case 3: return naive_seq;
    default: return nullptr;
    }
}

// eWiseAdd(A, B) (include/matrix_la.h:375-435) or, when `masked`,
// eWiseAdd(A, B, M) (272-335), on the reference's own code.
template <typename T>
int ewise_add_t(int masked, int64_t am, int64_t an, int64_t anz, const int* ar, const int* ac, const T* av,
                int64_t bnz, const int* br, const int* bc, const T* bv, int64_t mnz, const int* mr,
                const int* mc, int64_t* cm, int64_t* cn, int64_t* cnz, int** cr, int** cc, T** cv) {
    spMtx<T> A = make_csr<T>(am, an, anz, ar, ac, av);
    spMtx<T> B = make_csr<T>(am, an, bnz, br, bc, bv);
    spMtx<T> C;
    if (masked) {
        spMtx<T> M = make_csr<T>(am, an, mnz, mr, mc, nullptr);
        C = eWiseAdd<T, T>(A, B, M);
    } else {
        C = eWiseAdd<T>(A, B);
    }
    export_csr(C, cm, cn, cnz, cr, cc, cv);
    return 0;
}

}  // namespace

extern "C" {

void ref_free(void* p) { std::free(p); }

// Reads a Matrix Market file exactly as the reference CLI does
// (main.cpp:279-310 value type, matrix.h:280-417 reader, matrix.h:679-698
// adjacency), and optionally applies the CLI's symmetrisation
// build_symm_from_lower(extract_lower_triangle(.)) (main.cpp:221-222).
int ref_read_mtx(const char* path, int symmetrise, int64_t* m, int64_t* n,
                 int64_t* nnz, int** rst, int** col, int** val) {
    try {
        std::ifstream istr(path);
        std::string t;
        istr >> t >> t >> t >> t;
        istr.close();
        spMtx<int> adj;
        if (t == "real") {
            spMtx<double> g(path, "mtx");
            adj = build_adjacency_matrix(g);
        } else {
            spMtx<int> g(path, "mtx");
            adj = build_adjacency_matrix(g);
        }
        if (symmetrise) adj = build_symm_from_lower(extract_lower_triangle(adj));
        export_csr(adj, m, n, nnz, rst, col, val);
        return 0;
    } catch (...) {
        return 1;
    }
}

// Reads a graph file of `format` ("mtx", "bin", "graph", "rmat") with the
// value type the CLI picks for it (main.cpp:279-310) and returns the matrix
// exactly as read - before build_adjacency_matrix - with values widened to
// double and the four matcode bytes.
int ref_read_raw(const char* path, const char* format, int64_t* m, int64_t* n, int64_t* nnz,
                 int** rst, int** col, double** val, char* matcode) {
    try {
        GraphInfo info{"g", path, "", format};
        const std::string t = get_graph_val_type(path, info);
        spMtx<double> g;
        if (t == "real") {
            spMtx<double> r(path, format);
            g = r;
        } else {
            spMtx<int> r(path, format);
            g = spMtx<double>(r.m, r.n, r.nz);
            std::memcpy(g.Rst, r.Rst, sizeof(int) * (r.m + 1));
            for (size_t i = 0; i < r.nz; ++i) { g.Col[i] = r.Col[i]; g.Val[i] = r.Val[i]; }
            std::memcpy(g.matcode, r.matcode, 4);
        }
        std::memcpy(matcode, g.matcode, 4);
        export_csr(g, m, n, nnz, rst, col, val);
        return 0;
    } catch (...) {
        return 1;
    }
}

// The CLI's preparation of a graph file of any format: read, adjacency
// (matrix.h:679-698) and, when `symmetrise`, the lower-triangle
// symmetrisation every action but BC applies (main.cpp:221-222).
int ref_read_cli(const char* path, const char* format, int symmetrise, int64_t* m, int64_t* n,
                 int64_t* nnz, int** rst, int** col, int** val) {
    try {
        GraphInfo info{"g", path, "", format};
        const std::string t = get_graph_val_type(path, info);
        spMtx<int> adj;
        if (t == "real") {
            spMtx<double> g(path, format);
            adj = build_adjacency_matrix(g);
        } else {
            spMtx<int> g(path, format);
            adj = build_adjacency_matrix(g);
        }
        if (symmetrise) adj = build_symm_from_lower(extract_lower_triangle(adj));
        export_csr(adj, m, n, nnz, rst, col, val);
        return 0;
    } catch (...) {
        return 1;
    }
}

// The CLI's "tobinary" action (main.cpp:325-331): read `path` with the value
// type the CLI picks and write it with write_crs_to_bin (matrix.h:259-277).
int ref_tobinary(const char* path, const char* format, const char* out_path) {
    try {
        GraphInfo info{"g", path, "", format};
        const std::string t = get_graph_val_type(path, info);
        if (t == "real") {
            spMtx<double> g(path, format);
            return g.write_crs_to_bin(out_path) ? 1 : 0;
        }
        spMtx<int> g(path, format);
        return g.write_crs_to_bin(out_path) ? 1 : 0;
    } catch (...) {
        return 1;
    }
}

int ref_ewise_add_i32(int masked, int64_t am, int64_t an, int64_t anz, const int* ar, const int* ac,
                      const int* av, int64_t bnz, const int* br, const int* bc, const int* bv, int64_t mnz,
                      const int* mr, const int* mc, int64_t* cm, int64_t* cn, int64_t* cnz, int** cr, int** cc,
                      int** cv) {
    return ewise_add_t<int>(masked, am, an, anz, ar, ac, av, bnz, br, bc, bv, mnz, mr, mc, cm, cn, cnz, cr, cc, cv);
}

int ref_ewise_add_f64(int masked, int64_t am, int64_t an, int64_t anz, const int* ar, const int* ac,
                      const double* av, int64_t bnz, const int* br, const int* bc, const double* bv, int64_t mnz,
                      const int* mr, const int* mc, int64_t* cm, int64_t* cn, int64_t* cnz, int** cr, int** cc,
                      double** cv) {
    return ewise_add_t<double>(masked, am, an, anz, ar, ac, av, bnz, br, bc, bv, mnz, mr, mc, cm, cn, cnz, cr, cc,
                               cv);
}

// VxM (include/matrix_la.h:1286-1291): y[j] += A(i,j) * x[i].
int ref_vxm_f64(int64_t m, int64_t n, int64_t nnz, const int* rst, const int* col, const double* val,
                double* x, double* y) {
    spMtx<double> A = make_csr<double>(m, n, nnz, rst, col, val);
    VxM<double>(A, x, y);
    return 0;
}

int ref_vxm_i32(int64_t m, int64_t n, int64_t nnz, const int* rst, const int* col, const int* val, int* x,
                int* y) {
    spMtx<int> A = make_csr<int>(m, n, nnz, rst, col, val);
    VxM<int>(A, x, y);
    return 0;
}

// C<M> = A*B with the reference's mxm entry points; algo 0 msa, 1 mca,
// 2 heap, 3 naive (matrix_la.h:700-749, 586-641, 1013-1084, 1139-1277).
int ref_mxm_i32(int algo, int64_t am, int64_t an, int64_t anz, const int* ar, const int* ac, const int* av,
                int64_t bm, int64_t bn, int64_t bnz, const int* br, const int* bc, const int* bv,
                int64_t mm, int64_t mn, int64_t mnz, const int* mr, const int* mc, const int* mv,
                int64_t* cm, int64_t* cn, int64_t* cnz, int** cr, int** cc, int** cv) {
    spMtx<int> A = make_csr<int>(am, an, anz, ar, ac, av);
    spMtx<int> B = make_csr<int>(bm, bn, bnz, br, bc, bv);
    spMtx<int> M = make_csr<int>(mm, mn, mnz, mr, mc, mv);
    spMtx<int> C;
    if (run_mxm<int>(algo, A, B, M, C)) return 1;
    export_csr(C, cm, cn, cnz, cr, cc, cv);
    return 0;
}

int ref_mxm_f64(int algo, int64_t am, int64_t an, int64_t anz, const int* ar, const int* ac, const double* av,
                int64_t bm, int64_t bn, int64_t bnz, const int* br, const int* bc, const double* bv,
                int64_t mm, int64_t mn, int64_t mnz, const int* mr, const int* mc, const double* mv,
                int64_t* cm, int64_t* cn, int64_t* cnz, int** cr, int** cc, double** cv) {
    spMtx<double> A = make_csr<double>(am, an, anz, ar, ac, av);
    spMtx<double> B = make_csr<double>(bm, bn, bnz, br, bc, bv);
    spMtx<double> M = make_csr<double>(mm, mn, mnz, mr, mc, mv);
    spMtx<double> C;
    if (run_mxm<double>(algo, A, B, M, C)) return 1;
    export_csr(C, cm, cn, cnz, cr, cc, cv);
    return 0;
}

// C<!M> = A*B, matrix_la.h:788-891 (parallel branch).
int ref_cmask_i32(int64_t am, int64_t an, int64_t anz, const int* ar, const int* ac, const int* av,
                  int64_t bm, int64_t bn, int64_t bnz, const int* br, const int* bc, const int* bv,
                  int64_t mm, int64_t mn, int64_t mnz, const int* mr, const int* mc, const int* mv,
                  int64_t* cm, int64_t* cn, int64_t* cnz, int** cr, int** cc, int** cv) {
    spMtx<int> A = make_csr<int>(am, an, anz, ar, ac, av);
    spMtx<int> B = make_csr<int>(bm, bn, bnz, br, bc, bv);
    spMtx<int> M = make_csr<int>(mm, mn, mnz, mr, mc, mv);
    spMtx<int> C;
    mxmm_msa_cmask<int, int>(true, A, B, M, C);
    export_csr(C, cm, cn, cnz, cr, cc, cv);
    return 0;
}

int ref_cmask_f64(int64_t am, int64_t an, int64_t anz, const int* ar, const int* ac, const double* av,
                  int64_t bm, int64_t bn, int64_t bnz, const int* br, const int* bc, const double* bv,
                  int64_t mm, int64_t mn, int64_t mnz, const int* mr, const int* mc, const double* mv,
                  int64_t* cm, int64_t* cn, int64_t* cnz, int** cr, int** cc, double** cv) {
    spMtx<double> A = make_csr<double>(am, an, anz, ar, ac, av);
    spMtx<double> B = make_csr<double>(bm, bn, bnz, br, bc, bv);
    spMtx<double> M = make_csr<double>(mm, mn, mnz, mr, mc, mv);
    spMtx<double> C;
    mxmm_msa_cmask<double, double>(true, A, B, M, C);
    export_csr(C, cm, cn, cnz, cr, cc, cv);
    return 0;
}

// triangle_counting_masked_sandia (main.cpp:65-86) with the chosen mxmOp.
int64_t ref_tc_sandia(int algo, int64_t m, int64_t nnz, const int* rst, const int* col) {
    spMtx<int> A = make_csr<int>(m, m, nnz, rst, col, nullptr);
    op_t<int> op = ktruss_op(algo);
    if (!op) return -1;
    std::stringstream sink;
    auto* old = std::cout.rdbuf(sink.rdbuf());
    int64_t t = triangle_counting_masked_sandia(A, op, true);
    std::cout.rdbuf(old);
    return t;
}

// Row sums of C<L> = L*L (the per-row view of main.cpp:73-78).
int ref_tc_rows(int64_t m, int64_t nnz, const int* rst, const int* col, int64_t* rows) {
    spMtx<int> A = make_csr<int>(m, m, nnz, rst, col, nullptr);
    spMtx<int> L = extract_lower_triangle(A);
    spMtx<int> C;
    mxmm_msa<int, int>(true, L, L, L, C);
    for (size_t i = 0; i < C.m; ++i) {
        int64_t s = 0;
        for (int j = C.Rst[i]; j < C.Rst[i + 1]; ++j) s += C.Val[j];
        rows[i] = s;
    }
    return 0;
}

// k_truss (main.cpp:90-146); returns the iteration count it prints.
int ref_ktruss(int algo, int64_t m, int64_t nnz, const int* rst, const int* col, const int* val, int k,
               int64_t* cnz, int** cr, int** cc, int** cv, int* iters) {
    spMtx<int> A = make_csr<int>(m, m, nnz, rst, col, val);
    op_t<int> op = ktruss_op(algo);
    if (!op) return 1;
    std::stringstream sink;
    auto* old = std::cout.rdbuf(sink.rdbuf());
    spMtx<int> C = k_truss(A, k, op, true);
    std::cout.rdbuf(old);
    std::string s = sink.str();
    size_t p = s.find("Iterations:");
    *iters = (p == std::string::npos) ? -1 : std::atoi(s.c_str() + p + 11);
    int64_t cmm, cnn;
    export_csr(C, &cmm, &cnn, cnz, cr, cc, cv);
    C.nz = C.Rst ? C.Rst[C.m] : 0;
    return 0;
}

// betweenness_centrality_batch exactly as shipped: FP32, int32 path counts,
// sources 0..batch-1 (betweenness_centrality.h:125-237).
int ref_bc_batch_f32(int64_t m, int64_t nnz, const int* rst, const int* col, int64_t batch, float* bc) {
    spMtx<int> A = make_csr<int>(m, m, nnz, rst, col, nullptr);
    std::stringstream sink;
    auto* old = std::cerr.rdbuf(sink.rdbuf());
    std::vector<float> r = betweenness_centrality_batch(true, A, (size_t)batch);
    std::cerr.rdbuf(old);
    std::memcpy(bc, r.data(), sizeof(float) * m);
    return 0;
}

// betweenness_centrality exactly as shipped: every source, in blocks of
// blockSize (betweenness_centrality.h:5-123), FP32.
int ref_bc_all_f32(int64_t m, int64_t nnz, const int* rst, const int* col, int64_t block, float* bc) {
    spMtx<int> A = make_csr<int>(m, m, nnz, rst, col, nullptr);
    std::stringstream sink;
    auto* old = std::cerr.rdbuf(sink.rdbuf());
    std::vector<float> r = betweenness_centrality(true, A, (size_t)block);
    std::cerr.rdbuf(old);
    std::memcpy(bc, r.data(), sizeof(float) * m);
    return 0;
}

// The same batched algorithm (betweenness_centrality.h:161-228) run with the
// reference's own templates instantiated at double and an explicit source
// list; the dense conversion of Numsp is zero-filled (matrix.h:586-596 form).
int ref_bc_batch_f64(int64_t m, int64_t nnz, const int* rst, const int* col, const int* val,
                     int64_t nsrc, const int* sources, double* bc) {
    spMtx<int> Ai = make_csr<int>(m, m, nnz, rst, col, val);
    spMtx<double> A = convertType<double>(Ai);
    spMtx<double> AT = transpose(A);
    size_t n = (size_t)nsrc;
    size_t mxn = (size_t)m * n;
    // Numsp: identity over the sources (row = vertex, column = source index)
    spMtx<double> Numsp((size_t)m, n, n);
    std::vector<int> owner(m, -1);
    for (size_t j = 0; j < n; ++j) owner[sources[j]] = (int)j;
    {
        int p = 0;
        Numsp.Rst[0] = 0;
        for (int64_t v = 0; v < m; ++v) {
            if (owner[v] >= 0) { Numsp.Col[p] = owner[v]; Numsp.Val[p] = 1.0; ++p; }
            Numsp.Rst[v + 1] = p;
        }
    }
    // Front = transpose(rows of A at the sources)
    spMtx<double> AS(n, (size_t)m, 0);
    {
        size_t z = 0;
        for (size_t j = 0; j < n; ++j) z += A.Rst[sources[j] + 1] - A.Rst[sources[j]];
        AS.resizeVals(z);
        AS.Rst[0] = 0;
        size_t p = 0;
        for (size_t j = 0; j < n; ++j) {
            int s = sources[j];
            for (int q = A.Rst[s]; q < A.Rst[s + 1]; ++q) { AS.Col[p] = A.Col[q]; AS.Val[p] = A.Val[q]; ++p; }
            AS.Rst[j + 1] = (int)p;
        }
    }
    spMtx<double> Front = transpose(AS);
    spMtx<double> Fronttmp;
    std::vector<spMtx<double>> Sigmas((size_t)m + 1);
    size_t d = 0;
    do {
        Sigmas[d] = Front;
        Numsp = add_nointersect(Numsp, Front);
        mxmm_msa_cmask<double, double>(true, AT, Front, Numsp, Fronttmp);
        Front = Fronttmp;
        ++d;
    } while (Front.nz != 0);

    denseMtx<double> Numspd(Numsp);
    denseMtx<double> Nspinv((size_t)m, n), Bcu((size_t)m, n), W((size_t)m, n), Wbuf((size_t)m, n);
    for (size_t i = 0; i < mxn; ++i) Bcu.Val[i] = 1.0;
    for (size_t i = 0; i < mxn; ++i) W.Val[i] = 0.0;
    for (size_t i = 0; i < mxn; ++i) Nspinv.Val[i] = Numspd.Val[i] != 0.0 ? 1.0 / Numspd.Val[i] : 0.0;
    for (size_t k = d - 1; k > 0; --k) {
        eWiseMult(Nspinv, Bcu, Sigmas[k], W);
        mxmm_spd(A, W, Sigmas[k - 1], W, Wbuf);
        fuseEWiseMultAdd(W, Numspd, Bcu);
    }
    for (int64_t i = 0; i < m; ++i) {
        double s = 0.0;
        for (size_t j = 0; j < n; ++j) s += Bcu.Val[(size_t)n * i + j];
        bc[i] = s - (double)n;
    }
    return 0;
}

}  // extern "C"
