// graphalgo_gb300.hpp - C++ drop-in for UAlex322/GraphAlgo's masked-SpGEMM
// path, running on the GB300 through the C ABI in graphalgo_gb300.h.
//
// It re-exposes the reference's types and signatures:
//   spMtx<T>, denseMtx<T>                     (include/matrix.h:23-666)
//   mxmm_msa / mxmm_mca / mxmm_heap / mxmm_naive (+ mxmm_hybrid, mxmm_tri),
//   mxmm_msa_cmask, mxmm_spd,
//   add_nointersect, eWiseMult, fuseEWiseMultAdd, transpose  (include/matrix_la.h)
//   extract_lower_triangle, extract_upper_triangle, build_symm_from_lower,
//   build_adjacency_matrix, convertType       (include/matrix.h:668-792)
//   triangle_counting_masked_sandia / _lu / _vertex, k_truss  (src/main.cpp:14-146)
//   betweenness_centrality_batch, betweenness_centrality
//                                             (include/betweenness_centrality.h)
// so that `mxmOp<int> op = ga::mxmm_msa<int>;` and the callers compile
// unchanged inside `namespace ga` (or with `using namespace ga;`).
//
// Data stays in host spMtx/denseMtx objects as in the reference; each call
// uploads its operands, runs on the device and downloads the result. The
// loops of k_truss and betweenness_centrality_batch run entirely on the
// device. The `isParallel` flag is accepted and ignored (the GPU is always
// parallel). Errors throw ga::error.
//
// Link with -lgraphalgo_gb300.
#pragma once

#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "graphalgo_gb300.h"

namespace ga {

struct error : std::runtime_error {
    int code;
    error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// ------------------------------------------------------------------ context
// One context per host thread, created on first use on device 0 (or the
// device given to set_device before that).
class Context {
public:
    static Context& get() {
        thread_local Context c;
        return c;
    }
    static void set_device(int d) { get().device_ = d; }
    ga_ctx handle() {
        if (!ctx_) {
            int rc = ga_ctx_create(device_, nullptr, &ctx_);
            if (rc != GA_OK) throw error(rc, std::string("ga_ctx_create: ") + ga_status_string(rc));
        }
        return ctx_;
    }
    ~Context() {
        if (ctx_) ga_ctx_destroy(ctx_);
    }

private:
    Context() = default;
    ga_ctx ctx_ = nullptr;
    int device_ = 0;
};

inline ga_ctx ctx() { return Context::get().handle(); }

inline void check(int rc) {
    if (rc != GA_OK) throw error(rc, ga_last_error(ctx()));
}

template <typename T> struct dtype_of;
template <> struct dtype_of<int32_t> { static constexpr ga_dtype value = GA_INT32; };
template <> struct dtype_of<int64_t> { static constexpr ga_dtype value = GA_INT64; };
template <> struct dtype_of<float> { static constexpr ga_dtype value = GA_FP32; };
template <> struct dtype_of<double> { static constexpr ga_dtype value = GA_FP64; };
template <> struct dtype_of<uint8_t> { static constexpr ga_dtype value = GA_UINT8; };

// ------------------------------------------------------------------ spMtx
// CSR matrix with the reference's public layout: m x n, nz entries, Rst
// (m+1 row starts), Col (nz column indices, ascending per row), Val.
template <typename ValT>
class spMtx {
public:
    size_t m = 0, n = 0, nz = 0, capacity = 0;
    char matcode[4] = {'M', 'C', 'I', 'G'};
    int* Rst = nullptr;
    int* Col = nullptr;
    ValT* Val = nullptr;

    spMtx() {}
    spMtx(size_t m_, size_t n_) : m(m_), n(n_) { Rst = new int[m + 1](); }
    spMtx(size_t m_, size_t n_, size_t nz_) : m(m_), n(n_), nz(nz_), capacity(nz_) {
        Rst = new int[m + 1]();
        Col = new int[nz ? nz : 1];
        Val = new ValT[nz ? nz : 1]();
    }
    spMtx(const spMtx& o) : m(o.m), n(o.n), nz(o.nz), capacity(o.nz) {
        std::memcpy(matcode, o.matcode, 4);
        Rst = new int[m + 1];
        std::memcpy(Rst, o.Rst, sizeof(int) * (m + 1));
        Col = new int[nz ? nz : 1];
        if (nz) std::memcpy(Col, o.Col, sizeof(int) * nz);
        if (o.Val) {
            Val = new ValT[nz ? nz : 1];
            if (nz) std::memcpy(Val, o.Val, sizeof(ValT) * nz);
        }
    }
    spMtx(spMtx&& o) noexcept { take(o); }
    spMtx& operator=(const spMtx& o) {
        if (this != &o) {
            spMtx t(o);
            release();
            take(t);
        }
        return *this;
    }
    spMtx& operator=(spMtx&& o) noexcept {
        if (this != &o) {
            release();
            take(o);
        }
        return *this;
    }
    ~spMtx() { release(); }

    // grow-only storage, contents not preserved (include/matrix.h:107-127)
    void resizeVals(size_t newNz) {
        if (newNz > capacity) {
            delete[] Col;
            delete[] Val;
            Col = new int[newNz];
            Val = new ValT[newNz];
            capacity = newNz;
        }
        nz = newNz;
    }
    void resizeRows(size_t newM) {
        if (m != newM || !Rst) {
            delete[] Rst;
            Rst = new int[newM + 1]();
            m = newM;
        }
    }
    template <typename ValT2>
    void copyPattern(const spMtx<ValT2>& s) {
        resizeRows(s.m);
        std::memcpy(Rst, s.Rst, sizeof(int) * (m + 1));
        n = s.n;
        resizeVals(s.nz);
        if (nz) std::memcpy(Col, s.Col, sizeof(int) * nz);
    }
    spMtx extractRows(size_t begin, size_t end) const {
        spMtx r(end - begin, n, (size_t)(Rst[end] - Rst[begin]));
        for (size_t i = 0; i <= end - begin; ++i) r.Rst[i] = Rst[i + begin] - Rst[begin];
        std::memcpy(r.Col, Col + Rst[begin], sizeof(int) * r.nz);
        std::memcpy(r.Val, Val + Rst[begin], sizeof(ValT) * r.nz);
        return r;
    }
    bool operator==(const spMtx& o) const {
        if (m != o.m || n != o.n || nz != o.nz) return false;
        for (size_t i = 0; i <= m; ++i)
            if (Rst[i] != o.Rst[i]) return false;
        for (size_t j = 0; j < nz; ++j)
            if (Col[j] != o.Col[j] || Val[j] != o.Val[j]) return false;
        return true;
    }

private:
    void release() {
        delete[] Rst;
        delete[] Col;
        delete[] Val;
        Rst = nullptr; Col = nullptr; Val = nullptr;
    }
    void take(spMtx& o) {
        m = o.m; n = o.n; nz = o.nz; capacity = o.capacity;
        std::memcpy(matcode, o.matcode, 4);
        Rst = o.Rst; Col = o.Col; Val = o.Val;
        o.Rst = nullptr; o.Col = nullptr; o.Val = nullptr;
        o.m = o.n = o.nz = o.capacity = 0;
    }
};

// ---------------------------------------------------------------- denseMtx
template <typename ValT>
class denseMtx {
public:
    size_t m = 0, n = 0, capacity = 0;
    ValT* Val = nullptr;

    denseMtx() {}
    denseMtx(size_t m_, size_t n_) : m(m_), n(n_), capacity(m_ * n_) { Val = new ValT[capacity ? capacity : 1](); }
    denseMtx(const denseMtx& o) : denseMtx(o.m, o.n) { std::memcpy(Val, o.Val, sizeof(ValT) * m * n); }
    denseMtx(denseMtx&& o) noexcept : m(o.m), n(o.n), capacity(o.capacity), Val(o.Val) { o.Val = nullptr; }
    // dense copy of a sparse matrix, zero elsewhere (include/matrix.h:585-596)
    template <typename ValT2>
    explicit denseMtx(const spMtx<ValT2>& s) : denseMtx(s.m, s.n) {
        for (size_t i = 0; i < s.m; ++i)
            for (int k = s.Rst[i]; k < s.Rst[i + 1]; ++k) Val[n * i + (size_t)s.Col[k]] = (ValT)s.Val[k];
    }
    denseMtx& operator=(denseMtx&& o) noexcept {
        std::swap(m, o.m); std::swap(n, o.n); std::swap(capacity, o.capacity); std::swap(Val, o.Val);
        return *this;
    }
    denseMtx& operator=(const denseMtx& o) {
        if (this != &o) {
            resize(o.m, o.n);
            std::memcpy(Val, o.Val, sizeof(ValT) * m * n);
        }
        return *this;
    }
    ~denseMtx() { delete[] Val; }
    void resize(size_t newM, size_t newN) {
        m = newM;
        n = newN;
        if (capacity < m * n) {
            delete[] Val;
            capacity = m * n;
            Val = new ValT[capacity]();
        }
    }
};

// ------------------------------------------------------------ device copies
namespace detail {

struct DevCsr {
    ga_csr h = nullptr;
    DevCsr() = default;
    explicit DevCsr(ga_csr x) : h(x) {}
    DevCsr(const DevCsr&) = delete;
    DevCsr& operator=(const DevCsr&) = delete;
    DevCsr(DevCsr&& o) noexcept : h(o.h) { o.h = nullptr; }
    ~DevCsr() {
        if (h) ga_csr_free(ctx(), h);
    }
};

struct DevDense {
    ga_dense h = nullptr;
    DevDense() = default;
    explicit DevDense(ga_dense x) : h(x) {}
    DevDense(const DevDense&) = delete;
    DevDense(DevDense&& o) noexcept : h(o.h) { o.h = nullptr; }
    ~DevDense() {
        if (h) ga_dense_free(ctx(), h);
    }
};

template <typename T>
DevCsr upload(const spMtx<T>& A) {
    ga_csr h = nullptr;
    check(ga_csr_upload(ctx(), (int64_t)A.m, (int64_t)A.n, (int64_t)A.Rst[A.m], A.Rst, A.Col, A.Val,
                        dtype_of<T>::value, &h));
    return DevCsr(h);
}

template <typename T>
void download(ga_csr h, spMtx<T>& C) {
    int64_t m, n, nnz;
    int dt;
    check(ga_csr_info(h, &m, &n, &nnz, &dt));
    C.resizeRows((size_t)m);
    C.resizeVals((size_t)nnz);
    C.n = (size_t)n;
    check(ga_csr_download(ctx(), h, C.Rst, C.Col, C.Val));
}

template <typename T>
DevDense upload(const denseMtx<T>& D) {
    ga_dense h = nullptr;
    check(ga_dense_create(ctx(), (int64_t)D.m, (int64_t)D.n, dtype_of<T>::value, D.Val, &h));
    return DevDense(h);
}

template <typename T>
void download(ga_dense h, denseMtx<T>& D) {
    int64_t m, n;
    int dt;
    check(ga_dense_info(h, &m, &n, &dt));
    D.resize((size_t)m, (size_t)n);
    check(ga_dense_download(ctx(), h, D.Val));
}

template <typename T, typename U>
spMtx<T> mask_as(const spMtx<U>& M) {
    // a structural mask: only the pattern is used, so values become ones
    spMtx<T> R;
    R.copyPattern(M);
    for (size_t j = 0; j < R.nz; ++j) R.Val[j] = (T)1;
    return R;
}

template <typename T, typename U>
void masked(ga_algo algo, const spMtx<T>& A, const spMtx<T>& B, const spMtx<U>& M, spMtx<T>& C) {
    DevCsr a = upload(A), b = upload(B);
    DevCsr mk = upload(mask_as<T>(M));
    ga_csr c = nullptr;
    check(ga_mxm_masked(ctx(), algo, a.h, b.h, mk.h, &c));
    DevCsr cc(c);
    download(c, C);
}

}  // namespace detail

template <typename T>
using mxmOp = void (*)(bool, const spMtx<T>&, const spMtx<T>&, const spMtx<T>&, spMtx<T>&);

// ------------------------------------------------------ masked SpGEMM family
// C<M> = A*B, C takes M's pattern (include/matrix_la.h:700-713).
template <typename T, typename U>
void mxmm_msa(bool, const spMtx<T>& A, const spMtx<T>& B, const spMtx<U>& M, spMtx<T>& C) {
    detail::masked(GA_MSA, A, B, M, C);
}
// include/matrix_la.h:586-599
template <typename T, typename U>
void mxmm_mca(bool, const spMtx<T>& A, const spMtx<T>& B, const spMtx<U>& M, spMtx<T>& C) {
    detail::masked(GA_MCA, A, B, M, C);
}
// include/matrix_la.h:1013-1028 (values start from zero)
template <typename T>
void mxmm_heap(bool, const spMtx<T>& A, const spMtx<T>& B, const spMtx<T>& M, spMtx<T>& C) {
    detail::masked(GA_HEAP, A, B, M, C);
}
// include/matrix_la.h:1139-1277
template <typename T>
void mxmm_naive(bool, const spMtx<T>& A, const spMtx<T>& B, const spMtx<T>& M, spMtx<T>& C) {
    detail::masked(GA_NAIVE, A, B, M, C);
}
// Not in the reference: per row the cheaper of MSA and inner products
// (GA_HYBRID), and triangle listing (GA_TRI: C<A> = A*A of a symmetric 0/1
// matrix, the k-truss support; other operands run GA_HYBRID). Same results.
template <typename T>
void mxmm_hybrid(bool, const spMtx<T>& A, const spMtx<T>& B, const spMtx<T>& M, spMtx<T>& C) {
    detail::masked(GA_HYBRID, A, B, M, C);
}
template <typename T>
void mxmm_tri(bool, const spMtx<T>& A, const spMtx<T>& B, const spMtx<T>& M, spMtx<T>& C) {
    detail::masked(GA_TRI, A, B, M, C);
}
// C<!M> = A*B with a new sorted pattern (include/matrix_la.h:788-798)
template <typename T, typename U>
void mxmm_msa_cmask(bool, const spMtx<T>& A, const spMtx<T>& B, const spMtx<U>& M, spMtx<T>& C) {
    detail::DevCsr a = detail::upload(A), b = detail::upload(B);
    detail::DevCsr mk = detail::upload(detail::mask_as<T>(M));
    ga_csr c = nullptr;
    check(ga_mxm_cmask(ctx(), a.h, b.h, mk.h, &c));
    detail::DevCsr cc(c);
    detail::download(c, C);
}
// dense C<M> = A*B; the result is written to Cbuf and swapped into C, as in
// the reference (include/matrix_la.h:241-270)
template <typename T, typename U>
void mxmm_spd(const spMtx<T>& A, const denseMtx<T>& B, const spMtx<U>& M, denseMtx<T>& C, denseMtx<T>& Cbuf) {
    detail::DevCsr a = detail::upload(A);
    detail::DevCsr mk = detail::upload(detail::mask_as<T>(M));
    detail::DevDense b = detail::upload(B);
    ga_dense c = nullptr;
    check(ga_dense_create(ctx(), (int64_t)A.m, (int64_t)B.n, dtype_of<T>::value, nullptr, &c));
    detail::DevDense cd(c);
    check(ga_mxm_spd(ctx(), a.h, b.h, mk.h, c));
    detail::download(c, Cbuf);
    std::swap(C.Val, Cbuf.Val);
    std::swap(C.capacity, Cbuf.capacity);
    C.m = Cbuf.m;
    C.n = Cbuf.n;
}

// ---------------------------------------------------------- element-wise
template <typename T>
spMtx<T> add_nointersect(const spMtx<T>& A, const spMtx<T>& B) {
    detail::DevCsr a = detail::upload(A), b = detail::upload(B);
    ga_csr c = nullptr;
    check(ga_add_nointersect(ctx(), a.h, b.h, &c));
    detail::DevCsr cc(c);
    spMtx<T> C;
    detail::download(c, C);
    return C;
}
template <typename T, typename U>
void eWiseMult(const denseMtx<T>& A, const denseMtx<T>& B, const spMtx<U>& M, const denseMtx<T>& C) {
    detail::DevDense a = detail::upload(A), b = detail::upload(B);
    detail::DevCsr mk = detail::upload(detail::mask_as<T>(M));
    ga_dense c = nullptr;
    check(ga_dense_create(ctx(), (int64_t)C.m, (int64_t)C.n, dtype_of<T>::value, nullptr, &c));
    detail::DevDense cd(c);
    check(ga_ewise_mult_masked(ctx(), a.h, b.h, mk.h, c));
    check(ga_dense_download(ctx(), c, C.Val));
}
template <typename T>
void fuseEWiseMultAdd(const denseMtx<T>& A, const denseMtx<T>& B, denseMtx<T>& C) {
    detail::DevDense a = detail::upload(A), b = detail::upload(B), c = detail::upload(C);
    check(ga_fuse_ewise_mult_add(ctx(), a.h, b.h, c.h));
    check(ga_dense_download(ctx(), c.h, C.Val));
}

// ------------------------------------------------------------- graph prep
namespace detail {
template <typename T, typename F>
spMtx<T> unary(const spMtx<T>& A, F fn) {
    DevCsr a = upload(A);
    ga_csr c = nullptr;
    check(fn(ctx(), a.h, &c));
    DevCsr cc(c);
    spMtx<T> C;
    download(c, C);
    return C;
}
}  // namespace detail

template <typename T>
spMtx<T> transpose(const spMtx<T>& A) { return detail::unary(A, ga_transpose); }
template <typename T>
spMtx<T> extract_lower_triangle(const spMtx<T>& A) { return detail::unary(A, ga_extract_lower); }
template <typename T>
spMtx<T> extract_upper_triangle(const spMtx<T>& A) { return detail::unary(A, ga_extract_upper); }
template <typename T>
spMtx<T> build_symm_from_lower(const spMtx<T>& L) { return detail::unary(L, ga_symm_from_lower); }

template <typename T>
spMtx<int> build_adjacency_matrix(const spMtx<T>& G) {
    spMtx<int> R;
    R.copyPattern(G);
    std::memcpy(R.matcode, G.matcode, 4);
    R.matcode[2] = 'I';
    for (size_t j = 0; j < R.nz; ++j) R.Val[j] = 1;
    return R;
}

template <typename T2, typename T1>
spMtx<T2> convertType(const spMtx<T1>& s) {
    spMtx<T2> r;
    r.copyPattern(s);
    for (size_t j = 0; j < s.nz; ++j) r.Val[j] = (T2)s.Val[j];
    return r;
}

// ---------------------------------------------------------------- callers
namespace detail {
inline ga_algo algo_of(mxmOp<int> op) {
    if (op == static_cast<mxmOp<int>>(&mxmm_msa<int, int>)) return GA_MSA;
    if (op == static_cast<mxmOp<int>>(&mxmm_mca<int, int>)) return GA_MCA;
    if (op == static_cast<mxmOp<int>>(&mxmm_heap<int>)) return GA_HEAP;
    if (op == static_cast<mxmOp<int>>(&mxmm_naive<int>)) return GA_NAIVE;
    if (op == static_cast<mxmOp<int>>(&mxmm_hybrid<int>)) return GA_HYBRID;
    if (op == static_cast<mxmOp<int>>(&mxmm_tri<int>)) return GA_TRI;
    throw error(GA_ERR_INVALID_ARG,
                "mxmOp must be ga::mxmm_msa, mxmm_mca, mxmm_heap, mxmm_naive, mxmm_hybrid or mxmm_tri");
}
}  // namespace detail

// src/main.cpp:65-86: C<L> = L*L summed
inline int64_t triangle_counting_masked_sandia(const spMtx<int>& A, mxmOp<int> op, bool = true) {
    detail::DevCsr a = detail::upload(A);
    int64_t total = 0;
    check(ga_tc(ctx(), detail::algo_of(op), a.h, &total, nullptr));
    return total;
}
// triangle count with the warp-intersection kernel and per-row counts
inline int64_t triangle_counting_dot(const spMtx<int>& A, std::vector<int64_t>* per_row = nullptr) {
    detail::DevCsr a = detail::upload(A);
    int64_t total = 0;
    if (per_row) per_row->assign(A.m, 0);
    check(ga_tc(ctx(), GA_DOT, a.h, &total, per_row ? per_row->data() : nullptr));
    return total;
}
// src/main.cpp:40-62: C<A> = L*U summed and halved
inline int64_t triangle_counting_masked_lu(const spMtx<int>& A, mxmOp<int> op, bool = true) {
    detail::DevCsr a = detail::upload(A);
    int64_t total = 0;
    check(ga_tc_lu(ctx(), detail::algo_of(op), a.h, &total));
    return total;
}
// src/main.cpp:14-37: per-vertex (A*A<A> row sums) / 2; caller owns the array
inline int* triangle_counting_vertex(const spMtx<int>& A, mxmOp<int> op, bool = true) {
    detail::DevCsr a = detail::upload(A);
    int* out = new int[A.m];
    check(ga_tc_vertex(ctx(), detail::algo_of(op), a.h, out));
    return out;
}
// src/main.cpp:90-146
inline spMtx<int> k_truss(const spMtx<int>& A, int k, mxmOp<int> op, bool = true, int* iterations = nullptr) {
    detail::DevCsr a = detail::upload(A);
    ga_csr c = nullptr;
    int iters = 0;
    check(ga_ktruss(ctx(), detail::algo_of(op), a.h, k, &c, &iters));
    detail::DevCsr cc(c);
    spMtx<int> C;
    detail::download(c, C);
    if (iterations) *iterations = iters;
    return C;
}

// include/betweenness_centrality.h:125-237 for an explicit source list, FP64
inline std::vector<double> betweenness_centrality_sources(const spMtx<int>& A, const std::vector<int>& sources) {
    if (A.m != A.n) throw "non-square matrix; BC is only for square matrices";
    detail::DevCsr a = detail::upload(A);
    std::vector<double> bc(A.m, 0.0);
    check(ga_bc(ctx(), a.h, sources.data(), (int64_t)sources.size(), bc.data()));
    return bc;
}
// the reference's signature: sources 0..batch-1, scores returned as float
inline std::vector<float> betweenness_centrality_batch(bool, const spMtx<int>& A, size_t batchSize) {
    size_t n = std::min(A.n, batchSize);
    std::vector<int> src(n);
    for (size_t j = 0; j < n; ++j) src[j] = (int)j;
    std::vector<double> d = betweenness_centrality_sources(A, src);
    return std::vector<float>(d.begin(), d.end());
}
// all sources in blocks of blockSize (include/betweenness_centrality.h:5-123),
// accumulated on the device (ga_bc_all); blockSize 0 is refused (the
// reference would loop forever), blocks above 1,024 sources run as device
// batches of at most 1,024 with the same sums
inline std::vector<float> betweenness_centrality(bool, const spMtx<int>& A, size_t blockSize) {
    if (A.m != A.n) throw "non-square matrix; BC is only for square matrices";
    detail::DevCsr a = detail::upload(A);
    std::vector<double> bc(A.m, 0.0);
    check(ga_bc_all(ctx(), a.h, (int64_t)blockSize, bc.data()));
    return std::vector<float>(bc.begin(), bc.end());
}

}  // namespace ga
