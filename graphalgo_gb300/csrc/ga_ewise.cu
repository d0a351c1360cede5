// Element-wise operations on sparse matrices and matrix-vector products: the
// GraphBLAS-style operations the reference declares in include/matrix_la.h
// (eWiseAdd 272-435, eWiseMult 438-533, multScalar 535-541, MxV / VxM
// 1279-1291) without its callers using them.
//
// Every output entry finds its place independently: row merges use a binary
// search of each entry's column in the other operand's row, and a prefix sum
// over "kept" flags gives positions, so hub rows need no serial merge.
// MxV walks each row in order on one thread and VxM is MxV over the
// transpose, so floating-point sums keep the reference's order of terms.
#include "ga_device.cuh"

namespace ga {

__device__ __forceinline__ bool holds(const int32_t* c, int n, int32_t j, int& at) {
    at = lower_bound_i32(c, n, j);
    return at < n && c[at] == j;
}

// bonly[q] = 1 for a B entry whose column A's row lacks.
__global__ void k_union_flags(const int32_t* __restrict__ ar, const int32_t* __restrict__ ac,
                              const int32_t* __restrict__ br, const int32_t* __restrict__ bc, int64_t m,
                              int32_t* __restrict__ bonly) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
        const int32_t a0 = ar[i], an = ar[i + 1] - a0;
        for (int32_t q = br[i] + lane; q < br[i + 1]; q += 32) {
            int at;
            bonly[q] = !holds(ac + a0, an, bc[q], at);
        }
    }
}

__global__ void k_union_count(const int32_t* __restrict__ ar, const int32_t* __restrict__ br,
                              const int32_t* __restrict__ bs, int64_t m, int32_t* __restrict__ cnt) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        cnt[i] = (ar[i + 1] - ar[i]) + (bs[br[i + 1]] - bs[br[i]]);
}

// Union of the rows: an A entry lands after the row's A entries before it
// and the B-only entries with smaller columns; a B-only entry after the
// B-only entries before it and the A entries with smaller columns.
template <typename T>
__global__ void k_union_fill(const int32_t* __restrict__ ar, const int32_t* __restrict__ ac,
                             const T* __restrict__ av, const int32_t* __restrict__ br,
                             const int32_t* __restrict__ bc, const T* __restrict__ bv,
                             const int32_t* __restrict__ bonly, const int32_t* __restrict__ bs, int64_t m,
                             const int32_t* __restrict__ cr, int32_t* __restrict__ cc, T* __restrict__ cv) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
        const int32_t a0 = ar[i], an = ar[i + 1] - a0, b0 = br[i], bn = br[i + 1] - b0, o = cr[i];
        const int32_t base = bs[b0];
        for (int32_t t = lane; t < an; t += 32) {
            const int32_t c = ac[a0 + t];
            int at;
            const bool both = holds(bc + b0, bn, c, at);
            const int32_t p = o + t + (bs[b0 + at] - base);
            cc[p] = c;
            cv[p] = both ? (T)(av[a0 + t] + bv[b0 + at]) : av[a0 + t];
        }
        for (int32_t t = lane; t < bn; t += 32) {
            if (!bonly[b0 + t]) continue;
            const int32_t c = bc[b0 + t];
            const int32_t p = o + (bs[b0 + t] - base) + lower_bound_i32(ac + a0, an, c);
            cc[p] = c;
            cv[p] = bv[b0 + t];
        }
    }
}

// Masked sum at every mask entry: (0 + A(i,j)) + B(i,j), kept when nonzero.
template <typename T>
__device__ __forceinline__ T masked_sum(const int32_t* ac, const T* av, int32_t a0, int32_t an, const int32_t* bc,
                                        const T* bv, int32_t b0, int32_t bn, int32_t j) {
    T v = (T)0;
    int at;
    if (holds(ac + a0, an, j, at)) v = (T)(v + av[a0 + at]);
    if (holds(bc + b0, bn, j, at)) v = (T)(v + bv[b0 + at]);
    return v;
}

template <typename T>
__global__ void k_madd_flags(const int32_t* __restrict__ ar, const int32_t* __restrict__ ac,
                             const T* __restrict__ av, const int32_t* __restrict__ br,
                             const int32_t* __restrict__ bc, const T* __restrict__ bv,
                             const int32_t* __restrict__ mr, const int32_t* __restrict__ mc, int64_t m,
                             int32_t* __restrict__ keep) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
        const int32_t a0 = ar[i], an = ar[i + 1] - a0, b0 = br[i], bn = br[i + 1] - b0;
        for (int32_t q = mr[i] + lane; q < mr[i + 1]; q += 32)
            keep[q] = masked_sum<T>(ac, av, a0, an, bc, bv, b0, bn, mc[q]) != (T)0;
    }
}

template <typename T>
__global__ void k_madd_fill(const int32_t* __restrict__ ar, const int32_t* __restrict__ ac,
                            const T* __restrict__ av, const int32_t* __restrict__ br,
                            const int32_t* __restrict__ bc, const T* __restrict__ bv,
                            const int32_t* __restrict__ mr, const int32_t* __restrict__ mc, int64_t m,
                            const int32_t* __restrict__ keep, const int32_t* __restrict__ ks,
                            int32_t* __restrict__ cc, T* __restrict__ cv) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
        const int32_t a0 = ar[i], an = ar[i + 1] - a0, b0 = br[i], bn = br[i + 1] - b0;
        for (int32_t q = mr[i] + lane; q < mr[i + 1]; q += 32) {
            if (!keep[q]) continue;
            cc[ks[q]] = mc[q];
            cv[ks[q]] = masked_sum<T>(ac, av, a0, an, bc, bv, b0, bn, mc[q]);
        }
    }
}

// keep[q] = 1 for an A entry whose column B's row (and M's, if given) holds.
__global__ void k_mult_flags(const int32_t* __restrict__ ar, const int32_t* __restrict__ ac,
                             const int32_t* __restrict__ br, const int32_t* __restrict__ bc,
                             const int32_t* __restrict__ mr, const int32_t* __restrict__ mc, int64_t m,
                             int32_t* __restrict__ keep) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
        const int32_t b0 = br[i], bn = br[i + 1] - b0;
        const int32_t m0 = mr ? mr[i] : 0, mn = mr ? mr[i + 1] - m0 : 0;
        for (int32_t q = ar[i] + lane; q < ar[i + 1]; q += 32) {
            int at;
            bool k = holds(bc + b0, bn, ac[q], at);
            if (k && mr) k = holds(mc + m0, mn, ac[q], at);
            keep[q] = k;
        }
    }
}

template <typename T>
__global__ void k_mult_fill(const int32_t* __restrict__ ar, const int32_t* __restrict__ ac,
                            const T* __restrict__ av, const int32_t* __restrict__ br,
                            const int32_t* __restrict__ bc, const T* __restrict__ bv, int64_t m,
                            const int32_t* __restrict__ keep, const int32_t* __restrict__ ks,
                            int32_t* __restrict__ cc, T* __restrict__ cv) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
        const int32_t b0 = br[i], bn = br[i + 1] - b0;
        for (int32_t q = ar[i] + lane; q < ar[i + 1]; q += 32) {
            if (!keep[q]) continue;
            int at;
            holds(bc + b0, bn, ac[q], at);
            cc[ks[q]] = ac[q];
            cv[ks[q]] = (T)(av[q] * bv[b0 + at]);
        }
    }
}

// out[i] = s[idx[i]] for i <= m (row starts from a scan over entries).
__global__ void k_gather_starts(const int32_t* __restrict__ idx, const int32_t* __restrict__ s, int64_t m,
                                int32_t* __restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= m; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = s[idx[i]];
}

template <typename T>
__global__ void k_scale(T* __restrict__ v, int64_t n, double alpha) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        v[q] = (T)(__dmul_rn((double)v[q], alpha));
}

// y[i] += A(i,j) * x[j], each row's terms in order on one thread.
template <typename T>
__global__ void k_mxv(const int32_t* __restrict__ ar, const int32_t* __restrict__ ac, const T* __restrict__ av,
                      const T* __restrict__ x, int64_t m, T* __restrict__ y) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        T acc = y[i];
        for (int32_t q = ar[i]; q < ar[i + 1]; ++q) acc = mul_add_separate<T>(acc, av[q], x[ac[q]]);
        y[i] = acc;
    }
}

static void check_pair(ga_csr A, ga_csr B, ga_csr M, const char* what) {
    GA_REQUIRE(A->m == B->m && A->n == B->n, GA_ERR_SHAPE, std::string(what) + ": shapes differ");
    GA_REQUIRE(!M || (M->m == A->m && M->n == A->n), GA_ERR_SHAPE, std::string(what) + ": mask shape differs");
    GA_REQUIRE(A->dtype == B->dtype, GA_ERR_DTYPE, std::string(what) + ": dtypes differ");
}

// Row starts and entry arrays of a result whose entries are the kept ones
// of an operand's entry list (`idx` = that operand's row starts).
static ga_csr kept_result(ga_ctx ctx, ga_csr shape, const int32_t* idx, int64_t entries, DBuf<int32_t>& keep,
                          DBuf<int32_t>& ks, ga_dtype dt) {
    scan_exclusive_i32(ctx, keep.p, ks.p, entries);
    const int64_t nnz = entries ? read_i32(ctx, ks.p + entries) : 0;
    ga_csr C = csr_alloc(ctx, shape->m, shape->n, nnz, dt);
    k_gather_starts<<<grid_for(shape->m + 1, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(idx, ks.p, shape->m,
                                                                                             C->rst);
    post_launch("gather_starts");
    return C;
}

static ga_csr ewise_add(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr M) {
    check_pair(A, B, M, "eWiseAdd");
    ProfScope ps(ctx, "ewise_add");
    const int gw = grid_for(A->m * 32, 256, ctx->num_sms * 16);
    if (M) {
        DBuf<int32_t> keep(ctx, (size_t)M->nnz + 1), ks(ctx, (size_t)M->nnz + 1);
        if (M->nnz) {
            GA_DISPATCH_DTYPE(A->dtype, T, {
                k_madd_flags<T><<<gw, 256, 0, ctx->stream>>>(A->rst, A->col, static_cast<const T*>(A->val), B->rst,
                                                             B->col, static_cast<const T*>(B->val), M->rst, M->col,
                                                             A->m, keep.p);
            });
            post_launch("madd_flags");
        }
        ga_csr C = kept_result(ctx, A, M->rst, M->nnz, keep, ks, A->dtype);
        try {
            if (C->nnz) {
                GA_DISPATCH_DTYPE(A->dtype, T, {
                    k_madd_fill<T><<<gw, 256, 0, ctx->stream>>>(A->rst, A->col, static_cast<const T*>(A->val), B->rst,
                                                                B->col, static_cast<const T*>(B->val), M->rst, M->col,
                                                                A->m, keep.p, ks.p, C->col, static_cast<T*>(C->val));
                });
                post_launch("madd_fill");
            }
            GA_CUDA(cudaStreamSynchronize(ctx->stream));
        } catch (...) {
            csr_destroy(ctx, C);
            throw;
        }
        return C;
    }
    DBuf<int32_t> bonly(ctx, (size_t)B->nnz + 1), bs(ctx, (size_t)B->nnz + 1), cnt(ctx, (size_t)A->m + 1);
    if (B->nnz) {
        k_union_flags<<<gw, 256, 0, ctx->stream>>>(A->rst, A->col, B->rst, B->col, A->m, bonly.p);
        post_launch("union_flags");
    }
    scan_exclusive_i32(ctx, bonly.p, bs.p, B->nnz);
    k_union_count<<<grid_for(A->m, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(A->rst, B->rst, bs.p, A->m, cnt.p);
    post_launch("union_count");
    scan_exclusive_i32(ctx, cnt.p, cnt.p, A->m);
    const int64_t nnz = A->m ? read_i32(ctx, cnt.p + A->m) : 0;
    ga_csr C = csr_alloc(ctx, A->m, A->n, nnz, A->dtype);
    try {
        GA_CUDA(cudaMemcpyAsync(C->rst, cnt.p, sizeof(int32_t) * (A->m + 1), cudaMemcpyDeviceToDevice, ctx->stream));
        if (nnz) {
            GA_DISPATCH_DTYPE(A->dtype, T, {
                k_union_fill<T><<<gw, 256, 0, ctx->stream>>>(A->rst, A->col, static_cast<const T*>(A->val), B->rst,
                                                             B->col, static_cast<const T*>(B->val), bonly.p, bs.p,
                                                             A->m, C->rst, C->col, static_cast<T*>(C->val));
            });
            post_launch("union_fill");
        }
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
    } catch (...) {
        csr_destroy(ctx, C);
        throw;
    }
    return C;
}

static ga_csr ewise_mult(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr M) {
    check_pair(A, B, M, "eWiseMult");
    ProfScope ps(ctx, "ewise_mult");
    const int gw = grid_for(A->m * 32, 256, ctx->num_sms * 16);
    DBuf<int32_t> keep(ctx, (size_t)A->nnz + 1), ks(ctx, (size_t)A->nnz + 1);
    if (A->nnz) {
        k_mult_flags<<<gw, 256, 0, ctx->stream>>>(A->rst, A->col, B->rst, B->col, M ? M->rst : nullptr,
                                                  M ? M->col : nullptr, A->m, keep.p);
        post_launch("mult_flags");
    }
    ga_csr C = kept_result(ctx, A, A->rst, A->nnz, keep, ks, A->dtype);
    try {
        if (C->nnz) {
            GA_DISPATCH_DTYPE(A->dtype, T, {
                k_mult_fill<T><<<gw, 256, 0, ctx->stream>>>(A->rst, A->col, static_cast<const T*>(A->val), B->rst,
                                                            B->col, static_cast<const T*>(B->val), A->m, keep.p, ks.p,
                                                            C->col, static_cast<T*>(C->val));
            });
            post_launch("mult_fill");
        }
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
    } catch (...) {
        csr_destroy(ctx, C);
        throw;
    }
    return C;
}

static void mxv(ga_ctx ctx, ga_csr A, ga_dense x, ga_dense y) {
    GA_REQUIRE(x->m * x->n == A->n && y->m * y->n == A->m, GA_ERR_SHAPE, "MxV: vector lengths differ from A");
    GA_REQUIRE(x->dtype == A->dtype && y->dtype == A->dtype, GA_ERR_DTYPE, "MxV: dtypes differ");
    GA_REQUIRE(x->val != y->val, GA_ERR_INVALID_ARG, "MxV: y may not alias x");
    ProfScope ps(ctx, "mxv");
    GA_DISPATCH_DTYPE(A->dtype, T, {
        k_mxv<T><<<grid_for(A->m, 128, ctx->num_sms * 16), 128, 0, ctx->stream>>>(
            A->rst, A->col, static_cast<const T*>(A->val), static_cast<const T*>(x->val), A->m,
            static_cast<T*>(y->val));
    });
    post_launch("mxv");
}

}  // namespace ga

using namespace ga;

extern "C" {

int ga_ewise_add(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr M, ga_csr* C) {
    if (!ctx || !A || !B || !C) return GA_ERR_INVALID_ARG;
    *C = nullptr;
    GA_API_BODY(ctx, *C = ewise_add(ctx, A, B, M));
}

int ga_ewise_mult(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr M, ga_csr* C) {
    if (!ctx || !A || !B || !C) return GA_ERR_INVALID_ARG;
    *C = nullptr;
    GA_API_BODY(ctx, *C = ewise_mult(ctx, A, B, M));
}

int ga_mult_scalar(ga_ctx ctx, ga_csr A, double alpha) {
    if (!ctx || !A) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        ProfScope ps(ctx, "mult_scalar");
        if (A->nnz) {
            GA_DISPATCH_DTYPE(A->dtype, T, {
                k_scale<T><<<grid_for(A->nnz, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(static_cast<T*>(A->val),
                                                                                            A->nnz, alpha);
            });
            post_launch("scale");
        }
        A->unit = -1;
    });
}

int ga_mxv(ga_ctx ctx, ga_csr A, ga_dense x, ga_dense y) {
    if (!ctx || !A || !x || !y) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, mxv(ctx, A, x, y));
}

int ga_vxm(ga_ctx ctx, ga_csr A, ga_dense x, ga_dense y) {
    if (!ctx || !A || !x || !y) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        GA_REQUIRE(x->m * x->n == A->m && y->m * y->n == A->n, GA_ERR_SHAPE, "VxM: vector lengths differ from A");
        ga_csr T = transpose_csr(ctx, A);
        try {
            mxv(ctx, T, x, y);
            GA_CUDA(cudaStreamSynchronize(ctx->stream));
        } catch (...) {
            csr_destroy(ctx, T);
            throw;
        }
        csr_destroy(ctx, T);
    });
}

}  // extern "C"
