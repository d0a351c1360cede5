/*
 * CPU oracle: plain-C restatement of the reference's masked-SpGEMM path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h). It is the checker for the CUDA
 * path and the timed CPU baseline ("port") of bench.py; the product never
 * uses it. Every function cites the reference lines it restates
 * (UAlex322/GraphAlgo, paths relative to the project root). OpenMP row
 * parallelism mirrors the reference's own `omp parallel for` loops so that the
 * baseline timing is that of the reference's algorithm on all host cores.
 *
 * Parity: pinned against the unmodified reference (oracle/_ref) and the
 * committed golden fixtures by tests/test_oracle_pin.py.
 */
#include "oracle.h"

#include <stdlib.h>
#include <stdio.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

void or_free(void* p) { free(p); }

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void or_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

static void* xmalloc(size_t bytes) { return malloc(bytes ? bytes : 1); }
static void* xcalloc(size_t count, size_t size) { return calloc(count ? count : 1, size ? size : 1); }

static int cmp_int(const void* a, const void* b) {
    int x = *(const int*)a, y = *(const int*)b;
    return (x > y) - (x < y);
}

/* -------------------------------------------------------------------------
 * Type-generic kernels, instantiated for i32, i64, f32, f64.
 * ------------------------------------------------------------------------- */
#define OR_DEFINE(T, S)                                                                   \
                                                                                          \
/* C<M> = A*B, pattern of C = pattern of M (structural mask).                             \
 * Restates _mxmm_msa_parallel, include/matrix_la.h:715-749: a dense per-thread           \
 * accumulator of length B.n, mask columns zeroed on row entry (728-729), every           \
 * product scattered (732-740), mask columns gathered (743-746). */                       \
void or_mxm_masked_##S(int64_t m, int64_t bn, const int* ar, const int* ac, const T* av,  \
                       const int* br, const int* bc, const T* bv, const int* mr,          \
                       const int* mc, T* cv) {                                            \
    _Pragma("omp parallel")                                                               \
    {                                                                                     \
        T* acc = (T*)xcalloc((size_t)bn, sizeof(T));                                      \
        _Pragma("omp for schedule(dynamic, 32)")                                          \
        for (int64_t i = 0; i < m; ++i) {                                                 \
            for (int j = mr[i]; j < mr[i + 1]; ++j) acc[mc[j]] = (T)0;                    \
            for (int t = ar[i]; t < ar[i + 1]; ++t) {                                     \
                int k = ac[t];                                                            \
                T a = av ? av[t] : (T)1;                                                  \
                for (int j = br[k]; j < br[k + 1]; ++j)                                   \
                    acc[bc[j]] += a * (bv ? bv[j] : (T)1);                                \
            }                                                                             \
            for (int j = mr[i]; j < mr[i + 1]; ++j) cv[j] = acc[mc[j]];                   \
        }                                                                                 \
        free(acc);                                                                        \
    }                                                                                     \
}                                                                                         \
                                                                                          \
/* C<!M> = A*B: new pattern = structural product columns not in M's row, sorted.         \
 * Restates _mxmm_msa_cmask_parallel, include/matrix_la.h:800-891: a symbolic pass        \
 * counting distinct product columns minus those in the mask row (814-832), a             \
 * prefix sum (838-846), and a numeric pass where the first product sets the value       \
 * and later ones add (866-875), then the touched columns are sorted (881-887). */        \
int or_mxm_cmask_##S(int64_t m, int64_t bn, const int* ar, const int* ac, const T* av,    \
                     const int* br, const int* bc, const T* bv, const int* mr,            \
                     const int* mc, int** cr_out, int** cc_out, T** cv_out,               \
                     int64_t* cnz_out) {                                                  \
    int* cr = (int*)xcalloc((size_t)m + 1, sizeof(int));                                  \
    _Pragma("omp parallel")                                                               \
    {                                                                                     \
        char* state = (char*)xcalloc((size_t)bn, 1);                                      \
        int* touched = (int*)xmalloc(sizeof(int) * (size_t)bn);                           \
        _Pragma("omp for schedule(dynamic, 64)")                                          \
        for (int64_t i = 0; i < m; ++i) {                                                 \
            int nt = 0;                                                                   \
            for (int t = ar[i]; t < ar[i + 1]; ++t) {                                     \
                int k = ac[t];                                                            \
                for (int j = br[k]; j < br[k + 1]; ++j)                                   \
                    if (!state[bc[j]]) { state[bc[j]] = 1; touched[nt++] = bc[j]; }       \
            }                                                                             \
            int row_nz = nt;                                                              \
            for (int j = mr[i]; j < mr[i + 1]; ++j)                                       \
                if (state[mc[j]]) --row_nz;                                               \
            cr[i + 1] = row_nz;                                                           \
            for (int q = 0; q < nt; ++q) state[touched[q]] = 0;                           \
        }                                                                                 \
        free(state);                                                                      \
        free(touched);                                                                    \
    }                                                                                     \
    for (int64_t i = 0; i < m; ++i) cr[i + 1] += cr[i];                                   \
    int64_t nnz = cr[m];                                                                  \
    int* cc = (int*)xmalloc(sizeof(int) * (size_t)nnz);                                   \
    T* cv = (T*)xmalloc(sizeof(T) * (size_t)nnz);                                         \
    _Pragma("omp parallel")                                                               \
    {                                                                                     \
        /* 0 = allowed, 1 = masked out, 2 = set */                                        \
        char* state = (char*)xcalloc((size_t)bn, 1);                                      \
        T* val = (T*)xcalloc((size_t)bn, sizeof(T));                                      \
        int* touched = (int*)xmalloc(sizeof(int) * (size_t)bn);                           \
        _Pragma("omp for schedule(dynamic, 256)")                                         \
        for (int64_t i = 0; i < m; ++i) {                                                 \
            int nt = 0;                                                                   \
            for (int j = mr[i]; j < mr[i + 1]; ++j) state[mc[j]] = 1;                     \
            for (int t = ar[i]; t < ar[i + 1]; ++t) {                                     \
                int k = ac[t];                                                            \
                T a = av ? av[t] : (T)1;                                                  \
                for (int j = br[k]; j < br[k + 1]; ++j) {                                 \
                    int col = bc[j];                                                      \
                    T b = bv ? bv[j] : (T)1;                                              \
                    if (state[col] == 0) {                                                \
                        state[col] = 2; touched[nt++] = col; val[col] = a * b;            \
                    } else if (state[col] == 2) {                                         \
                        val[col] += a * b;                                                \
                    }                                                                     \
                }                                                                         \
            }                                                                             \
            for (int j = mr[i]; j < mr[i + 1]; ++j) state[mc[j]] = 0;                     \
            qsort(touched, (size_t)nt, sizeof(int), cmp_int);                             \
            int p = cr[i];                                                                \
            for (int q = 0; q < nt; ++q) {                                                \
                int col = touched[q];                                                     \
                cc[p] = col; cv[p] = val[col]; ++p;                                       \
                val[col] = (T)0; state[col] = 0;                                          \
            }                                                                             \
        }                                                                                 \
        free(state); free(val); free(touched);                                            \
    }                                                                                     \
    *cr_out = cr; *cc_out = cc; *cv_out = cv; *cnz_out = nnz;                             \
    return 0;                                                                             \
}                                                                                         \
                                                                                          \
/* C<M> = A*B with B and C dense (m x n, row-major); C is zero outside M.                 \
 * Restates mxmm_spd, include/matrix_la.h:241-270: zero the output row (257-259),         \
 * then for each A entry add a*B[j][c] at every mask column c (260-267). */               \
void or_mxm_spd_##S(int64_t m, int64_t n, const int* ar, const int* ac, const T* av,      \
                    const T* B, const int* mr, const int* mc, T* C) {                     \
    _Pragma("omp parallel for schedule(dynamic, 64)")                                     \
    for (int64_t i = 0; i < m; ++i) {                                                     \
        T* crow = C + (size_t)n * (size_t)i;                                              \
        for (int64_t c = 0; c < n; ++c) crow[c] = (T)0;                                   \
        for (int q = ar[i]; q < ar[i + 1]; ++q) {                                         \
            int j = ac[q];                                                                \
            T a = av ? av[q] : (T)1;                                                      \
            const T* brow = B + (size_t)n * (size_t)j;                                    \
            for (int k = mr[i]; k < mr[i + 1]; ++k) crow[mc[k]] += a * brow[mc[k]];       \
        }                                                                                 \
    }                                                                                     \
}                                                                                         \
                                                                                          \
/* Union of two CSR matrices with disjoint patterns, rows merged by column.               \
 * Restates add_nointersect, include/matrix_la.h:337-372 (ties take B's entry). */        \
int or_add_nointersect_##S(int64_t m, const int* ar, const int* ac, const T* av,          \
                           const int* br, const int* bc, const T* bv, int** cr_out,       \
                           int** cc_out, T** cv_out, int64_t* cnz_out) {                  \
    int* cr = (int*)xmalloc(sizeof(int) * ((size_t)m + 1));                               \
    cr[0] = 0;                                                                            \
    for (int64_t i = 1; i <= m; ++i) cr[i] = ar[i] + br[i];                               \
    int64_t nnz = cr[m];                                                                  \
    int* cc = (int*)xmalloc(sizeof(int) * (size_t)nnz);                                   \
    T* cv = (T*)xmalloc(sizeof(T) * (size_t)nnz);                                         \
    _Pragma("omp parallel for schedule(dynamic, 64)")                                     \
    for (int64_t i = 0; i < m; ++i) {                                                     \
        int x = ar[i], y = br[i], p = cr[i];                                              \
        while (x < ar[i + 1] && y < br[i + 1]) {                                          \
            if (ac[x] < bc[y]) { cc[p] = ac[x]; cv[p] = av[x]; ++x; }                     \
            else { cc[p] = bc[y]; cv[p] = bv[y]; ++y; }                                   \
            ++p;                                                                          \
        }                                                                                 \
        while (x < ar[i + 1] && p < cr[i + 1]) { cc[p] = ac[x]; cv[p] = av[x]; ++x; ++p; } \
        while (y < br[i + 1] && p < cr[i + 1]) { cc[p] = bc[y]; cv[p] = bv[y]; ++y; ++p; } \
    }                                                                                     \
    *cr_out = cr; *cc_out = cc; *cv_out = cv; *cnz_out = nnz;                             \
    return 0;                                                                             \
}                                                                                         \
                                                                                          \
/* C<M> = A .* B on dense m x n matrices; C is zeroed first.                              \
 * Restates eWiseMult(dense, dense, mask), include/matrix_la.h:200-219. */                \
void or_ewise_mult_masked_##S(int64_t m, int64_t n, const T* A, const T* B,               \
                              const int* mr, const int* mc, T* C) {                       \
    _Pragma("omp parallel for schedule(static, 64)")                                      \
    for (int64_t i = 0; i < m; ++i) {                                                     \
        T* crow = C + (size_t)n * (size_t)i;                                              \
        for (int64_t c = 0; c < n; ++c) crow[c] = (T)0;                                   \
    }                                                                                     \
    _Pragma("omp parallel for schedule(dynamic, 64)")                                     \
    for (int64_t i = 0; i < m; ++i)                                                       \
        for (int j = mr[i]; j < mr[i + 1]; ++j) {                                         \
            size_t idx = (size_t)n * (size_t)i + (size_t)mc[j];                           \
            C[idx] = A[idx] * B[idx];                                                     \
        }                                                                                 \
}                                                                                         \
                                                                                          \
/* C += A .* B element-wise. Restates fuseEWiseMultAdd, include/matrix_la.h:192-198. */   \
void or_fuse_ewise_mult_add_##S(int64_t count, const T* A, const T* B, T* C) {            \
    _Pragma("omp parallel for schedule(static, 4096)")                                    \
    for (int64_t i = 0; i < count; ++i) C[i] += A[i] * B[i];                              \
}                                                                                         \
                                                                                          \
/* Counting-sort transpose. Restates transpose(spMtx), include/matrix_la.h:166-190. */    \
int or_transpose_##S(int64_t m, int64_t n, const int* ar, const int* ac, const T* av,     \
                     int** cr_out, int** cc_out, T** cv_out) {                            \
    int64_t nnz = ar[m];                                                                  \
    int* cr = (int*)xcalloc((size_t)n + 1, sizeof(int));                                  \
    int* cc = (int*)xmalloc(sizeof(int) * (size_t)nnz);                                   \
    T* cv = (T*)xmalloc(sizeof(T) * (size_t)nnz);                                         \
    for (int64_t q = 0; q < nnz; ++q) ++cr[ac[q] + 1];                                    \
    for (int64_t r = 0; r < n; ++r) cr[r + 1] += cr[r];                                   \
    int* pos = (int*)xmalloc(sizeof(int) * ((size_t)n + 1));                              \
    memcpy(pos, cr, sizeof(int) * ((size_t)n + 1));                                       \
    for (int64_t i = 0; i < m; ++i)                                                       \
        for (int q = ar[i]; q < ar[i + 1]; ++q) {                                         \
            int p = pos[ac[q]]++;                                                         \
            cc[p] = (int)i; cv[p] = av ? av[q] : (T)1;                                    \
        }                                                                                 \
    free(pos);                                                                            \
    *cr_out = cr; *cc_out = cc; *cv_out = cv;                                             \
    return 0;                                                                             \
}                                                                                         \
                                                                                          \
/* Strict lower triangle: the leading entries of each (sorted) row with col < i.          \
 * Restates extract_lower_triangle, include/matrix.h:736-763. */                          \
int or_extract_lower_##S(int64_t m, const int* ar, const int* ac, const T* av,            \
                         int** cr_out, int** cc_out, T** cv_out, int64_t* cnz_out) {      \
    int* cr = (int*)xmalloc(sizeof(int) * ((size_t)m + 1));                               \
    cr[0] = 0;                                                                            \
    for (int64_t i = 0; i < m; ++i) {                                                     \
        int r = ar[i];                                                                    \
        while (r < ar[i + 1] && ac[r] < i) ++r;                                           \
        cr[i + 1] = cr[i] + (r - ar[i]);                                                  \
    }                                                                                     \
    int64_t nnz = cr[m];                                                                  \
    int* cc = (int*)xmalloc(sizeof(int) * (size_t)nnz);                                   \
    T* cv = (T*)xmalloc(sizeof(T) * (size_t)nnz);                                         \
    for (int64_t i = 0; i < m; ++i) {                                                     \
        int len = cr[i + 1] - cr[i];                                                      \
        memcpy(cc + cr[i], ac + ar[i], sizeof(int) * (size_t)len);                        \
        for (int q = 0; q < len; ++q) cv[cr[i] + q] = av ? av[ar[i] + q] : (T)1;          \
    }                                                                                     \
    *cr_out = cr; *cc_out = cc; *cv_out = cv; *cnz_out = nnz;                             \
    return 0;                                                                             \
}                                                                                         \
                                                                                          \
/* Strict upper triangle: the trailing entries of each row with col > i.                  \
 * Restates extract_upper_triangle, include/matrix.h:765-792. */                          \
int or_extract_upper_##S(int64_t m, const int* ar, const int* ac, const T* av,            \
                         int** cr_out, int** cc_out, T** cv_out, int64_t* cnz_out) {      \
    int* cr = (int*)xmalloc(sizeof(int) * ((size_t)m + 1));                               \
    cr[0] = 0;                                                                            \
    for (int64_t i = 0; i < m; ++i) {                                                     \
        int r = ar[i];                                                                    \
        while (r < ar[i + 1] && ac[r] <= i) ++r;                                          \
        cr[i + 1] = cr[i] + (ar[i + 1] - r);                                              \
    }                                                                                     \
    int64_t nnz = cr[m];                                                                  \
    int* cc = (int*)xmalloc(sizeof(int) * (size_t)nnz);                                   \
    T* cv = (T*)xmalloc(sizeof(T) * (size_t)nnz);                                         \
    for (int64_t i = 0; i < m; ++i) {                                                     \
        int len = cr[i + 1] - cr[i];                                                      \
        int off = ar[i + 1] - len;                                                        \
        memcpy(cc + cr[i], ac + off, sizeof(int) * (size_t)len);                          \
        for (int q = 0; q < len; ++q) cv[cr[i] + q] = av ? av[off + q] : (T)1;            \
    }                                                                                     \
    *cr_out = cr; *cc_out = cc; *cv_out = cv; *cnz_out = nnz;                             \
    return 0;                                                                             \
}                                                                                         \
                                                                                          \
/* S = L + L^T by merging each row of L with the same row of its transpose.               \
 * Restates build_symm_from_lower, include/matrix.h:700-734. */                           \
int or_symm_from_lower_##S(int64_t m, const int* ar, const int* ac, const T* av,          \
                           int** cr_out, int** cc_out, T** cv_out, int64_t* cnz_out) {    \
    int *ur, *uc; T* uv;                                                                  \
    or_transpose_##S(m, m, ar, ac, av, &ur, &uc, &uv);                                    \
    int64_t nnz = 2 * (int64_t)ar[m];                                                     \
    int* cr = (int*)xmalloc(sizeof(int) * ((size_t)m + 1));                               \
    int* cc = (int*)xmalloc(sizeof(int) * (size_t)nnz);                                   \
    T* cv = (T*)xmalloc(sizeof(T) * (size_t)nnz);                                         \
    int64_t p = 0;                                                                        \
    cr[0] = 0;                                                                            \
    for (int64_t i = 0; i < m; ++i) {                                                     \
        int x = ar[i], y = ur[i];                                                         \
        while (x < ar[i + 1] && y < ur[i + 1]) {                                          \
            if (ac[x] < uc[y]) { cc[p] = ac[x]; cv[p] = av ? av[x] : (T)1; ++x; }         \
            else { cc[p] = uc[y]; cv[p] = uv[y]; ++y; }                                   \
            ++p;                                                                          \
        }                                                                                 \
        while (x < ar[i + 1]) { cc[p] = ac[x]; cv[p] = av ? av[x] : (T)1; ++x; ++p; }     \
        while (y < ur[i + 1]) { cc[p] = uc[y]; cv[p] = uv[y]; ++y; ++p; }                 \
        cr[i + 1] = (int)p;                                                               \
    }                                                                                     \
    free(ur); free(uc); free(uv);                                                         \
    *cr_out = cr; *cc_out = cc; *cv_out = cv; *cnz_out = p;                               \
    return 0;                                                                             \
}

OR_DEFINE(int32_t, i32)
OR_DEFINE(int64_t, i64)
OR_DEFINE(float, f32)
OR_DEFINE(double, f64)
#undef OR_DEFINE

/* -------------------------------------------------------------------------
 * Element-wise operations and matrix-vector products that the reference
 * declares but its callers never use (include/matrix_la.h:272-541,
 * 1279-1291). Where the reference's code has slips, the intended operation
 * is restated and the slip named.
 * ------------------------------------------------------------------------- */
static int find_col(const int* c, int b, int e, int j) {
    while (b < e) {
        int mid = (b + e) >> 1;
        if (c[mid] < j) b = mid + 1; else e = mid;
    }
    return b;
}

#define OR_DEFINE_EWISE(T, S)                                                             \
/* Without a mask: eWiseAdd(A, B), include/matrix_la.h:375-435, the union of the rows     \
 * with A + B where both hold a column. With a mask: eWiseAdd(A, B, M), 272-335: for     \
 * every mask entry v = (0 + A(i,j)) + B(i,j), absent entries skipped, kept when v != 0  \
 * (the reference indexes B's values by A.Col at 291 and 316; B.Col is meant). */        \
int or_ewise_add_##S(int64_t m, const int* ar, const int* ac, const T* av,                \
                     const int* br, const int* bc, const T* bv, const int* mr,            \
                     const int* mc, int** cr_out, int** cc_out, T** cv_out,               \
                     int64_t* cnz_out) {                                                  \
    int* cr = (int*)xmalloc(sizeof(int) * ((size_t)m + 1));                               \
    size_t cap = 0;                                                                       \
    for (int64_t i = 0; i < m; ++i)                                                       \
        cap += mr ? (size_t)(mr[i + 1] - mr[i])                                           \
                  : (size_t)(ar[i + 1] - ar[i] + br[i + 1] - br[i]);                      \
    int* cc = (int*)xmalloc(sizeof(int) * cap);                                           \
    T* cv = (T*)xmalloc(sizeof(T) * cap);                                                 \
    int64_t p = 0;                                                                        \
    cr[0] = 0;                                                                            \
    for (int64_t i = 0; i < m; ++i) {                                                     \
        if (mr) {                                                                         \
            for (int q = mr[i]; q < mr[i + 1]; ++q) {                                     \
                int j = mc[q];                                                            \
                int x = find_col(ac, ar[i], ar[i + 1], j);                                \
                int y = find_col(bc, br[i], br[i + 1], j);                                \
                T v = (T)0;                                                               \
                if (x < ar[i + 1] && ac[x] == j) v = v + av[x];                           \
                if (y < br[i + 1] && bc[y] == j) v = v + bv[y];                           \
                if (v != (T)0) { cc[p] = j; cv[p] = v; ++p; }                             \
            }                                                                             \
        } else {                                                                          \
            int x = ar[i], y = br[i];                                                     \
            while (x < ar[i + 1] || y < br[i + 1]) {                                      \
                if (y >= br[i + 1] || (x < ar[i + 1] && ac[x] < bc[y])) {                 \
                    cc[p] = ac[x]; cv[p] = av[x]; ++x;                                    \
                } else if (x >= ar[i + 1] || bc[y] < ac[x]) {                             \
                    cc[p] = bc[y]; cv[p] = bv[y]; ++y;                                    \
                } else {                                                                  \
                    cc[p] = ac[x]; cv[p] = av[x] + bv[y]; ++x; ++y;                       \
                }                                                                         \
                ++p;                                                                      \
            }                                                                             \
        }                                                                                 \
        cr[i + 1] = (int)p;                                                               \
    }                                                                                     \
    *cr_out = cr; *cc_out = cc; *cv_out = cv; *cnz_out = p;                               \
    return 0;                                                                             \
}                                                                                         \
                                                                                          \
/* eWiseMult(A, B), include/matrix_la.h:438-483, and eWiseMult(A, B, M), 486-533: the     \
 * columns every operand holds, value A * B. (The reference's unmasked fill loop          \
 * advances i instead of its output index, 470, and its masked count loop steps the      \
 * mask twice per match, 497-504.) */                                                    \
int or_ewise_mult_##S(int64_t m, const int* ar, const int* ac, const T* av,               \
                      const int* br, const int* bc, const T* bv, const int* mr,           \
                      const int* mc, int** cr_out, int** cc_out, T** cv_out,              \
                      int64_t* cnz_out) {                                                 \
    int* cr = (int*)xmalloc(sizeof(int) * ((size_t)m + 1));                               \
    int* cc = (int*)xmalloc(sizeof(int) * (size_t)ar[m]);                                 \
    T* cv = (T*)xmalloc(sizeof(T) * (size_t)ar[m]);                                       \
    int64_t p = 0;                                                                        \
    cr[0] = 0;                                                                            \
    for (int64_t i = 0; i < m; ++i) {                                                     \
        for (int x = ar[i]; x < ar[i + 1]; ++x) {                                         \
            int j = ac[x];                                                                \
            int y = find_col(bc, br[i], br[i + 1], j);                                    \
            if (y >= br[i + 1] || bc[y] != j) continue;                                   \
            if (mr) {                                                                     \
                int z = find_col(mc, mr[i], mr[i + 1], j);                                \
                if (z >= mr[i + 1] || mc[z] != j) continue;                               \
            }                                                                             \
            cc[p] = j; cv[p] = av[x] * bv[y]; ++p;                                        \
        }                                                                                 \
        cr[i + 1] = (int)p;                                                               \
    }                                                                                     \
    *cr_out = cr; *cc_out = cc; *cv_out = cv; *cnz_out = p;                               \
    return 0;                                                                             \
}                                                                                         \
                                                                                          \
/* multScalar, include/matrix_la.h:535-541: every value times alpha, in place, the       \
 * product formed in double and converted back to T as `T *= double` does. */            \
void or_mult_scalar_##S(int64_t nnz, T* v, double alpha) {                                \
    for (int64_t q = 0; q < nnz; ++q) v[q] = (T)((double)v[q] * alpha);                   \
}                                                                                         \
                                                                                          \
/* MxV, include/matrix_la.h:1279-1284: y[i] += A(i,j) * x[j] over each row in order      \
 * (the reference reads a G.Xadj member that spMtx does not have; Rst is meant). */       \
void or_mxv_##S(int64_t m, const int* ar, const int* ac, const T* av, const T* x, T* y) { \
    for (int64_t i = 0; i < m; ++i)                                                       \
        for (int q = ar[i]; q < ar[i + 1]; ++q) {                                         \
            T prod = av[q] * x[ac[q]];                                                    \
            y[i] = y[i] + prod;                                                           \
        }                                                                                 \
}                                                                                         \
                                                                                          \
/* VxM, include/matrix_la.h:1286-1291: y[j] += A(i,j) * x[i], rows in ascending order. */ \
void or_vxm_##S(int64_t m, const int* ar, const int* ac, const T* av, const T* x, T* y) { \
    for (int64_t i = 0; i < m; ++i)                                                       \
        for (int q = ar[i]; q < ar[i + 1]; ++q) {                                         \
            T prod = av[q] * x[i];                                                        \
            y[ac[q]] = y[ac[q]] + prod;                                                   \
        }                                                                                 \
}

OR_DEFINE_EWISE(int32_t, i32)
OR_DEFINE_EWISE(int64_t, i64)
OR_DEFINE_EWISE(float, f32)
OR_DEFINE_EWISE(double, f64)
#undef OR_DEFINE_EWISE

/* -------------------------------------------------------------------------
 * Callers of the masked SpGEMM.
 * ------------------------------------------------------------------------- */

/* triangle_counting_masked_sandia, src/main.cpp:65-86: L = strict lower
 * triangle of A (67), C<L> = L*L (73), total = sum of C's values (76-78).
 * rows[i] = sum of row i of C. Values of A are taken as 1, as the CLI's
 * build_adjacency_matrix (include/matrix.h:679-698) makes them. */
int64_t or_tc_sandia(int64_t m, const int* rst, const int* col, int64_t* rows) {
    int *lr, *lc; int32_t* lv; int64_t lnz;
    or_extract_lower_i32(m, rst, col, NULL, &lr, &lc, &lv, &lnz);
    int32_t* cv = (int32_t*)xmalloc(sizeof(int32_t) * (size_t)lnz);
    or_mxm_masked_i32(m, m, lr, lc, lv, lr, lc, lv, lr, lc, cv);
    int64_t total = 0;
    for (int64_t i = 0; i < m; ++i) {
        int64_t s = 0;
        for (int j = lr[i]; j < lr[i + 1]; ++j) s += cv[j];
        if (rows) rows[i] = s;
        total += s;
    }
    free(lr); free(lc); free(lv); free(cv);
    return total;
}

/* k_truss, src/main.cpp:90-146: C = A (91); each iteration Tmp<C> = C*C (102),
 * keep entries with Tmp >= k-2 as 1 (106-117), stop when the count is unchanged
 * (120-123; the returned matrix is C, whose values are A's when that happens at
 * the first iteration), else swap (126). At most m iterations (100). */
/* Gustavson products P = sum over entries (i,j) of C of nnz(C_j) */
static int64_t products_of(int64_t m, const int* cr, const int* cc) {
    int64_t p = 0;
    for (int64_t i = 0; i < m; ++i)
        for (int q = cr[i]; q < cr[i + 1]; ++q) p += cr[cc[q] + 1] - cr[cc[q]];
    return p;
}

/* The reference CLI's reading of a Matrix Market graph (src/main.cpp:279-331
 * with read_mtx_to_crs, include/matrix.h:280-417): entries read one token at
 * a time with stdio (the reference extracts them with iostream >>),
 * self-loops dropped, symmetric files mirrored, rows placed by a counting
 * pass; then build_adjacency_matrix (all values 1) and, when `symmetrise`,
 * build_symm_from_lower(extract_lower_triangle(.)). Serial, as the
 * reference's reader is. Returns 0, or 1 when the file cannot be read. */
int or_read_mtx_cli(const char* path, int symmetrise, int64_t* m_out, int64_t* nnz_out, int** rst_out,
                    int** col_out) {
    FILE* f = fopen(path, "r");
    if (!f) return 1;
    char line[1024];
    if (!fgets(line, sizeof line, f)) { fclose(f); return 1; }
    int pattern = strstr(line, "pattern") != NULL, sym = strstr(line, "symmetric") != NULL;
    long long m = 0, n = 0, nz = 0;
    for (;;) {
        if (!fgets(line, sizeof line, f)) { fclose(f); return 1; }
        if (line[0] == '%') continue;
        if (sscanf(line, "%lld %lld %lld", &m, &n, &nz) == 3) break;
    }
    if (m != n) { fclose(f); return 1; }
    size_t cap = (size_t)(sym ? 2 * nz : nz);
    int* ra = (int*)xmalloc(sizeof(int) * cap);
    int* ca = (int*)xmalloc(sizeof(int) * cap);
    int* deg = (int*)xcalloc((size_t)m + 1, sizeof(int));
    size_t cur = 0;
    for (long long e = 0; e < nz; ++e) {
        long long r, c;
        double v;
        int got = pattern ? fscanf(f, "%lld %lld", &r, &c) : fscanf(f, "%lld %lld %lf", &r, &c, &v);
        if (got != (pattern ? 2 : 3)) break;
        if (r == c) continue;
        ra[cur] = (int)(r - 1); ca[cur++] = (int)(c - 1); ++deg[r];
        if (sym) { ra[cur] = (int)(c - 1); ca[cur++] = (int)(r - 1); ++deg[c]; }
    }
    fclose(f);
    int* rst = (int*)xmalloc(sizeof(int) * ((size_t)m + 1));
    int* fill = (int*)xmalloc(sizeof(int) * ((size_t)m + 1));
    rst[0] = 0;
    for (long long i = 0; i < m; ++i) rst[i + 1] = rst[i] + deg[i + 1];
    memcpy(fill, rst, sizeof(int) * ((size_t)m + 1));
    int* col = (int*)xmalloc(sizeof(int) * (cur ? cur : 1));
    for (size_t q = 0; q < cur; ++q) col[fill[ra[q]]++] = ca[q];
    free(ra); free(ca); free(deg); free(fill);
    if (symmetrise) {
        int *lr, *lc, *sr, *sc; int32_t *lv, *sv; int64_t lnz, snz;
        or_extract_lower_i32(m, rst, col, NULL, &lr, &lc, &lv, &lnz);
        or_symm_from_lower_i32(m, lr, lc, lv, &sr, &sc, &sv, &snz);
        free(lr); free(lc); free(lv); free(sv); free(rst); free(col);
        rst = sr; col = sc;
    }
    *m_out = m; *nnz_out = rst[m]; *rst_out = rst; *col_out = col;
    return 0;
}

int or_ktruss(int64_t m, const int* rst, const int* col, const int* val, int k,
              int** cr_out, int** cc_out, int** cv_out, int64_t* cnz_out, int* iters) {
    return or_ktruss_ex(m, rst, col, val, k, cr_out, cc_out, cv_out, cnz_out, iters, NULL);
}

int or_ktruss_ex(int64_t m, const int* rst, const int* col, const int* val, int k,
                 int** cr_out, int** cc_out, int** cv_out, int64_t* cnz_out, int* iters, int64_t* products) {
    int64_t prod = 0;
    int64_t nnz = rst[m];
    int* cr = (int*)xmalloc(sizeof(int) * ((size_t)m + 1));
    int* cc = (int*)xmalloc(sizeof(int) * (size_t)nnz);
    int* cv = (int*)xmalloc(sizeof(int) * (size_t)nnz);
    memcpy(cr, rst, sizeof(int) * ((size_t)m + 1));
    memcpy(cc, col, sizeof(int) * (size_t)nnz);
    for (int64_t q = 0; q < nnz; ++q) cv[q] = val ? val[q] : 1;
    int64_t cnz = nnz;
    int total = 0;
    int* tv = (int*)xmalloc(sizeof(int) * (size_t)(nnz ? nnz : 1));
    int* tr = (int*)xmalloc(sizeof(int) * ((size_t)m + 1));
    int* tc = (int*)xmalloc(sizeof(int) * (size_t)(nnz ? nnz : 1));
    for (int64_t t = 0; t < m; ++t) {
        if (products) prod += products_of(m, cr, cc);
        or_mxm_masked_i32(m, m, cr, cc, cv, cr, cc, cv, cr, cc, tv);
        int64_t p = 0;
        tr[0] = 0;
        for (int64_t i = 0; i < m; ++i) {
            for (int j = cr[i]; j < cr[i + 1]; ++j)
                if (tv[j] >= k - 2) { tc[p] = cc[j]; tv[p] = 1; ++p; }
            tr[i + 1] = (int)p;
        }
        if (p == cnz) { total = (int)t + 1; break; }
        /* swap C and Tmp */
        int* s;
        s = cr; cr = tr; tr = s;
        s = cc; cc = tc; tc = s;
        s = cv; cv = tv; tv = s;
        cnz = p;
    }
    free(tv); free(tr); free(tc);
    *cr_out = cr; *cc_out = cc; *cv_out = cv; *cnz_out = cnz; *iters = total;
    if (products) *products = prod;
    return 0;
}

/* betweenness_centrality_batch, include/betweenness_centrality.h:125-237,
 * restated in FP64 for an explicit list of distinct sources.
 *  setup (161-173): Numsp = identity over the sources, Front = rows of A at the
 *      sources, transposed (vertex x source);
 *  forward (176-192): Sigmas[d] = Front; Numsp = Numsp (+) Front;
 *      Front<!Numsp> = A^T * Front; until Front is empty;
 *  backward (195-218): Bcu = 1, W<Sigmas[k]> = Bcu ./ Numsp,
 *      W<Sigmas[k-1]> = A * W, Bcu += W .* Numsp, for k = d-1 .. 1;
 *  reduction (220-228): bc[i] = sum_j Bcu[i][j] - nsrc.
 * The dense copy of Numsp is zero-filled (include/matrix.h:585-596 form). */
int or_bc_batch(int64_t m, const int* rst, const int* col, const int* val,
                int64_t nsrc, const int* sources, double* bc) {
    int64_t nnz = rst[m];
    int64_t ns = nsrc;
    double* av = (double*)xmalloc(sizeof(double) * (size_t)nnz);
    for (int64_t q = 0; q < nnz; ++q) av[q] = val ? (double)val[q] : 1.0;
    int *tr, *tc; double* tv;
    or_transpose_f64(m, m, rst, col, av, &tr, &tc, &tv);

    /* Numsp: entry (sources[j], j) = 1 */
    int* owner = (int*)xmalloc(sizeof(int) * (size_t)m);
    for (int64_t v = 0; v < m; ++v) owner[v] = -1;
    for (int64_t j = 0; j < ns; ++j) owner[sources[j]] = (int)j;
    int* nr = (int*)xmalloc(sizeof(int) * ((size_t)m + 1));
    int* nc = (int*)xmalloc(sizeof(int) * (size_t)ns);
    double* nv = (double*)xmalloc(sizeof(double) * (size_t)ns);
    nr[0] = 0;
    for (int64_t v = 0, p = 0; v < m; ++v) {
        if (owner[v] >= 0) { nc[p] = owner[v]; nv[p] = 1.0; ++p; }
        nr[v + 1] = (int)p;
    }
    /* Front = transpose(A rows at the sources) */
    int* sr = (int*)xmalloc(sizeof(int) * ((size_t)ns + 1));
    int64_t snz = 0;
    for (int64_t j = 0; j < ns; ++j) snz += rst[sources[j] + 1] - rst[sources[j]];
    int* sc = (int*)xmalloc(sizeof(int) * (size_t)snz);
    double* sv = (double*)xmalloc(sizeof(double) * (size_t)snz);
    sr[0] = 0;
    for (int64_t j = 0, p = 0; j < ns; ++j) {
        int s = sources[j];
        for (int q = rst[s]; q < rst[s + 1]; ++q) { sc[p] = col[q]; sv[p] = av[q]; ++p; }
        sr[j + 1] = (int)p;
    }
    int *fr, *fc; double* fv;
    or_transpose_f64(ns, m, sr, sc, sv, &fr, &fc, &fv);
    free(sr); free(sc); free(sv);

    /* forward sweep */
    int64_t cap = 16, d = 0;
    int** Sr = (int**)xmalloc(sizeof(int*) * (size_t)cap);
    int** Sc = (int**)xmalloc(sizeof(int*) * (size_t)cap);
    for (;;) {
        if (d == cap) {
            cap *= 2;
            Sr = (int**)realloc(Sr, sizeof(int*) * (size_t)cap);
            Sc = (int**)realloc(Sc, sizeof(int*) * (size_t)cap);
        }
        Sr[d] = fr; Sc[d] = fc;  /* Sigmas[d] = Front (pattern; values live in Numsp) */
        int *ur, *uc; double* uv; int64_t unz;
        or_add_nointersect_f64(m, nr, nc, nv, fr, fc, fv, &ur, &uc, &uv, &unz);
        free(nr); free(nc); free(nv);
        nr = ur; nc = uc; nv = uv;
        int *xr, *xc; double* xv; int64_t xnz;
        or_mxm_cmask_f64(m, ns, tr, tc, tv, fr, fc, fv, nr, nc, &xr, &xc, &xv, &xnz);
        free(fv);
        fr = xr; fc = xc; fv = xv;
        ++d;
        if (xnz == 0) break;
    }
    free(fr); free(fc); free(fv);

    /* backward sweep on dense m x ns matrices */
    size_t mxn = (size_t)m * (size_t)ns;
    double* sigd = (double*)xcalloc(mxn, sizeof(double));
    for (int64_t v = 0; v < m; ++v)
        for (int q = nr[v]; q < nr[v + 1]; ++q) sigd[(size_t)ns * v + nc[q]] = nv[q];
    double* inv = (double*)xmalloc(sizeof(double) * mxn);
    double* bcu = (double*)xmalloc(sizeof(double) * mxn);
    double* W = (double*)xcalloc(mxn, sizeof(double));
    double* W2 = (double*)xcalloc(mxn, sizeof(double));
    for (size_t i = 0; i < mxn; ++i) bcu[i] = 1.0;
    for (size_t i = 0; i < mxn; ++i) inv[i] = sigd[i] != 0.0 ? 1.0 / sigd[i] : 0.0;
    for (int64_t k = d - 1; k > 0; --k) {
        or_ewise_mult_masked_f64(m, ns, inv, bcu, Sr[k], Sc[k], W);
        or_mxm_spd_f64(m, ns, rst, col, av, W, Sr[k - 1], Sc[k - 1], W2);
        or_fuse_ewise_mult_add_f64((int64_t)mxn, W2, sigd, bcu);
    }
    for (int64_t i = 0; i < m; ++i) {
        double s = 0.0;
        for (int64_t j = 0; j < ns; ++j) s += bcu[(size_t)ns * i + j];
        bc[i] = s - (double)ns;
    }
    for (int64_t q = 0; q < d; ++q) { free(Sr[q]); free(Sc[q]); }
    free(Sr); free(Sc);
    free(sigd); free(inv); free(bcu); free(W); free(W2);
    free(nr); free(nc); free(nv);
    free(tr); free(tc); free(tv);
    free(owner); free(av);
    return 0;
}

/* All-source BC, betweenness_centrality (include/betweenness_centrality.h:
 * 5-123): the sources in blocks of `block` (the last block ragged), each
 * block run as the batched algorithm over sources i..i+n-1
 * (betweenness_centrality.h:44-54 sets Numsp's identity rows i..i+n-1 and
 * Front = transpose(A.extractRows(i, i+n))), its row sums minus n added
 * into bc (:103-111). FP64. */
int or_bc_all(int64_t m, const int* rst, const int* col, const int* val, int64_t block, double* bc) {
    if (block < 1) return -1;
    double* part = (double*)xmalloc(sizeof(double) * (size_t)(m ? m : 1));
    int* src = (int*)xmalloc(sizeof(int) * (size_t)(block < m ? block : (m ? m : 1)));
    for (int64_t v = 0; v < m; ++v) bc[v] = 0.0;
    for (int64_t i = 0; i < m; i += block) {
        const int64_t n = m - i < block ? m - i : block;
        for (int64_t j = 0; j < n; ++j) src[j] = (int)(i + j);
        or_bc_batch(m, rst, col, val, n, src, part);
        for (int64_t v = 0; v < m; ++v) bc[v] += part[v];
    }
    free(part);
    free(src);
    return 0;
}
