/*
 * CPU oracle: a plain-C restatement of the reference (UAlex322/GraphAlgo)
 * algorithms on the masked-SpGEMM path.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py may load this library, and only as
 * the checker or the timed CPU baseline. The product (graphalgo_gb300) never
 * links, loads or calls it.
 *
 * Parity pinned: tests/test_oracle_pin.py checks every function here against
 * the unmodified reference (oracle/_ref/libref.so, built by oracle/build_ref.sh)
 * and against the committed golden fixtures in tests/golden/.
 *
 * Conventions (as in the reference's spMtx, include/matrix.h:23-33):
 * CSR with int32 row starts (m+1) and int32 column indices, columns sorted
 * strictly ascending inside each row. Value types: i32, i64, f32, f64.
 * Functions that create a new pattern return malloc'd arrays; free them with
 * or_free().
 */
#ifndef GA_ORACLE_H
#define GA_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

void or_free(void* p);
int or_num_threads(void);
void or_set_num_threads(int n);

#define OR_DECL(T, S)                                                              \
    void or_mxm_masked_##S(int64_t m, int64_t bn, const int* ar, const int* ac,    \
                           const T* av, const int* br, const int* bc, const T* bv, \
                           const int* mr, const int* mc, T* cv);                   \
    int or_mxm_cmask_##S(int64_t m, int64_t bn, const int* ar, const int* ac,      \
                         const T* av, const int* br, const int* bc, const T* bv,   \
                         const int* mr, const int* mc, int** cr, int** cc, T** cv, \
                         int64_t* cnz);                                            \
    void or_mxm_spd_##S(int64_t m, int64_t n, const int* ar, const int* ac,        \
                        const T* av, const T* B, const int* mr, const int* mc,     \
                        T* C);                                                     \
    int or_add_nointersect_##S(int64_t m, const int* ar, const int* ac,            \
                               const T* av, const int* br, const int* bc,          \
                               const T* bv, int** cr, int** cc, T** cv,            \
                               int64_t* cnz);                                      \
    void or_ewise_mult_masked_##S(int64_t m, int64_t n, const T* A, const T* B,    \
                                  const int* mr, const int* mc, T* C);             \
    void or_fuse_ewise_mult_add_##S(int64_t count, const T* A, const T* B, T* C);  \
    int or_transpose_##S(int64_t m, int64_t n, const int* ar, const int* ac,       \
                         const T* av, int** cr, int** cc, T** cv);                 \
    int or_extract_lower_##S(int64_t m, const int* ar, const int* ac, const T* av, \
                             int** cr, int** cc, T** cv, int64_t* cnz);            \
    int or_extract_upper_##S(int64_t m, const int* ar, const int* ac, const T* av, \
                             int** cr, int** cc, T** cv, int64_t* cnz);            \
    int or_symm_from_lower_##S(int64_t m, const int* ar, const int* ac,            \
                               const T* av, int** cr, int** cc, T** cv,            \
                               int64_t* cnz);

#define OR_DECL_EWISE(T, S)                                                            \
    int or_ewise_add_##S(int64_t m, const int* ar, const int* ac, const T* av,           \
                         const int* br, const int* bc, const T* bv, const int* mr,       \
                         const int* mc, int** cr, int** cc, T** cv, int64_t* cnz);       \
    int or_ewise_mult_##S(int64_t m, const int* ar, const int* ac, const T* av,          \
                          const int* br, const int* bc, const T* bv, const int* mr,      \
                          const int* mc, int** cr, int** cc, T** cv, int64_t* cnz);      \
    void or_mult_scalar_##S(int64_t nnz, T* v, double alpha);                            \
    void or_mxv_##S(int64_t m, const int* ar, const int* ac, const T* av, const T* x,    \
                    T* y);                                                               \
    void or_vxm_##S(int64_t m, const int* ar, const int* ac, const T* av, const T* x,    \
                    T* y);
OR_DECL_EWISE(int32_t, i32)
OR_DECL_EWISE(int64_t, i64)
OR_DECL_EWISE(float, f32)
OR_DECL_EWISE(double, f64)
#undef OR_DECL_EWISE

OR_DECL(int32_t, i32)
OR_DECL(int64_t, i64)
OR_DECL(float, f32)
OR_DECL(double, f64)
#undef OR_DECL

/* Triangle count, Sandia form C<L> = L*L with L = strict lower triangle of A;
 * rows (optional, length m) receives the row sums of C. */
/* Seeded R-MAT graph, the same as the product's generator (oracle/gen.c). */
int or_gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed, int64_t* m_out,
                int64_t* nnz_out, int** rst_out, int** col_out);
int64_t or_tc_sandia(int64_t m, const int* rst, const int* col, int64_t* rows);

/* The reference CLI's reading of a Matrix Market graph file: read_mtx_to_crs,
 * build_adjacency_matrix and, when `symmetrise`, the lower-triangle
 * symmetrisation (pattern in *rst / *col, free with or_free). */
int or_read_mtx_cli(const char* path, int symmetrise, int64_t* m, int64_t* nnz, int** rst, int** col);

/* k-truss by iterated support Tmp<C> = C*C and pruning below k-2.
 * val may be NULL (all ones). Returns 0 on success; *iters is the count the
 * reference prints. */
int or_ktruss(int64_t m, const int* rst, const int* col, const int* val, int k,
              int** cr, int** cc, int** cv, int64_t* cnz, int* iters);
/* Same, also returning the Gustavson product count summed over the
 * iterations' support products (products may be NULL). */
int or_ktruss_ex(int64_t m, const int* rst, const int* col, const int* val, int k,
                 int** cr, int** cc, int** cv, int64_t* cnz, int* iters, int64_t* products);

/* Batched betweenness centrality in FP64 over an explicit source list.
 * val may be NULL (all ones). bc has length m. */
/* All-source BC in blocks (betweenness_centrality.h:5-123), FP64. */
int or_bc_all(int64_t m, const int* rst, const int* col, const int* val, int64_t block, double* bc);
int or_bc_batch(int64_t m, const int* rst, const int* col, const int* val,
                int64_t nsrc, const int* sources, double* bc);

#ifdef __cplusplus
}
#endif
#endif
