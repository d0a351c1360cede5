/*
 * graphalgo_gb300 — GB300-native (sm_103a) masked sparse matrix-matrix
 * multiply C<M> = A*B over CSR graphs, and its callers (triangle counting,
 * k-truss, batched betweenness centrality).
 *
 * C ABI. Plain pointers and sizes; every call returns an int status (GA_OK = 0)
 * and ga_last_error(ctx) gives the message. No C++ exception crosses it.
 *
 * Drop-in for UAlex322/GraphAlgo's masked-SpGEMM path. The reference's plugin
 * seam is the function-pointer type
 *     template<T> using mxmOp = void(*)(bool, const spMtx<T>&, const spMtx<T>&,
 *                                       const spMtx<T>&, spMtx<T>&);
 * (src/main.cpp:11-12); include/graphalgo_gb300.hpp re-exposes those exact
 * signatures on top of this ABI. Each entry point below names the reference
 * function it replaces.
 *
 * Data model. A CSR matrix (the reference's spMtx<T>, include/matrix.h:23-33)
 * lives in device memory behind a ga_csr handle: int32 row starts (m+1),
 * int32 column indices sorted strictly ascending within each row, values of
 * one ga_dtype. Masks are structural (only the pattern of M matters), as in
 * every reference entry point. Dense matrices (denseMtx<T>,
 * include/matrix.h:561-666) are row-major behind a ga_dense handle.
 *
 * Threading. One ga_ctx per host thread. Calls are ordered on the context's
 * CUDA stream; functions that return host results synchronise that stream.
 */
#ifndef GRAPHALGO_GB300_H
#define GRAPHALGO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GA_API __attribute__((visibility("default")))

typedef struct ga_ctx_s* ga_ctx;
typedef struct ga_csr_s* ga_csr;
typedef struct ga_dense_s* ga_dense;

/* value types (the reference's T: int for graphs, float/double for BC) */
typedef enum {
    GA_INT32 = 0,
    GA_INT64 = 1,
    GA_FP32 = 2,
    GA_FP64 = 3,
    GA_UINT8 = 4
} ga_dtype;

/* masked-SpGEMM variants: the reference's four mxmOp implementations,
 * plus an inner-product (sorted-list intersection) form */
typedef enum {
    GA_MSA = 0,   /* mxmm_msa,   include/matrix_la.h:700-749 */
    GA_MCA = 1,   /* mxmm_mca,   include/matrix_la.h:586-641 */
    GA_HEAP = 2,  /* mxmm_heap,  include/matrix_la.h:1013-1084 (sorted merges of B rows with the mask row
                     here: by a lane, by 32 lanes over slices, or by the whole warp, galloping) */
    GA_NAIVE = 3, /* mxmm_naive, include/matrix_la.h:1139-1277 */
    GA_DOT = 4,   /* inner-product form: each mask entry (i,j) is A_i . (B^T)_j by warp
                     sorted-list intersection (B^T built on the fly unless B is
                     symmetric); TC's dot kernel; k-truss support (symmetric A) */
    GA_AUTO = 5,  /* the autotuner's choice of variant and schedule (ga_autotune) */
    GA_HYBRID = 6, /* per output row, the cheaper of MSA (Gustavson work: the row's
                     products) and the inner-product form (work: sum over its mask
                     entries of min(|A_i|, |B^T_j|)), decided while binning */
    GA_TRI = 7     /* triangle listing, for C<A> = A*A with A one symmetric int32
                     matrix of unit values (the k-truss support): vertices ranked
                     by (degree, index), each triangle found once as a wedge of
                     increasing rank and counted on its three edges; any other
                     operands (and k-truss from non-unit values) run GA_HYBRID */
} ga_algo;

/* status codes */
enum {
    GA_OK = 0,
    GA_ERR_INVALID_ARG = 1,
    GA_ERR_INVALID_CSR = 2, /* unsorted / out-of-range / malformed CSR */
    GA_ERR_SHAPE = 3,       /* dimensions do not agree */
    GA_ERR_DTYPE = 4,       /* value types do not agree or are unsupported */
    GA_ERR_CUDA = 5,        /* a CUDA runtime call failed */
    GA_ERR_OOM = 6,         /* device allocation failed (or was injected) */
    GA_ERR_NO_DEVICE = 7,   /* no CUDA device / the kernels are not loadable */
    GA_ERR_TIMEOUT = 8,     /* a bounded device wait expired */
    GA_ERR_UNSUPPORTED = 9,
    GA_ERR_ADMISSION = 10,  /* request refused: HBM bound exceeded */
    GA_ERR_CANCELLED = 11   /* request cancelled before it started */
};

/* ------------------------------------------------------------------ context */
/* stream may be NULL (the context creates its own non-blocking stream) or a
 * cudaStream_t owned by the caller. */
GA_API int ga_ctx_create(int device, void* stream, ga_ctx* out);
GA_API int ga_ctx_destroy(ga_ctx ctx);
GA_API const char* ga_last_error(ga_ctx ctx);
GA_API const char* ga_status_string(int status);
GA_API int ga_ctx_sync(ga_ctx ctx);
GA_API int ga_ctx_stream(ga_ctx ctx, void** stream);
GA_API int ga_device_count(int* count);
GA_API int ga_version(int* major, int* minor);

/* Context options. GA_OPT_DEVICE_LOOPS (default 1): run the k-truss and BC
 * iteration loops as CUDA graphs with device-side WHILE conditions (no host
 * round trip per iteration); 0 runs the same kernels from a host loop.
 * GA_OPT_PROFILE: when 1, each kernel launch is bracketed by CUDA events and
 * ga_ctx_kernel_stats reports per-kernel totals. GA_OPT_FAIL_ALLOC_AFTER:
 * fault injection for tests — the N-th device allocation from now on fails
 * with GA_ERR_OOM (-1 disables). GA_OPT_KNN_TILED: when 1, ga_gen_knn_batch
 * uses its tiled kernel (the one for graphs above 4,096 points) for every
 * graph; both kernels give the same graphs. Masked-product schedule (what
 * the autotuner chooses; results do not depend on it):
 * GA_OPT_MXM_WARP_FLOPS (32768): output rows with at most this many
 * Gustavson products (and at most 256 mask entries) are computed by one
 * warp, larger rows by CTAs; GA_OPT_MXM_HEAVY_FLOPS (2^20): CTA work of rows
 * with at least this many products is scheduled first;
 * GA_OPT_MXM_CTAS_PER_SM (0 = as many as fit): persistent grid size;
 * GA_OPT_DOT_CHUNK (8): mask entries per warp task of the inner-product form;
 * GA_OPT_HYBRID_RATIO (16): GA_HYBRID sends a row to the inner-product form
 * when its inner-product work times this is below its Gustavson work;
 * GA_OPT_TRI_ORDER (0): GA_TRI ranks vertices by degree (0; power-law
 * graphs) or by index (1; unions of small graphs).
 * GA_OPT_KT_FRONTIER (1): the GA_TRI k-truss of one matrix lists the
 * triangles once and then, per iteration, only the triangles of the edges it
 * prunes, lowering the supports they touch (same edge sets and iteration
 * counts); 0 lists every triangle again in every iteration.
 * GA_OPT_BC_BACKWARD (0): how BC's backward sweep reads the dependency
 * rows W[w] of a vertex's next-level neighbours: 0 gathers, the rows of
 * four neighbours in flight at once; 1 bulk copies (cp.async.bulk) of whole
 * rows into shared memory, two batches of four rows in flight per warp
 * (used for even source counts up to 128, else 0 runs); 2 one neighbour at
 * a time. Results are the same. */
enum { GA_OPT_DEVICE_LOOPS = 1, GA_OPT_PROFILE = 2, GA_OPT_FAIL_ALLOC_AFTER = 3, GA_OPT_KNN_TILED = 4,
       GA_OPT_MXM_WARP_FLOPS = 5, GA_OPT_MXM_HEAVY_FLOPS = 6, GA_OPT_MXM_CTAS_PER_SM = 7, GA_OPT_DOT_CHUNK = 8,
       GA_OPT_HYBRID_RATIO = 9, GA_OPT_TRI_ORDER = 10, GA_OPT_KT_FRONTIER = 11, GA_OPT_BC_BACKWARD = 12 };
GA_API int ga_ctx_set_option(ga_ctx ctx, int option, int64_t value);

/* Per-kernel timing collected while GA_OPT_PROFILE is on. Writes up to `cap`
 * records; *count receives the number of distinct kernels. */
typedef struct {
    char name[48];
    int64_t launches;
    double total_ms;
} ga_kernel_stat;
GA_API int ga_ctx_kernel_stats(ga_ctx ctx, ga_kernel_stat* out, int cap, int* count);
GA_API int ga_ctx_reset_kernel_stats(ga_ctx ctx);

/* Stream-ordered device timer: ga_timer_start records an event on the
 * context's stream; ga_timer_stop records another, synchronises and returns
 * the elapsed milliseconds. */
GA_API int ga_timer_start(ga_ctx ctx);
GA_API int ga_timer_stop(ga_ctx ctx, double* ms);

/* Free / total device memory as the CUDA runtime sees it. */
GA_API int ga_mem_info(ga_ctx ctx, int64_t* free_bytes, int64_t* total_bytes);
/* Device bytes the context's allocations hold now and at most since the last
 * reset (requested sizes; reset_peak != 0 sets the peak to the current use). */
GA_API int ga_ctx_mem_stats(ga_ctx ctx, int64_t* in_use, int64_t* peak, int reset_peak);

/* Work counters accumulated on the device by every masked-SpGEMM launch of
 * this context (MSA / MCA / HEAP / DOT): Gustavson products P = sum over A entries
 * (i,k) of nnz(B_k) (the work of the reference's C<M> = A*B), mask entries,
 * launches, A entries, rows, and the products the kernels actually processed
 * (fewer than P when a k-truss support product only evaluates the upper
 * triangle of a symmetric matrix and mirrors it; for HEAP the B entries its
 * merges compared, the galloping merges skipping runs that cannot meet the
 * mask), and the list entries the
 * inner-product intersections walked (DOT, and the hybrid form's
 * inner-product rows), and for GA_TRI the wedges it looked up and the
 * triangles it found; for the frontier k-truss (GA_TRI, after its one
 * listing) the pruned edges whose triangles it walked, the row entries it
 * probed and the triangles it destroyed. They feed the GFLOP/s (2P)
 * and byte models. out has GA_CTR_COUNT entries; reset != 0 zeroes them
 * after reading. Synchronises the stream. */
enum { GA_CTR_PRODUCTS = 0, GA_CTR_MASK_ENTRIES = 1, GA_CTR_LAUNCHES = 2, GA_CTR_A_ENTRIES = 3,
       GA_CTR_ROWS = 4, GA_CTR_EXECUTED = 5, GA_CTR_EXECUTED_DOT = 6, GA_CTR_WEDGES = 7,
       GA_CTR_TRIANGLES = 8, GA_CTR_FRONT_EDGES = 9, GA_CTR_FRONT_PROBES = 10, GA_CTR_FRONT_TRIANGLES = 11,
       GA_CTR_COUNT = 12 };
GA_API int ga_ctx_work_counters(ga_ctx ctx, int64_t* out, int reset);

/* Kernel launches issued by this library in this process so far (counted on
 * the host; a launch captured into a CUDA graph counts once, when captured). */
GA_API int64_t ga_kernel_launches(void);

/* Writes a device buffer larger than the L2 cache (256 MiB) on the context
 * stream, so the next timed step starts with a cold L2. */
GA_API int ga_ctx_flush_l2(ga_ctx ctx);

/* Page-lock (or release) host memory the caller owns, for fast async copies
 * (cudaHostRegister / cudaHostUnregister). */
GA_API int ga_host_register(void* ptr, size_t bytes);
GA_API int ga_host_unregister(void* ptr);

/* --------------------------------------------------------------- CSR handle */
/* Upload a host CSR (spMtx::Rst/Col/Val). val may be NULL: all ones.
 * The pattern is validated on the device (monotone row starts, in-range and
 * strictly ascending columns); a malformed matrix gives GA_ERR_INVALID_CSR.
 * Replaces the spMtx constructors / copy (include/matrix.h:56-80). */
GA_API int ga_csr_upload(ga_ctx ctx, int64_t m, int64_t n, int64_t nnz,
                         const int32_t* rst, const int32_t* col, const void* val,
                         ga_dtype dtype, ga_csr* out);
/* Same from device pointers (copied on the device); no host traffic. */
GA_API int ga_csr_from_device(ga_ctx ctx, int64_t m, int64_t n, int64_t nnz,
                              const int32_t* d_rst, const int32_t* d_col, const void* d_val,
                              ga_dtype dtype, ga_csr* out);
GA_API int ga_csr_info(ga_csr A, int64_t* m, int64_t* n, int64_t* nnz, int* dtype);
/* Copy back into caller-allocated host arrays (rst: m+1, col/val: nnz).
 * Any of the three may be NULL to skip it. */
GA_API int ga_csr_download(ga_ctx ctx, ga_csr A, int32_t* rst, int32_t* col, void* val);
/* Asynchronous download on the context's copy stream: it starts once the
 * work queued so far on the context's stream is done and overlaps with work
 * queued after it. Host buffers should be page-locked (ga_host_register)
 * for the copy to be asynchronous. ga_ctx_copy_sync waits for every
 * download; ga_csr_free on a handle orders its free after them. */
GA_API int ga_csr_download_async(ga_ctx ctx, ga_csr A, int32_t* rst, int32_t* col, void* val);
GA_API int ga_ctx_copy_sync(ga_ctx ctx);
GA_API int ga_csr_device_ptrs(ga_csr A, void** rst, void** col, void** val);
GA_API int ga_csr_free(ga_ctx ctx, ga_csr A);
/* Declares whether A is symmetric (pattern and values), which the
 * triangle-listing and inner-product forms, the symmetric k-truss loop and
 * BC otherwise check on the device once per handle (a search per entry for
 * its mirror). symmetric = 1: no check is run; A must be symmetric (a false
 * declaration gives wrong results). 0: A is treated as not symmetric. -1:
 * the check runs again on the next use. No counterpart in the reference
 * (its CLI symmetrises the graphs it reads, src/main.cpp:221-222). */
GA_API int ga_csr_set_symmetric(ga_ctx ctx, ga_csr A, int symmetric);
/* Deep copy, optionally converting the value type
 * (convertType, include/matrix.h:668-677). */
GA_API int ga_csr_convert(ga_ctx ctx, ga_csr A, ga_dtype dtype, ga_csr* out);

/* ------------------------------------------------------------- dense handle */
GA_API int ga_dense_create(ga_ctx ctx, int64_t m, int64_t n, ga_dtype dtype, const void* host_vals,
                           ga_dense* out);
GA_API int ga_dense_download(ga_ctx ctx, ga_dense D, void* host_vals);
GA_API int ga_dense_info(ga_dense D, int64_t* m, int64_t* n, int* dtype);
GA_API int ga_dense_device_ptr(ga_dense D, void** vals);
GA_API int ga_dense_free(ga_ctx ctx, ga_dense D);
/* Dense copy of a sparse matrix, zero-filled elsewhere
 * (denseMtx(const spMtx&), include/matrix.h:585-596). */
GA_API int ga_dense_from_csr(ga_ctx ctx, ga_csr A, ga_dense* out);

/* -------------------------------------------------------- masked SpGEMM */
/* C<M> = A*B, structural mask: C has M's pattern (row starts and columns of
 * M), values sum_k A[i][k]*B[k][j] or an explicit 0.
 * Replaces mxmm_msa / mxmm_mca / mxmm_heap / mxmm_naive
 * (include/matrix_la.h:700-713, 586-599, 1013-1028, 1139-1277).
 * A, B share a dtype; M may have any dtype. *C is a new handle. */
GA_API int ga_mxm_masked(ga_ctx ctx, ga_algo algo, ga_csr A, ga_csr B, ga_csr M, ga_csr* C);
/* Same, writing only the values into a caller-provided device array aligned
 * with M's pattern (length nnz(M), A's dtype). No allocation of C. */
GA_API int ga_mxm_masked_vals(ga_ctx ctx, ga_algo algo, ga_csr A, ga_csr B, ga_csr M, void* d_cvals);

/* Allocation-free C<M> = A*B (no counterpart in the reference). For callers
 * that cannot allocate device memory when they need the product: an
 * application that hands the whole device-memory budget to its own arena at
 * start-up and lets no library allocate, or a latency-critical caller that
 * cannot accept the device-wide synchronisation cudaMalloc / cudaFree may
 * cause. Every argument is a device pointer the caller owns: CSR arrays of
 * A (m x k), B (k x n) and the mask M (m x n, mask_nnz entries, structural),
 * and c_val (mask_nnz values of `dtype`, aligned with M's pattern). No
 * context and no allocation: the kernel's scratch lives in one fixed 16 MiB
 * device array inside this library, which every GPU that loads the library
 * keeps until the process exits. algo is GA_MSA, GA_MCA or GA_HEAP, run with
 * the default schedule (a context's tuned schedule does not apply here);
 * b_unit != 0 promises that B's values are all 1, and GA_MSA / GA_MCA then do
 * not read b_val (GA_HEAP always does: b_val may be NULL only for the other
 * two). The work runs on `stream` (NULL: the default stream) and is not
 * synchronised. Returns GA_ERR_INVALID_ARG for a NULL array and when the
 * scratch this shape needs
 * - 256 + 4(m+1) + 16 + 16 min(m(1 + ceil(n/2^17)) + mask_nnz/4096 + 1,
 * mask_nnz + 1) bytes - exceeds 16 MiB (about 460k rows when n <= 2^17).
 * The first call on a device looks up the array's device address for that
 * device; make that first call before any stream capture. Calls share the
 * array: two calls whose work overlaps on the GPU race with each other, so
 * order them on one stream (each call clears what must start at zero). */
GA_API int ga_mxm_masked_noalloc(void* stream, ga_algo algo, int64_t m, int64_t k, int64_t n,
                                 const int32_t* a_rst, const int32_t* a_col, const void* a_val,
                                 const int32_t* b_rst, const int32_t* b_col, const void* b_val,
                                 const int32_t* m_rst, const int32_t* m_col, int64_t mask_nnz,
                                 ga_dtype dtype, int b_unit, void* c_val);

/* C<!M> = A*B: the structural product minus M's pattern, columns sorted.
 * Replaces mxmm_msa_cmask (include/matrix_la.h:788-891). An empty M gives
 * the unmasked product. */
GA_API int ga_mxm_cmask(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr M, ga_csr* C);

/* Dense C<M> = A*B with B and C dense (m x n); C is zero outside M.
 * Replaces mxmm_spd (include/matrix_la.h:241-270). C may not alias B. */
GA_API int ga_mxm_spd(ga_ctx ctx, ga_csr A, ga_dense B, ga_csr M, ga_dense C);

/* ------------------------------------------------------ element-wise helpers */
/* Union of two matrices with disjoint patterns (include/matrix_la.h:337-372). */
GA_API int ga_add_nointersect(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr* C);
/* Dense C<M> = A .* B, zero elsewhere (include/matrix_la.h:200-219). */
GA_API int ga_ewise_mult_masked(ga_ctx ctx, ga_dense A, ga_dense B, ga_csr M, ga_dense C);
/* Dense C += A .* B (include/matrix_la.h:192-198). */
GA_API int ga_fuse_ewise_mult_add(ga_ctx ctx, ga_dense A, ga_dense B, ga_dense C);

/* --------------------------------- sparse element-wise and matrix-vector
 * The GraphBLAS-style operations the reference declares but its callers
 * never use (include/matrix_la.h:272-541, 1279-1291), with the intended
 * semantics where its code slips (named in the oracle's restatement).
 * A, B (and M) have equal shapes; A and B equal dtypes; M is a pattern. */
/* M NULL: eWiseAdd(A, B), matrix_la.h:375-435: the union of the rows, A + B
 * where both hold a column. M given: eWiseAdd(A, B, M), 272-335: at every
 * mask entry (0 + A(i,j)) + B(i,j), kept when nonzero. */
GA_API int ga_ewise_add(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr M, ga_csr* C);
/* eWiseMult(A, B [, M]), matrix_la.h:438-533: the columns every operand
 * holds, value A * B. */
GA_API int ga_ewise_mult(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr M, ga_csr* C);
/* multScalar, matrix_la.h:535-541: A's values times alpha in place (formed
 * in double, converted back to A's type). */
GA_API int ga_mult_scalar(ga_ctx ctx, ga_csr A, double alpha);
/* MxV, matrix_la.h:1279-1284: y += A x (x: A.n values, y: A.m values, any
 * dense shape of that size, A's dtype); each row's terms summed in order. */
GA_API int ga_mxv(ga_ctx ctx, ga_csr A, ga_dense x, ga_dense y);
/* VxM, matrix_la.h:1286-1291: y += x^T A (x: A.m values, y: A.n values),
 * each column's terms summed in row order. */
GA_API int ga_vxm(ga_ctx ctx, ga_csr A, ga_dense x, ga_dense y);

/* ------------------------------------------------------------ graph prep */
GA_API int ga_transpose(ga_ctx ctx, ga_csr A, ga_csr* AT);          /* matrix_la.h:166-190 */
GA_API int ga_extract_lower(ga_ctx ctx, ga_csr A, ga_csr* L);       /* matrix.h:736-763 */
GA_API int ga_extract_upper(ga_ctx ctx, ga_csr A, ga_csr* U);       /* matrix.h:765-792 */
GA_API int ga_symm_from_lower(ga_ctx ctx, ga_csr L, ga_csr* S);     /* matrix.h:700-734 */
/* All values set to 1 as int32 (build_adjacency_matrix, matrix.h:679-698). */
GA_API int ga_adjacency(ga_ctx ctx, ga_csr A, ga_csr* adj);

/* ------------------------------------------------- edge lists and files
 * Ingestion builds the CSR on the device: entries are counted and placed
 * per row, each row is sorted by column, and duplicate (i, j) entries merge
 * onto the value of the earliest one in input order (the product's kernels
 * need strictly ascending columns; the reference keeps duplicates, which
 * files that follow the Matrix Market rules never hold).
 * The flags select the reference CLI's preparation steps. */
enum {
    GA_EDGES_MIRROR = 1,     /* each kept edge (i, j) also stored as (j, i), right after it
                                (symmetric Matrix Market files, matrix.h:339-346) */
    GA_EDGES_DROP_LOOPS = 2, /* drop (i, i) (the Matrix Market reader, matrix.h:355-358) */
    GA_EDGES_LOWER_SYMM = 4, /* keep i > j only and mirror: build_symm_from_lower(
                                extract_lower_triangle(.)), src/main.cpp:221-222 */
    GA_EDGES_UNIT = 8        /* int32 values, all 1: build_adjacency_matrix, matrix.h:679-698 */
};
/* Edge list (src[e], dst[e], val[e] of `dtype`; val NULL: all 1) to an
 * m x n CSR. Host arrays; ga_csr_from_device_edges takes device arrays.
 * An endpoint outside the matrix gives GA_ERR_INVALID_ARG. */
GA_API int ga_csr_from_edges(ga_ctx ctx, int64_t m, int64_t n, int64_t ne, const int32_t* src,
                             const int32_t* dst, const void* val, ga_dtype dtype, int flags, ga_csr* out);
GA_API int ga_csr_from_device_edges(ga_ctx ctx, int64_t m, int64_t n, int64_t ne, const int32_t* src,
                                    const int32_t* dst, const void* val, ga_dtype dtype, int flags,
                                    ga_csr* out);
/* Matrix Market coordinate file, as spMtx(filename, "mtx") reads it
 * (matrix.h:280-417): the body is parsed on the device; self-loops are
 * dropped, symmetric files mirrored; real files give GA_FP64 values,
 * integer files GA_INT32, pattern files GA_INT32 ones (src/main.cpp:279-310).
 * `flags` may add GA_EDGES_LOWER_SYMM and GA_EDGES_UNIT (the CLI's
 * preparation). Complex or array files and non-square matrices are refused
 * (matrix.h:301-309). `matcode` (4 bytes, may be NULL) receives the file's
 * Matrix Market type code. Real values are correctly rounded (equal to
 * strtod's). */
GA_API int ga_read_mtx(ga_ctx ctx, const char* path, int flags, char* matcode, ga_csr* out);
/* Binary CSR file of write_crs_to_bin (matrix.h:259-277, 441-482): matcode,
 * m, n, nz as 8-byte integers, Rst, Col, Val; values are doubles when
 * matcode[2] is 'R', int32 otherwise. Rows are sorted and duplicates merged
 * as above; `flags` as for ga_read_mtx. */
GA_API int ga_read_bin(ga_ctx ctx, const char* path, int flags, char* matcode, ga_csr* out);
/* Writes A (GA_INT32 or GA_FP64) in that layout; `matcode` NULL writes
 * "MCIG" / "MCRG". */
GA_API int ga_write_bin(ga_ctx ctx, ga_csr A, const char* matcode, const char* path);

/* ------------------------------------------------------------ algorithms */
/* Triangle count of an undirected graph given as symmetric adjacency A.
 * algo GA_MSA/MCA/HEAP/NAIVE: C<L> = L*L with that variant, L = strict lower
 * triangle of A, total = sum of C (triangle_counting_masked_sandia,
 * src/main.cpp:65-86); GA_DOT: the same counts by warp-level sorted-list
 * intersections; GA_TRI: by listing every triangle once (a symmetric A; any
 * other A takes the Sandia form with GA_HYBRID); GA_HYBRID and GA_AUTO as
 * for the masked product. per_row (host, length m, may be NULL) receives the row sums
 * of C<L> = L*L: triangles whose largest vertex is that row. Values of A are
 * ignored (the reference CLI makes them 1, src/main.cpp:335). */
GA_API int ga_tc(ga_ctx ctx, ga_algo algo, ga_csr A, int64_t* total, int64_t* per_row);
/* Device-result variant: writes the total into d_total (int64, device) and
 * per-row counts into d_per_row (device, length m, may be NULL); no sync. */
GA_API int ga_tc_device(ga_ctx ctx, ga_algo algo, ga_csr A, int64_t* d_total, int64_t* d_per_row);
/* Other TC forms: C<A> = L*U summed and halved (triangle_counting_masked_lu,
 * src/main.cpp:40-62), and per-vertex counts (A*A<A> row sums)/2
 * (triangle_counting_vertex, src/main.cpp:14-37; per_vertex has length m). */
GA_API int ga_tc_lu(ga_ctx ctx, ga_algo algo, ga_csr A, int64_t* total);
GA_API int ga_tc_vertex(ga_ctx ctx, ga_algo algo, ga_csr A, int32_t* per_vertex);

/* k-truss (src/main.cpp:90-146): iterate Tmp<C> = C*C with the chosen
 * variant, keep entries >= k-2 as 1, stop when nnz is unchanged. The loop
 * stays on the device. *C is the returned matrix; *iters the iteration count
 * the reference prints (0 if it did not converge within m iterations).
 * A must be int32. */
GA_API int ga_ktruss(ga_ctx ctx, ga_algo algo, ga_csr A, int k, ga_csr* C, int* iters);

/* k-truss sweep: C_k for k = kmin, kmin + 1, ... until C_k is empty, each
 * C_k and its iteration count equal to ga_ktruss(C_{k-1}, k) (the
 * reference's k_truss, src/main.cpp:90-146, applied to the previous
 * result). ga_ktruss_sweep_next returns the next C_k (the caller frees it)
 * with its k and iteration count, and *C = NULL once the empty truss has
 * been returned. With GA_TRI (or GA_AUTO choosing it) on a symmetric matrix
 * of unit values the k-truss state stays on the device from one k to the
 * next: the triangles are listed once for the whole sweep and each k starts
 * from the supports the previous k left; other cases run one ga_ktruss per
 * k. A is copied by ga_ktruss_sweep_begin; free the sweep before its
 * context. No counterpart in the reference (its CLI runs one k per call). */
typedef struct ga_kt_sweep_s* ga_kt_sweep;
GA_API int ga_ktruss_sweep_begin(ga_ctx ctx, ga_algo algo, ga_csr A, int kmin, ga_kt_sweep* sweep);
GA_API int ga_ktruss_sweep_next(ga_kt_sweep sweep, ga_csr* C, int* k, int* iters);
GA_API int ga_ktruss_sweep_free(ga_kt_sweep sweep);

/* Batched betweenness centrality (betweenness_centrality_batch,
 * include/betweenness_centrality.h:125-237) for an explicit list of distinct
 * sources, path counts and dependencies in FP64. bc (host, length m). The
 * reference itself uses sources 0..batch-1. A must be square without
 * self-loops; values are used as the reference's algebra uses them. */
GA_API int ga_bc(ga_ctx ctx, ga_csr A, const int32_t* sources, int64_t nsrc, double* bc);
/* Device-result variant (bc: device array of length m, overwritten). */
GA_API int ga_bc_device(ga_ctx ctx, ga_csr A, const int32_t* d_sources, int64_t nsrc, double* d_bc);
/* All-source betweenness centrality (betweenness_centrality,
 * include/betweenness_centrality.h:5-123): sources 0..m-1 in blocks of
 * `block` (>= 1), each block's scores added into bc (host, length m) on the
 * device, FP64. The reference adds each block's row sums minus the block's
 * size; that is the block's dependency sum, which is what is added here.
 * Blocks larger than 1,024 sources run as consecutive device batches of at
 * most 1,024 (BC is a sum over sources: the block size changes only the
 * order of the additions). GA_ERR_INVALID_ARG for block < 1. */
GA_API int ga_bc_all(ga_ctx ctx, ga_csr A, int64_t block, double* bc);
/* Device-result variant (bc: device array of length m, overwritten). */
GA_API int ga_bc_all_device(ga_ctx ctx, ga_csr A, int64_t block, double* d_bc);

/* -------------------------------------------------------------- autotuner */
/* Times candidate schedules — MSA with three warp/CTA bin thresholds and
 * two grid sizes, MCA, the inner-product form with three chunk sizes, the
 * hybrid form with three ratios, and triangle listing where the operands
 * are one symmetric 0/1 matrix — on the caller's problem (L2 flushed before
 * each run) and keeps the fastest for problems of the same signature
 * (device, kind, half-octave size buckets, symmetry and unit values) in a
 * process-wide cache; GA_AUTO calls use it, tuning
 * on first use. Kinds: GA_TUNE_KTRUSS (the support product C<A> = A*A of
 * k-truss), GA_TUNE_PRODUCT (A*B masked by M), GA_TUNE_TC (triangle count
 * of A). force != 0 re-tunes. Tuning launches are not counted in the work
 * counters. No counterpart in the reference (its variant is a CLI flag). */
enum { GA_TUNE_KTRUSS = 0, GA_TUNE_PRODUCT = 1, GA_TUNE_TC = 2 };
typedef struct {
    int algo;               /* chosen ga_algo */
    int64_t warp_max_flops, heavy_flops;
    int ctas_per_sm, dot_chunk;
    int64_t hybrid_ratio;
    double ms;              /* its time on the problem */
    double default_ms;      /* the default schedule (MSA) on the same problem */
    int candidates;
    int cached;             /* 1: taken from the cache, no timing run */
    int tri_order;          /* GA_OPT_TRI_ORDER of the choice */
} ga_tune_result;
GA_API int ga_autotune(ga_ctx ctx, int kind, ga_csr A, ga_csr B, ga_csr M, int force, ga_tune_result* out);
/* The same restricted to one variant (GA_MSA, GA_MCA, GA_DOT, GA_HYBRID or
 * GA_TRI; -1: any):
 * tunes that variant's schedule only. To run it, set the result's schedule
 * with ga_ctx_set_option and call with that variant. */
GA_API int ga_autotune_variant(ga_ctx ctx, int kind, int algo, ga_csr A, ga_csr B, ga_csr M, int force,
                               ga_tune_result* out);
/* The process-wide tuning cache as a text file (one line per problem
 * signature and its choice), so later processes start tuned: save writes
 * every entry, load adds the file's entries (a malformed file loads nothing
 * and gives GA_ERR_INVALID_ARG), clear empties the cache. entries (may be
 * NULL) receives the number written or read. */
GA_API int ga_tune_save(const char* path, int64_t* entries);
GA_API int ga_tune_load(const char* path, int64_t* entries);
GA_API int ga_tune_clear(void);

/* ------------------------------------------------------ batched graphs */
/* Many independent graphs as one block-diagonal matrix: rows (and columns)
 * of graph g are voff[g] .. voff[g+1]-1. The batched calls run each kernel
 * once over the whole union (the masked-SpGEMM work queue holds the row bins
 * of every graph) and return per-graph results equal to running each graph
 * alone. No counterpart in the reference, whose callers take one graph. */
/* Concatenate `count` CSR handles of one dtype into a block-diagonal U;
 * voff (host, count+1 entries, may be NULL) receives the row offsets. */
GA_API int ga_csr_block_diag(ga_ctx ctx, int64_t count, const ga_csr* parts, ga_csr* U, int64_t* voff);
/* Seeded k-NN graphs built on the device: graph g has n[g] points (1..4096)
 * i.i.d. N(0,1) in dim[g] dimensions (1..32), each linked to its k nearest
 * by FP32 Euclidean distance (self excluded, ties to the smaller index),
 * symmetrised by union; int32 unit values, rows sorted. Returns the union
 * and its row offsets (voff, host, count+1). */
GA_API int ga_gen_knn_batch(ga_ctx ctx, int64_t count, const int32_t* n, const int32_t* dim, int k,
                            uint64_t seed, ga_csr* U, int64_t* voff);
/* Per-graph triangle counts (totals: host, count entries) of a block-diagonal
 * union of symmetric adjacency matrices, as ga_tc would give for each graph. */
GA_API int ga_batch_tc(ga_ctx ctx, ga_algo algo, ga_csr U, int64_t count, const int64_t* voff, int64_t* totals);
/* Per-graph k-truss of a block-diagonal union (int32, all values 1): one
 * device loop prunes every graph, a graph stops changing once it converged,
 * and iters (host, count entries) receives each graph's iteration count as
 * ga_ktruss reports it. *C is the union of the per-graph results. */
GA_API int ga_batch_ktruss(ga_ctx ctx, ga_algo algo, ga_csr U, int64_t count, const int64_t* voff, int k,
                           ga_csr* C, int* iters);
/* The same with one k per graph (k: host, count entries). */
GA_API int ga_batch_ktruss_k(ga_ctx ctx, ga_algo algo, ga_csr U, int64_t count, const int64_t* voff, const int* k,
                             ga_csr* C, int* iters);
/* Batched BC over a block-diagonal union: graph g's sources are
 * sources[soff[g] .. soff[g+1]) (vertex indices within graph g, distinct;
 * soff: host, count+1 entries, at most 1,024 sources per graph). No path
 * leaves a graph, so the j-th sources of all graphs share one column of the
 * per-(vertex, source) state: it holds union vertices x the largest source
 * count. bc (host, length m of the union) holds in graph g's rows the
 * scores ga_bc gives for graph g and its sources alone (FP64, up to the
 * order of the sums). */
GA_API int ga_batch_bc(ga_ctx ctx, ga_csr U, int64_t count, const int64_t* voff, const int64_t* soff,
                       const int32_t* sources, double* bc);

/* ------------------------------------------------------- request server */
/* Serves triangle-count, k-truss and BC requests on device-resident graphs
 * as they arrive. Worker threads each own a context (stream), so calls of
 * different workers overlap on the device. Every request has an upper bound
 * on the device bytes its call allocates (ga_request_bytes_bound); a worker
 * starts the oldest queued request only while the bounds of the calls in
 * flight plus its own fit in the HBM budget, and a request whose bound alone
 * exceeds the budget completes with GA_ERR_ADMISSION. With coalesce on, a
 * worker that takes a request on a small graph also takes the queued
 * requests of the same type on small graphs and serves them with one
 * batched call (ga_batch_tc, ga_batch_ktruss_k with one k per graph,
 * ga_batch_bc); each request gets the result it gets alone. workers = 1
 * with coalesce = 0 is the plain sequential form. No counterpart in the
 * reference (one graph per run). */
typedef struct ga_server_s* ga_server;
enum { GA_REQ_TC = 0, GA_REQ_KTRUSS = 1, GA_REQ_BC = 2 };
typedef struct {
    int workers;                   /* worker threads (1..64); 0: 4 */
    int coalesce;                  /* 1: batch queued requests on small graphs */
    int tc_algo;                   /* ga_algo of TC (any; GA_AUTO: tuned per graph, GA_TRI for batched calls) */
    int ktruss_algo;               /* ga_algo of k-truss (GA_MSA, GA_MCA, GA_HEAP, GA_DOT, GA_HYBRID, GA_TRI,
                                      GA_AUTO as for TC) */
    int64_t hbm_budget;            /* bytes the calls in flight may hold; 0: 80% of free memory at creation */
    int64_t coalesce_nnz;          /* graphs with at most this many stored entries are batched; 0: 2^20 */
    int64_t coalesce_max_nnz;      /* stored entries of one batched union at most; 0: 2^22 (several groups
                                      keep several workers busy) */
    int64_t coalesce_max_requests; /* requests served by one batched call at most; 0: 4096 */
    int64_t bc_group_pairs;        /* batched BC keeps state per (union vertex, source column): union
                                      vertices x (largest source count of a request + 1) + sources
                                      of one group at most; 0: 2^25 */
} ga_server_config;
typedef struct {
    int status;                /* GA_OK, the call's error code, or GA_ERR_ADMISSION */
    int type, graph;
    int64_t tc_total;          /* TC: triangles */
    int iters;                 /* k-truss: iteration count as ga_ktruss reports it */
    int64_t truss_nnz;         /* k-truss: stored entries of the result */
    const int32_t* truss_rst;  /* k-truss result (m+1 row starts) when requested, else NULL */
    const int32_t* truss_col;  /* its columns */
    const double* bc;          /* BC: scores (length m) */
    double t_submit, t_start, t_end; /* seconds on the server's clock */
    int batch_size;            /* requests served by the same call */
    int worker;
    int64_t bytes_bound;
    const char* error;         /* message when status != GA_OK */
} ga_server_result;
typedef struct {
    int64_t submitted, completed, failed, rejected;
    int64_t calls, batched_calls, batched_requests, max_group, max_in_flight;
    int64_t budget, reserved, peak_reserved, queued;
    int64_t cancelled;
} ga_server_stats;
/* Upper bound on the device bytes of one request (type GA_REQ_*, graph of m
 * vertices and nnz stored entries; param = number of BC sources). */
GA_API int ga_request_bytes_bound(int type, int64_t m, int64_t nnz, int64_t param, int64_t* bytes);
/* cfg may be NULL (defaults). */
GA_API int ga_server_create(int device, const ga_server_config* cfg, ga_server* srv);
/* Waits for every queued request, then stops the workers. */
GA_API int ga_server_destroy(ga_server srv);
/* Uploads a symmetric adjacency matrix (host CSR, values 1) once; it stays
 * resident and its bytes come out of the budget. */
GA_API int ga_server_add_graph(ga_server srv, int64_t m, const int32_t* rst, const int32_t* col, int* graph_id);
/* The same from a device CSR of context ctx (same device; copied on the
 * device, ctx's stream synchronised first; A stays the caller's), or from a
 * graph file (".mtx" / ".bin" by extension, read on the device with the
 * reference CLI's preparation: adjacency and lower-triangle symmetrisation,
 * src/main.cpp:221-222), so a pool loads without host CSR builds. */
GA_API int ga_server_add_graph_device(ga_server srv, ga_ctx ctx, ga_csr A, int* graph_id);
GA_API int ga_server_add_graph_file(ga_server srv, const char* path, int* graph_id);
/* Vertex count and stored entries of a resident graph (either may be NULL). */
GA_API int ga_server_graph_info(ga_server srv, int graph, int64_t* m, int64_t* nnz);
/* Queues a request: GA_REQ_TC, GA_REQ_KTRUSS (k), or GA_REQ_BC (sources,
 * copied). want_edges: keep the k-truss edge set for ga_server_wait. */
GA_API int ga_server_submit(ga_server srv, int type, int graph, int k, const int32_t* sources, int nsrc,
                            int want_edges, int64_t* req_id);
/* Blocks until the request is done (timeout_s <= 0: no limit; else
 * GA_ERR_TIMEOUT). The result's arrays stay valid until ga_server_release. */
GA_API int ga_server_wait(ga_server srv, int64_t req_id, double timeout_s, ga_server_result* res);
GA_API int ga_server_release(ga_server srv, int64_t req_id);
/* Cancels a request that is still queued: it completes at once with status
 * GA_ERR_CANCELLED (wait and release it as any other). A request that has
 * started runs to completion: GA_ERR_UNSUPPORTED. */
GA_API int ga_server_cancel(ga_server srv, int64_t req_id);
/* Blocks until the queue is empty and no call is in flight. */
GA_API int ga_server_drain(ga_server srv, double timeout_s);
GA_API int ga_server_get_stats(ga_server srv, ga_server_stats* stats);

/* ------------------------------------------------------ synthetic graphs */
/* Seeded generators producing sorted, duplicate-free, loop-free symmetric
 * int32 CSR on the host (arrays allocated with malloc; free with
 * ga_host_free). R-MAT and Erdos-Renyi output depends only on the seed;
 * the k-NN points use the C library's log/cos and so the host's libm.
 *  R-MAT: scale, edge factor, quadrant probabilities a, b, c (d = 1-a-b-c).
 *  Erdos-Renyi G(n, m): m distinct undirected edges.
 *  k-NN: n points i.i.d. N(0,1) in dim dimensions, k nearest neighbours by
 *  Euclidean distance (self excluded), symmetrised by union. */
GA_API int ga_gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed,
                       int64_t* m, int64_t* nnz, int32_t** rst, int32_t** col);
/* The same R-MAT graph as ga_gen_rmat (bit for bit), generated and built on
 * the device: edges from the same random streams, then mirrored, loops
 * dropped, rows sorted and duplicates merged by the ingestion kernels. */
GA_API int ga_gen_rmat_device(ga_ctx ctx, int scale, int edge_factor, double a, double b, double c, uint64_t seed,
                              ga_csr* out);
GA_API int ga_gen_er(int64_t n, int64_t edges, uint64_t seed, int64_t* m, int64_t* nnz, int32_t** rst,
                     int32_t** col);
GA_API int ga_gen_knn(int64_t n, int dim, int k, uint64_t seed, int64_t* m, int64_t* nnz, int32_t** rst,
                      int32_t** col);
GA_API void ga_host_free(void* p);

#ifdef __cplusplus
}
#endif
#endif /* GRAPHALGO_GB300_H */
