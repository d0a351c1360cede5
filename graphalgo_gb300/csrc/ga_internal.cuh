// Internal declarations shared by the CUDA translation units of
// libgraphalgo_gb300.so. Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>
#include <map>
#include <stdexcept>
#include <unordered_map>

#include "../../include/graphalgo_gb300.h"

namespace ga {

// ------------------------------------------------------------------ errors
struct Error {
    int code;
    std::string msg;
};

[[noreturn]] void fail(int code, const std::string& msg);
void check_cuda(cudaError_t e, const char* what, const char* file, int line);
#define GA_CUDA(expr) ::ga::check_cuda((expr), #expr, __FILE__, __LINE__)
#define GA_REQUIRE(cond, code, msg) \
    do {                            \
        if (!(cond)) ::ga::fail((code), (msg)); \
    } while (0)

// --------------------------------------------------------------- device info
constexpr int kWarp = 32;
constexpr int32_t kEmpty = -1;  // empty hash-table key

// ------------------------------------------------------------------ context
struct PendingTiming {
    const char* name;
    cudaEvent_t start, stop;
};

struct KStat {
    int64_t launches = 0;
    double total_ms = 0.0;
};

// Schedule parameters of the masked products (options or autotuner).
struct MxmTune {
    int64_t warp_max_flops = 32768;  // rows with more Gustavson products go to a CTA
    int64_t heavy_flops = 1 << 20;   // CTA items of rows with at least this many products run first
    int ctas_per_sm = 0;             // persistent grid: CTAs per SM (0: as many as fit)
    int dot_chunk = 8;               // inner-product form: mask entries per warp task
    int64_t hybrid_ratio = 16;       // hybrid form: a row goes to the inner product when its
                                     // inner-product work x this is below its Gustavson work
    int tri_order = 0;               // triangle listing: vertex ranks by degree (0) or index (1)
};

}  // namespace ga

struct ga_ctx_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int num_sms = 0;
    int cc_major = 0, cc_minor = 0;
    size_t smem_optin = 0;  // max dynamic shared memory per block (opt-in)
    cudaMemPool_t pool = nullptr;
    std::string last_error;
    // options
    bool device_loops = true;
    bool profile = false;
    int64_t fail_alloc_after = -1;  // fault injection
    bool knn_tiled = false;         // k-NN generator: tiled kernel for every graph
    bool kt_frontier = true;        // GA_TRI k-truss: incremental support after the first listing
    int bc_backward = 0;            // BC backward sweep: W rows by gathers (0), bulk copies (1), one at a time (2)
    ga::MxmTune tune;               // masked-product schedule
    // profiling
    std::vector<ga::PendingTiming> pending;
    std::vector<cudaEvent_t> event_pool;
    std::map<std::string, ga::KStat> kstats;
    cudaEvent_t timer_start = nullptr, timer_stop = nullptr;
    // pinned host word for small read-backs
    int64_t* h_pinned = nullptr;
    bool capturing = false;
    // device work counters (GA_CTR_*), accumulated by the masked-SpGEMM binning
    unsigned long long* d_counters = nullptr;
    // scratch written to evict the L2 between benchmark steps
    void* l2_flush = nullptr;
    size_t l2_flush_bytes = 0;
    // device bytes this context holds (requested sizes) and their high-water mark
    // asynchronous downloads: a copy stream, the event its copies wait for and
    // the event marking the last one done (created on first use)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copy_ready = nullptr, copy_done = nullptr;
    std::unordered_map<void*, size_t> live;
    int64_t bytes_in_use = 0;
    int64_t bytes_peak = 0;
    // device loops captured once and relaunched (run_cached_loop), by slot
    void* loop_cache[4] = {};
};

namespace ga {
// Frees the context's cached loop graphs and their device buffers.
void destroy_loop_caches(ga_ctx ctx);
}  // namespace ga

struct ga_csr_s {
    int64_t m = 0, n = 0, nnz = 0;
    ga_dtype dtype = GA_INT32;
    int32_t* rst = nullptr;
    int32_t* col = nullptr;
    void* val = nullptr;
    size_t cap = 0;  // allocated entries of col/val
    int unit = -1;   // all values equal 1: -1 unknown, 0 no, 1 yes
    int sym = -1;    // pattern and values symmetric: -1 unknown, 0 no, 1 yes
    cudaEvent_t copied = nullptr;  // the handle's last download on the copy stream
};

struct ga_dense_s {
    int64_t m = 0, n = 0;
    ga_dtype dtype = GA_FP64;
    void* val = nullptr;
};

namespace ga {

size_t dtype_size(ga_dtype t);
bool dtype_valid(int t);

// -------------------------------------------------------------- allocation
void* dalloc(ga_ctx ctx, size_t bytes);
void dfree(ga_ctx ctx, void* p);

template <typename T>
T* dalloc_t(ga_ctx ctx, size_t count) {
    return static_cast<T*>(dalloc(ctx, count * sizeof(T)));
}

// RAII device buffer, freed stream-ordered on the context's stream.
template <typename T>
struct DBuf {
    ga_ctx ctx = nullptr;
    T* p = nullptr;
    size_t count = 0;
    DBuf() = default;
    DBuf(ga_ctx c, size_t n) : ctx(c), p(dalloc_t<T>(c, n)), count(n) {}
    ~DBuf() {
        if (p) dfree(ctx, p);
    }
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : ctx(o.ctx), p(o.p), count(o.count) { o.p = nullptr; }
    DBuf& operator=(DBuf&& o) noexcept {
        if (this != &o) {
            if (p) dfree(ctx, p);
            ctx = o.ctx; p = o.p; count = o.count; o.p = nullptr;
        }
        return *this;
    }
    T* release() {
        T* r = p;
        p = nullptr;
        return r;
    }
};

// CSR handle helpers
ga_csr csr_alloc(ga_ctx ctx, int64_t m, int64_t n, int64_t nnz, ga_dtype dt);
void csr_destroy(ga_ctx ctx, ga_csr A);

// ------------------------------------------------------------- profiling
// Begin/end a named kernel region on the context stream (no-op unless the
// GA_OPT_PROFILE option is on and no graph capture is running).
int prof_begin(ga_ctx ctx, const char* name);  // returns a token for prof_end (-1: off)
void prof_end(ga_ctx ctx, int token);
struct ProfScope {
    ga_ctx ctx;
    int token;
    ProfScope(ga_ctx c, const char* name) : ctx(c), token(prof_begin(c, name)) {}
    ~ProfScope() { prof_end(ctx, token); }
};
void post_launch(const char* name);

// ------------------------------------------------------------- primitives
// Exclusive prefix sum of `n` int32 counts into out[0..n] (out[n] = total).
// in and out may alias. Launch sizes depend only on n (graph-capturable).
void scan_exclusive_i32(ga_ctx ctx, const int32_t* in, int32_t* out, int64_t n);
// Same for int64.
void scan_exclusive_i64(ga_ctx ctx, const int64_t* in, int64_t* out, int64_t n);
// Scratch bytes needed by the scans above for n elements.
size_t scan_scratch_bytes(int64_t n);

// Fills `count` values of type `dt` with 1.
void fill_ones(ga_ctx ctx, void* vals, int64_t count, ga_dtype dt);

// Validates a device CSR; throws GA_ERR_INVALID_CSR when malformed.
void validate_csr(ga_ctx ctx, const int32_t* rst, const int32_t* col, int64_t m, int64_t n, int64_t nnz);
// The same checks as bits: 1 row starts not a monotone 0..nnz sequence,
// 2 a column out of range, 4 columns not strictly ascending in some row.
int csr_check_bits(ga_ctx ctx, const int32_t* rst, const int32_t* col, int64_t m, int64_t n, int64_t nnz);

// Sorts each CSR row segment by key (payload follows): rows of up to 256
// entries by one warp in registers, up to 8,192 by a CTA's bitonic sort in
// shared memory, longer ones by one CTA each (sorted pieces, then
// merge-path merges). nnz: entries of the whole matrix.
void sort_rows_by_key(ga_ctx ctx, const int32_t* rst, int64_t m, int32_t* key, int32_t* pay, int64_t nnz);

// k-truss on a single matrix (batch == nullptr) or on a block-diagonal union
// of graphs with per-graph convergence (see ga_batch_ktruss).
struct KtBatch {
    int64_t ngraphs = 0;
    const int32_t* voff = nullptr;   // first row of each graph (ngraphs + 1)
    const int32_t* gid = nullptr;    // graph of each row
    const int32_t* nvert = nullptr;  // vertices per graph
    int32_t* nnz_g = nullptr;        // current stored entries per graph
    int32_t* iters_g = nullptr;      // reported iteration count per graph
    int32_t* done_g = nullptr;       // graph finished (converged, or stopped after n_g iterations)
    const int32_t* kg = nullptr;     // per-graph k (nullptr: the call's k for every graph)
};
ga_csr ktruss_impl(ga_ctx ctx, ga_algo algo, ga_csr A, int k, int* iters_out, const KtBatch* batch);

// Device state of a k-truss loop.
struct KtState {
    int32_t nnz;        // nnz of C
    int32_t t;          // iteration index
    int32_t iters;      // reported iteration count
    int32_t swapped;    // this iteration replaced C by the pruned matrix
    int32_t done;
    int32_t first_vals; // C still carries A's values (no swap yet)
};

// Triangle-listing k-truss with the orientation kept in C itself: for the
// whole loop every row of C is stored as [entries whose column is ranked
// above the row | the rest], both parts in column order, so each row's
// oriented list is its first ocount entries and the prune's compaction keeps
// the layout. Buffers (all from tri_kt_bytes):
struct TriKt {
    int32_t* crank;     // cap: rank of each entry's column, aligned with C
    int32_t* tcrank;    // cap: its compacted copy
    int32_t* ocount;    // m + 1: oriented entries per row
    int32_t* tstart;    // m + 2: tasks per row, scanned into task starts
    int32_t* task_row;  // cap / 16 + m + 1: row of each task
    int32_t* dpos;      // m + 1: position of each row's diagonal entry, -1 if none
    void* scan_scr;
};
size_t tri_kt_bytes(int64_t m, int64_t cap);
void tri_kt_carve(void* scratch, int64_t m, int64_t cap, TriKt* t);
// Before the loop: ranks, the partition of every row (tmp_col: cap entries,
// tmp_flag: cap + 1), the mirror index in that layout, diagonal positions,
// tasks per row. row_of must hold every entry's row.
void tri_kt_setup(ga_ctx ctx, ga_csr C, const int32_t* row_of, int32_t* mir, int32_t* tmp_col, int32_t* tmp_flag,
                  const TriKt& t, int64_t cap);
// One support evaluation: counts at the oriented entries of sup (cap).
void tri_kt_support(ga_ctx ctx, ga_csr C, int32_t* sup, const TriKt& t, int64_t cap);
// Keep flags from the support (k, or the batch's per-graph k / finished
// graphs), with the upper-triangle work counters.
void tri_kt_flags(ga_ctx ctx, ga_csr C, const int32_t* row_of, const int32_t* mir, const int32_t* sup,
                  const TriKt& t, int64_t cap, int k, const KtBatch* batch, int32_t* flag);
// After the flags' scan (pos): compaction of C into tc / tr with rows (trow)
// and new positions (pos_new), and of the resident arrays; rows of a batch's
// finished graphs get no tasks in the next iteration.
void tri_kt_scatter(ga_ctx ctx, ga_csr C, const int32_t* pos, const int32_t* row_of, const TriKt& t, int64_t cap,
                    int32_t* tc, int32_t* tr, int32_t* pos_new, int32_t* trow, const KtBatch* batch);
// With the iteration's swap: C <- the pruned matrix (tr, tc, values 1), and
// rows, mirrors (mir_new), column ranks and diagonal positions follow it.
void tri_kt_copyback(ga_ctx ctx, ga_csr C, const KtState* st, const int32_t* tr, const int32_t* tc,
                     const int32_t* trow, const int32_t* mir_new, const int32_t* pos_new, int32_t* row_of,
                     int32_t* mir, const TriKt& t, int64_t cap);
// After the loop: every row back in column order.
void tri_kt_finish(ga_ctx ctx, ga_csr C, const int32_t* row_of, const TriKt& t, int32_t* tmp_col);

// Frontier form of the triangle-listing k-truss of one matrix (symmetric,
// values 1), after tri_kt_setup: the triangles are listed once, then every
// iteration prunes the edges whose support is below k - 2 and lowers the
// supports of the edges that shared a triangle with them. Buffers: sup, oid,
// f0, f1, tc (cap each), flag (cap + 1), state (cap bytes), tr (m + 1), scan
// scratch. Leaves C pruned with its rows in column order; returns the
// reference's iteration count.
struct TriFrontBufs {
    int32_t* sup;
    int32_t* flag;
    int32_t* tr;
    int32_t* tc;
    int32_t* oid;
    int32_t* f0;
    int32_t* f1;
    uint8_t* state;
    void* scan_scr;
};
// With `batch`: every graph of the union with its own k, iteration count
// (batch->iters_g) and iteration bound; the loop runs while a graph iterates.
int tri_kt_frontier(ga_ctx ctx, ga_csr C, int k, const int32_t* row_of, const int32_t* mir, const TriKt& t,
                    int64_t cap, const TriFrontBufs& b, const KtBatch* batch);
// The same state kept between calls: run(k) iterates for one k (the first
// call lists the triangles; a later call, one matrix only, takes a larger k
// and continues from the supports the previous k left, so a sweep k = kmin,
// kmin + 1, ... lists the triangles once); compact() writes the kept
// entries, rows in column order, to b.tc / b.tr and returns their number and
// the iteration count of the last run (one host synchronisation).
class TriFront {
public:
    TriFront(ga_ctx ctx, ga_csr C, const int32_t* row_of, const int32_t* mir, const TriKt& t, int64_t cap,
             const TriFrontBufs& b, const KtBatch* batch);
    ~TriFront();
    TriFront(const TriFront&) = delete;
    TriFront& operator=(const TriFront&) = delete;
    void run(int k);
    int64_t compact(int* iters);

private:
    struct Impl;
    Impl* impl_;
};

// Autotuned algorithm resolution: GA_AUTO becomes the cached (or freshly
// tuned) variant, and ctx->tune its schedule; other values pass through.
// Callers hold a TuneScope so the context's schedule is restored afterwards.
ga_algo resolve_ktruss_algo(ga_ctx ctx, ga_algo algo, ga_csr A);
ga_algo resolve_tc_algo(ga_ctx ctx, ga_algo algo, ga_csr A);
ga_algo resolve_mxm_algo(ga_ctx ctx, ga_algo algo, ga_csr A, ga_csr B, ga_csr M);
struct TuneScope {
    ga_ctx ctx;
    MxmTune saved;
    explicit TuneScope(ga_ctx c) : ctx(c), saved(c->tune) {}
    ~TuneScope() { ctx->tune = saved; }
};
// Position of the first entry with column >= i in each row (rows sorted).
void upper_starts(ga_ctx ctx, ga_csr A, int32_t* ust);
// Row index of every entry; position of every entry's mirror (j, i) in a
// symmetric pattern.
void expand_rows(ga_ctx ctx, ga_csr A, int32_t* row_of);
void mirror_index(ga_ctx ctx, ga_csr A, const int32_t* row_of, int32_t* mir);

// Triangle-listing support product (GA_TRI) of a symmetric int32 matrix
// whose values are all 1. tri_support_launch allocates nothing (capturable):
// C's entry count is read on the device (at most cap), row_of / mir are the
// row and mirror position of every entry, pos has cap + 1 entries, scratch
// tri_scratch_bytes(C->m, cap) bytes; sup receives C·C at C's entries.
// upper_counts: work counters as for an upper-triangle support product.
// tri_prepare ranks the vertices by C's degrees into the scratch; it runs
// once before the evaluations (any ranking gives the same counts).
size_t tri_scratch_bytes(int64_t m, int64_t cap);
void tri_prepare(ga_ctx ctx, ga_csr C, void* scratch, int64_t cap);
void tri_support_launch(ga_ctx ctx, ga_csr C, const int32_t* row_of, const int32_t* mir, int32_t* pos,
                        int32_t* sup, void* scratch, int64_t cap, bool upper_counts);
// A, B and M one symmetric int32 matrix with unit values (synchronises the
// stream the first time a handle is checked).
bool tri_applies(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr M);
void tri_masked_into(ga_ctx ctx, ga_csr A, int32_t* sup);
// Triangle count of a symmetric pattern (diagonal ignored) into *d_total
// (added to) and, when given, per row the triangles whose largest vertex
// index is the row (zeroed first): the row sums of C<L> = L·L.
void tri_count(ga_ctx ctx, ga_csr A, unsigned long long* d_total, unsigned long long* d_per_row);

// device-side transpose (counting sort; rows of the result sorted)
ga_csr transpose_csr(ga_ctx ctx, ga_csr A);
ga_csr extract_tri(ga_ctx ctx, ga_csr A, bool lower);
ga_csr copy_csr(ga_ctx ctx, ga_csr A, ga_dtype to);

// Masked SpGEMM into caller-provided value storage aligned with M.
void mxm_masked_into(ga_ctx ctx, ga_algo algo, ga_csr A, ga_csr B, ga_csr M, void* d_cvals);
ga_csr mxm_cmask(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr M);
// hybrid: room for the hybrid form's inner-product tasks too.
size_t mxm_scratch_bytes(int64_t m, int64_t n, int64_t mask_nnz, bool hybrid = true);
// unit_a / unit_b: A's / B's values are all ones (skips value loads).
// GA_HYBRID: Bt holds B^T (B itself when B is symmetric).
void mxm_masked_launch(ga_ctx ctx, ga_algo algo, ga_csr A, ga_csr B, ga_csr M, void* d_cvals, void* scratch,
                       int64_t cap_nnz, bool unit_b, const int32_t* mask_row_end = nullptr, bool unit_a = false,
                       ga_csr Bt = nullptr);
// Inner-product masked product (GA_DOT): Bt holds B^T (B itself when B is
// symmetric); unit: A's and B's values are all ones. Allocates nothing.
// With mask_row_end, M->rst holds row starts of the mask and
// mask_row_end - 1 the row partition of M's column array.
void mxm_dot_launch(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr Bt, ga_csr M, void* d_cvals, bool unit,
                    const int32_t* mask_row_end);
// True when every stored value of A equals 1 (computed once per handle and
// cached; synchronises the stream the first time).
bool csr_unit_values(ga_ctx ctx, ga_csr A);
// True when A is square and every (i, j, v) has a matching (j, i, v)
// (synchronises the stream).
bool csr_is_symmetric(ga_ctx ctx, ga_csr A);
// Batched BC over the block-diagonal union U of `count` graphs (host vertex
// offsets voff), graph g with the sources [soff[g], soff[g+1]) of the host
// array `sources` (indices within graph g); scores of U's rows into d_bc.
void bc_union_device(ga_ctx ctx, ga_csr U, int64_t count, const int64_t* voff, const int64_t* soff,
                     const int32_t* sources, double* d_bc);
void scan_exclusive_i32_scratch(ga_ctx ctx, const int32_t* in, int32_t* out, int64_t n, void* scratch);

// Read one device value to the host (synchronises the stream).
int64_t read_i64(ga_ctx ctx, const int64_t* d);
int32_t read_i32(ga_ctx ctx, const int32_t* d);

int grid_for(int64_t work, int block, int max_blocks = 1 << 20);

}  // namespace ga

// Entry-point wrapper: runs `body`, maps ga::Error / std::bad_alloc / other
// exceptions to status codes and records the message on the context.
#define GA_API_BODY(ctx, ...)                                        \
    do {                                                             \
        try {                                                        \
            __VA_ARGS__;                                             \
            return GA_OK;                                            \
        } catch (const ::ga::Error& e) {                             \
            if (ctx) (ctx)->last_error = e.msg;                      \
            return e.code;                                           \
        } catch (const std::bad_alloc&) {                            \
            if (ctx) (ctx)->last_error = "host allocation failed";   \
            return GA_ERR_OOM;                                       \
        } catch (const std::exception& e) {                          \
            if (ctx) (ctx)->last_error = e.what();                   \
            return GA_ERR_INVALID_ARG;                               \
        }                                                            \
    } while (0)
