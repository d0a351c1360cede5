// Callers of the masked SpGEMM: triangle counting (Sandia L*L, L*U and
// per-vertex forms, plus the warp-intersection dot-product form) and the
// device-resident k-truss loop. Also the CUDA-graph loop driver.
#include "ga_device.cuh"
#include "ga_loop.cuh"

#include <memory>

namespace ga {

// ============================================================ loop driver
void run_device_loop(ga_ctx ctx, const std::function<void(const LoopCtl&)>& body, int64_t max_host_iters) {
    DBuf<int> cont(ctx, 1);
    LoopCtl ctl;
    ctl.cont = cont.p;
    ctl.use_handle = 0;
    ctl.handle = 0;
    if (!ctx->device_loops) {
        int* h = reinterpret_cast<int*>(ctx->h_pinned);
        for (int64_t it = 0; it < max_host_iters; ++it) {
            body(ctl);
            GA_CUDA(cudaMemcpyAsync(h, cont.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
            GA_CUDA(cudaStreamSynchronize(ctx->stream));
            if (*h == 0) return;
        }
        fail(GA_ERR_TIMEOUT, "device loop did not finish within its iteration bound");
    }
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool capture_failed = false;
    GA_CUDA(cudaGraphCreate(&graph, 0));
    try {
        GA_CUDA(cudaGraphConditionalHandleCreate(&ctl.handle, graph, 1, cudaGraphCondAssignDefault));
        ctl.use_handle = 1;
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = ctl.handle;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        GA_CUDA(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp));
        cudaGraph_t bodyg = cp.conditional.phGraph_out[0];
        GA_CUDA(cudaStreamBeginCaptureToGraph(ctx->stream, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
        ctx->capturing = true;
        try {
            body(ctl);
        } catch (...) {
            ctx->capturing = false;
            capture_failed = true;
            cudaGraph_t dummy;
            cudaStreamEndCapture(ctx->stream, &dummy);
            cudaGetLastError();
            throw;
        }
        ctx->capturing = false;
        cudaGraph_t captured = nullptr;
        GA_CUDA(cudaStreamEndCapture(ctx->stream, &captured));
        GA_CUDA(cudaGraphInstantiate(&exec, graph, 0));
        {
            ProfScope ps(ctx, "device_loop_graph");
            GA_CUDA(cudaGraphLaunch(exec, ctx->stream));
        }
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
    } catch (...) {
        if (exec) cudaGraphExecDestroy(exec);
        // A graph whose conditional body was left by a failed capture is not
        // destroyed (destroying it crashed the driver); it leaks on this
        // error path only.
        if (!capture_failed) cudaGraphDestroy(graph);
        throw;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
}

namespace {
struct CachedLoop {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int* cont = nullptr;   // the loop's continue flag (host-loop mode)
    void* args = nullptr;  // the call's parameters
    size_t args_bytes = 0;
    LoopCtl ctl{};
};

CachedLoop* cache_slot(ga_ctx ctx, int slot) {
    GA_REQUIRE(slot >= 0 && slot < 4, GA_ERR_INVALID_ARG, "loop cache slot out of range");
    if (!ctx->loop_cache[slot]) ctx->loop_cache[slot] = new CachedLoop();
    CachedLoop* c = static_cast<CachedLoop*>(ctx->loop_cache[slot]);
    if (!c->cont) GA_CUDA(cudaMalloc(&c->cont, sizeof(int)));
    return c;
}
}  // namespace

void* cached_loop_args(ga_ctx ctx, int slot, size_t bytes) {
    CachedLoop* c = cache_slot(ctx, slot);
    if (c->args_bytes < bytes) {
        GA_REQUIRE(c->exec == nullptr, GA_ERR_INVALID_ARG, "loop parameters grew after capture");
        if (c->args) GA_CUDA(cudaFree(c->args));
        c->args = nullptr;
        GA_CUDA(cudaMalloc(&c->args, bytes));
        c->args_bytes = bytes;
    }
    return c->args;
}

void run_cached_loop(ga_ctx ctx, int slot, const std::function<void(const LoopCtl&)>& body, int64_t max_host_iters) {
    if (!ctx->device_loops) {
        run_device_loop(ctx, body, max_host_iters);
        return;
    }
    CachedLoop* c = cache_slot(ctx, slot);
    if (!c->exec) {
        cudaGraph_t graph = nullptr;
        bool capture_failed = false;
        GA_CUDA(cudaGraphCreate(&graph, 0));
        try {
            c->ctl.cont = c->cont;
            GA_CUDA(cudaGraphConditionalHandleCreate(&c->ctl.handle, graph, 1, cudaGraphCondAssignDefault));
            c->ctl.use_handle = 1;
            cudaGraphNodeParams cp = {};
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = c->ctl.handle;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            cudaGraphNode_t node;
            GA_CUDA(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp));
            cudaGraph_t bodyg = cp.conditional.phGraph_out[0];
            GA_CUDA(cudaStreamBeginCaptureToGraph(ctx->stream, bodyg, nullptr, nullptr, 0,
                                                  cudaStreamCaptureModeRelaxed));
            ctx->capturing = true;
            try {
                body(c->ctl);
            } catch (...) {
                ctx->capturing = false;
                capture_failed = true;
                cudaGraph_t dummy;
                cudaStreamEndCapture(ctx->stream, &dummy);
                cudaGetLastError();
                throw;
            }
            ctx->capturing = false;
            cudaGraph_t captured = nullptr;
            GA_CUDA(cudaStreamEndCapture(ctx->stream, &captured));
            GA_CUDA(cudaGraphInstantiate(&c->exec, graph, 0));
            c->graph = graph;
        } catch (...) {
            // as in run_device_loop: a graph left by a failed capture is not destroyed
            if (!capture_failed) cudaGraphDestroy(graph);
            c->exec = nullptr;
            throw;
        }
    }
    {
        ProfScope ps(ctx, "device_loop_graph");
        GA_CUDA(cudaGraphLaunch(c->exec, ctx->stream));
    }
}

void destroy_loop_caches(ga_ctx ctx) {
    for (void*& p : ctx->loop_cache) {
        CachedLoop* c = static_cast<CachedLoop*>(p);
        if (!c) continue;
        if (c->exec) cudaGraphExecDestroy(c->exec);
        if (c->graph) cudaGraphDestroy(c->graph);
        if (c->cont) cudaFree(c->cont);
        if (c->args) cudaFree(c->args);
        delete c;
        p = nullptr;
    }
}

// ==================================================== triangle counting
constexpr int kTcThreads = 256;
constexpr int kTcChunk = 8;  // edges (i, j) of one L row per work unit

// Dot-product form of the triangle count, straight from A (rows sorted, no
// extraction of L): the strictly lower part of row i is L_i = A_i[0, low_i)
// with low_i = ust[i] - rst[i]. For an edge (i, j) = (i, L_i[t]), the
// triangles (i, j, k) with k < j are |L_i[0..t) ∩ L_j| (only entries below j
// can meet L_j). Warps take kTcChunk consecutive entries of A (a chunk finds
// its row by a binary search of the row starts, upper entries are skipped).
// The shorter list is walked 32 entries at a time, one per lane; the longer
// one is held in registers when it has at most 32 entries (searched by
// shuffles), else, when 32 or more entries are walked, as the last entries
// of 32 buckets (the shuffle search picks the bucket, a binary search in
// memory finishes), else searched in memory; __ballot_sync/__popc count the
// hits. per_row[i] = triangles whose largest vertex is i (the row
// sums of the reference's C<L> = L*L). No host synchronisation.
__global__ void __launch_bounds__(kTcThreads) k_tc_dot(const int32_t* __restrict__ ar, const int32_t* __restrict__ ac,
                                                       const int32_t* __restrict__ ust, int64_t m,
                                                       unsigned long long* __restrict__ total,
                                                       unsigned long long* __restrict__ per_row) {
    const int lane = threadIdx.x & 31;
    const unsigned FULL = 0xffffffffu;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t nnz = ar[m];
    unsigned long long acc_total = 0;
    for (int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; c * kTcChunk < nnz; c += warps) {
        const int32_t q0 = (int32_t)(c * kTcChunk);
        const int32_t q1 = (int32_t)min((int64_t)q0 + kTcChunk, nnz);
        int i = upper_bound_i32(ar, (int)m + 1, q0) - 1;
        unsigned long long row_cnt = 0;
        for (int32_t q = q0; q < q1; ++q) {
            while (q >= ar[i + 1]) {
                if (lane == 0 && row_cnt && per_row) atomicAdd(&per_row[i], row_cnt);
                acc_total += row_cnt;
                row_cnt = 0;
                ++i;
            }
            const int32_t ib = ar[i];
            const int t = q - ib;
            if (t == 0 || q >= ust[i]) continue;  // first lower entry meets nothing; upper part skipped
            const int32_t j = __ldg(ac + q);
            const int32_t jb = ar[j], jn = ust[j] - jb;
            if (jn == 0) continue;
            const bool walk_j = jn <= t;  // walk the shorter list
            const int32_t* W = walk_j ? ac + jb : ac + ib;
            const int32_t* S = walk_j ? ac + ib : ac + jb;
            const int wn = walk_j ? jn : t, sn = walk_j ? t : jn;
            const bool small = sn <= 32, bucketed = !small && wn >= 32;
            int32_t key = INT32_MAX;
            if (small) {
                key = lane < sn ? __ldg(S + lane) : INT32_MAX;
            } else if (bucketed) {
                const int hi_b = (int)(((int64_t)(lane + 1) * sn) >> 5);
                key = __ldg(S + hi_b - 1);
            }
            unsigned long long cnt = 0;
            for (int base = 0; base < wn; base += 32) {
                const int e = base + lane;
                const int32_t x = e < wn ? __ldg(W + e) : INT32_MAX;
                const int b = (small || bucketed) ? warp_lower_bound(key, x) : 0;
                bool hit = false;
                if (small) {
                    const int32_t y = __shfl_sync(FULL, key, b & 31);
                    hit = e < wn && b < sn && y == x;
                } else if (bucketed) {
                    if (e < wn && b < 32) {
                        const int lo_b = (int)(((int64_t)b * sn) >> 5);
                        const int hi_b = (int)(((int64_t)(b + 1) * sn) >> 5);
                        const int pos = lo_b + lower_bound_i32(S + lo_b, hi_b - lo_b, x);
                        hit = pos < hi_b && __ldg(S + pos) == x;
                    }
                } else if (e < wn) {
                    const int pos = lower_bound_i32(S, sn, x);
                    hit = pos < sn && __ldg(S + pos) == x;
                }
                cnt += __popc(__ballot_sync(FULL, hit));
            }
            row_cnt += cnt;
        }
        if (lane == 0 && row_cnt && per_row) atomicAdd(&per_row[i], row_cnt);
        acc_total += row_cnt;
    }
    if (lane == 0 && acc_total) atomicAdd(total, acc_total);
}

// Row sums of C (int32) into per_row and the total.
__global__ void k_row_sums(const int32_t* __restrict__ cr, const int32_t* __restrict__ cv, int64_t m,
                           int64_t* __restrict__ per_row, unsigned long long* __restrict__ total) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    unsigned long long acc = 0;
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
        long long s = 0;
        for (int32_t q = cr[i] + lane; q < cr[i + 1]; q += 32) s += cv[q];
        s = warp_sum<long long>(s);
        if (lane == 0) {
            if (per_row) per_row[i] = s;
            acc += (unsigned long long)s;
        }
    }
    if (lane == 0 && acc) atomicAdd(total, acc);
}

// per-vertex: (row sum as int) >> 1, the reference's int arithmetic
__global__ void k_row_sums_half_i32(const int32_t* __restrict__ cr, const int32_t* __restrict__ cv, int64_t m,
                                    int32_t* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
        int s = 0;
        for (int32_t q = cr[i] + lane; q < cr[i + 1]; q += 32) s += cv[q];
        s = warp_sum<int>(s);
        if (lane == 0) out[i] = s >> 1;
    }
}

static ga_csr adjacency_of(ga_ctx ctx, ga_csr A) {
    ga_csr C = csr_alloc(ctx, A->m, A->n, A->nnz, GA_INT32);
    GA_CUDA(cudaMemcpyAsync(C->rst, A->rst, sizeof(int32_t) * (A->m + 1), cudaMemcpyDeviceToDevice, ctx->stream));
    if (A->nnz)
        GA_CUDA(cudaMemcpyAsync(C->col, A->col, sizeof(int32_t) * A->nnz, cudaMemcpyDeviceToDevice, ctx->stream));
    fill_ones(ctx, C->val, A->nnz, GA_INT32);
    C->unit = 1;
    return C;
}

struct CsrGuard {
    ga_ctx ctx; ga_csr a;
    CsrGuard(ga_ctx c, ga_csr x) : ctx(c), a(x) {}
    ~CsrGuard() { csr_destroy(ctx, a); }
};

static void tc_device(ga_ctx ctx, ga_algo algo, ga_csr A, int64_t* d_total, int64_t* d_per_row) {
    GA_REQUIRE(A->m == A->n, GA_ERR_SHAPE, "triangle counting needs a square matrix");
    TuneScope tscope(ctx);
    algo = resolve_tc_algo(ctx, algo, A);
    unsigned long long* tot = reinterpret_cast<unsigned long long*>(d_total);
    GA_CUDA(cudaMemsetAsync(tot, 0, sizeof(unsigned long long), ctx->stream));
    if (A->m == 0) return;
    if (algo == GA_TRI) {
        // triangle listing on a symmetric pattern; other matrices take the
        // Sandia form with the hybrid product
        if (csr_is_symmetric(ctx, A)) {
            tri_count(ctx, A, tot, reinterpret_cast<unsigned long long*>(d_per_row));
            return;
        }
        algo = GA_HYBRID;
    }
    if (algo == GA_DOT) {
        const int64_t m = A->m;
        DBuf<int32_t> ust(ctx, (size_t)m + 1);
        upper_starts(ctx, A, ust.p);
        if (d_per_row) GA_CUDA(cudaMemsetAsync(d_per_row, 0, sizeof(int64_t) * m, ctx->stream));
        if (A->nnz == 0) return;
        ProfScope ps(ctx, "tc_dot");
        k_tc_dot<<<grid_for((A->nnz + kTcChunk - 1) / kTcChunk * 32, kTcThreads, ctx->num_sms * 16), kTcThreads, 0,
                   ctx->stream>>>(A->rst, A->col, ust.p, m, tot, reinterpret_cast<unsigned long long*>(d_per_row));
        post_launch("tc_dot");
        return;
    }
    ga_csr L0 = extract_tri(ctx, A, true);
    CsrGuard g0(ctx, L0);
    // Sandia form with a masked-SpGEMM variant on the unit-valued L
    ga_csr L = adjacency_of(ctx, L0);
    CsrGuard g1(ctx, L);
    DBuf<int32_t> cv(ctx, (size_t)L->nnz + 1);
    mxm_masked_into(ctx, algo, L, L, L, cv.p);
    ProfScope ps(ctx, "tc_row_sums");
    k_row_sums<<<grid_for(A->m * 32, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(L->rst, cv.p, A->m, d_per_row,
                                                                                   tot);
    post_launch("row_sums");
}

// ============================================================== k-truss

// Rows of graphs that have finished (batched k-truss) keep every entry.
__device__ __forceinline__ bool kt_keep_all(const int32_t* gid, const int32_t* done_g, int64_t i) {
    return gid != nullptr && done_g[gid[i]] != 0;
}

// Row of entry q: the maintained row index when there is one, else a binary
// search of the row starts.
__device__ __forceinline__ int64_t kt_row(const int32_t* cr, int64_t m, const int32_t* row_of, int64_t q) {
    return row_of ? row_of[q] : upper_bound_i32(cr, (int)m + 1, (int32_t)q) - 1;
}

// Prune, step 1 (one thread per entry): keep flag of every entry of C
// (support >= k-2, or the entry's graph has finished), 0 past C's end up to
// cap so the exclusive scan over cap entries gives new positions.
__global__ void k_kt_flags(const int32_t* __restrict__ cr, const int32_t* __restrict__ sup, int64_t m, int k,
                           int64_t cap, int32_t* __restrict__ flag, const int32_t* __restrict__ gid,
                           const int32_t* __restrict__ done_g, const int32_t* __restrict__ row_of,
                           const int32_t* __restrict__ kg) {
    const int64_t cur = cr[m];
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < cap; q += (int64_t)gridDim.x * blockDim.x) {
        int32_t keep = 0;
        if (q < cur) {
            if (kg) {  // per-graph k (batches)
                const int g = gid[kt_row(cr, m, row_of, q)];
                keep = done_g[g] != 0 || sup[q] >= kg[g] - 2;
            } else {
                keep = sup[q] >= k - 2;
                if (!keep && gid) keep = kt_keep_all(gid, done_g, kt_row(cr, m, row_of, q));
            }
        }
        flag[q] = keep;
    }
}

// Prune, step 2, after the exclusive scan `pos` of the flags: kept entries
// move to pos[q] (columns, and their rows when tracked), pos_new[q] is the
// new position or -1, and the new row starts are tr[i] = pos[cr[i]].
__global__ void k_kt_scatter(const int32_t* __restrict__ cr, const int32_t* __restrict__ cc,
                             const int32_t* __restrict__ pos, int64_t m, int32_t* __restrict__ tc,
                             int32_t* __restrict__ tr, int32_t* __restrict__ pos_new, int32_t* __restrict__ trow,
                             const int32_t* __restrict__ row_of) {
    const int64_t cur = cr[m];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < cur || q <= m; q += stride) {
        if (q <= m) tr[q] = pos[cr[q]];
        if (q < cur) {
            const int32_t d = pos[q];
            const bool keep = pos[q + 1] != d;
            if (keep) {
                tc[d] = cc[q];
                if (trow) trow[d] = row_of[q];
            }
            if (pos_new) pos_new[q] = keep ? d : -1;
        }
    }
}

// Batched k-truss bookkeeping after iteration t, one block per graph: a graph
// whose kept count equals its current count has converged (iterations t+1);
// otherwise it was pruned and stops after n_g iterations (reported as 0),
// as the reference's loop bound does (src/main.cpp:100).
__global__ void k_kt_graph_update(const KtState* st, const int32_t* __restrict__ tr, KtBatch b) {
    const int t = st->t;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < b.ngraphs; g += (int64_t)gridDim.x * blockDim.x) {
        if (b.done_g[g]) continue;
        const int32_t kept = tr[b.voff[g + 1]] - tr[b.voff[g]];
        if (kept == b.nnz_g[g]) {
            b.iters_g[g] = t + 1;
            b.done_g[g] = 1;
        } else {
            b.nnz_g[g] = kept;
            if (t + 1 >= b.nvert[g]) {
                b.iters_g[g] = 0;
                b.done_g[g] = 1;
            }
        }
    }
}

__global__ void k_kt_finalize(KtState* st, const int32_t* __restrict__ tr, int64_t m, LoopCtl ctl) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int32_t nnz_new = tr[m];
    if (nnz_new == st->nnz) {
        st->iters = st->t + 1;
        st->swapped = 0;
        st->done = 1;
    } else {
        st->nnz = nnz_new;
        st->swapped = 1;
        st->first_vals = 0;
        st->t += 1;
        if ((int64_t)st->t >= m) {
            st->iters = 0;
            st->done = 1;
        }
    }
    loop_continue(ctl, st->done == 0);
}

// C <- pruned matrix (rows, columns, values 1) when the iteration swapped.
__global__ void k_kt_copyback(const KtState* st, const int32_t* __restrict__ tr, const int32_t* __restrict__ tc,
                              int64_t m, int32_t* __restrict__ cr, int32_t* __restrict__ cc,
                              int32_t* __restrict__ cv) {
    if (!st->swapped) return;
    const int64_t nnz = st->nnz;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q <= m || q < nnz; q += stride) {
        if (q <= m) cr[q] = tr[q];
        if (q < nnz) { cc[q] = tc[q]; cv[q] = 1; }
    }
}

// Position of the first entry of row i with column >= i (rows sorted).
// With gid / done_g (batched k-truss), rows of graphs that have finished get
// an empty upper part: their support is not needed again (they keep every
// entry), so the product skips them.
__global__ void k_upper_start(const int32_t* __restrict__ cr, const int32_t* __restrict__ cc, int64_t m,
                              int32_t* __restrict__ ust, const int32_t* __restrict__ gid = nullptr,
                              const int32_t* __restrict__ done_g = nullptr) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t b = cr[i], n = cr[i + 1] - b;
        ust[i] = kt_keep_all(gid, done_g, i) ? b + n : b + lower_bound_i32(cc + b, n, (int32_t)i);
    }
}

// Row index of every entry.
__global__ void k_expand_rows(const int32_t* __restrict__ cr, int64_t m, int32_t* __restrict__ row_of) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps)
        for (int32_t q = cr[i] + lane; q < cr[i + 1]; q += 32) row_of[q] = (int32_t)i;
}

// Position of each entry's mirror (j, i) in a symmetric pattern.
__global__ void k_mirror_index(const int32_t* __restrict__ cr, const int32_t* __restrict__ cc,
                               const int32_t* __restrict__ row_of, int64_t nnz, int32_t* __restrict__ mir) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x) {
        const int32_t i = row_of[q], j = cc[q];
        const int32_t jb = cr[j], jn = cr[j + 1] - jb;
        mir[q] = jb + lower_bound_i32(cc + jb, jn, i);
    }
}

// The support of a symmetric C is symmetric: lower entries (column below the
// row) take the value computed for their mirror in the upper triangle.
__global__ void k_gather_lower(const KtState* st, const int32_t* __restrict__ cc, const int32_t* __restrict__ row_of,
                               const int32_t* __restrict__ mir, int32_t* __restrict__ sup) {
    const int64_t nnz = st->nnz;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x)
        if (cc[q] < row_of[q]) sup[q] = sup[mir[q]];
}

// Mirror positions after a prune: a kept entry's mirror is kept too (equal
// support), so its new mirror is the mirror's new position.
__global__ void k_mirror_update(const KtState* st, const int32_t* __restrict__ pos_new,
                                const int32_t* __restrict__ mir, int32_t* __restrict__ mir_new) {
    const int64_t nnz = st->nnz;  // before the prune
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x) {
        const int32_t p = pos_new[q];
        if (p >= 0) mir_new[p] = pos_new[mir[q]];
    }
}

// Row index and mirror arrays follow C when the iteration swapped.
__global__ void k_kt_copyback_aux(const KtState* st, const int32_t* __restrict__ trow,
                                  const int32_t* __restrict__ mir_new, int32_t* __restrict__ row_of,
                                  int32_t* __restrict__ mir) {
    if (!st->swapped) return;
    const int64_t nnz = st->nnz;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x) {
        row_of[q] = trow[q];
        mir[q] = mir_new[q];
    }
}

void expand_rows(ga_ctx ctx, ga_csr A, int32_t* row_of) {
    k_expand_rows<<<grid_for(A->m * 32, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(A->rst, A->m, row_of);
    post_launch("expand_rows");
}

void mirror_index(ga_ctx ctx, ga_csr A, const int32_t* row_of, int32_t* mir) {
    if (A->nnz == 0) return;
    k_mirror_index<<<grid_for(A->nnz, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(A->rst, A->col, row_of,
                                                                                     A->nnz, mir);
    post_launch("mirror_index");
}

void upper_starts(ga_ctx ctx, ga_csr A, int32_t* ust) {
    k_upper_start<<<grid_for(A->m, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(A->rst, A->col, A->m, ust);
    post_launch("kt_upper_start");
}

ga_csr ktruss_impl(ga_ctx ctx, ga_algo algo, ga_csr A, int k, int* iters_out, const KtBatch* batch) {
    GA_REQUIRE(A->m == A->n, GA_ERR_SHAPE, "k-truss needs a square matrix");
    GA_REQUIRE(A->dtype == GA_INT32, GA_ERR_DTYPE, "k-truss needs int32 values (spMtx<int>)");
    TuneScope tscope(ctx);
    algo = resolve_ktruss_algo(ctx, algo, A);
    GA_REQUIRE(algo == GA_MSA || algo == GA_MCA || algo == GA_HEAP || algo == GA_NAIVE || algo == GA_DOT ||
                   algo == GA_HYBRID || algo == GA_TRI,
               GA_ERR_INVALID_ARG, "k-truss: unknown algorithm");
    const int64_t m = A->m;
    // C = A (a copy; its pattern shrinks in place)
    ga_csr C = copy_csr(ctx, A, GA_INT32);
    try {
        if (m == 0) {
            if (iters_out) *iters_out = 0;
            return C;
        }
        const int64_t cap = A->nnz > 0 ? A->nnz : 1;
        // eflag: keep flags of the entries, scanned in place into new positions
        DBuf<int32_t> sup(ctx, (size_t)cap), eflag(ctx, (size_t)cap + 1), tr(ctx, (size_t)m + 1), tc(ctx, (size_t)cap);
        DBuf<unsigned char> scan_scr(ctx, scan_scratch_bytes(cap));
        DBuf<KtState> st(ctx, 1);
        KtState h0 = {};
        h0.nnz = (int32_t)A->nnz;
        h0.first_vals = 1;
        GA_CUDA(cudaMemcpyAsync(st.p, &h0, sizeof(KtState), cudaMemcpyHostToDevice, ctx->stream));
        // C's values are A's at the first iteration and ones afterwards
        const bool unit = csr_unit_values(ctx, A);
        // For a symmetric A every C stays symmetric, and so does its support:
        // only the upper triangle (columns >= i) is multiplied, the lower
        // triangle is mirrored. Same values, about half the products.
        const bool upper = algo != GA_NAIVE && csr_is_symmetric(ctx, A);
        // Triangle listing when C is symmetric with unit values; else the
        // hybrid form (symmetric) or MSA.
        const bool tri = algo == GA_TRI && upper && unit;
        if (algo == GA_TRI && !tri) algo = upper ? GA_HYBRID : GA_MSA;
        GA_REQUIRE(upper || (algo != GA_DOT && algo != GA_HYBRID), GA_ERR_UNSUPPORTED,
                   "k-truss with GA_DOT or GA_HYBRID needs a symmetric matrix");
        DBuf<unsigned char> mxm_scr(ctx, tri ? tri_kt_bytes(m, cap) : mxm_scratch_bytes(m, m, cap));
        TriKt tk{};
        if (tri) tri_kt_carve(mxm_scr.p, m, cap, &tk);
        const size_t aux = upper ? (size_t)cap : 1;
        DBuf<int32_t> ust(ctx, upper && !tri ? (size_t)m + 1 : 1);
        DBuf<int32_t> row_of(ctx, aux), mir(ctx, aux), pos_new(ctx, aux), trow(ctx, aux), mir_new(ctx, aux);
        ga_csr_s Cu;  // C with row starts moved to the upper part
        const int grid_rows = grid_for(m * 32, 256, ctx->num_sms * 16);
        const int grid_copy = grid_for(m + cap, 256, ctx->num_sms * 8);
        const int grid_ent = grid_for(cap, 256, ctx->num_sms * 16);
        if (upper) {
            // row of every entry and the position of its mirror, kept up to
            // date through the prunes
            k_expand_rows<<<grid_rows, 256, 0, ctx->stream>>>(C->rst, m, row_of.p);
            post_launch("kt_expand_rows");
            if (tri) {
                // rows partitioned [ranked above the row | the rest] for the whole loop
                tri_kt_setup(ctx, C, row_of.p, mir.p, tc.p, eflag.p, tk, cap);
                if (ctx->kt_frontier) {
                    // one listing, then only the triangles of the pruned edges
                    const TriFrontBufs fb{sup.p, eflag.p, tr.p, tc.p, pos_new.p, trow.p, mir_new.p,
                                          reinterpret_cast<uint8_t*>(tk.tcrank), scan_scr.p};
                    const int it = tri_kt_frontier(ctx, C, k, row_of.p, mir.p, tk, cap, fb, batch);
                    C->unit = 1;
                    C->sym = 1;
                    if (iters_out) *iters_out = it;
                    return C;
                }
            } else {
                k_mirror_index<<<grid_ent, 256, 0, ctx->stream>>>(C->rst, C->col, row_of.p, C->nnz, mir.p);
                post_launch("kt_mirror_index");
            }
        }
        auto body = [&](const LoopCtl& ctl) {
            // Tmp<C> = C*C, values aligned with C's pattern
            if (algo == GA_NAIVE) {
                mxm_masked_into(ctx, algo, C, C, C, sup.p);
            } else if (tri) {
                tri_kt_support(ctx, C, sup.p, tk, cap);
            } else if (upper) {
                k_upper_start<<<grid_for(m, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(
                    C->rst, C->col, m, ust.p, batch ? batch->gid : nullptr, batch ? batch->done_g : nullptr);
                post_launch("kt_upper_start");
                Cu = *C;
                Cu.rst = ust.p;
                if (algo == GA_DOT) mxm_dot_launch(ctx, C, C, C, &Cu, sup.p, unit, C->rst + 1);
                else mxm_masked_launch(ctx, algo, C, C, &Cu, sup.p, mxm_scr.p, cap, unit, C->rst + 1, unit,
                                       algo == GA_HYBRID ? C : nullptr);
                k_gather_lower<<<grid_ent, 256, 0, ctx->stream>>>(st.p, C->col, row_of.p, mir.p, sup.p);
                post_launch("kt_gather_lower");
            } else {
                mxm_masked_launch(ctx, algo, C, C, C, sup.p, mxm_scr.p, cap, unit, nullptr, unit);
            }
            // prune: keep flags, their exclusive scan (new positions), scatter
            const int32_t* gid = batch ? batch->gid : nullptr;
            const int32_t* done_g = batch ? batch->done_g : nullptr;
            if (tri) {
                tri_kt_flags(ctx, C, row_of.p, mir.p, sup.p, tk, cap, k, batch, eflag.p);
            } else {
                k_kt_flags<<<grid_ent, 256, 0, ctx->stream>>>(C->rst, sup.p, m, k, cap, eflag.p, gid, done_g,
                                                              upper ? row_of.p : nullptr,
                                                              batch ? batch->kg : nullptr);
                post_launch("kt_flags");
            }
            scan_exclusive_i32_scratch(ctx, eflag.p, eflag.p, cap, scan_scr.p);
            if (tri) {
                tri_kt_scatter(ctx, C, eflag.p, row_of.p, tk, cap, tc.p, tr.p, pos_new.p, trow.p, batch);
            } else {
                k_kt_scatter<<<grid_copy, 256, 0, ctx->stream>>>(C->rst, C->col, eflag.p, m, tc.p, tr.p,
                                                                 upper ? pos_new.p : nullptr,
                                                                 upper ? trow.p : nullptr,
                                                                 upper ? row_of.p : nullptr);
                post_launch("kt_scatter");
            }
            if (batch) {
                k_kt_graph_update<<<grid_for(batch->ngraphs, 128, ctx->num_sms * 4), 128, 0, ctx->stream>>>(
                    st.p, tr.p, *batch);
                post_launch("kt_graph_update");
            }
            if (upper) {
                k_mirror_update<<<grid_ent, 256, 0, ctx->stream>>>(st.p, pos_new.p, mir.p, mir_new.p);
                post_launch("kt_mirror_update");
            }
            k_kt_finalize<<<1, 32, 0, ctx->stream>>>(st.p, tr.p, m, ctl);
            post_launch("kt_finalize");
            if (tri) {
                tri_kt_copyback(ctx, C, st.p, tr.p, tc.p, trow.p, mir_new.p, pos_new.p, row_of.p, mir.p, tk, cap);
                return;
            }
            k_kt_copyback<<<grid_copy, 256, 0, ctx->stream>>>(st.p, tr.p, tc.p, m, C->rst, C->col,
                                                              static_cast<int32_t*>(C->val));
            post_launch("kt_copyback");
            if (upper) {
                k_kt_copyback_aux<<<grid_ent, 256, 0, ctx->stream>>>(st.p, trow.p, mir_new.p, row_of.p, mir.p);
                post_launch("kt_copyback_aux");
            }
        };
        const bool saved = ctx->device_loops;
        if (algo == GA_NAIVE) ctx->device_loops = false;  // naive allocates per call
        try {
            ProfScope ps(ctx, "ktruss_loop");
            run_device_loop(ctx, body, m + 1);
        } catch (...) {
            ctx->device_loops = saved;
            throw;
        }
        ctx->device_loops = saved;
        KtState hs;
        GA_CUDA(cudaMemcpyAsync(&hs, st.p, sizeof(KtState), cudaMemcpyDeviceToHost, ctx->stream));
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
        C->nnz = hs.nnz;
        if (tri) tri_kt_finish(ctx, C, row_of.p, tk, tc.p);  // rows back in column order
        C->unit = unit ? 1 : -1;
        C->sym = upper ? 1 : -1;  // pruning a symmetric matrix by a symmetric support keeps it symmetric
        if (iters_out) *iters_out = hs.iters;
    } catch (...) {
        csr_destroy(ctx, C);
        throw;
    }
    return C;
}

// ------------------------------------------------------------ k-truss sweep
// C_k = k-truss of A for k = kmin, kmin + 1, ... until C_k is empty, each
// C_k equal to k_truss(C_{k-1}, k) (src/main.cpp:90-146). For a symmetric
// 0/1 matrix with triangle listing the frontier state stays on the device
// from one k to the next: the triangles are listed once for the whole
// sweep, and each k starts from the supports the previous k left. Otherwise
// every k is one ga_ktruss call on the previous result.
struct KtSweep {
    ga_ctx ctx = nullptr;
    ga_algo algo = GA_MSA;
    int k = 0;
    bool finished = false;
    ga_csr cur = nullptr;  // stage by stage: the next k's input
    bool fused = false;
    ga_csr W = nullptr;    // fused: A's copy, rows partitioned for the whole sweep
    int64_t cap = 0;
    DBuf<int32_t> sup, eflag, tr, tc, row_of, mir, oid, f0, f1;
    DBuf<uint8_t> state;
    DBuf<unsigned char> scan_scr, tri_scr;
    TriKt tk{};
    std::unique_ptr<TriFront> front;

    ~KtSweep() {
        front.reset();
        if (cur) csr_destroy(ctx, cur);
        if (W) csr_destroy(ctx, W);
    }

    void begin(ga_algo a, ga_csr A, int kmin) {
        GA_REQUIRE(A->m == A->n, GA_ERR_SHAPE, "k-truss needs a square matrix");
        GA_REQUIRE(A->dtype == GA_INT32, GA_ERR_DTYPE, "k-truss needs int32 values (spMtx<int>)");
        algo = a;
        k = kmin;
        const int64_t m = A->m;
        ga_algo r = GA_MSA;
        {
            TuneScope tscope(ctx);
            r = resolve_ktruss_algo(ctx, a, A);
        }
        fused = r == GA_TRI && ctx->kt_frontier && m > 0 && A->nnz > 0 && csr_is_symmetric(ctx, A) &&
                csr_unit_values(ctx, A);
        if (!fused) {
            cur = copy_csr(ctx, A, GA_INT32);
            return;
        }
        W = copy_csr(ctx, A, GA_INT32);
        cap = W->nnz;
        sup = DBuf<int32_t>(ctx, (size_t)cap);
        eflag = DBuf<int32_t>(ctx, (size_t)cap + 1);
        tr = DBuf<int32_t>(ctx, (size_t)m + 1);
        tc = DBuf<int32_t>(ctx, (size_t)cap);
        row_of = DBuf<int32_t>(ctx, (size_t)cap);
        mir = DBuf<int32_t>(ctx, (size_t)cap);
        oid = DBuf<int32_t>(ctx, (size_t)cap);
        f0 = DBuf<int32_t>(ctx, (size_t)cap);
        f1 = DBuf<int32_t>(ctx, (size_t)cap);
        state = DBuf<uint8_t>(ctx, (size_t)cap);
        scan_scr = DBuf<unsigned char>(ctx, scan_scratch_bytes(cap + 1));
        tri_scr = DBuf<unsigned char>(ctx, tri_kt_bytes(m, cap));
        setup_front();
    }

    // The frontier state on W (its rows partitioned by rank, its mirror
    // index; the first run lists W's triangles). The buffers keep the size
    // of the sweep's first matrix; a rebuilt W is smaller.
    void setup_front() {
        cap = W->nnz;
        tri_kt_carve(tri_scr.p, W->m, cap, &tk);
        expand_rows(ctx, W, row_of.p);
        tri_kt_setup(ctx, W, row_of.p, mir.p, tc.p, eflag.p, tk, cap);
        const TriFrontBufs fb{sup.p, eflag.p, tr.p, tc.p, oid.p, f0.p, f1.p, state.p, scan_scr.p};
        front.reset(new TriFront(ctx, W, row_of.p, mir.p, tk, cap, fb, nullptr));
    }

    // Entries never move inside the state, so once a k-truss keeps at most
    // half of W's entries the state is rebuilt on it: every per-k pass (the
    // reseed, the keep flags, the output) then runs over the live entries,
    // at the price of one listing of the smaller graph.
    void maybe_rebuild(ga_csr Ck) {
        if (Ck->nnz == 0 || Ck->nnz * 2 > W->nnz) return;
        front.reset();
        ga_csr nw = copy_csr(ctx, Ck, GA_INT32);
        nw->unit = 1;
        nw->sym = 1;
        csr_destroy(ctx, W);
        W = nw;
        setup_front();
    }

    // The next C_k (owned by the caller), or nullptr after the empty one.
    ga_csr next(int* k_out, int* iters) {
        if (k_out) *k_out = k;
        if (iters) *iters = 0;
        if (finished) return nullptr;
        ga_csr out = nullptr;
        int it = 0;
        if (fused) {
            front->run(k);
            const int64_t kept = front->compact(&it);
            const int64_t m = W->m;
            out = csr_alloc(ctx, m, m, kept, GA_INT32);
            try {
                GA_CUDA(cudaMemcpyAsync(out->rst, tr.p, sizeof(int32_t) * (size_t)(m + 1), cudaMemcpyDeviceToDevice,
                                        ctx->stream));
                if (kept)
                    GA_CUDA(cudaMemcpyAsync(out->col, tc.p, sizeof(int32_t) * (size_t)kept, cudaMemcpyDeviceToDevice,
                                            ctx->stream));
                fill_ones(ctx, out->val, kept, GA_INT32);
            } catch (...) {
                csr_destroy(ctx, out);
                throw;
            }
            out->unit = 1;
            out->sym = 1;
            maybe_rebuild(out);
        } else {
            ga_csr res = ktruss_impl(ctx, algo, cur, k, &it, nullptr);
            csr_destroy(ctx, cur);
            cur = res;
            out = copy_csr(ctx, res, GA_INT32);
            out->unit = res->unit;
            out->sym = res->sym;
        }
        if (iters) *iters = it;
        if (out->nnz == 0) finished = true;
        ++k;
        return out;
    }
};

}  // namespace ga

struct ga_kt_sweep_s : ga::KtSweep {};

using namespace ga;

extern "C" {

int ga_ktruss_sweep_begin(ga_ctx ctx, ga_algo algo, ga_csr A, int kmin, ga_kt_sweep* sweep) {
    if (!ctx || !A || !sweep) return GA_ERR_INVALID_ARG;
    *sweep = nullptr;
    ga_kt_sweep_s* s = nullptr;
    GA_API_BODY(ctx, {
        s = new ga_kt_sweep_s();
        s->ctx = ctx;
        try {
            s->begin(algo, A, kmin);
        } catch (...) {
            delete s;
            throw;
        }
        *sweep = s;
    });
}

int ga_ktruss_sweep_next(ga_kt_sweep sweep, ga_csr* C, int* k, int* iters) {
    if (!sweep || !C) return GA_ERR_INVALID_ARG;
    *C = nullptr;
    ga_ctx ctx = sweep->ctx;
    GA_API_BODY(ctx, *C = sweep->next(k, iters));
}

int ga_ktruss_sweep_free(ga_kt_sweep sweep) {
    if (!sweep) return GA_OK;
    ga_ctx ctx = sweep->ctx;
    GA_API_BODY(ctx, delete sweep);
}

int ga_tc_device(ga_ctx ctx, ga_algo algo, ga_csr A, int64_t* d_total, int64_t* d_per_row) {
    if (!ctx || !A || !d_total) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, tc_device(ctx, algo, A, d_total, d_per_row));
}

int ga_tc(ga_ctx ctx, ga_algo algo, ga_csr A, int64_t* total, int64_t* per_row) {
    if (!ctx || !A || !total) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        DBuf<int64_t> d_total(ctx, 1);
        DBuf<int64_t> d_rows(ctx, per_row ? (size_t)A->m + 1 : 1);
        tc_device(ctx, algo, A, d_total.p, per_row ? d_rows.p : nullptr);
        if (per_row && A->m)
            GA_CUDA(cudaMemcpyAsync(per_row, d_rows.p, sizeof(int64_t) * A->m, cudaMemcpyDeviceToHost, ctx->stream));
        *total = read_i64(ctx, d_total.p);
    });
}

int ga_tc_lu(ga_ctx ctx, ga_algo algo, ga_csr A, int64_t* total) {
    if (!ctx || !A || !total) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        GA_REQUIRE(A->m == A->n, GA_ERR_SHAPE, "triangle counting needs a square matrix");
        GA_REQUIRE(algo != GA_DOT, GA_ERR_INVALID_ARG, "the L*U form takes a masked-SpGEMM variant");
        ga_csr Aa = adjacency_of(ctx, A);
        CsrGuard ga(ctx, Aa);
        ga_csr L = extract_tri(ctx, Aa, true);
        CsrGuard gl(ctx, L);
        ga_csr U = transpose_csr(ctx, L);
        CsrGuard gu(ctx, U);
        DBuf<int32_t> cv(ctx, (size_t)Aa->nnz + 1);
        mxm_masked_into(ctx, algo, L, U, Aa, cv.p);
        DBuf<int64_t> d_total(ctx, 1);
        GA_CUDA(cudaMemsetAsync(d_total.p, 0, sizeof(int64_t), ctx->stream));
        k_row_sums<<<grid_for(A->m * 32, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(
            Aa->rst, cv.p, A->m, nullptr, reinterpret_cast<unsigned long long*>(d_total.p));
        post_launch("row_sums");
        *total = read_i64(ctx, d_total.p) >> 1;
    });
}

int ga_tc_vertex(ga_ctx ctx, ga_algo algo, ga_csr A, int32_t* per_vertex) {
    if (!ctx || !A || !per_vertex) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        GA_REQUIRE(A->m == A->n, GA_ERR_SHAPE, "triangle counting needs a square matrix");
        GA_REQUIRE(algo != GA_DOT, GA_ERR_INVALID_ARG, "the per-vertex form takes a masked-SpGEMM variant");
        ga_csr Aa = adjacency_of(ctx, A);
        CsrGuard ga(ctx, Aa);
        DBuf<int32_t> cv(ctx, (size_t)Aa->nnz + 1);
        mxm_masked_into(ctx, algo, Aa, Aa, Aa, cv.p);
        DBuf<int32_t> out(ctx, (size_t)A->m + 1);
        k_row_sums_half_i32<<<grid_for(A->m * 32, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(Aa->rst, cv.p,
                                                                                                A->m, out.p);
        post_launch("row_sums_half");
        GA_CUDA(cudaMemcpyAsync(per_vertex, out.p, sizeof(int32_t) * A->m, cudaMemcpyDeviceToHost, ctx->stream));
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int ga_ktruss(ga_ctx ctx, ga_algo algo, ga_csr A, int k, ga_csr* C, int* iters) {
    if (!ctx || !A || !C) return GA_ERR_INVALID_ARG;
    *C = nullptr;
    GA_API_BODY(ctx, *C = ktruss_impl(ctx, algo, A, k, iters, nullptr));
}

}  // extern "C"
