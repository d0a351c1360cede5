// Callers of the masked SpGEMM: triangle counting (Sandia L*L, L*U and
// per-vertex forms, plus the warp-intersection dot-product form) and the
// device-resident k-truss loop. Also the CUDA-graph loop driver.
#include "ga_device.cuh"
#include "ga_loop.cuh"

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
        cudaGraphDestroy(graph);
        throw;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
}

// ==================================================== triangle counting
constexpr int kTcThreads = 256;
constexpr int kTcWarps = kTcThreads / 32;
constexpr int kTcRowSmem = 1024;  // L row entries staged in shared memory per warp

// Dot-product form over L (strict lower triangle, rows sorted): for each row
// i and each j in L_i, |L_i ∩ L_j| counted by warp-level sorted-list
// intersection. Only the prefix L_i[0..t) (entries < j) can meet L_j. The
// shorter list is walked 32 entries at a time, one per lane, each lane
// binary-searches the longer one, and __ballot_sync/__popc count the hits.
// Rows are fetched dynamically so hub rows do not stall a static schedule.
// per_row[i] = triangles whose largest vertex is i (the row sums of the
// reference's C<L> = L*L).
__global__ void __launch_bounds__(kTcThreads) k_tc_dot(const int32_t* __restrict__ lr, const int32_t* __restrict__ lc,
                                                       int64_t m, int* __restrict__ next_row,
                                                       unsigned long long* __restrict__ total,
                                                       int64_t* __restrict__ per_row) {
    __shared__ int32_t buf[kTcWarps][kTcRowSmem];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned FULL = 0xffffffffu;
    unsigned long long acc_total = 0;
    while (true) {
        int i = 0;
        if (lane == 0) i = atomicAdd(next_row, 1);
        i = __shfl_sync(FULL, i, 0);
        if (i >= m) break;
        const int32_t lb = lr[i], ln = lr[i + 1] - lb;
        const int32_t* Li;
        if (ln <= kTcRowSmem) {
            for (int t = lane; t < ln; t += 32) buf[wid][t] = lc[lb + t];
            __syncwarp();
            Li = buf[wid];
        } else {
            Li = lc + lb;
        }
        long long cnt = 0;
        for (int t = 1; t < ln; ++t) {
            const int32_t j = Li[t];
            const int32_t jb = lr[j], jn = lr[j + 1] - jb;
            if (jn == 0) continue;
            if (jn <= t) {
                for (int base = 0; base < jn; base += 32) {
                    int q = base + lane;
                    bool hit = false;
                    if (q < jn) {
                        int32_t x = __ldg(lc + jb + q);
                        int p = lower_bound_i32(Li, t, x);
                        hit = p < t && Li[p] == x;
                    }
                    unsigned bal = __ballot_sync(FULL, hit);
                    cnt += __popc(bal);
                }
            } else {
                const int32_t* Lj = lc + jb;
                for (int base = 0; base < t; base += 32) {
                    int q = base + lane;
                    bool hit = false;
                    if (q < t) {
                        int32_t x = Li[q];
                        int p = lower_bound_i32(Lj, jn, x);
                        hit = p < jn && __ldg(Lj + p) == x;
                    }
                    unsigned bal = __ballot_sync(FULL, hit);
                    cnt += __popc(bal);
                }
            }
        }
        if (lane == 0) {
            if (per_row) per_row[i] = cnt;
            acc_total += (unsigned long long)cnt;
        }
        __syncwarp();
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
    unsigned long long* tot = reinterpret_cast<unsigned long long*>(d_total);
    GA_CUDA(cudaMemsetAsync(tot, 0, sizeof(unsigned long long), ctx->stream));
    if (A->m == 0) return;
    ga_csr L0 = extract_tri(ctx, A, true);
    CsrGuard g0(ctx, L0);
    if (algo == GA_DOT) {
        DBuf<int> next(ctx, 1);
        GA_CUDA(cudaMemsetAsync(next.p, 0, sizeof(int), ctx->stream));
        if (d_per_row) GA_CUDA(cudaMemsetAsync(d_per_row, 0, sizeof(int64_t) * A->m, ctx->stream));
        ProfScope ps(ctx, "tc_dot");
        k_tc_dot<<<ctx->num_sms * 8, kTcThreads, 0, ctx->stream>>>(L0->rst, L0->col, A->m, next.p, tot, d_per_row);
        post_launch("tc_dot");
        return;
    }
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
struct KtState {
    int32_t nnz;        // nnz of C
    int32_t t;          // iteration index
    int32_t iters;      // reported iteration count
    int32_t swapped;    // this iteration replaced C by the pruned matrix
    int32_t done;
    int32_t first_vals; // C still carries A's values (no swap yet)
};

__global__ void k_kt_count(const int32_t* __restrict__ cr, const int32_t* __restrict__ sup, int64_t m, int k,
                           int32_t* __restrict__ cnt) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
        int c = 0;
        for (int32_t q = cr[i] + lane; q < cr[i + 1]; q += 32) c += sup[q] >= k - 2;
        c = warp_sum<int>(c);
        if (lane == 0) cnt[i] = c;
    }
}

// Keep entries with support >= k-2, in order (ballot compaction per row).
__global__ void k_kt_compact(const int32_t* __restrict__ cr, const int32_t* __restrict__ cc,
                             const int32_t* __restrict__ sup, const int32_t* __restrict__ tr, int64_t m, int k,
                             int32_t* __restrict__ tc) {
    const int lane = threadIdx.x & 31;
    const unsigned FULL = 0xffffffffu;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
        int32_t o = tr[i];
        const int32_t b = cr[i], e = cr[i + 1];
        for (int32_t base = b; base < e; base += 32) {
            int32_t q = base + lane;
            bool keep = q < e && sup[q] >= k - 2;
            unsigned bal = __ballot_sync(FULL, keep);
            if (keep) tc[o + __popc(bal & ((1u << lane) - 1u))] = cc[q];
            o += __popc(bal);
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

static ga_csr ktruss(ga_ctx ctx, ga_algo algo, ga_csr A, int k, int* iters_out) {
    GA_REQUIRE(A->m == A->n, GA_ERR_SHAPE, "k-truss needs a square matrix");
    GA_REQUIRE(A->dtype == GA_INT32, GA_ERR_DTYPE, "k-truss needs int32 values (spMtx<int>)");
    GA_REQUIRE(algo == GA_MSA || algo == GA_MCA || algo == GA_HEAP || algo == GA_NAIVE, GA_ERR_INVALID_ARG,
               "k-truss: unknown algorithm");
    const int64_t m = A->m;
    // C = A (a copy; its pattern shrinks in place)
    ga_csr C = copy_csr(ctx, A, GA_INT32);
    try {
        if (m == 0) {
            if (iters_out) *iters_out = 0;
            return C;
        }
        const int64_t cap = A->nnz > 0 ? A->nnz : 1;
        DBuf<int32_t> sup(ctx, (size_t)cap), cnt(ctx, (size_t)m + 1), tr(ctx, (size_t)m + 1), tc(ctx, (size_t)cap);
        DBuf<unsigned char> scan_scr(ctx, scan_scratch_bytes(m));
        DBuf<unsigned char> mxm_scr(ctx, mxm_scratch_bytes(m, m, cap));
        DBuf<KtState> st(ctx, 1);
        KtState h0 = {};
        h0.nnz = (int32_t)A->nnz;
        h0.first_vals = 1;
        GA_CUDA(cudaMemcpyAsync(st.p, &h0, sizeof(KtState), cudaMemcpyHostToDevice, ctx->stream));
        // C's values are A's at the first iteration and ones afterwards
        const bool unit = csr_unit_values(ctx, A);
        const int grid_rows = grid_for(m * 32, 256, ctx->num_sms * 16);
        const int grid_copy = grid_for(m + cap, 256, ctx->num_sms * 8);
        auto body = [&](const LoopCtl& ctl) {
            // Tmp<C> = C*C, values aligned with C's pattern
            if (algo == GA_NAIVE) mxm_masked_into(ctx, algo, C, C, C, sup.p);
            else mxm_masked_launch(ctx, algo, C, C, C, sup.p, mxm_scr.p, cap, unit);
            k_kt_count<<<grid_rows, 256, 0, ctx->stream>>>(C->rst, sup.p, m, k, cnt.p);
            post_launch("kt_count");
            scan_exclusive_i32_scratch(ctx, cnt.p, tr.p, m, scan_scr.p);
            k_kt_compact<<<grid_rows, 256, 0, ctx->stream>>>(C->rst, C->col, sup.p, tr.p, m, k, tc.p);
            post_launch("kt_compact");
            k_kt_finalize<<<1, 32, 0, ctx->stream>>>(st.p, tr.p, m, ctl);
            post_launch("kt_finalize");
            k_kt_copyback<<<grid_copy, 256, 0, ctx->stream>>>(st.p, tr.p, tc.p, m, C->rst, C->col,
                                                              static_cast<int32_t*>(C->val));
            post_launch("kt_copyback");
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
        C->unit = unit ? 1 : -1;
        if (iters_out) *iters_out = hs.iters;
    } catch (...) {
        csr_destroy(ctx, C);
        throw;
    }
    return C;
}

}  // namespace ga

using namespace ga;

extern "C" {

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
    GA_API_BODY(ctx, *C = ktruss(ctx, algo, A, k, iters));
}

}  // extern "C"
