// Masked SpGEMM C<M> = A*B (structural mask, C has M's pattern).
//
// Design (one pass, no symbolic phase: the output pattern is M's):
//  1. k_row_bin: one warp per output row computes the mask length m_i and the
//     Gustavson product count P_i = sum_{k in A_i} nnz(B_k); rows with an
//     empty mask are skipped, rows with no products get explicit zeros, the
//     rest go to a warp queue (short mask rows, few products) or a CTA queue
//     (long mask rows or many products; mask rows longer than kCtaSlots are
//     split into slot chunks, each chunk restricted to its column range).
//  2. k_mxm_masked: a persistent kernel (one wave of CTAs sized by occupancy)
//     drains the CTA queue, then each warp drains the warp queue. Per row the
//     accumulator is indexed by mask slot and lives in shared memory.
//     The column -> slot lookup is the variant:
//       GA_MSA  : open-addressing hash of the mask row in shared memory;
//       GA_MCA  : binary search of the sorted mask row in shared memory
//                 (the reference MCA walks the mask row, matrix_la.h:625-632);
//       GA_HEAP : warp-cooperative sorted merge of each B row against the
//                 mask row (replaces the priority-queue merge,
//                 matrix_la.h:1030-1084).
//     MSA and MCA flatten the products of 32 A entries across the warp's
//     lanes (a warp scan of the B row lengths, then each lane walks the
//     flattened index), so hub rows of B keep every lane busy and B's column
//     stream is read coalesced.
// Integer results are exact and equal across variants; floating-point sums
// are accumulated with shared-memory atomics (order not fixed).
#include "ga_device.cuh"

namespace ga {

constexpr int kMxmThreads = 512;
constexpr int kMxmWarps = kMxmThreads / 32;
constexpr int kCtaSlots = 4096;      // mask slots per CTA work item
constexpr int kCtaTblBits = 13;      // 8192-entry hash table
constexpr int kWarpSlots = 128;      // mask slots per warp row
constexpr int kWarpTblBits = 8;      // 256-entry hash table
constexpr int64_t kWarpMaxFlops = 1 << 16;  // rows above this go to a CTA

struct MxmQueue {
    int32_t warp_count;
    int32_t cta_count;
    int32_t warp_next;
    int32_t cta_next;
    unsigned long long flops;  // total products (reported)
};

template <typename T, typename A>
struct MxmArgs {
    const int32_t* ar; const int32_t* ac; const T* av;
    const int32_t* br; const int32_t* bc; const T* bv;
    const int32_t* mr; const int32_t* mc;
    T* cv;
    int64_t m;
    MxmQueue* q;
    int32_t* warp_rows;
    int2* cta_items;
};

__global__ void k_reset_queue(MxmQueue* q) {
    if (threadIdx.x == 0) {
        q->warp_count = 0; q->cta_count = 0; q->warp_next = 0; q->cta_next = 0; q->flops = 0ull;
    }
}

// ------------------------------------------------------------------ binning
template <typename T, typename A>
__global__ void k_row_bin(MxmArgs<T, A> p) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    unsigned long long my_flops = 0;
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < p.m; i += warps) {
        int32_t mb = p.mr[i], me = p.mr[i + 1];
        int32_t mi = me - mb;
        if (mi == 0) continue;
        int32_t ab = p.ar[i], ae = p.ar[i + 1];
        long long f = 0;
        for (int32_t t = ab + lane; t < ae; t += 32) {
            int32_t k = p.ac[t];
            f += p.br[k + 1] - p.br[k];
        }
        f = warp_sum<long long>(f);
        if (f == 0) {
            for (int32_t q = mb + lane; q < me; q += 32) p.cv[q] = (T)0;
            continue;
        }
        if (lane == 0) {
            my_flops += (unsigned long long)f;
            if (mi <= kWarpSlots && f <= kWarpMaxFlops) {
                int pos = atomicAdd(&p.q->warp_count, 1);
                p.warp_rows[pos] = (int32_t)i;
            } else {
                int chunks = (mi + kCtaSlots - 1) / kCtaSlots;
                int pos = atomicAdd(&p.q->cta_count, chunks);
                for (int c = 0; c < chunks; ++c) p.cta_items[pos + c] = make_int2((int)i, c);
            }
        }
    }
    if (lane == 0 && my_flops) atomicAdd(&p.q->flops, my_flops);
}

// ------------------------------------------------------------------ lookups
enum { LK_HASH = 0, LK_BSEARCH = 1, LK_MERGE = 2 };

struct SlotTable {
    int32_t* keys;    // hash keys (LK_HASH) or sorted mask columns (others)
    uint16_t* slots;  // hash payload (LK_HASH)
    int bits;
    int ns;           // slots in this item
    int32_t lo, hi;   // column range of the item
};

template <int LK>
__device__ __forceinline__ int slot_of(const SlotTable& t, int32_t c) {
    if (LK == LK_HASH) {
        return hash_find<uint16_t>(t.keys, t.slots, t.bits, c);
    } else {
        if (c < t.lo || c > t.hi) return -1;
        int pos = lower_bound_i32(t.keys, t.ns, c);
        return (pos < t.ns && t.keys[pos] == c) ? pos : -1;
    }
}

// Products of A entries [t, t+32) (lane-strided group) for one output row,
// flattened over the warp. s_incl/s_off/s_a are this warp's 32-entry scratch.
template <int LK, typename T, typename A>
__device__ __forceinline__ void group_products(const MxmArgs<T, A>& p, int32_t t_first, int32_t t_end,
                                               const SlotTable& tbl, A* acc, bool clip, int* s_incl, int* s_off,
                                               A* s_a) {
    const int lane = threadIdx.x & 31;
    int32_t t = t_first + lane;
    int len = 0;
    int32_t bs = 0;
    A av = (A)0;
    if (t < t_end) {
        int32_t k = p.ac[t];
        av = to_acc<T, A>(p.av[t]);
        bs = p.br[k];
        int32_t be = p.br[k + 1];
        if (clip) {
            int n = be - bs;
            int lo = lower_bound_i32(p.bc + bs, n, tbl.lo);
            int hi = upper_bound_i32(p.bc + bs, n, tbl.hi);
            be = bs + hi;
            bs = bs + lo;
        }
        len = be - bs;
    }
    int incl = warp_incl_scan(len);
    int total = __shfl_sync(0xffffffffu, incl, 31);
    s_incl[lane] = incl;
    s_off[lane] = bs - (incl - len);
    s_a[lane] = av;
    __syncwarp();
    int q = 0;
    for (int pidx = lane; pidx < total; pidx += 32) {
        while (s_incl[q] <= pidx) ++q;
        int32_t j = pidx + s_off[q];
        int32_t c = __ldg(p.bc + j);
        int slot = slot_of<LK>(tbl, c);
        if (slot >= 0) atomic_add_acc<A>(&acc[slot], s_a[q] * to_acc<T, A>(__ldg(p.bv + j)));
    }
    __syncwarp();
}

// Warp-cooperative sorted merge of B row k (columns [bs, be)) against the
// item's sorted mask columns; matches add a*b into the slot accumulator.
template <typename T, typename A>
__device__ __forceinline__ void merge_row(const MxmArgs<T, A>& p, int32_t bs, int32_t be, A av,
                                          const SlotTable& tbl, A* acc) {
    const int lane = threadIdx.x & 31;
    const unsigned FULL = 0xffffffffu;
    if (bs >= be) return;
    int32_t x0 = __ldg(p.bc + bs);
    int yc = lower_bound_i32(tbl.keys, tbl.ns, x0);
    int32_t xb = bs;
    while (xb < be && yc < tbl.ns) {
        int32_t x = (xb + lane < be) ? __ldg(p.bc + xb + lane) : INT32_MAX;
        int32_t y = (yc + lane < tbl.ns) ? tbl.keys[yc + lane] : INT32_MAX;
        int r = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            int32_t yy = __shfl_sync(FULL, y, r + step - 1);
            if (yy < x) r += step;
        }
        int32_t y31 = __shfl_sync(FULL, y, 31);
        if (r == 31 && y31 < x) r = 32;
        int32_t yr = __shfl_sync(FULL, y, r & 31);
        if (r < 32 && yr == x && x != INT32_MAX)
            atomic_add_acc<A>(&acc[yc + r], av * to_acc<T, A>(__ldg(p.bv + xb + lane)));
        int32_t x31 = __shfl_sync(FULL, x, 31);
        if (x31 <= y31) xb += 32; else yc += 32;
    }
}

template <typename A>
struct MxmSmem {
    static constexpr size_t cta_bytes =
        (size_t)(1 << kCtaTblBits) * sizeof(int32_t) + (size_t)(1 << kCtaTblBits) * sizeof(uint16_t) +
        (size_t)kCtaSlots * sizeof(A);
    static constexpr size_t warp_one = (size_t)(1 << kWarpTblBits) * sizeof(int32_t) +
                                       (size_t)(1 << kWarpTblBits) * sizeof(uint16_t) + (size_t)kWarpSlots * sizeof(A);
    static constexpr size_t warp_bytes = warp_one * kMxmWarps;
    static constexpr size_t scratch_bytes = (size_t)kMxmWarps * 32 * (2 * sizeof(int) + sizeof(A));
    static constexpr size_t total = (cta_bytes > warp_bytes ? cta_bytes : warp_bytes) + scratch_bytes;
};

template <int LK, typename T, typename A>
__global__ void __launch_bounds__(kMxmThreads, 2) k_mxm_masked(MxmArgs<T, A> p) {
    extern __shared__ __align__(16) unsigned char smem[];
    using SM = MxmSmem<A>;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int* s_incl = reinterpret_cast<int*>(smem + (SM::total - SM::scratch_bytes)) + wid * 32;
    int* s_off = reinterpret_cast<int*>(smem + (SM::total - SM::scratch_bytes)) + kMxmWarps * 32 + wid * 32;
    A* s_a = reinterpret_cast<A*>(smem + (SM::total - SM::scratch_bytes) + (size_t)kMxmWarps * 32 * 2 * sizeof(int)) +
             wid * 32;
    __shared__ int s_item;

    // ------------------------------------------------------------ CTA items
    {
        const int TBL = 1 << kCtaTblBits;
        int32_t* keys = reinterpret_cast<int32_t*>(smem);
        uint16_t* slots = reinterpret_cast<uint16_t*>(smem + TBL * sizeof(int32_t));
        A* acc = reinterpret_cast<A*>(smem + TBL * (sizeof(int32_t) + sizeof(uint16_t)));
        for (int t = threadIdx.x; t < TBL; t += blockDim.x) keys[t] = kEmpty;
        const int ncta = p.q->cta_count;
        while (true) {
            if (threadIdx.x == 0) s_item = atomicAdd(&p.q->cta_next, 1);
            __syncthreads();
            const int it = s_item;
            if (it >= ncta) break;
            const int2 item = p.cta_items[it];
            const int64_t i = item.x;
            const int32_t mb = p.mr[i], mi = p.mr[i + 1] - mb;
            const int s0 = item.y * kCtaSlots;
            const int ns = min(kCtaSlots, mi - s0);
            const int32_t* mcol = p.mc + mb + s0;
            SlotTable tbl;
            tbl.keys = keys; tbl.slots = slots; tbl.bits = kCtaTblBits; tbl.ns = ns;
            tbl.lo = __ldg(mcol); tbl.hi = __ldg(mcol + ns - 1);
            if (LK == LK_HASH) {
                for (int s = threadIdx.x; s < ns; s += blockDim.x)
                    hash_insert<uint16_t>(keys, slots, kCtaTblBits, __ldg(mcol + s), (uint16_t)s);
            } else {
                for (int s = threadIdx.x; s < ns; s += blockDim.x) keys[s] = __ldg(mcol + s);
            }
            for (int s = threadIdx.x; s < ns; s += blockDim.x) acc[s] = (A)0;
            __syncthreads();
            const bool clip = mi > kCtaSlots;
            const int32_t ab = p.ar[i], ae = p.ar[i + 1];
            if (LK == LK_MERGE) {
                for (int32_t t = ab + wid; t < ae; t += kMxmWarps) {
                    int32_t k = __ldg(p.ac + t);
                    A av = to_acc<T, A>(__ldg(p.av + t));
                    int32_t bs = __ldg(p.br + k), be = __ldg(p.br + k + 1);
                    merge_row<T, A>(p, bs, be, av, tbl, acc);
                }
            } else {
                for (int32_t g = ab + wid * 32; g < ae; g += kMxmWarps * 32)
                    group_products<LK, T, A>(p, g, ae, tbl, acc, clip, s_incl, s_off, s_a);
            }
            __syncthreads();
            for (int s = threadIdx.x; s < ns; s += blockDim.x) p.cv[mb + s0 + s] = from_acc<T, A>(acc[s]);
            if (LK == LK_HASH) {
                for (int t = threadIdx.x; t < TBL; t += blockDim.x) keys[t] = kEmpty;
            }
            __syncthreads();
        }
    }

    // ----------------------------------------------------------- warp rows
    {
        const int TBL = 1 << kWarpTblBits;
        unsigned char* base = smem + wid * SM::warp_one;
        int32_t* keys = reinterpret_cast<int32_t*>(base);
        uint16_t* slots = reinterpret_cast<uint16_t*>(base + TBL * sizeof(int32_t));
        A* acc = reinterpret_cast<A*>(base + TBL * (sizeof(int32_t) + sizeof(uint16_t)));
        for (int t = lane; t < TBL; t += 32) keys[t] = kEmpty;
        __syncwarp();
        const int nwarp = p.q->warp_count;
        while (true) {
            int r = 0;
            if (lane == 0) r = atomicAdd(&p.q->warp_next, 1);
            r = __shfl_sync(0xffffffffu, r, 0);
            if (r >= nwarp) break;
            const int64_t i = p.warp_rows[r];
            const int32_t mb = p.mr[i], mi = p.mr[i + 1] - mb;
            const int32_t* mcol = p.mc + mb;
            SlotTable tbl;
            tbl.keys = keys; tbl.slots = slots; tbl.bits = kWarpTblBits; tbl.ns = mi;
            tbl.lo = __ldg(mcol); tbl.hi = __ldg(mcol + mi - 1);
            if (LK == LK_HASH) {
                for (int s = lane; s < mi; s += 32)
                    hash_insert<uint16_t>(keys, slots, kWarpTblBits, __ldg(mcol + s), (uint16_t)s);
            } else {
                for (int s = lane; s < mi; s += 32) keys[s] = __ldg(mcol + s);
            }
            for (int s = lane; s < mi; s += 32) acc[s] = (A)0;
            __syncwarp();
            const int32_t ab = p.ar[i], ae = p.ar[i + 1];
            if (LK == LK_MERGE) {
                for (int32_t t = ab; t < ae; ++t) {
                    int32_t k = __ldg(p.ac + t);
                    A av = to_acc<T, A>(__ldg(p.av + t));
                    merge_row<T, A>(p, __ldg(p.br + k), __ldg(p.br + k + 1), av, tbl, acc);
                }
            } else {
                for (int32_t g = ab; g < ae; g += 32)
                    group_products<LK, T, A>(p, g, ae, tbl, acc, false, s_incl, s_off, s_a);
            }
            __syncwarp();
            for (int s = lane; s < mi; s += 32) p.cv[mb + s] = from_acc<T, A>(acc[s]);
            if (LK == LK_HASH) {
                for (int t = lane; t < TBL; t += 32) keys[t] = kEmpty;
            }
            __syncwarp();
        }
    }
}

// Launch the masked product for one value type and lookup variant.
template <int LK, typename T>
static void launch_masked(ga_ctx ctx, ga_csr A_, ga_csr B_, ga_csr M_, T* cv, MxmQueue* q, int32_t* warp_rows,
                          int2* cta_items) {
    using Ac = typename Acc<T>::type;
    MxmArgs<T, Ac> p;
    p.ar = A_->rst; p.ac = A_->col; p.av = static_cast<const T*>(A_->val);
    p.br = B_->rst; p.bc = B_->col; p.bv = static_cast<const T*>(B_->val);
    p.mr = M_->rst; p.mc = M_->col;
    p.cv = cv; p.m = M_->m; p.q = q; p.warp_rows = warp_rows; p.cta_items = cta_items;
    {
        ProfScope ps(ctx, "mxm_row_bin");
        int grid = grid_for(p.m * 32, 256, ctx->num_sms * 16);
        k_row_bin<T, Ac><<<grid, 256, 0, ctx->stream>>>(p);
        post_launch("mxm_row_bin");
    }
    const size_t smem = MxmSmem<Ac>::total;
    auto kern = k_mxm_masked<LK, T, Ac>;
    GA_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    GA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kMxmThreads, smem));
    if (per_sm < 1) per_sm = 1;
    const char* name = LK == LK_HASH ? "mxm_msa" : LK == LK_BSEARCH ? "mxm_mca" : "mxm_heap_merge";
    ProfScope ps(ctx, name);
    kern<<<ctx->num_sms * per_sm, kMxmThreads, smem, ctx->stream>>>(p);
    post_launch(name);
}

void naive_masked_into(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr M, void* d_cvals);

size_t mxm_scratch_bytes(int64_t m, int64_t mask_nnz) {
    const int64_t cap_cta = m + mask_nnz / kCtaSlots + 1;
    return 256 + sizeof(int32_t) * (size_t)(m + 1) + sizeof(int2) * (size_t)cap_cta + 64;
}

// Non-allocating launch (usable inside captured loops): `scratch` holds
// mxm_scratch_bytes(M->m, max nnz(M)) bytes. Resets the queue itself.
void mxm_masked_launch(ga_ctx ctx, ga_algo algo, ga_csr A, ga_csr B, ga_csr M, void* d_cvals, void* scratch) {
    GA_REQUIRE(algo == GA_MSA || algo == GA_MCA || algo == GA_HEAP, GA_ERR_INVALID_ARG, "mxm: unknown algorithm");
    unsigned char* s = static_cast<unsigned char*>(scratch);
    MxmQueue* q = reinterpret_cast<MxmQueue*>(s);
    int32_t* warp_rows = reinterpret_cast<int32_t*>(s + 256);
    size_t off = 256 + sizeof(int32_t) * (size_t)(M->m + 1);
    off = (off + 15) & ~(size_t)15;
    int2* cta_items = reinterpret_cast<int2*>(s + off);
    k_reset_queue<<<1, 32, 0, ctx->stream>>>(q);
    post_launch("mxm_reset_queue");
    GA_DISPATCH_DTYPE(A->dtype, T, {
        T* cv = static_cast<T*>(d_cvals);
        if (algo == GA_MSA) launch_masked<LK_HASH, T>(ctx, A, B, M, cv, q, warp_rows, cta_items);
        else if (algo == GA_MCA) launch_masked<LK_BSEARCH, T>(ctx, A, B, M, cv, q, warp_rows, cta_items);
        else launch_masked<LK_MERGE, T>(ctx, A, B, M, cv, q, warp_rows, cta_items);
    });
}

void mxm_masked_into(ga_ctx ctx, ga_algo algo, ga_csr A, ga_csr B, ga_csr M, void* d_cvals) {
    GA_REQUIRE(A->n == B->m, GA_ERR_SHAPE, "mxm: A.n != B.m");
    GA_REQUIRE(M->m == A->m && M->n == B->n, GA_ERR_SHAPE, "mxm: mask shape differs from A*B");
    GA_REQUIRE(A->dtype == B->dtype, GA_ERR_DTYPE, "mxm: A and B dtypes differ");
    if (M->nnz == 0 || M->m == 0) return;
    if (algo == GA_NAIVE) {
        naive_masked_into(ctx, A, B, M, d_cvals);
        return;
    }
    DBuf<unsigned char> scratch(ctx, mxm_scratch_bytes(M->m, M->nnz));
    mxm_masked_launch(ctx, algo, A, B, M, d_cvals, scratch.p);
}

}  // namespace ga

using namespace ga;

extern "C" {

int ga_mxm_masked_vals(ga_ctx ctx, ga_algo algo, ga_csr A, ga_csr B, ga_csr M, void* d_cvals) {
    if (!ctx || !A || !B || !M || (!d_cvals && M->nnz)) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, mxm_masked_into(ctx, algo, A, B, M, d_cvals));
}

int ga_mxm_masked(ga_ctx ctx, ga_algo algo, ga_csr A, ga_csr B, ga_csr M, ga_csr* C) {
    if (!ctx || !A || !B || !M || !C) return GA_ERR_INVALID_ARG;
    *C = nullptr;
    GA_API_BODY(ctx, {
        GA_REQUIRE(A->dtype == B->dtype, GA_ERR_DTYPE, "mxm: A and B dtypes differ");
        ga_csr R = csr_alloc(ctx, M->m, M->n, M->nnz, A->dtype);
        try {
            GA_CUDA(cudaMemcpyAsync(R->rst, M->rst, sizeof(int32_t) * (M->m + 1), cudaMemcpyDeviceToDevice,
                                    ctx->stream));
            if (M->nnz)
                GA_CUDA(cudaMemcpyAsync(R->col, M->col, sizeof(int32_t) * M->nnz, cudaMemcpyDeviceToDevice,
                                        ctx->stream));
            mxm_masked_into(ctx, algo, A, B, M, R->val);
        } catch (...) {
            csr_destroy(ctx, R);
            throw;
        }
        *C = R;
    });
}

}  // extern "C"
