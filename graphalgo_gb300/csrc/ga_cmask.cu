// Complemented-mask SpGEMM C<!M> = A*B (new pattern, sorted columns) and the
// "naive" masked product built on it (full product, then a mask gather).
//
// Two passes over the same per-row machinery, as the reference does
// (matrix_la.h:800-891): a symbolic pass counts each row's output columns,
// a prefix sum gives the row starts, a numeric pass fills columns and values.
// One CTA per row (grid-stride). A row whose product count P_i is at most
// kHashMax uses a shared-memory hash of its product columns; the surviving
// keys (not in M's row) are sorted with a block bitonic sort. Longer rows are
// processed in column windows of kWin columns with a dense shared-memory
// accumulator and bitmap, which yields sorted output directly.
#include "ga_device.cuh"

namespace ga {

constexpr int kCmThreads = 256;
constexpr int kCmWarps = kCmThreads / 32;
constexpr int kHashMax = 2048;          // products handled by the hash path
constexpr int kHashBitsMax = 12;        // 4096-entry table
constexpr int kWin = 4096;              // columns per dense window

template <typename T>
struct CmArgs {
    const int32_t* ar; const int32_t* ac; const T* av;
    const int32_t* br; const int32_t* bc; const T* bv;
    const int32_t* mr; const int32_t* mc;  // mr == nullptr: no mask
    int64_t m;
    const int64_t* flops;  // P_i per row
    int32_t* cnt;          // symbolic output
    const int32_t* cr;     // numeric: row starts
    int32_t* cc; T* cv;    // numeric outputs
};

__global__ void k_cm_flops(const int32_t* __restrict__ ar, const int32_t* __restrict__ ac,
                           const int32_t* __restrict__ br, int64_t m, int64_t* __restrict__ flops) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
        long long f = 0;
        for (int32_t t = ar[i] + lane; t < ar[i + 1]; t += 32) {
            int32_t k = ac[t];
            f += br[k + 1] - br[k];
        }
        f = warp_sum<long long>(f);
        if (lane == 0) flops[i] = f;
    }
}

__device__ __forceinline__ bool in_mask(const int32_t* mc, int32_t mb, int32_t me, int32_t c) {
    int n = me - mb;
    int p = lower_bound_i32(mc + mb, n, c);
    return p < n && mc[mb + p] == c;
}

// Visit every product (col, a*b) of row i whose column lies in [lo, hi],
// flattened over the lanes of each warp; warps take groups of 32 A entries.
template <bool CLIP, typename T, typename Fn>
__device__ __forceinline__ void foreach_product(const CmArgs<T>& p, int64_t i, int32_t lo, int32_t hi, int* s_incl,
                                                int* s_off, T* s_a, Fn fn) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int32_t ab = p.ar[i], ae = p.ar[i + 1];
    for (int32_t g = ab + wid * 32; g < ae; g += kCmWarps * 32) {
        int32_t t = g + lane;
        int len = 0;
        int32_t bs = 0;
        T a = (T)0;
        if (t < ae) {
            int32_t k = p.ac[t];
            a = p.av[t];
            bs = p.br[k];
            int32_t be = p.br[k + 1];
            if (CLIP) {
                int n = be - bs;
                int l = lower_bound_i32(p.bc + bs, n, lo);
                int h = upper_bound_i32(p.bc + bs, n, hi);
                be = bs + h;
                bs = bs + l;
            }
            len = be - bs;
        }
        int incl = warp_incl_scan(len);
        int total = __shfl_sync(0xffffffffu, incl, 31);
        s_incl[lane] = incl;
        s_off[lane] = bs - (incl - len);
        s_a[lane] = a;
        __syncwarp();
        int q = 0;
        for (int x = lane; x < total; x += 32) {
            while (s_incl[q] <= x) ++q;
            int32_t j = x + s_off[q];
            fn(__ldg(p.bc + j), s_a[q], j);
        }
        __syncwarp();
    }
}

// Block-wide exclusive scan of one int per thread.
__device__ __forceinline__ int block_scan_int(int v, int* warp_tot, int* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = warp_incl_scan(v);
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int w = lane < kCmWarps ? warp_tot[lane] : 0;
        int y = warp_incl_scan(w);
        if (lane < kCmWarps) warp_tot[lane] = y - w;
        if (lane == kCmWarps - 1) *total = y;
    }
    __syncthreads();
    int r = x - v + warp_tot[wid];
    __syncthreads();
    return r;
}

template <typename T>
struct CmSmem {
    static constexpr size_t hash_bytes = (size_t)(1 << kHashBitsMax) * (sizeof(int32_t) + sizeof(T)) +
                                         (size_t)(1 << kHashBitsMax) * (sizeof(int32_t) + sizeof(T));
    static constexpr size_t win_bytes = (size_t)kWin * sizeof(T) + (size_t)(kWin / 32) * sizeof(uint32_t);
    static constexpr size_t scratch = (size_t)kCmWarps * 32 * (2 * sizeof(int) + sizeof(T));
    static constexpr size_t total = (hash_bytes > win_bytes ? hash_bytes : win_bytes) + scratch;
};

template <bool NUMERIC, typename T>
__global__ void __launch_bounds__(kCmThreads) k_cmask(CmArgs<T> p) {
    extern __shared__ __align__(16) unsigned char smem[];
    using SM = CmSmem<T>;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned char* scr = smem + (SM::total - SM::scratch);
    int* s_incl = reinterpret_cast<int*>(scr) + wid * 32;
    int* s_off = reinterpret_cast<int*>(scr) + kCmWarps * 32 + wid * 32;
    T* s_a = reinterpret_cast<T*>(scr + (size_t)kCmWarps * 32 * 2 * sizeof(int)) + wid * 32;
    __shared__ int s_wt[32];
    __shared__ int s_total;
    __shared__ int32_t s_lo, s_hi;
    (void)lane;

    for (int64_t i = blockIdx.x; i < p.m; i += gridDim.x) {
        const int64_t P = p.flops[i];
        const int32_t mb = p.mr ? p.mr[i] : 0, me = p.mr ? p.mr[i + 1] : 0;
        if (P == 0) {
            if (!NUMERIC && threadIdx.x == 0) p.cnt[i] = 0;
            continue;
        }
        if (P <= kHashMax) {
            // ---------------------------------------------------- hash path
            int bits = 6;
            while ((1 << bits) < 2 * P) ++bits;
            const int TBL = 1 << bits;
            const uint32_t mask = TBL - 1;
            int32_t* keys = reinterpret_cast<int32_t*>(smem);
            T* vals = reinterpret_cast<T*>(smem + (size_t)(1 << kHashBitsMax) * sizeof(int32_t));
            int32_t* sk = reinterpret_cast<int32_t*>(smem + (size_t)(1 << kHashBitsMax) * (sizeof(int32_t) + sizeof(T)));
            T* sv = reinterpret_cast<T*>(reinterpret_cast<unsigned char*>(sk) + (size_t)(1 << kHashBitsMax) * sizeof(int32_t));
            for (int t = threadIdx.x; t < TBL; t += blockDim.x) {
                keys[t] = kEmpty;
                if (NUMERIC) vals[t] = (T)0;
            }
            __syncthreads();
            foreach_product<false, T>(p, i, 0, 0, s_incl, s_off, s_a, [&](int32_t c, T a, int32_t j) {
                uint32_t h = hash_col(c) >> (32 - bits);
                while (true) {
                    int32_t prev = atomicCAS(&keys[h], kEmpty, c);
                    if (prev == kEmpty || prev == c) {
                        if (NUMERIC) atomicAdd(&vals[h], a * __ldg(p.bv + j));
                        break;
                    }
                    h = (h + 1) & mask;
                }
            });
            __syncthreads();
            // survivors: present and not in the mask row; TBL <= 4096 so each
            // of the 256 threads owns at most 16 consecutive entries
            const int per = (TBL + kCmThreads - 1) / kCmThreads;
            const int t0 = threadIdx.x * per;
            int mine = 0;
            for (int u = 0; u < per; ++u) {
                int t = t0 + u;
                if (t < TBL && keys[t] != kEmpty && !in_mask(p.mc, mb, me, keys[t])) ++mine;
            }
            int pos = block_scan_int(mine, s_wt, &s_total);
            const int count = s_total;
            if (!NUMERIC) {
                if (threadIdx.x == 0) p.cnt[i] = count;
                __syncthreads();
                continue;
            }
            for (int u = 0; u < per; ++u) {
                int t = t0 + u;
                if (t < TBL && keys[t] != kEmpty && !in_mask(p.mc, mb, me, keys[t])) {
                    sk[pos] = keys[t];
                    sv[pos] = vals[t];
                    ++pos;
                }
            }
            int p2 = 1;
            while (p2 < count) p2 <<= 1;
            __syncthreads();
            for (int t = count + threadIdx.x; t < p2; t += blockDim.x) sk[t] = INT32_MAX;
            __syncthreads();
            for (int k = 2; k <= p2; k <<= 1) {
                for (int j = k >> 1; j > 0; j >>= 1) {
                    for (int t = threadIdx.x; t < p2; t += blockDim.x) {
                        int x = t ^ j;
                        if (x > t) {
                            bool up = (t & k) == 0;
                            int32_t a = sk[t], b = sk[x];
                            if ((a > b) == up) {
                                sk[t] = b; sk[x] = a;
                                T va = sv[t]; sv[t] = sv[x]; sv[x] = va;
                            }
                        }
                    }
                    __syncthreads();
                }
            }
            const int32_t o = p.cr[i];
            for (int t = threadIdx.x; t < count; t += blockDim.x) {
                p.cc[o + t] = sk[t];
                p.cv[o + t] = sv[t];
            }
            __syncthreads();
        } else {
            // ------------------------------------------- windowed dense path
            T* acc = reinterpret_cast<T*>(smem);
            uint32_t* bits = reinterpret_cast<uint32_t*>(smem + (size_t)kWin * sizeof(T));
            // column range of the products
            if (threadIdx.x == 0) { s_lo = INT32_MAX; s_hi = -1; }
            __syncthreads();
            {
                int32_t lo = INT32_MAX, hi = -1;
                for (int32_t t = p.ar[i] + threadIdx.x; t < p.ar[i + 1]; t += blockDim.x) {
                    int32_t k = p.ac[t];
                    int32_t b = p.br[k], e = p.br[k + 1];
                    if (e > b) {
                        lo = min(lo, p.bc[b]);
                        hi = max(hi, p.bc[e - 1]);
                    }
                }
                atomicMin(&s_lo, lo);
                atomicMax(&s_hi, hi);
            }
            __syncthreads();
            const int32_t lo_all = s_lo, hi_all = s_hi;
            int running = 0;
            for (int64_t w0 = lo_all; w0 <= hi_all; w0 += kWin) {
                const int32_t wlo = (int32_t)w0;
                const int32_t whi = (int32_t)((w0 + kWin - 1) < (int64_t)hi_all ? (w0 + kWin - 1) : (int64_t)hi_all);
                for (int t = threadIdx.x; t < kWin / 32; t += blockDim.x) bits[t] = 0u;
                if (NUMERIC)
                    for (int t = threadIdx.x; t < kWin; t += blockDim.x) acc[t] = (T)0;
                __syncthreads();
                foreach_product<true, T>(p, i, wlo, whi, s_incl, s_off, s_a, [&](int32_t c, T a, int32_t j) {
                    int d = c - wlo;
                    atomicOr(&bits[d >> 5], 1u << (d & 31));
                    if (NUMERIC) atomicAdd(&acc[d], a * __ldg(p.bv + j));
                });
                __syncthreads();
                // drop the mask row's columns inside the window
                if (p.mr) {
                    int n = me - mb;
                    int s = lower_bound_i32(p.mc + mb, n, wlo);
                    for (int q = s + threadIdx.x; q < n; q += blockDim.x) {
                        int32_t c = p.mc[mb + q];
                        if (c > whi) break;
                        int d = c - wlo;
                        atomicAnd(&bits[d >> 5], ~(1u << (d & 31)));
                    }
                }
                __syncthreads();
                // kWin/32 = 128 words over 256 threads: one word per thread
                uint32_t word = threadIdx.x < kWin / 32 ? bits[threadIdx.x] : 0u;
                int pos = block_scan_int(__popc(word), s_wt, &s_total);
                const int wcount = s_total;
                if (NUMERIC) {
                    const int32_t o = p.cr[i] + running + pos;
                    int r = 0;
                    while (word) {
                        int b = __ffs(word) - 1;
                        word &= word - 1;
                        int d = threadIdx.x * 32 + b;
                        p.cc[o + r] = wlo + d;
                        p.cv[o + r] = acc[d];
                        ++r;
                    }
                }
                running += wcount;
                __syncthreads();
            }
            if (!NUMERIC && threadIdx.x == 0) p.cnt[i] = running;
            __syncthreads();
        }
    }
}

template <typename T>
static ga_csr cmask_typed(ga_ctx ctx, ga_csr A, ga_csr B, const int32_t* mr, const int32_t* mc) {
    CmArgs<T> p;
    p.ar = A->rst; p.ac = A->col; p.av = static_cast<const T*>(A->val);
    p.br = B->rst; p.bc = B->col; p.bv = static_cast<const T*>(B->val);
    p.mr = mr; p.mc = mc; p.m = A->m;
    DBuf<int64_t> flops(ctx, (size_t)A->m + 1);
    DBuf<int32_t> cnt(ctx, (size_t)A->m + 1);
    p.flops = flops.p; p.cnt = cnt.p;
    {
        ProfScope ps(ctx, "cmask_flops");
        k_cm_flops<<<grid_for(A->m * 32, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(A->rst, A->col, B->rst, A->m,
                                                                                        flops.p);
        post_launch("cmask_flops");
    }
    const size_t smem = CmSmem<T>::total;
    GA_CUDA(cudaFuncSetAttribute(k_cmask<false, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    GA_CUDA(cudaFuncSetAttribute(k_cmask<true, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 1;
    GA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cmask<true, T>, kCmThreads, smem));
    if (per_sm < 1) per_sm = 1;
    const int grid = (int)std::min<int64_t>(A->m > 0 ? A->m : 1, (int64_t)ctx->num_sms * per_sm);
    if (A->m > 0) {
        ProfScope ps(ctx, "cmask_symbolic");
        k_cmask<false, T><<<grid, kCmThreads, smem, ctx->stream>>>(p);
        post_launch("cmask_symbolic");
    }
    DBuf<int32_t> rst(ctx, (size_t)A->m + 1);
    if (A->m > 0) scan_exclusive_i32(ctx, cnt.p, rst.p, A->m);
    else GA_CUDA(cudaMemsetAsync(rst.p, 0, sizeof(int32_t), ctx->stream));
    int64_t nnz = read_i32(ctx, rst.p + A->m);
    ga_csr C = csr_alloc(ctx, A->m, B->n, nnz, A->dtype);
    try {
        GA_CUDA(cudaMemcpyAsync(C->rst, rst.p, sizeof(int32_t) * (A->m + 1), cudaMemcpyDeviceToDevice, ctx->stream));
        if (nnz) {
            p.cr = C->rst; p.cc = C->col; p.cv = static_cast<T*>(C->val);
            ProfScope ps(ctx, "cmask_numeric");
            k_cmask<true, T><<<grid, kCmThreads, smem, ctx->stream>>>(p);
            post_launch("cmask_numeric");
        }
    } catch (...) {
        csr_destroy(ctx, C);
        throw;
    }
    return C;
}

ga_csr mxm_cmask(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr M) {
    GA_REQUIRE(A->n == B->m, GA_ERR_SHAPE, "cmask: A.n != B.m");
    GA_REQUIRE(!M || (M->m == A->m && M->n == B->n), GA_ERR_SHAPE, "cmask: mask shape differs from A*B");
    GA_REQUIRE(A->dtype == B->dtype, GA_ERR_DTYPE, "cmask: A and B dtypes differ");
    const int32_t* mr = M ? M->rst : nullptr;
    const int32_t* mc = M ? M->col : nullptr;
    ga_csr C = nullptr;
    switch (A->dtype) {
    case GA_INT32: C = cmask_typed<int32_t>(ctx, A, B, mr, mc); break;
    case GA_INT64: C = cmask_typed<unsigned long long>(ctx, A, B, mr, mc); break;
    case GA_FP32: C = cmask_typed<float>(ctx, A, B, mr, mc); break;
    case GA_FP64: C = cmask_typed<double>(ctx, A, B, mr, mc); break;
    case GA_UINT8: fail(GA_ERR_DTYPE, "cmask: uint8 values are not supported");
    }
    C->dtype = A->dtype;
    return C;
}

// ----------------------------------------------------------- naive variant
// C<M> = A*B by the full product followed by a gather of the mask entries
// (mxmm_naive, include/matrix_la.h:1139-1277): each mask entry binary-searches
// its column in the product row; absent entries are 0.
template <typename T>
__global__ void k_mask_gather(const int32_t* __restrict__ pr, const int32_t* __restrict__ pc,
                              const T* __restrict__ pv, const int32_t* __restrict__ mr,
                              const int32_t* __restrict__ mc, int64_t m, T* __restrict__ cv) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
        int32_t b = pr[i], n = pr[i + 1] - b;
        for (int32_t q = mr[i] + lane; q < mr[i + 1]; q += 32) {
            int32_t c = mc[q];
            int p = lower_bound_i32(pc + b, n, c);
            cv[q] = (p < n && pc[b + p] == c) ? pv[b + p] : (T)0;
        }
    }
}

void naive_masked_into(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr M, void* d_cvals) {
    GA_REQUIRE(A->dtype != GA_UINT8, GA_ERR_DTYPE, "naive: uint8 values are not supported");
    ProfScope ps(ctx, "mxm_naive");
    ga_csr P = mxm_cmask(ctx, A, B, nullptr);
    try {
        GA_DISPATCH_DTYPE(A->dtype, T, {
            k_mask_gather<T><<<grid_for(M->m * 32, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(
                P->rst, P->col, static_cast<const T*>(P->val), M->rst, M->col, M->m, static_cast<T*>(d_cvals));
        });
        post_launch("mask_gather");
    } catch (...) {
        csr_destroy(ctx, P);
        throw;
    }
    csr_destroy(ctx, P);
}

}  // namespace ga

using namespace ga;

extern "C" int ga_mxm_cmask(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr M, ga_csr* C) {
    if (!ctx || !A || !B || !M || !C) return GA_ERR_INVALID_ARG;
    *C = nullptr;
    GA_API_BODY(ctx, *C = mxm_cmask(ctx, A, B, M));
}
