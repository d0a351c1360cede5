// CSR primitives: prefix sums, type conversion, transpose, triangle
// extraction, symmetrisation, element-wise ops and the sparse x dense
// product used by the BC backward sweep.
#include "ga_device.cuh"

#include <cstring>

namespace ga {

// =================================================================== scans
// Tiles of kScanItems per block: each thread owns kScanPer consecutive items.
constexpr int kScanThreads = 512;
constexpr int kScanPer = 8;
constexpr int kScanTile = kScanThreads * kScanPer;

template <typename T>
__device__ __forceinline__ T block_excl_scan(T v, T* warp_tot, T* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        T t = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += t;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        T w = lane < nw ? warp_tot[lane] : (T)0;
        T y = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            T t = __shfl_up_sync(0xffffffffu, y, d);
            if (lane >= d) y += t;
        }
        if (lane < nw) warp_tot[lane] = y - w;
        if (lane == nw - 1) *total = y;
    }
    __syncthreads();
    T r = x - v + warp_tot[wid];
    __syncthreads();
    return r;
}

// Per-tile sums.
template <typename T>
__global__ void k_scan_reduce(const T* __restrict__ in, int64_t n, T* __restrict__ sums) {
    __shared__ T wt[32];
    __shared__ T tot;
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPer;
    T s = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; ++k)
        if (base + k < n) s += in[base + k];
    block_excl_scan<T>(s, wt, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// Scan each tile and add its offset; offs == nullptr means a single tile.
// Writes out[n] = grand total from the tile that owns index n-1.
template <typename T>
__global__ void k_scan_tiles(const T* in, T* out, int64_t n, const T* __restrict__ offs) {
    __shared__ T wt[32];
    __shared__ T tot;
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPer;
    T v[kScanPer];
    T s = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
        v[k] = (base + k < n) ? in[base + k] : (T)0;
        s += v[k];
    }
    T run = block_excl_scan<T>(s, wt, &tot);  // includes a __syncthreads after all reads
    T off = offs ? offs[blockIdx.x] : (T)0;
    run += off;
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 0 && (int64_t)(blockIdx.x + 1) * kScanTile >= n) out[n] = off + tot;
}

template <typename T>
static void scan_rec(ga_ctx ctx, const T* in, T* out, int64_t n, T* scratch) {
    if (n <= kScanTile) {
        k_scan_tiles<T><<<1, kScanThreads, 0, ctx->stream>>>(in, out, n, nullptr);
        post_launch("scan_tiles");
        return;
    }
    int64_t tiles = (n + kScanTile - 1) / kScanTile;
    T* sums = scratch;  // tiles + 1 entries, then the next level's scratch
    k_scan_reduce<T><<<(unsigned)tiles, kScanThreads, 0, ctx->stream>>>(in, n, sums);
    post_launch("scan_reduce");
    scan_rec<T>(ctx, sums, sums, tiles, scratch + tiles + 1);
    k_scan_tiles<T><<<(unsigned)tiles, kScanThreads, 0, ctx->stream>>>(in, out, n, sums);
    post_launch("scan_tiles");
}

size_t scan_scratch_bytes(int64_t n) {
    size_t items = 0;
    while (n > kScanTile) {
        int64_t tiles = (n + kScanTile - 1) / kScanTile;
        items += (size_t)tiles + 1;
        n = tiles;
    }
    return (items + 1) * sizeof(int64_t);
}

void scan_exclusive_i32(ga_ctx ctx, const int32_t* in, int32_t* out, int64_t n) {
    DBuf<char> scratch(ctx, scan_scratch_bytes(n));
    scan_rec<int32_t>(ctx, in, out, n, reinterpret_cast<int32_t*>(scratch.p));
}

void scan_exclusive_i64(ga_ctx ctx, const int64_t* in, int64_t* out, int64_t n) {
    DBuf<char> scratch(ctx, scan_scratch_bytes(n));
    scan_rec<int64_t>(ctx, in, out, n, reinterpret_cast<int64_t*>(scratch.p));
}

void scan_exclusive_i32_scratch(ga_ctx ctx, const int32_t* in, int32_t* out, int64_t n, void* scratch) {
    scan_rec<int32_t>(ctx, in, out, n, reinterpret_cast<int32_t*>(scratch));
}

// ================================================================ fill/convert
template <typename T>
__global__ void k_fill(T* __restrict__ v, int64_t n, T x) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[i] = x;
}

void fill_ones(ga_ctx ctx, void* vals, int64_t count, ga_dtype dt) {
    if (count <= 0) return;
    int grid = grid_for(count, 256, ctx->num_sms * 8);
    GA_DISPATCH_DTYPE(dt, T, {
        k_fill<T><<<grid, 256, 0, ctx->stream>>>(static_cast<T*>(vals), count, (T)1);
    });
    post_launch("fill");
}

template <typename T>
__global__ void k_any_not_one(const T* __restrict__ v, int64_t n, int* __restrict__ flag) {
    bool bad = false;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        bad |= v[i] != (T)1;
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

bool csr_unit_values(ga_ctx ctx, ga_csr A) {
    if (A->unit >= 0) return A->unit == 1;
    if (A->nnz == 0) {
        A->unit = 1;
        return true;
    }
    DBuf<int> flag(ctx, 1);
    GA_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), ctx->stream));
    GA_DISPATCH_DTYPE(A->dtype, T, {
        k_any_not_one<T><<<grid_for(A->nnz, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(
            static_cast<const T*>(A->val), A->nnz, flag.p);
    });
    post_launch("unit_check");
    A->unit = read_i32(ctx, flag.p) ? 0 : 1;
    return A->unit == 1;
}

// Pattern and values symmetric: every (i, j, v) has a (j, i, v). One warp
// per chunk of 256 consecutive entries (balanced whatever the row lengths):
// the chunk's first and last rows by binary search of the row starts, each
// entry's row by a search between them. Only the entries above the diagonal
// search their mirror (in row j); the entries below it are counted, and the
// two counts must agree, which halves the searches.
constexpr int kSymChunk = 256;

template <typename T>
__global__ void k_check_symmetric(const int32_t* __restrict__ r, const int32_t* __restrict__ c,
                                  const T* __restrict__ v, int64_t m, int64_t nnz, int* __restrict__ flag) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t ch = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ch * kSymChunk < nnz; ch += warps) {
        const int32_t q0 = (int32_t)(ch * kSymChunk);
        const int32_t q1 = (int32_t)min(nnz, (int64_t)q0 + kSymChunk);
        const int i0 = upper_bound_i32(r, (int)m + 1, q0) - 1;
        const int i1 = upper_bound_i32(r, (int)m + 1, q1 - 1) - 1;
        bool bad = false;
        int upper = 0, lower = 0;
        for (int32_t q = q0 + lane; q < q1; q += 32) {
            const int i = i0 + upper_bound_i32(r + i0 + 1, i1 - i0, q);
            const int32_t j = c[q];
            if ((int64_t)j >= m) { bad = true; continue; }
            if (j < i) {
                ++lower;
                continue;
            }
            if (j == i) continue;
            // an entry above the diagonal: its mirror must be there, with the
            // same value (searched in row j, which for a power-law graph is
            // usually the shorter row: hubs have the low indices)
            ++upper;
            const int32_t jb = r[j], jn = r[j + 1] - jb;
            const int pos = lower_bound_i32(c + jb, jn, (int32_t)i);
            if (pos >= jn || c[jb + pos] != (int32_t)i || !(v[jb + pos] == v[q])) bad = true;
        }
        if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(flag, 1);
        // every upper entry has a distinct lower mirror; equal counts then
        // give every lower entry an upper one
        upper = warp_sum<int>(upper);
        lower = warp_sum<int>(lower);
        if (lane == 0 && upper != lower) atomicAdd(flag + 1, upper - lower);
    }
}

bool csr_is_symmetric(ga_ctx ctx, ga_csr A) {
    if (A->sym >= 0) return A->sym == 1;
    if (A->m != A->n) return false;
    if (A->nnz == 0) return true;
    // flag[0]: a missing or different mirror; flag[1]: upper minus lower entries
    DBuf<int> flag(ctx, 2);
    GA_CUDA(cudaMemsetAsync(flag.p, 0, 2 * sizeof(int), ctx->stream));
    GA_DISPATCH_DTYPE(A->dtype, T, {
        k_check_symmetric<T><<<grid_for((A->nnz + kSymChunk - 1) / kSymChunk * 32, 256, ctx->num_sms * 16), 256, 0,
                               ctx->stream>>>(A->rst, A->col, static_cast<const T*>(A->val), A->m, A->nnz, flag.p);
    });
    post_launch("check_symmetric");
    int h[2];
    GA_CUDA(cudaMemcpyAsync(h, flag.p, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    GA_CUDA(cudaStreamSynchronize(ctx->stream));
    A->sym = h[0] == 0 && h[1] == 0 ? 1 : 0;
    return A->sym == 1;
}

template <typename S, typename D>
__global__ void k_convert(const S* __restrict__ s, D* __restrict__ d, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        d[i] = (D)s[i];
}

ga_csr copy_csr(ga_ctx ctx, ga_csr A, ga_dtype to) {
    ga_csr C = csr_alloc(ctx, A->m, A->n, A->nnz, to);
    try {
        GA_CUDA(cudaMemcpyAsync(C->rst, A->rst, sizeof(int32_t) * (A->m + 1), cudaMemcpyDeviceToDevice,
                                ctx->stream));
        if (A->nnz) {
            GA_CUDA(cudaMemcpyAsync(C->col, A->col, sizeof(int32_t) * A->nnz, cudaMemcpyDeviceToDevice,
                                    ctx->stream));
            if (to == A->dtype) {
                GA_CUDA(cudaMemcpyAsync(C->val, A->val, dtype_size(to) * A->nnz, cudaMemcpyDeviceToDevice,
                                        ctx->stream));
            } else {
                int grid = grid_for(A->nnz, 256, ctx->num_sms * 8);
                GA_DISPATCH_DTYPE(A->dtype, S, {
                    GA_DISPATCH_DTYPE(to, D, {
                        k_convert<S, D><<<grid, 256, 0, ctx->stream>>>(static_cast<const S*>(A->val),
                                                                       static_cast<D*>(C->val), A->nnz);
                    });
                });
                post_launch("convert");
            }
        }
    } catch (...) {
        csr_destroy(ctx, C);
        throw;
    }
    return C;
}

// ================================================================ transpose
__global__ void k_count_cols(const int32_t* __restrict__ col, int64_t nnz, int32_t* __restrict__ cnt) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&cnt[col[q]], 1);
}

// Scatter: entry (i, j) goes to AT row j at an atomically reserved position;
// the row index is recorded with the source entry index for the sort.
__global__ void k_transpose_scatter(const int32_t* __restrict__ rst, const int32_t* __restrict__ col, int64_t m,
                                    int32_t* __restrict__ cursor, int32_t* __restrict__ trow,
                                    int32_t* __restrict__ tsrc) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
        for (int32_t q = rst[i] + lane; q < rst[i + 1]; q += 32) {
            int32_t p = atomicAdd(&cursor[col[q]], 1);
            trow[p] = (int32_t)i;
            tsrc[p] = q;
        }
    }
}

// Sort every row segment by key with a block-wide bitonic sort in shared
// memory; the payload follows its key. Rows longer than kSortCap are listed
// in long_rows (count in *nlong) for k_sort_long_rows.
constexpr int kSortCap = 8192;

// Block-wide bitonic sort of len <= kSortCap (key, payload) pairs at gk/gp,
// staged in sk/sp (shared, kSortCap entries each). All threads call it.
__device__ void block_sort_pairs(int32_t* gk, int32_t* gp, int len, int32_t* sk, int32_t* sp) {
    int p2 = 1;
    while (p2 < len) p2 <<= 1;
    for (int t = threadIdx.x; t < p2; t += blockDim.x) {
        if (t < len) { sk[t] = gk[t]; sp[t] = gp[t]; }
        else { sk[t] = INT32_MAX; sp[t] = 0; }
    }
    __syncthreads();
    for (int k = 2; k <= p2; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int t = threadIdx.x; t < p2; t += blockDim.x) {
                int x = t ^ j;
                if (x > t) {
                    bool up = (t & k) == 0;
                    int32_t a = sk[t], c = sk[x];
                    if ((a > c) == up) {
                        sk[t] = c; sk[x] = a;
                        int32_t pa = sp[t]; sp[t] = sp[x]; sp[x] = pa;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int t = threadIdx.x; t < len; t += blockDim.x) { gk[t] = sk[t]; gp[t] = sp[t]; }
    __syncthreads();
}

// Warp-wide bitonic sort of up to 32*K (key, payload) pairs held in
// registers, element e = r*32 + lane in register r of lane `lane` (a striped
// layout: loads and stores are coalesced). Pairs at distance j < 32 meet
// across lanes by shuffles, pairs at distance j >= 32 inside one thread.
// Padding elements hold INT32_MAX.
template <int K>
__device__ __forceinline__ void warp_bitonic(int32_t (&k)[K], int32_t (&v)[K]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int w = 2; w <= 32 * K; w <<= 1) {
#pragma unroll
        for (int j = w >> 1; j > 0; j >>= 1) {
            if (j >= 32) {
#pragma unroll
                for (int r = 0; r < K; ++r) {
                    const int r2 = r ^ (j >> 5);
                    if (r2 > r) {
                        const bool up = ((r * 32 + lane) & w) == 0;
                        if (up ? k[r] > k[r2] : k[r] < k[r2]) {
                            const int32_t tk = k[r]; k[r] = k[r2]; k[r2] = tk;
                            const int32_t tv = v[r]; v[r] = v[r2]; v[r2] = tv;
                        }
                    }
                }
            } else {
#pragma unroll
                for (int r = 0; r < K; ++r) {
                    const int32_t ok = __shfl_xor_sync(0xffffffffu, k[r], j);
                    const int32_t ov = __shfl_xor_sync(0xffffffffu, v[r], j);
                    const bool up = ((r * 32 + lane) & w) == 0, low = (lane & j) == 0;
                    // the lower element of an ascending pair keeps the smaller key
                    if (low == up ? ok < k[r] : ok > k[r]) {
                        k[r] = ok;
                        v[r] = ov;
                    }
                }
            }
        }
    }
}

template <int K>
__device__ __forceinline__ void warp_sort_row(int32_t* key, int32_t* pay, int len) {
    const int lane = threadIdx.x & 31;
    int32_t k[K], v[K];
#pragma unroll
    for (int r = 0; r < K; ++r) {
        const int e = r * 32 + lane;
        k[r] = e < len ? key[e] : INT32_MAX;
        v[r] = e < len ? pay[e] : 0;
    }
    warp_bitonic<K>(k, v);
#pragma unroll
    for (int r = 0; r < K; ++r) {
        const int e = r * 32 + lane;
        if (e < len) {
            key[e] = k[r];
            pay[e] = v[r];
        }
    }
}

// Rows of at most 256 entries: one warp each, in registers. Longer rows are
// listed for a CTA: up to kSortCap entries in `mid_rows` (k_sort_mid_rows),
// beyond that in `long_rows` (k_sort_long_rows).
__global__ void k_sort_rows(const int32_t* __restrict__ rst, int64_t m, int32_t* __restrict__ key,
                            int32_t* __restrict__ pay, int32_t* __restrict__ mid_rows, int* __restrict__ nmid,
                            int32_t* __restrict__ long_rows, int* __restrict__ nlong) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
        const int32_t b = rst[i], len = rst[i + 1] - b;
        if (len <= 1) continue;
        if (len <= 32) warp_sort_row<1>(key + b, pay + b, len);
        else if (len <= 64) warp_sort_row<2>(key + b, pay + b, len);
        else if (len <= 256) warp_sort_row<8>(key + b, pay + b, len);
        else if (lane == 0) {
            if (len > kSortCap) {
                long_rows[atomicAdd(nlong, 1)] = (int32_t)i;
                atomicMax(nlong + 1, len);
            } else {
                mid_rows[atomicAdd(nmid, 1)] = (int32_t)i;
            }
        }
    }
}

__global__ void k_sort_mid_rows(const int32_t* __restrict__ rst, const int32_t* __restrict__ rows,
                                const int* __restrict__ nrows, int32_t* __restrict__ key,
                                int32_t* __restrict__ pay) {
    extern __shared__ int32_t sm[];
    const int n = *nrows;
    for (int r = blockIdx.x; r < n; r += gridDim.x) {
        const int32_t i = rows[r];
        const int32_t b = rst[i];
        block_sort_pairs(key + b, pay + b, rst[i + 1] - b, sm, sm + kSortCap);
    }
}

// First i (A entries among the first d outputs) of the stable merge of
// sorted A[0, na) and B[0, nb): ties take A first.
__device__ __forceinline__ int32_t merge_split(const int32_t* A, int32_t na, const int32_t* B, int32_t nb,
                                               int32_t d) {
    int32_t lo = d > nb ? d - nb : 0, hi = d < na ? d : na;
    while (lo < hi) {
        const int32_t mid = (lo + hi) >> 1;
        if (A[mid] <= B[d - 1 - mid]) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Long rows, first step: CTA (r, c) sorts piece c (kSortCap entries) of
// listed row r in shared memory; pieces past the row's end exit.
__global__ void __launch_bounds__(512) k_sort_long_pieces(const int32_t* __restrict__ rst,
                                                          const int32_t* __restrict__ rows, int32_t* key,
                                                          int32_t* pay) {
    extern __shared__ int32_t sm[];
    const int32_t i = rows[blockIdx.x];
    const int32_t b = rst[i], L = rst[i + 1] - b;
    const int32_t c0 = (int32_t)blockIdx.y * kSortCap;
    if (c0 >= L) return;
    block_sort_pairs(key + b + c0, pay + b + c0, min(kSortCap, L - c0), sm, sm + kSortCap);
}

// Long rows, second step, one CTA per row: pairs of sorted runs merged
// (merge path: each thread finds its split of the output by a binary search
// and merges its share) between the row's place in key/pay and the same
// place in tkey/tpay, doubling the run length each pass.
__global__ void __launch_bounds__(512) k_sort_long_rows(const int32_t* __restrict__ rst,
                                                        const int32_t* __restrict__ rows, int32_t* key,
                                                        int32_t* pay, int32_t* tkey, int32_t* tpay) {
    const int32_t i = rows[blockIdx.x];
    const int32_t b = rst[i], L = rst[i + 1] - b;
    int32_t* k0 = key + b;
    int32_t* p0 = pay + b;
    int32_t* k1 = tkey + b;
    int32_t* p1 = tpay + b;
    for (int64_t w = kSortCap; w < L; w <<= 1) {
        for (int64_t s0 = 0; s0 < L; s0 += 2 * w) {
            const int32_t na = (int32_t)min(w, (int64_t)L - s0);
            const int32_t nb = (int32_t)min(w, (int64_t)L - s0 - na);
            const int32_t total = na + nb;
            const int32_t* A = k0 + s0;
            const int32_t* Ap = p0 + s0;
            const int32_t* B = A + na;
            const int32_t* Bp = Ap + na;
            const int32_t per = (total + (int32_t)blockDim.x - 1) / (int32_t)blockDim.x;
            const int32_t d0 = min(total, (int32_t)threadIdx.x * per), d1 = min(total, d0 + per);
            if (d0 >= d1) continue;
            int32_t ia = merge_split(A, na, B, nb, d0), ib = d0 - ia;
            for (int32_t o = d0; o < d1; ++o) {
                const bool take_a = ib >= nb || (ia < na && A[ia] <= B[ib]);
                k1[s0 + o] = take_a ? A[ia] : B[ib];
                p1[s0 + o] = take_a ? Ap[ia] : Bp[ib];
                if (take_a) ++ia; else ++ib;
            }
        }
        __syncthreads();
        int32_t* t = k0; k0 = k1; k1 = t;
        t = p0; p0 = p1; p1 = t;
    }
    if (k0 != key + b)
        for (int32_t t = threadIdx.x; t < L; t += blockDim.x) {
            key[b + t] = k0[t];
            pay[b + t] = p0[t];
        }
}

void sort_rows_by_key(ga_ctx ctx, const int32_t* rst, int64_t m, int32_t* key, int32_t* pay, int64_t nnz) {
    if (m <= 0 || nnz <= 1) return;
    ProfScope ps(ctx, "sort_rows");
    DBuf<int> counts(ctx, 3);  // medium rows, long rows, longest long row
    DBuf<int32_t> mid_rows(ctx, (size_t)m + 1), long_rows(ctx, (size_t)m + 1);
    GA_CUDA(cudaMemsetAsync(counts.p, 0, 3 * sizeof(int), ctx->stream));
    k_sort_rows<<<grid_for(m * 32, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(
        rst, m, key, pay, mid_rows.p, counts.p, long_rows.p, counts.p + 1);
    post_launch("sort_rows");
    const size_t smem = 2 * kSortCap * sizeof(int32_t);
    GA_CUDA(cudaFuncSetAttribute(k_sort_mid_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // 64 KB of shared memory per CTA: three CTAs per SM
    k_sort_mid_rows<<<ctx->num_sms * 3, 512, smem, ctx->stream>>>(rst, mid_rows.p, counts.p, key, pay);
    post_launch("sort_mid_rows");
    int h[3];
    GA_CUDA(cudaMemcpyAsync(h, counts.p, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
    GA_CUDA(cudaStreamSynchronize(ctx->stream));
    if (h[1] == 0) return;
    DBuf<int32_t> tkey(ctx, (size_t)nnz), tpay(ctx, (size_t)nnz);
    GA_CUDA(cudaFuncSetAttribute(k_sort_long_pieces, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    GA_REQUIRE((h[2] + kSortCap - 1) / kSortCap <= 65535, GA_ERR_INVALID_ARG, "sort: a row of over 536M entries");
    const dim3 pieces((unsigned)h[1], (unsigned)((h[2] + kSortCap - 1) / kSortCap));
    k_sort_long_pieces<<<pieces, 512, smem, ctx->stream>>>(rst, long_rows.p, key, pay);
    post_launch("sort_long_pieces");
    k_sort_long_rows<<<h[1], 512, 0, ctx->stream>>>(rst, long_rows.p, key, pay, tkey.p, tpay.p);
    post_launch("sort_long_rows");
    GA_CUDA(cudaStreamSynchronize(ctx->stream));
}

template <typename T>
__global__ void k_gather_vals(const int32_t* __restrict__ src, const T* __restrict__ v, T* __restrict__ out,
                              int64_t n) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        out[q] = v[src[q]];
}

ga_csr transpose_csr(ga_ctx ctx, ga_csr A) {
    ProfScope ps(ctx, "transpose");
    ga_csr T = csr_alloc(ctx, A->n, A->m, A->nnz, A->dtype);
    try {
        DBuf<int32_t> cnt(ctx, (size_t)A->n + 1);
        GA_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * (A->n + 1), ctx->stream));
        if (A->nnz) {
            k_count_cols<<<grid_for(A->nnz, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(A->col, A->nnz, cnt.p);
            post_launch("transpose_count");
        }
        scan_exclusive_i32(ctx, cnt.p, T->rst, A->n);
        if (A->nnz) {
            DBuf<int32_t> cursor(ctx, (size_t)A->n + 1);
            DBuf<int32_t> src(ctx, (size_t)A->nnz);
            GA_CUDA(cudaMemcpyAsync(cursor.p, T->rst, sizeof(int32_t) * (A->n + 1), cudaMemcpyDeviceToDevice,
                                    ctx->stream));
            k_transpose_scatter<<<grid_for(A->m * 32, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(
                A->rst, A->col, A->m, cursor.p, T->col, src.p);
            post_launch("transpose_scatter");
            sort_rows_by_key(ctx, T->rst, T->m, T->col, src.p, A->nnz);
            GA_DISPATCH_DTYPE(A->dtype, V, {
                k_gather_vals<V><<<grid_for(A->nnz, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(
                    src.p, static_cast<const V*>(A->val), static_cast<V*>(T->val), A->nnz);
            });
            post_launch("transpose_gather");
        }
    } catch (...) {
        csr_destroy(ctx, T);
        throw;
    }
    return T;
}

// ======================================================== triangle extraction
// Per row, the number of leading entries with col < i (lower) or trailing
// entries with col > i (upper); rows are sorted.
__global__ void k_tri_count(const int32_t* __restrict__ rst, const int32_t* __restrict__ col, int64_t m,
                            bool lower, int32_t* __restrict__ cnt, int32_t* __restrict__ first) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t b = rst[i], e = rst[i + 1];
        // first position with col >= i (lower) / col > i (upper)
        int32_t lo = b, hi = e;
        while (lo < hi) {
            int32_t mid = (lo + hi) >> 1;
            bool go_right = lower ? (col[mid] < (int32_t)i) : (col[mid] <= (int32_t)i);
            if (go_right) lo = mid + 1; else hi = mid;
        }
        if (lower) { cnt[i] = lo - b; first[i] = b; }
        else { cnt[i] = e - lo; first[i] = lo; }
    }
}

template <typename T>
__global__ void k_tri_copy(const int32_t* __restrict__ first, const int32_t* __restrict__ orst,
                           const int32_t* __restrict__ col, const T* __restrict__ val, int64_t m,
                           int32_t* __restrict__ ocol, T* __restrict__ oval) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
        int32_t s = first[i], o = orst[i], len = orst[i + 1] - orst[i];
        for (int32_t t = lane; t < len; t += 32) {
            ocol[o + t] = col[s + t];
            oval[o + t] = val[s + t];
        }
    }
}

ga_csr extract_tri(ga_ctx ctx, ga_csr A, bool lower) {
    ProfScope ps(ctx, lower ? "extract_lower" : "extract_upper");
    DBuf<int32_t> cnt(ctx, (size_t)A->m + 1), first(ctx, (size_t)A->m + 1), rst(ctx, (size_t)A->m + 1);
    k_tri_count<<<grid_for(A->m, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(A->rst, A->col, A->m, lower, cnt.p,
                                                                               first.p);
    post_launch("tri_count");
    scan_exclusive_i32(ctx, cnt.p, rst.p, A->m);
    int64_t nnz = read_i32(ctx, rst.p + A->m);
    ga_csr L = csr_alloc(ctx, A->m, A->n, nnz, A->dtype);
    try {
        GA_CUDA(cudaMemcpyAsync(L->rst, rst.p, sizeof(int32_t) * (A->m + 1), cudaMemcpyDeviceToDevice, ctx->stream));
        if (nnz) {
            GA_DISPATCH_DTYPE(A->dtype, T, {
                k_tri_copy<T><<<grid_for(A->m * 32, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(
                    first.p, rst.p, A->col, static_cast<const T*>(A->val), A->m, L->col, static_cast<T*>(L->val));
            });
            post_launch("tri_copy");
        }
    } catch (...) {
        csr_destroy(ctx, L);
        throw;
    }
    return L;
}

// ================================================== merge of two sorted rows
// C row i = merge of X row i and Y row i by column; on equal columns Y's entry
// comes first (the tie rule of build_symm_from_lower and add_nointersect,
// include/matrix.h:713-720, include/matrix_la.h:351-357). Every element finds
// its output position by a binary search in the other row.
template <typename T>
__global__ void k_merge_rows(const int32_t* __restrict__ xr, const int32_t* __restrict__ xc,
                             const T* __restrict__ xv, const int32_t* __restrict__ yr,
                             const int32_t* __restrict__ yc, const T* __restrict__ yv, int64_t m,
                             const int32_t* __restrict__ cr, int32_t* __restrict__ cc, T* __restrict__ cv) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
        int32_t xb = xr[i], xn = xr[i + 1] - xb;
        int32_t yb = yr[i], yn = yr[i + 1] - yb;
        int32_t o = cr[i];
        for (int32_t t = lane; t < xn; t += 32) {
            int32_t c = xc[xb + t];
            int p = upper_bound_i32(yc + yb, yn, c);
            cc[o + t + p] = c;
            cv[o + t + p] = xv[xb + t];
        }
        for (int32_t t = lane; t < yn; t += 32) {
            int32_t c = yc[yb + t];
            int p = lower_bound_i32(xc + xb, xn, c);
            cc[o + t + p] = c;
            cv[o + t + p] = yv[yb + t];
        }
    }
}

__global__ void k_add_rst(const int32_t* __restrict__ a, const int32_t* __restrict__ b, int64_t m,
                          int32_t* __restrict__ c) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= m; i += (int64_t)gridDim.x * blockDim.x)
        c[i] = a[i] + b[i];
}

static ga_csr merge_csr(ga_ctx ctx, ga_csr X, ga_csr Y) {
    ga_csr C = csr_alloc(ctx, X->m, X->n, X->nnz + Y->nnz, X->dtype);
    try {
        k_add_rst<<<grid_for(X->m + 1, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(X->rst, Y->rst, X->m, C->rst);
        post_launch("add_rst");
        if (C->nnz) {
            GA_DISPATCH_DTYPE(X->dtype, T, {
                k_merge_rows<T><<<grid_for(X->m * 32, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(
                    X->rst, X->col, static_cast<const T*>(X->val), Y->rst, Y->col, static_cast<const T*>(Y->val),
                    X->m, C->rst, C->col, static_cast<T*>(C->val));
            });
            post_launch("merge_rows");
        }
    } catch (...) {
        csr_destroy(ctx, C);
        throw;
    }
    return C;
}

// ================================================================ dense ops
template <typename T>
__global__ void k_scatter_dense(const int32_t* __restrict__ rst, const int32_t* __restrict__ col,
                                const T* __restrict__ val, int64_t m, int64_t n, T* __restrict__ D) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps)
        for (int32_t q = rst[i] + lane; q < rst[i + 1]; q += 32) D[(size_t)n * i + col[q]] = val[q];
}

// C<M> = A .* B (dense), zero elsewhere: one warp per row writes the zeros,
// then the mask entries.
template <typename T>
__global__ void k_ewise_mult_masked(const T* __restrict__ A, const T* __restrict__ B, const int32_t* __restrict__ mr,
                                    const int32_t* __restrict__ mc, int64_t m, int64_t n, T* __restrict__ C) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
        T* crow = C + (size_t)n * i;
        for (int64_t c = lane; c < n; c += 32) crow[c] = (T)0;
        __syncwarp();
        for (int32_t q = mr[i] + lane; q < mr[i + 1]; q += 32) {
            size_t idx = (size_t)n * i + mc[q];
            C[idx] = mul_add_separate<T>((T)0, A[idx], B[idx]);
        }
        __syncwarp();
    }
}

template <typename T>
__global__ void k_fuse_mult_add(const T* __restrict__ A, const T* __restrict__ B, T* __restrict__ C, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        C[i] = mul_add_separate<T>(C[i], A[i], B[i]);
}

// C<M> = A * B with dense B, C (n columns). One warp per row; each lane owns
// mask columns and accumulates over A's row in order, the summation order of
// mxmm_spd (include/matrix_la.h:260-267), so results match it bit for bit.
template <typename T>
__global__ void k_spd(const int32_t* __restrict__ ar, const int32_t* __restrict__ ac, const T* __restrict__ av,
                      const T* __restrict__ B, const int32_t* __restrict__ mr, const int32_t* __restrict__ mc,
                      int64_t m, int64_t n, T* __restrict__ C) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
        T* crow = C + (size_t)n * i;
        for (int64_t c = lane; c < n; c += 32) crow[c] = (T)0;
        __syncwarp();
        int32_t mb = mr[i], me = mr[i + 1];
        int32_t ab = ar[i], ae = ar[i + 1];
        for (int32_t q0 = mb; q0 < me; q0 += 32) {
            int32_t q = q0 + lane;
            if (q < me) {
                int32_t c = mc[q];
                T acc = (T)0;
                for (int32_t t = ab; t < ae; ++t) acc = mul_add_separate<T>(acc, av[t], B[(size_t)n * ac[t] + c]);
                crow[c] = acc;
            }
        }
        __syncwarp();
    }
}

}  // namespace ga

using namespace ga;

extern "C" {

int ga_transpose(ga_ctx ctx, ga_csr A, ga_csr* AT) {
    if (!ctx || !A || !AT) return GA_ERR_INVALID_ARG;
    *AT = nullptr;
    GA_API_BODY(ctx, *AT = transpose_csr(ctx, A));
}

int ga_extract_lower(ga_ctx ctx, ga_csr A, ga_csr* L) {
    if (!ctx || !A || !L) return GA_ERR_INVALID_ARG;
    *L = nullptr;
    GA_API_BODY(ctx, *L = extract_tri(ctx, A, true));
}

int ga_extract_upper(ga_ctx ctx, ga_csr A, ga_csr* U) {
    if (!ctx || !A || !U) return GA_ERR_INVALID_ARG;
    *U = nullptr;
    GA_API_BODY(ctx, *U = extract_tri(ctx, A, false));
}

int ga_symm_from_lower(ga_ctx ctx, ga_csr L, ga_csr* S) {
    if (!ctx || !L || !S) return GA_ERR_INVALID_ARG;
    *S = nullptr;
    GA_API_BODY(ctx, {
        GA_REQUIRE(L->m == L->n, GA_ERR_SHAPE, "build_symm_from_lower needs a square matrix");
        ProfScope ps(ctx, "symm_from_lower");
        ga_csr U = transpose_csr(ctx, L);
        try {
            *S = merge_csr(ctx, L, U);
        } catch (...) {
            csr_destroy(ctx, U);
            throw;
        }
        csr_destroy(ctx, U);
    });
}

int ga_adjacency(ga_ctx ctx, ga_csr A, ga_csr* adj) {
    if (!ctx || !A || !adj) return GA_ERR_INVALID_ARG;
    *adj = nullptr;
    GA_API_BODY(ctx, {
        ga_csr C = csr_alloc(ctx, A->m, A->n, A->nnz, GA_INT32);
        try {
            GA_CUDA(cudaMemcpyAsync(C->rst, A->rst, sizeof(int32_t) * (A->m + 1), cudaMemcpyDeviceToDevice,
                                    ctx->stream));
            if (A->nnz)
                GA_CUDA(cudaMemcpyAsync(C->col, A->col, sizeof(int32_t) * A->nnz, cudaMemcpyDeviceToDevice,
                                        ctx->stream));
            fill_ones(ctx, C->val, A->nnz, GA_INT32);
            C->unit = 1;
        } catch (...) {
            csr_destroy(ctx, C);
            throw;
        }
        *adj = C;
    });
}

int ga_add_nointersect(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr* C) {
    if (!ctx || !A || !B || !C) return GA_ERR_INVALID_ARG;
    *C = nullptr;
    GA_API_BODY(ctx, {
        GA_REQUIRE(A->m == B->m && A->n == B->n, GA_ERR_SHAPE, "add_nointersect: shapes differ");
        GA_REQUIRE(A->dtype == B->dtype, GA_ERR_DTYPE, "add_nointersect: dtypes differ");
        ProfScope ps(ctx, "add_nointersect");
        *C = merge_csr(ctx, A, B);
    });
}

int ga_dense_from_csr(ga_ctx ctx, ga_csr A, ga_dense* out) {
    if (!ctx || !A || !out) return GA_ERR_INVALID_ARG;
    *out = nullptr;
    GA_API_BODY(ctx, {
        ga_dense D = new ga_dense_s;
        D->m = A->m; D->n = A->n; D->dtype = A->dtype;
        size_t bytes = (size_t)A->m * A->n * dtype_size(A->dtype);
        try {
            D->val = dalloc(ctx, bytes);
            GA_CUDA(cudaMemsetAsync(D->val, 0, bytes, ctx->stream));
            GA_DISPATCH_DTYPE(A->dtype, T, {
                k_scatter_dense<T><<<grid_for(A->m * 32, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(
                    A->rst, A->col, static_cast<const T*>(A->val), A->m, A->n, static_cast<T*>(D->val));
            });
            post_launch("scatter_dense");
        } catch (...) {
            dfree(ctx, D->val);
            delete D;
            throw;
        }
        *out = D;
    });
}

int ga_ewise_mult_masked(ga_ctx ctx, ga_dense A, ga_dense B, ga_csr M, ga_dense C) {
    if (!ctx || !A || !B || !M || !C) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        GA_REQUIRE(A->m == B->m && A->n == B->n && C->m == A->m && C->n == A->n && M->m == A->m && M->n <= A->n,
                   GA_ERR_SHAPE, "eWiseMult: shapes differ");
        GA_REQUIRE(A->dtype == B->dtype && A->dtype == C->dtype, GA_ERR_DTYPE, "eWiseMult: dtypes differ");
        ProfScope ps(ctx, "ewise_mult_masked");
        GA_DISPATCH_DTYPE(A->dtype, T, {
            k_ewise_mult_masked<T><<<grid_for(A->m * 32, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(
                static_cast<const T*>(A->val), static_cast<const T*>(B->val), M->rst, M->col, A->m, A->n,
                static_cast<T*>(C->val));
        });
        post_launch("ewise_mult_masked");
    });
}

int ga_fuse_ewise_mult_add(ga_ctx ctx, ga_dense A, ga_dense B, ga_dense C) {
    if (!ctx || !A || !B || !C) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        GA_REQUIRE(A->m == B->m && A->n == B->n && C->m == A->m && C->n == A->n, GA_ERR_SHAPE,
                   "fuseEWiseMultAdd: shapes differ");
        GA_REQUIRE(A->dtype == B->dtype && A->dtype == C->dtype, GA_ERR_DTYPE, "fuseEWiseMultAdd: dtypes differ");
        ProfScope ps(ctx, "fuse_ewise_mult_add");
        int64_t n = A->m * A->n;
        GA_DISPATCH_DTYPE(A->dtype, T, {
            k_fuse_mult_add<T><<<grid_for(n, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(
                static_cast<const T*>(A->val), static_cast<const T*>(B->val), static_cast<T*>(C->val), n);
        });
        post_launch("fuse_mult_add");
    });
}

int ga_mxm_spd(ga_ctx ctx, ga_csr A, ga_dense B, ga_csr M, ga_dense C) {
    if (!ctx || !A || !B || !M || !C) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        GA_REQUIRE(B != C && B->val != C->val, GA_ERR_INVALID_ARG, "mxmm_spd: C may not alias B");
        GA_REQUIRE(A->n == B->m && M->m == A->m && C->m == A->m && C->n == B->n && M->n <= B->n, GA_ERR_SHAPE,
                   "mxmm_spd: shapes differ");
        GA_REQUIRE(A->dtype == B->dtype && B->dtype == C->dtype, GA_ERR_DTYPE, "mxmm_spd: dtypes differ");
        ProfScope ps(ctx, "spd");
        GA_DISPATCH_DTYPE(A->dtype, T, {
            k_spd<T><<<grid_for(A->m * 32, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(
                A->rst, A->col, static_cast<const T*>(A->val), static_cast<const T*>(B->val), M->rst, M->col, A->m,
                B->n, static_cast<T*>(C->val));
        });
        post_launch("spd");
    });
}

}  // extern "C"
