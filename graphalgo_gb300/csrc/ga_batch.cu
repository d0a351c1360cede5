// Batched execution: many independent graphs processed as one block-diagonal
// union, so a single launch of each kernel (and one captured k-truss loop)
// covers the whole batch. The masked-SpGEMM work queue then holds the row
// bins of every graph; per-graph results are recovered by segmented
// reductions over the graphs' row ranges.
//
// Also a seeded device generator of Gaussian k-nearest-neighbour graphs for
// whole batches (the batched workload's inputs).
#include "ga_device.cuh"

#include <vector>

namespace ga {

struct PartDesc {
    const int32_t* rst;
    const int32_t* col;
    const void* val;
    int32_t roff, coff, eoff, m, nnz;
};

template <typename T>
__global__ void k_block_diag(const PartDesc* __restrict__ parts, int64_t count, int32_t* __restrict__ rst,
                             int32_t* __restrict__ col, T* __restrict__ val) {
    for (int64_t g = blockIdx.x; g < count; g += gridDim.x) {
        const PartDesc d = parts[g];
        for (int32_t i = threadIdx.x; i < d.m; i += blockDim.x) rst[d.roff + i] = d.rst[i] + d.eoff;
        const T* v = static_cast<const T*>(d.val);
        for (int32_t q = threadIdx.x; q < d.nnz; q += blockDim.x) {
            col[d.eoff + q] = d.col[q] + d.coff;
            val[d.eoff + q] = v[q];
        }
    }
}

static ga_csr block_diag(ga_ctx ctx, int64_t count, const ga_csr* parts, int64_t* voff) {
    GA_REQUIRE(count >= 0, GA_ERR_INVALID_ARG, "block_diag: negative count");
    std::vector<PartDesc> desc((size_t)count);
    int64_t rows = 0, cols = 0, ents = 0;
    ga_dtype dt = count ? parts[0]->dtype : GA_INT32;
    bool unit = true, sym = true;
    for (int64_t g = 0; g < count; ++g) {
        const ga_csr P = parts[g];
        GA_REQUIRE(P != nullptr, GA_ERR_INVALID_ARG, "block_diag: NULL part");
        GA_REQUIRE(P->dtype == dt, GA_ERR_DTYPE, "block_diag: parts have different dtypes");
        GA_REQUIRE(rows + P->m < INT32_MAX && cols + P->n <= INT32_MAX && ents + P->nnz <= INT32_MAX,
                   GA_ERR_INVALID_ARG, "block_diag: the union exceeds the int32 index range");
        desc[(size_t)g] = PartDesc{P->rst, P->col, P->val, (int32_t)rows, (int32_t)cols, (int32_t)ents,
                                   (int32_t)P->m, (int32_t)P->nnz};
        if (voff) voff[g] = rows;
        unit = unit && P->unit == 1;
        sym = sym && P->sym == 1;
        rows += P->m;
        cols += P->n;
        ents += P->nnz;
    }
    if (voff) voff[count] = rows;
    ga_csr U = csr_alloc(ctx, rows, cols, ents, dt);
    try {
        if (count > 0) {
            DBuf<PartDesc> d(ctx, (size_t)count);
            GA_CUDA(cudaMemcpyAsync(d.p, desc.data(), sizeof(PartDesc) * count, cudaMemcpyHostToDevice, ctx->stream));
            GA_DISPATCH_DTYPE(dt, T, {
                k_block_diag<T><<<(unsigned)std::min<int64_t>(count, 65535), 256, 0, ctx->stream>>>(
                    d.p, count, U->rst, U->col, static_cast<T*>(U->val));
            });
            post_launch("block_diag");
            // synchronise before the host descriptor array goes away
            GA_CUDA(cudaStreamSynchronize(ctx->stream));
        }
        const int32_t last = (int32_t)ents;
        GA_CUDA(cudaMemcpyAsync(U->rst + rows, &last, sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
    } catch (...) {
        csr_destroy(ctx, U);
        throw;
    }
    U->unit = unit ? 1 : -1;
    U->sym = sym ? 1 : -1;  // known-symmetric blocks make a symmetric union
    return U;
}

// ------------------------------------------------------- k-NN batch generator
constexpr int kKnnThreads = 128;
constexpr int kKnnMaxN = 4096;
constexpr int kKnnMaxDim = 32;

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ double unit_uniform(uint64_t seed, uint64_t a, uint64_t b) {
    const uint64_t h = mix64(seed ^ mix64(a * 0x9E3779B97F4A7C15ull + b + 0x632BE59BD9B4E019ull));
    return ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);  // (0, 1)
}

// One thread per point: i.i.d. N(0,1) coordinates by Box-Muller over a
// counter-based hash of (seed, graph, point, coordinate pair).
__global__ void k_knn_points(const int32_t* __restrict__ voff, const int32_t* __restrict__ dim,
                             const int64_t* __restrict__ poff, int64_t ngraphs, int64_t npoints, uint64_t seed,
                             float* __restrict__ X) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < npoints; p += (int64_t)gridDim.x * blockDim.x) {
        const int g = upper_bound_i32(voff, (int)ngraphs + 1, (int32_t)p) - 1;
        const int64_t local = p - voff[g];
        const int d = dim[g];
        float* x = X + poff[g] + local * d;
        for (int c = 0; c < d; c += 2) {
            const double u1 = unit_uniform(seed, ((uint64_t)g << 32) | (uint64_t)local, (uint64_t)c);
            const double u2 = unit_uniform(seed ^ 0x5851F42D4C957F2Dull, ((uint64_t)g << 32) | (uint64_t)local,
                                           (uint64_t)c);
            const double r = sqrt(-2.0 * log(u1));
            x[c] = (float)(r * cos(6.283185307179586 * u2));
            if (c + 1 < d) x[c + 1] = (float)(r * sin(6.283185307179586 * u2));
        }
    }
}

// One CTA per point: squared distances to every point of its graph in shared
// memory, then k rounds of a block argmin (ties to the smaller index).
__global__ void __launch_bounds__(kKnnThreads) k_knn_select(const int32_t* __restrict__ voff,
                                                            const int32_t* __restrict__ dim,
                                                            const int64_t* __restrict__ poff, int64_t ngraphs,
                                                            const float* __restrict__ X, int k,
                                                            int32_t* __restrict__ nb) {
    __shared__ float dist[kKnnMaxN];
    __shared__ float me[kKnnMaxDim];
    __shared__ unsigned long long wmin[kKnnThreads / 32];
    const int64_t p = blockIdx.x;
    const int g = upper_bound_i32(voff, (int)ngraphs + 1, (int32_t)p) - 1;
    const int32_t base = voff[g];
    const int n = voff[g + 1] - base, d = dim[g];
    const int local = (int)(p - base);
    const float* Xg = X + poff[g];
    if (threadIdx.x < d) me[threadIdx.x] = Xg[(int64_t)local * d + threadIdx.x];
    __syncthreads();
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        float s = 0.f;
        const float* xj = Xg + (int64_t)j * d;
        for (int c = 0; c < d; ++c) {
            const float df = me[c] - xj[c];
            s = fmaf(df, df, s);
        }
        dist[j] = j == local ? INFINITY : s;
    }
    __syncthreads();
    const int kk = min(k, n - 1);
    for (int r = 0; r < kk; ++r) {
        unsigned long long best = ~0ull;
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            const unsigned long long key =
                ((unsigned long long)__float_as_uint(dist[j]) << 32) | (unsigned long long)(uint32_t)j;
            best = key < best ? key : best;
        }
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long other = __shfl_xor_sync(0xffffffffu, best, o);
            best = other < best ? other : best;
        }
        if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = best;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long b = wmin[0];
            for (int w = 1; w < kKnnThreads / 32; ++w) b = wmin[w] < b ? wmin[w] : b;
            const int j = (int)(uint32_t)(b & 0xffffffffull);
            nb[p * k + r] = base + j;
            dist[j] = INFINITY;
        }
        __syncthreads();
    }
    for (int r = kk + threadIdx.x; r < k; r += blockDim.x) nb[p * k + r] = -1;
}

// Graphs above kKnnMaxN points: one thread per query point, candidates
// staged in shared memory in tiles of kKnnTile points (coordinates padded
// to a multiple of 4 with zeros, which leaves every distance unchanged), and
// a sorted top-k list of (distance, index) keys per thread. The keys and the
// per-coordinate fmaf order are those of k_knn_select, so both kernels pick
// the same neighbours.
constexpr int kKnnTile = 256;
constexpr int kKnnMaxK = 64;

struct KnnTile {
    int32_t graph, first;  // graph and its first query point of this tile
};

__global__ void __launch_bounds__(kKnnThreads) k_knn_tiled(const KnnTile* __restrict__ tiles,
                                                           const int32_t* __restrict__ voff,
                                                           const int32_t* __restrict__ dim,
                                                           const int64_t* __restrict__ poff,
                                                           const float* __restrict__ X, int k,
                                                           int32_t* __restrict__ nb) {
    __shared__ __align__(16) float cand[kKnnTile * kKnnMaxDim];
    const KnnTile tl = tiles[blockIdx.x];
    const int32_t base = voff[tl.graph];
    const int n = voff[tl.graph + 1] - base, d = dim[tl.graph];
    const int dp = (d + 3) & ~3;
    const float* Xg = X + poff[tl.graph];
    const int local = tl.first + (int)threadIdx.x;
    const bool active = local < n;
    float q[kKnnMaxDim];
#pragma unroll
    for (int c = 0; c < kKnnMaxDim; ++c) q[c] = (active && c < d) ? Xg[(int64_t)local * d + c] : 0.f;
    const int kk = min(k, n - 1);
    float bd[kKnnMaxK];
    int bi[kKnnMaxK];
    int cnt = 0;
    float worst = INFINITY;
    int worst_i = INT32_MAX;
    for (int j0 = 0; j0 < n; j0 += kKnnTile) {
        const int tn = min(kKnnTile, n - j0);
        __syncthreads();
        for (int t = threadIdx.x; t < tn * dp; t += blockDim.x) {
            const int j = t / dp, c = t - j * dp;
            cand[t] = c < d ? Xg[(int64_t)(j0 + j) * d + c] : 0.f;
        }
        __syncthreads();
        if (!active || kk <= 0) continue;
        for (int j = 0; j < tn; ++j) {
            const float4* xj = reinterpret_cast<const float4*>(cand + j * dp);
            float s = 0.f;
#pragma unroll
            for (int c4 = 0; c4 < kKnnMaxDim / 4; ++c4) {
                if (4 * c4 < dp) {
                    const float4 x = xj[c4];
                    float df = q[4 * c4] - x.x;
                    s = fmaf(df, df, s);
                    df = q[4 * c4 + 1] - x.y;
                    s = fmaf(df, df, s);
                    df = q[4 * c4 + 2] - x.z;
                    s = fmaf(df, df, s);
                    df = q[4 * c4 + 3] - x.w;
                    s = fmaf(df, df, s);
                }
            }
            const int idx = j0 + j;
            if (idx == local) continue;
            if (cnt == kk && (s > worst || (s == worst && idx > worst_i))) continue;
            // insert (s, idx) into the sorted list
            int pos = cnt < kk ? cnt : kk - 1;
            while (pos > 0 && (bd[pos - 1] > s || (bd[pos - 1] == s && bi[pos - 1] > idx))) {
                bd[pos] = bd[pos - 1];
                bi[pos] = bi[pos - 1];
                --pos;
            }
            bd[pos] = s;
            bi[pos] = idx;
            if (cnt < kk) ++cnt;
            if (cnt == kk) {
                worst = bd[kk - 1];
                worst_i = bi[kk - 1];
            }
        }
    }
    if (!active) return;
    const int64_t p = (int64_t)base + local;
    for (int r = 0; r < k; ++r) nb[p * k + r] = r < cnt ? base + bi[r] : -1;
}

// Symmetrise the directed k-NN lists: row counts, fill both directions,
// sort rows, drop duplicates.
__global__ void k_knn_count(const int32_t* __restrict__ nb, int64_t npoints, int k, int32_t* __restrict__ cnt) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < npoints * k; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = nb[e];
        if (v < 0) continue;
        atomicAdd(&cnt[e / k], 1);
        atomicAdd(&cnt[v], 1);
    }
}

__global__ void k_knn_fill(const int32_t* __restrict__ nb, int64_t npoints, int k, int32_t* __restrict__ cursor,
                           int32_t* __restrict__ col) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < npoints * k; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = nb[e];
        if (v < 0) continue;
        const int32_t u = (int32_t)(e / k);
        col[atomicAdd(&cursor[u], 1)] = v;
        col[atomicAdd(&cursor[v], 1)] = u;
    }
}

__global__ void k_unique_count(const int32_t* __restrict__ rst, const int32_t* __restrict__ col, int64_t m,
                               int32_t* __restrict__ cnt) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        int c = 0;
        for (int32_t q = rst[i]; q < rst[i + 1]; ++q) c += (q == rst[i] || col[q] != col[q - 1]);
        cnt[i] = c;
    }
}

__global__ void k_unique_fill(const int32_t* __restrict__ rst, const int32_t* __restrict__ col, int64_t m,
                              const int32_t* __restrict__ orst, int32_t* __restrict__ ocol) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t o = orst[i];
        for (int32_t q = rst[i]; q < rst[i + 1]; ++q)
            if (q == rst[i] || col[q] != col[q - 1]) ocol[o++] = col[q];
    }
}

static ga_csr gen_knn_batch(ga_ctx ctx, int64_t count, const int32_t* n, const int32_t* dim, int k, uint64_t seed,
                            int64_t* voff_out) {
    GA_REQUIRE(count >= 1 && k >= 1 && k <= kKnnMaxK, GA_ERR_INVALID_ARG, "knn batch: need count >= 1 and 1 <= k <= 64");
    bool large = false;
    std::vector<int32_t> voff((size_t)count + 1);
    std::vector<int64_t> poff((size_t)count + 1);
    int64_t np = 0, nc = 0;
    for (int64_t g = 0; g < count; ++g) {
        GA_REQUIRE(n[g] >= 1 && n[g] <= (1 << 24), GA_ERR_INVALID_ARG, "knn batch: graph sizes must be 1..2^24");
        large = large || n[g] > kKnnMaxN;
        GA_REQUIRE(dim[g] >= 1 && dim[g] <= kKnnMaxDim, GA_ERR_INVALID_ARG, "knn batch: dimensions must be 1..32");
        voff[(size_t)g] = (int32_t)np;
        poff[(size_t)g] = nc;
        np += n[g];
        nc += (int64_t)n[g] * dim[g];
        GA_REQUIRE(np * (2 * (int64_t)k + 1) < INT32_MAX, GA_ERR_INVALID_ARG, "knn batch: too many points");
    }
    voff[(size_t)count] = (int32_t)np;
    poff[(size_t)count] = nc;
    if (voff_out)
        for (int64_t g = 0; g <= count; ++g) voff_out[g] = voff[(size_t)g];
    DBuf<int32_t> d_voff(ctx, (size_t)count + 1), d_dim(ctx, (size_t)count);
    DBuf<int64_t> d_poff(ctx, (size_t)count + 1);
    GA_CUDA(cudaMemcpyAsync(d_voff.p, voff.data(), sizeof(int32_t) * (count + 1), cudaMemcpyHostToDevice, ctx->stream));
    GA_CUDA(cudaMemcpyAsync(d_dim.p, dim, sizeof(int32_t) * count, cudaMemcpyHostToDevice, ctx->stream));
    GA_CUDA(cudaMemcpyAsync(d_poff.p, poff.data(), sizeof(int64_t) * (count + 1), cudaMemcpyHostToDevice, ctx->stream));
    DBuf<float> X(ctx, (size_t)nc);
    DBuf<int32_t> nb(ctx, (size_t)np * k);
    {
        ProfScope ps(ctx, "knn_points");
        k_knn_points<<<grid_for(np, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(d_voff.p, d_dim.p, d_poff.p, count,
                                                                                np, seed, X.p);
        post_launch("knn_points");
    }
    {
        ProfScope ps(ctx, "knn_select");
        if (!large && !ctx->knn_tiled) {
            k_knn_select<<<(unsigned)np, kKnnThreads, 0, ctx->stream>>>(d_voff.p, d_dim.p, d_poff.p, count, X.p, k,
                                                                      nb.p);
            post_launch("knn_select");
        } else {
            std::vector<KnnTile> tl;
            for (int64_t g = 0; g < count; ++g)
                for (int32_t f = 0; f < n[g]; f += kKnnThreads) tl.push_back(KnnTile{(int32_t)g, f});
            DBuf<KnnTile> d_tl(ctx, tl.size());
            GA_CUDA(cudaMemcpyAsync(d_tl.p, tl.data(), sizeof(KnnTile) * tl.size(), cudaMemcpyHostToDevice,
                                    ctx->stream));
            k_knn_tiled<<<(unsigned)tl.size(), kKnnThreads, 0, ctx->stream>>>(d_tl.p, d_voff.p, d_dim.p, d_poff.p,
                                                                            X.p, k, nb.p);
            post_launch("knn_tiled");
            GA_CUDA(cudaStreamSynchronize(ctx->stream));  // the host tile table goes out of scope
        }
    }
    DBuf<int32_t> cnt(ctx, (size_t)np + 1), rst(ctx, (size_t)np + 1), cursor(ctx, (size_t)np + 1);
    GA_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * (np + 1), ctx->stream));
    k_knn_count<<<grid_for(np * k, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(nb.p, np, k, cnt.p);
    post_launch("knn_count");
    scan_exclusive_i32(ctx, cnt.p, rst.p, np);
    const int32_t total = read_i32(ctx, rst.p + np);
    DBuf<int32_t> col(ctx, (size_t)total + 1), pay(ctx, (size_t)total + 1);
    GA_CUDA(cudaMemcpyAsync(cursor.p, rst.p, sizeof(int32_t) * (np + 1), cudaMemcpyDeviceToDevice, ctx->stream));
    k_knn_fill<<<grid_for(np * k, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(nb.p, np, k, cursor.p, col.p);
    post_launch("knn_fill");
    sort_rows_by_key(ctx, rst.p, np, col.p, pay.p, total);
    k_unique_count<<<grid_for(np, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(rst.p, col.p, np, cnt.p);
    post_launch("unique_count");
    DBuf<int32_t> orst(ctx, (size_t)np + 1);
    scan_exclusive_i32(ctx, cnt.p, orst.p, np);
    const int32_t nnz = read_i32(ctx, orst.p + np);
    ga_csr U = csr_alloc(ctx, np, np, nnz, GA_INT32);
    try {
        GA_CUDA(cudaMemcpyAsync(U->rst, orst.p, sizeof(int32_t) * (np + 1), cudaMemcpyDeviceToDevice, ctx->stream));
        k_unique_fill<<<grid_for(np, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(rst.p, col.p, np, orst.p, U->col);
        post_launch("unique_fill");
        fill_ones(ctx, U->val, nnz, GA_INT32);
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
    } catch (...) {
        csr_destroy(ctx, U);
        throw;
    }
    U->unit = 1;
    U->sym = 1;
    return U;
}

// ------------------------------------------------------------- batched TC / k-truss
__global__ void k_segment_sums(const int64_t* __restrict__ rows, const int32_t* __restrict__ voff, int64_t ngraphs,
                               int64_t* __restrict__ out) {
    __shared__ long long part[8];
    for (int64_t g = blockIdx.x; g < ngraphs; g += gridDim.x) {
        long long s = 0;
        for (int32_t i = voff[g] + threadIdx.x; i < voff[g + 1]; i += blockDim.x) s += rows[i];
        s = warp_sum<long long>(s);
        if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            long long t = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
            out[g] = t;
        }
        __syncthreads();
    }
}

__global__ void k_batch_setup(const int32_t* __restrict__ rst, const int32_t* __restrict__ voff, int64_t ngraphs,
                              int32_t* __restrict__ gid, int32_t* __restrict__ nvert, int32_t* __restrict__ nnz_g,
                              int32_t* __restrict__ iters_g, int32_t* __restrict__ done_g) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ngraphs; g += (int64_t)gridDim.x * blockDim.x) {
        const int32_t b = voff[g], e = voff[g + 1];
        nvert[g] = e - b;
        nnz_g[g] = rst[e] - rst[b];
        iters_g[g] = 0;
        done_g[g] = e == b;  // an empty graph reports 0 iterations, as the single-graph loop does
    }
    const int64_t m = voff[ngraphs];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        gid[i] = upper_bound_i32(voff, (int)ngraphs + 1, (int32_t)i) - 1;
}

static void check_voff(ga_csr U, int64_t count, const int64_t* voff) {
    GA_REQUIRE(count >= 1 && voff != nullptr, GA_ERR_INVALID_ARG, "batch: need at least one graph and offsets");
    GA_REQUIRE(voff[0] == 0 && voff[count] == U->m, GA_ERR_INVALID_ARG, "batch: offsets must run from 0 to m");
    for (int64_t g = 0; g < count; ++g)
        GA_REQUIRE(voff[g] <= voff[g + 1], GA_ERR_INVALID_ARG, "batch: offsets must be non-decreasing");
}

static DBuf<int32_t> upload_voff(ga_ctx ctx, int64_t count, const int64_t* voff) {
    std::vector<int32_t> v((size_t)count + 1);
    for (int64_t g = 0; g <= count; ++g) v[(size_t)g] = (int32_t)voff[g];
    DBuf<int32_t> d(ctx, (size_t)count + 1);
    GA_CUDA(cudaMemcpyAsync(d.p, v.data(), sizeof(int32_t) * (count + 1), cudaMemcpyHostToDevice, ctx->stream));
    GA_CUDA(cudaStreamSynchronize(ctx->stream));
    return d;
}

}  // namespace ga

using namespace ga;

extern "C" {

int ga_csr_block_diag(ga_ctx ctx, int64_t count, const ga_csr* parts, ga_csr* out, int64_t* voff) {
    if (!ctx || !out || (count > 0 && !parts)) return GA_ERR_INVALID_ARG;
    *out = nullptr;
    GA_API_BODY(ctx, *out = block_diag(ctx, count, parts, voff));
}

int ga_gen_knn_batch(ga_ctx ctx, int64_t count, const int32_t* n, const int32_t* dim, int k, uint64_t seed,
                     ga_csr* out, int64_t* voff) {
    if (!ctx || !out || !n || !dim) return GA_ERR_INVALID_ARG;
    *out = nullptr;
    GA_API_BODY(ctx, *out = gen_knn_batch(ctx, count, n, dim, k, seed, voff));
}

int ga_batch_tc(ga_ctx ctx, ga_algo algo, ga_csr U, int64_t count, const int64_t* voff, int64_t* totals) {
    if (!ctx || !U || !totals) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        check_voff(U, count, voff);
        DBuf<int32_t> dv = upload_voff(ctx, count, voff);
        DBuf<int64_t> d_total(ctx, 1), rows(ctx, (size_t)U->m + 1), per(ctx, (size_t)count);
        ProfScope ps(ctx, "batch_tc");
        int rc = ga_tc_device(ctx, algo, U, d_total.p, rows.p);
        if (rc != GA_OK) fail(rc, ctx->last_error);
        k_segment_sums<<<(unsigned)std::min<int64_t>(count, 65535), 256, 0, ctx->stream>>>(rows.p, dv.p, count, per.p);
        post_launch("segment_sums");
        GA_CUDA(cudaMemcpyAsync(totals, per.p, sizeof(int64_t) * count, cudaMemcpyDeviceToHost, ctx->stream));
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

static int batch_ktruss(ga_ctx ctx, ga_algo algo, ga_csr U, int64_t count, const int64_t* voff, int k,
                        const int* k_per_graph, ga_csr* C, int* iters) {
    if (!ctx || !U || !C || !iters) return GA_ERR_INVALID_ARG;
    *C = nullptr;
    GA_API_BODY(ctx, {
        check_voff(U, count, voff);
        GA_REQUIRE(U->dtype == GA_INT32, GA_ERR_DTYPE, "batched k-truss needs int32 values");
        GA_REQUIRE(csr_unit_values(ctx, U), GA_ERR_INVALID_ARG, "batched k-truss needs adjacency (all-ones) values");
        GA_REQUIRE(algo != GA_NAIVE, GA_ERR_UNSUPPORTED, "batched k-truss runs MSA, MCA, HEAP or DOT");
        DBuf<int32_t> dv = upload_voff(ctx, count, voff);
        DBuf<int32_t> gid(ctx, (size_t)U->m + 1), nvert(ctx, (size_t)count), nnz_g(ctx, (size_t)count),
            iters_g(ctx, (size_t)count), done_g(ctx, (size_t)count), kg(ctx, k_per_graph ? (size_t)count : 1);
        if (k_per_graph)
            GA_CUDA(cudaMemcpyAsync(kg.p, k_per_graph, sizeof(int32_t) * count, cudaMemcpyHostToDevice, ctx->stream));
        k_batch_setup<<<grid_for(count + U->m, 128, ctx->num_sms * 8), 128, 0, ctx->stream>>>(U->rst, dv.p, count, gid.p,
                                                                                     nvert.p, nnz_g.p, iters_g.p,
                                                                                     done_g.p);
        post_launch("batch_setup");
        KtBatch b;
        b.ngraphs = count; b.voff = dv.p; b.gid = gid.p; b.nvert = nvert.p;
        b.nnz_g = nnz_g.p; b.iters_g = iters_g.p; b.done_g = done_g.p;
        b.kg = k_per_graph ? kg.p : nullptr;
        ProfScope ps(ctx, "batch_ktruss");
        *C = ktruss_impl(ctx, algo, U, k, nullptr, &b);
        GA_CUDA(cudaMemcpyAsync(iters, iters_g.p, sizeof(int32_t) * count, cudaMemcpyDeviceToHost, ctx->stream));
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int ga_batch_ktruss(ga_ctx ctx, ga_algo algo, ga_csr U, int64_t count, const int64_t* voff, int k, ga_csr* C,
                    int* iters) {
    return batch_ktruss(ctx, algo, U, count, voff, k, nullptr, C, iters);
}

int ga_batch_ktruss_k(ga_ctx ctx, ga_algo algo, ga_csr U, int64_t count, const int64_t* voff, const int* k,
                      ga_csr* C, int* iters) {
    if (!k) return GA_ERR_INVALID_ARG;
    return batch_ktruss(ctx, algo, U, count, voff, 0, k, C, iters);
}

int ga_batch_bc(ga_ctx ctx, ga_csr U, int64_t count, const int64_t* voff, const int64_t* soff,
                const int32_t* sources, double* bc) {
    if (!ctx || !U || !soff || !bc) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        check_voff(U, count, voff);
        DBuf<double> d_bc(ctx, (size_t)(U->m > 0 ? U->m : 1));
        bc_union_device(ctx, U, count, voff, soff, sources, d_bc.p);
        if (U->m)
            GA_CUDA(cudaMemcpyAsync(bc, d_bc.p, sizeof(double) * U->m, cudaMemcpyDeviceToHost, ctx->stream));
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

}  // extern "C"
