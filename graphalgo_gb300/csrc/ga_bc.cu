// Batched betweenness centrality (betweenness_centrality_batch,
// include/betweenness_centrality.h:125-237) with FP64 path counts and
// dependencies, device-resident from the first frontier to the scores.
//
// Layout (vertex x source pairs, ns = number of sources):
//  * an append-only entry store (source index, sigma, bcu = 1 + delta), one
//    record per discovered (vertex, source) pair, grouped per (level, vertex);
//  * per level, a list of frontier rows (vertex, first entry, length) - the
//    reference's Sigmas[d];
//  * a visited bitmap per vertex (ns bits) - the reference's Numsp pattern;
//  * a dense m x ns FP64 matrix W used by the backward sweep.
// Forward level (Front<!Numsp> = A^T * Front, matrix_la.h:800-891 fused with
// add_nointersect, matrix_la.h:337-372): one warp per unvisited vertex pulls
// the frontier entries of its in-neighbours into a shared-memory accumulator
// over the sources, skips sources already visited, and appends the new
// frontier row to the store (stream compaction by atomic reservation).
// Backward level k (betweenness_centrality.h:203-218): W<S[k]> = bcu/sigma,
// then for every row of S[k-1]: acc = A * W restricted to its sources,
// bcu += acc * sigma, and bc[v] += acc * sigma (the final row sum,
// betweenness_centrality.h:220-228, accumulated as it is produced).
// Both sweeps run as device loops (CUDA-graph WHILE nodes).
//
// Source columns. Column j of the state holds source j, except in a batch
// over the block-diagonal union of several graphs: there column j holds the
// j-th source of every graph at once. A source only reaches the vertices of
// its own graph, so each (vertex, column) pair still belongs to one source,
// and the state is (union vertices) x (largest source count of a graph)
// instead of x (all sources). The columns a graph has no source for are
// marked visited on its vertices before the first level.
#include "ga_device.cuh"
#include "ga_loop.cuh"

#include <algorithm>

namespace ga {

constexpr int kBcThreads = 256;
constexpr int kBcWarps = kBcThreads / 32;
constexpr int kBcMaxSources = 1024;

struct BcState {
    int32_t d;        // current forward level
    int32_t depth;    // number of non-empty levels (forward result)
    int32_t k;        // backward level
    int32_t done;
    // entries appended so far (store size, low 32 bits) and frontier rows
    // appended so far (high 32 bits): one atomic reserves both
    unsigned long long er;
    int32_t overflow;
    int32_t mode;          // forward direction of the current level: 0 pull, 1 push
    int32_t ntouched;      // vertices reached by the current push level
    int32_t stalled;       // a bulk copy of the backward sweep did not complete in time
    int32_t nhrows;        // backward level: heavy rows listed in hrows
    unsigned long long cur_work, next_work;  // sum over frontier rows of entries x out-degree
};

struct BcArgs {
    const int32_t* atr; const int32_t* atc; const double* atv;  // A^T (in-neighbours)
    const int32_t* ar; const int32_t* ac; const double* av;     // A (out-neighbours)
    int64_t m;
    int ns, words;                                              // source columns, 32-bit words per vertex
    int nsrc;                                                   // sources (level-0 entries)
    const int32_t* sources;
    const int32_t* scol;                                        // column of each source (nullptr: its index)
    BcState* st;
    int32_t* level_rows;    // level_rows[d] = first row of level d
    int32_t* cur_start[2];  // per vertex, per parity: first entry of its frontier row
    int32_t* cur_len[2];
    uint32_t* vbits;        // m x words
    int32_t* vcnt;          // sources that reached each vertex
    int32_t* es; double* ev; double* ed;  // store: source, sigma, bcu
    int32_t* rv; int32_t* rs; int32_t* rl; // rows: vertex, start, length
    int64_t cap_entries, cap_rows;
    double* W;              // m x ns
    uint32_t* inlvl;        // m bits: vertex has entries at the level being swept
    double* bc;
    const int32_t* heavy_in;  // vertices with more than kBcHeavyDeg in-neighbours
    int nheavy_in;
    int64_t nnz;            // stored entries of A (direction choice)
    uint32_t* tbits;        // push levels: m x words, sources that reached each vertex
    int32_t* tlist;         // push levels: vertices reached, in order of first touch
    int32_t* tmark;         // push levels: vertex already listed
    int32_t* hrows;         // backward level: rows of S[k-1] whose vertex has more than kBcHeavyDeg neighbours
};

// A level pushes (frontier rows scatter along their out-edges with global
// atomics) when its frontier's work, entries x out-degree, is below
// nnz / kBcPushDiv; otherwise every unvisited vertex pulls (no atomics on
// global memory, but a pass over all in-edges).
constexpr unsigned long long kBcPushDiv = 8;

__global__ void k_bc_init(BcArgs p) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < p.nsrc; j += gridDim.x * blockDim.x) {
        int v = p.sources[j];
        const int c = p.scol ? p.scol[j] : j;
        p.es[j] = c;
        p.ev[j] = 1.0;
        p.ed[j] = 1.0;
        atomicOr(&p.vbits[(size_t)v * p.words + (c >> 5)], 1u << (c & 31));
        atomicAdd(&p.vcnt[v], 1);
        p.cur_start[0][v] = j;
        p.cur_len[0][v] = 1;
        atomicAdd(&p.st->next_work, (unsigned long long)(p.ar[v + 1] - p.ar[v]));
    }
}

__global__ void k_bc_state_init(BcArgs p) {
    p.st->d = 0; p.st->depth = 0; p.st->k = 0; p.st->done = 0;
    p.st->er = (unsigned long long)p.nsrc; p.st->overflow = 0;
    p.st->mode = 0; p.st->ntouched = 0; p.st->stalled = 0; p.st->nhrows = 0;
    p.st->cur_work = 0; p.st->next_work = 0;
    p.level_rows[0] = 0;
}

// Batches with packed columns: on the vertices of graph g (union rows
// [voff[g], voff[g+1])), the columns at and above its source count are
// marked visited, so no entry is ever made there and the vertex counts as
// reached by every column once its own sources have reached it.
__global__ void k_bc_previsit(BcArgs p, const int64_t* __restrict__ voff, const int32_t* __restrict__ gsrc,
                              int64_t count) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < p.m; v += (int64_t)gridDim.x * blockDim.x) {
        int64_t lo = 0, hi = count;  // the graph g with voff[g] <= v < voff[g+1]
        while (hi - lo > 1) {
            const int64_t mid = (lo + hi) >> 1;
            if (voff[mid] <= v) lo = mid; else hi = mid;
        }
        const int have = gsrc[lo];
        for (int w = 0; w < p.words; ++w) {
            const int c0 = w * 32;
            uint32_t bits = 0u;
            if (have <= c0) bits = 0xffffffffu;
            else if (have < c0 + 32) bits = ~((1u << (have - c0)) - 1u);
            if (c0 + 32 > p.ns) bits &= (p.ns - c0 >= 32) ? 0xffffffffu : ((1u << (p.ns - c0)) - 1u);
            p.vbits[(size_t)v * p.words + w] = bits;
        }
        p.vcnt[v] = p.ns - have;
    }
}

// Level start: the frontier's work decides the direction.
__global__ void k_bc_level_begin(BcArgs p) {
    BcState* st = p.st;
    if (st->done) return;
    st->cur_work = st->next_work;
    st->next_work = 0;
    st->ntouched = 0;
    st->mode = st->cur_work * kBcPushDiv < (unsigned long long)p.nnz ? 1 : 0;
}

// Vertices with more than kBcHeavyDeg neighbours are handled by a whole CTA
// (their neighbour lists are split over the CTA's warps).
constexpr int kBcHeavyDeg = 1024;

// Frontier entries of the in-neighbours in group [g, g+32) of vertex v,
// flattened over the warp (segment found by ballot/OR + popcount), added to
// acc for sources v has not reached yet.
template <bool UNIT>
__device__ __forceinline__ void bc_pull_group(const BcArgs& p, const int32_t* curS, const int32_t* curL, int32_t g,
                                              int32_t ae, const uint32_t* vis, double* acc, uint32_t* touched,
                                              int* s_incl, int* s_off, double* s_a) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int32_t t = g + lane;
    int len = 0, bs = 0;
    double a = 0.0;
    if (t < ae) {
        const int32_t u = __ldg(p.atc + t);
        len = curL[u];
        if (len) {
            bs = curS[u];
            a = UNIT ? 1.0 : __ldg(p.atv + t);
        }
    }
    const unsigned nz = __ballot_sync(FULL, len > 0);
    if (nz == 0) return;
    const int nseg = __popc(nz);
    const int incl = warp_incl_scan(len);
    const int total = __shfl_sync(FULL, incl, 31);
    if (len > 0) {
        const int rank = __popc(nz & ((1u << lane) - 1u));
        s_incl[rank] = incl;
        s_off[rank] = bs - (incl - len);
        s_a[rank] = a;
    }
    __syncwarp();
    const int my_end = lane < nseg ? s_incl[lane] - 1 : INT32_MAX;
    const unsigned lt = (1u << lane) - 1u;
    int q_base = 0;
    for (int base = 0; base < total; base += 32) {
        const int e = my_end - base;
        const unsigned bm = __reduce_or_sync(FULL, (e >= 0 && e < 32) ? (1u << e) : 0u);
        const int x = base + lane;
        if (x < total) {
            const int q = q_base + __popc(bm & lt);
            const int32_t j = x + s_off[q];
            const int s = p.es[j];
            if (!(vis[s >> 5] & (1u << (s & 31)))) {
                atomicAdd(&acc[s], s_a[q] * p.ev[j]);
                atomicOr(&touched[s >> 5], 1u << (s & 31));
            }
        }
        q_base += __popc(bm);
    }
    __syncwarp();
}

// Appends v's new frontier row (its touched sources, in source order) by one
// warp; resets acc/touched. Lane 0 adds the row's next-level work (entries x
// out-degree) to `work`, which the caller adds to the level total once.
__device__ __forceinline__ void bc_emit_row(const BcArgs& p, int64_t v, int32_t* nxtS, int32_t* nxtL,
                                            const uint32_t* vis, double* acc, uint32_t* touched,
                                            unsigned long long& work) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint32_t word = lane < p.words ? touched[lane] : 0u;
    const int cnt = __popc(word);
    const int excl = warp_incl_scan(cnt) - cnt;
    const int count = __shfl_sync(FULL, excl + cnt, 31);
    if (count == 0) {
        if (lane == 0) nxtL[v] = 0;
        return;
    }
    int start = 0;
    if (lane == 0) {
        const unsigned long long old = atomicAdd(&p.st->er, (1ull << 32) | (unsigned long long)count);
        start = (int)(old & 0xffffffffull);
        const int r = (int)(old >> 32);
        if ((int64_t)start + count > p.cap_entries || (int64_t)r >= p.cap_rows) {
            atomicExch(&p.st->overflow, 1);
            start = -1;
        } else {
            p.rv[r] = (int32_t)v; p.rs[r] = start; p.rl[r] = count;
            p.vcnt[v] += count;
            work += (unsigned long long)count * (unsigned long long)(p.ar[v + 1] - p.ar[v]);
        }
        nxtS[v] = start;
        nxtL[v] = start < 0 ? 0 : count;
    }
    start = __shfl_sync(FULL, start, 0);
    if (start >= 0 && word) {
        int pos = start + excl;
        uint32_t w = word;
        while (w) {
            const int b = __ffs(w) - 1;
            w &= w - 1;
            const int s = lane * 32 + b;
            p.es[pos] = s;
            p.ev[pos] = acc[s];
            p.ed[pos] = 1.0;
            ++pos;
        }
        p.vbits[(size_t)v * p.words + lane] = vis[lane] | word;
    }
    __syncwarp();
    for (int s = lane; s < p.ns; s += 32) acc[s] = 0.0;
    if (lane < p.words) touched[lane] = 0u;
    __syncwarp();
}

// One forward level: dynamic per-warp shared memory = acc[ns] doubles +
// touched[words] + visited[words] + 32-entry flattening scratch. Heavy
// vertices first, one per CTA with all warps pulling into warp 0's
// accumulator; then the rest, one per warp.
template <bool UNIT>
__global__ void __launch_bounds__(kBcThreads) k_bc_forward(BcArgs p) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const size_t per_warp = ((size_t)p.ns * sizeof(double) + 2 * (size_t)p.words * sizeof(uint32_t) +
                             32 * (2 * sizeof(int) + sizeof(double)) + 15) & ~(size_t)15;
    auto region = [&](int w, double*& acc, uint32_t*& touched, uint32_t*& vis, int*& s_incl, int*& s_off,
                      double*& s_a) {
        unsigned char* base = smem + w * per_warp;
        acc = reinterpret_cast<double*>(base);
        touched = reinterpret_cast<uint32_t*>(base + (size_t)p.ns * sizeof(double));
        vis = touched + p.words;
        s_incl = reinterpret_cast<int*>(vis + p.words);
        s_off = s_incl + 32;
        s_a = reinterpret_cast<double*>(s_off + 32);
    };
    double* acc; uint32_t* touched; uint32_t* vis; int* s_incl; int* s_off; double* s_a;
    region(wid, acc, touched, vis, s_incl, s_off, s_a);
    double* acc0; uint32_t* touched0; uint32_t* vis0; int* i0; int* o0; double* a0;
    region(0, acc0, touched0, vis0, i0, o0, a0);

    if (p.st->done || p.st->mode != 0) return;
    unsigned long long work = 0;  // lane 0: next-level work of the rows this warp emits
    const int d = p.st->d;
    const int par = d & 1;
    const int32_t* curS = p.cur_start[par];
    const int32_t* curL = p.cur_len[par];
    int32_t* nxtS = p.cur_start[par ^ 1];
    int32_t* nxtL = p.cur_len[par ^ 1];

    for (int s = lane; s < p.ns; s += 32) acc[s] = 0.0;
    if (lane < p.words) touched[lane] = 0u;
    __syncthreads();

    // heavy vertices: the CTA's warps split the in-neighbours
    for (int h = blockIdx.x; h < p.nheavy_in; h += gridDim.x) {
        const int64_t v = p.heavy_in[h];
        const bool active = p.vcnt[v] < p.ns;  // uniform over the CTA
        if (active) {
            if (wid == 0 && lane < p.words) vis0[lane] = p.vbits[(size_t)v * p.words + lane];
            __syncthreads();
            const int32_t ab = p.atr[v], ae = p.atr[v + 1];
            for (int32_t g = ab + wid * 32; g < ae; g += kBcWarps * 32)
                bc_pull_group<UNIT>(p, curS, curL, g, ae, vis0, acc0, touched0, s_incl, s_off, s_a);
            __syncthreads();
            if (wid == 0) bc_emit_row(p, v, nxtS, nxtL, vis0, acc0, touched0, work);
        } else if (threadIdx.x == 0) {
            nxtL[v] = 0;
        }
        __syncthreads();
    }

    // the rest: warp w takes the vertices w, w + W, w + 2W, ... (W warps in
    // the grid), 32 of them at a time: each lane checks one (heavy vertices
    // were done above; one that every source has reached, or without
    // in-neighbours, gets an empty next row), then the warp pulls the others
    // one by one
    const unsigned FULL = 0xffffffffu;
    const int64_t warps = (int64_t)gridDim.x * kBcWarps;
    for (int64_t v0 = (int64_t)blockIdx.x * kBcWarps + wid; v0 < p.m; v0 += warps * 32) {
        const int64_t vl = v0 + (int64_t)lane * warps;
        int32_t lab = 0, lae = 0;
        bool act = false;
        if (vl < p.m) {
            lab = p.atr[vl];
            lae = p.atr[vl + 1];
            if (lae - lab <= kBcHeavyDeg) {
                act = lae > lab && p.vcnt[vl] < p.ns;
                if (!act) nxtL[vl] = 0;
            }
        }
        unsigned am = __ballot_sync(FULL, act);
        while (am) {
            const int src = __ffs(am) - 1;
            am &= am - 1;
            const int64_t v = v0 + (int64_t)src * warps;
            const int32_t ab = __shfl_sync(FULL, lab, src), ae = __shfl_sync(FULL, lae, src);
            if (lane < p.words) vis[lane] = p.vbits[(size_t)v * p.words + lane];
            __syncwarp();
            for (int32_t g = ab; g < ae; g += 32)
                bc_pull_group<UNIT>(p, curS, curL, g, ae, vis, acc, touched, s_incl, s_off, s_a);
            bc_emit_row(p, v, nxtS, nxtL, vis, acc, touched, work);
        }
    }
    if (lane == 0 && work) atomicAdd(&p.st->next_work, work);
}

// Push level, one frontier row (vertex u, entries [e0, e0+len)) and the
// out-neighbours [t0, t1) of u, lanes over neighbours 32 at a time (group
// stride `step`): for every entry (source s, sigma) and neighbour w that s has
// not reached, W[w][s] += A[u][w] * sigma, and w's touched bit for s is set;
// the first touch of w lists it.
template <bool UNIT>
__device__ __forceinline__ void bc_push_row(const BcArgs& p, int32_t e0, int32_t len, int32_t t0, int32_t t1,
                                            int32_t step) {
    const int lane = threadIdx.x & 31;
    for (int32_t g = t0; g < t1; g += step) {
        const int32_t t = g + lane;
        if (t >= t1) continue;
        const int32_t w = __ldg(p.ac + t);
        const double a = UNIT ? 1.0 : __ldg(p.av + t);
        const uint32_t* vis = p.vbits + (size_t)w * p.words;
        for (int e = 0; e < len; ++e) {
            const int s = p.es[e0 + e];
            const uint32_t bit = 1u << (s & 31);
            if (vis[s >> 5] & bit) continue;
            atomicAdd(&p.W[(size_t)w * p.ns + s], a * p.ev[e0 + e]);
            const uint32_t old = atomicOr(&p.tbits[(size_t)w * p.words + (s >> 5)], bit);
            if (old == 0u && atomicExch(&p.tmark[w], 1) == 0) p.tlist[atomicAdd(&p.st->ntouched, 1)] = w;
        }
    }
}

// Frontier items of level d: the sources at level 0, else the rows found
// while level d-1 ran, [level_rows[d-1], level_rows[d]).
__device__ __forceinline__ void bc_frontier_item(const BcArgs& p, int d, int64_t it, int32_t& u, int32_t& e0,
                                                 int32_t& len) {
    if (d == 0) {
        u = p.sources[it]; e0 = (int32_t)it; len = 1;
    } else {
        const int64_t r = p.level_rows[d - 1] + it;
        u = p.rv[r]; e0 = p.rs[r]; len = p.rl[r];
    }
}

template <bool UNIT>
__global__ void __launch_bounds__(kBcThreads) k_bc_push(BcArgs p) {
    const BcState* st = p.st;
    if (st->done || st->mode != 1) return;
    const int d = st->d;
    const int wid = threadIdx.x >> 5;
    const int64_t items = d == 0 ? p.nsrc : (int64_t)p.level_rows[d] - p.level_rows[d - 1];
    // rows of high-degree vertices: the CTA's warps split the neighbours
    for (int64_t it = blockIdx.x; it < items; it += gridDim.x) {
        int32_t u, e0, len;
        bc_frontier_item(p, d, it, u, e0, len);
        const int32_t ab = p.ar[u], ae = p.ar[u + 1];
        if (ae - ab <= kBcHeavyDeg) continue;
        bc_push_row<UNIT>(p, e0, len, ab + wid * 32, ae, kBcWarps * 32);
    }
    const int64_t warps = (int64_t)gridDim.x * kBcWarps;
    for (int64_t it = (int64_t)blockIdx.x * kBcWarps + wid; it < items; it += warps) {
        int32_t u, e0, len;
        bc_frontier_item(p, d, it, u, e0, len);
        const int32_t ab = p.ar[u], ae = p.ar[u + 1];
        if (ae - ab > kBcHeavyDeg) continue;
        bc_push_row<UNIT>(p, e0, len, ab, ae, 32);
    }
}

// Push level, after the scatter: every vertex's next-frontier length is
// cleared, then each reached vertex appends its row (one warp each) from its
// W row and touched bits, which are reset.
__global__ void k_bc_push_clear(BcArgs p) {
    const BcState* st = p.st;
    if (st->done || st->mode != 1) return;
    int32_t* nxtL = p.cur_len[(st->d & 1) ^ 1];
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < p.m; v += (int64_t)gridDim.x * blockDim.x)
        nxtL[v] = 0;
}

__global__ void __launch_bounds__(kBcThreads) k_bc_push_emit(BcArgs p) {
    const BcState* st = p.st;
    if (st->done || st->mode != 1) return;
    const int lane = threadIdx.x & 31;
    const int par = st->d & 1;
    int32_t* nxtS = p.cur_start[par ^ 1];
    int32_t* nxtL = p.cur_len[par ^ 1];
    const int n = st->ntouched;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    unsigned long long work = 0;  // lane 0: next-level work of the rows this warp emits
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
        const int32_t w = p.tlist[i];
        bc_emit_row(p, w, nxtS, nxtL, p.vbits + (size_t)w * p.words, p.W + (size_t)w * p.ns,
                    p.tbits + (size_t)w * p.words, work);
        if (lane == 0) p.tmark[w] = 0;
    }
    if (lane == 0 && work) atomicAdd(&p.st->next_work, work);
}

__global__ void k_bc_forward_finalize(BcArgs p, LoopCtl ctl) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    BcState* st = p.st;
    bool more = false;
    if (!st->done) {
        const int d = st->d;
        const int32_t rows = (int32_t)(st->er >> 32);
        if (st->overflow || rows == p.level_rows[d]) {
            st->depth = d;
            st->done = 1;
        } else {
            p.level_rows[d + 1] = rows;
            st->d = d + 1;
            if ((int64_t)st->d > p.m) { st->depth = st->d; st->done = 1; }
            else more = true;
        }
    }
    if (!more) st->k = st->depth - 1;
    loop_continue(ctl, more);
}

// W<S[k]> = bcu / sigma and mark the level's vertices (set = true), or clear
// both again (set = false).
__global__ void k_bc_set_w(BcArgs p, bool set) {
    const int k = p.st->k;
    if (k < 1) return;
    const int lane = threadIdx.x & 31;
    const int32_t r0 = p.level_rows[k], r1 = p.level_rows[k + 1];
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t r = r0 + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); r < r1; r += warps) {
        const int32_t v = p.rv[r], s0 = p.rs[r], n = p.rl[r];
        double* wrow = p.W + (size_t)v * p.ns;
        for (int e = lane; e < n; e += 32) {
            int s = p.es[s0 + e];
            wrow[s] = set ? p.ed[s0 + e] / p.ev[s0 + e] : 0.0;
        }
        if (lane == 0) {
            if (set) atomicOr(&p.inlvl[v >> 5], 1u << (v & 31));
            else atomicAnd(&p.inlvl[v >> 5], ~(1u << (v & 31)));
        }
    }
    // before the backward level: the heavy rows of S[k-1], listed so that
    // the CTAs of the backward kernel can share them out
    if (set) {
        const int32_t q0 = p.level_rows[k - 1];
        for (int64_t r = q0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < r0;
             r += (int64_t)gridDim.x * blockDim.x) {
            const int32_t v = p.rv[r];
            if (p.ar[v + 1] - p.ar[v] > kBcHeavyDeg) p.hrows[atomicAdd(&p.st->nhrows, 1)] = (int32_t)r;
        }
    }
}

constexpr int kBcPer = 4;  // row entries per lane per pass of the backward sweep

// How the backward sweep reads the W rows of a row's level-k neighbours
// (GA_OPT_BC_BACKWARD): 0 gathers of up to kBcHits neighbours' rows issued
// together; 1 bulk copies of whole W rows into shared memory, two batches of
// kBcHits rows in flight per warp (needs an even source count of at most
// kBcBulkMaxCols and a 16-byte aligned W); 2 one neighbour at a time.
enum { kBcBwdGather = 0, kBcBwdBulk = 1, kBcBwdSingle = 2 };
constexpr int kBcHits = 4;
constexpr int kBcBulkMaxCols = 128;
constexpr long long kBcWaitCycles = 2000000000ll;  // about a second at 2 GHz

// The hit lanes of one group (bit mask `hits`) in ascending order, up to
// kBcHits of them: their neighbours and values, broadcast to the warp.
__device__ __forceinline__ int bc_take_hits(unsigned& hits, int32_t w, double a, int32_t (&ws)[kBcHits],
                                            double (&as)[kBcHits]) {
    const unsigned FULL = 0xffffffffu;
    int n = 0;
#pragma unroll
    for (int h = 0; h < kBcHits; ++h) {
        ws[h] = -1;
        as[h] = 0.0;
        if (hits) {  // warp-uniform
            const int src = __ffs(hits) - 1;
            hits &= hits - 1;
            ws[h] = __shfl_sync(FULL, w, src);
            as[h] = __shfl_sync(FULL, a, src);
            n = h + 1;
        }
    }
    return n;
}

// Per-warp state of the bulk form: two stages of kBcHits W rows in shared
// memory, one barrier per stage and its expected parity.
struct BcRing {
    double* rows;    // 2 * kBcHits rows of ns doubles
    uint64_t* bar;   // 2 barriers
    uint32_t phase;  // bit s: parity the next wait on stage s expects
    bool ok;         // false once a wait ran out
};

// acc[u] += sum over out-neighbours t in [t0, t1) step `stride` (groups of
// 32 fetched together, level-k neighbours picked by ballot) of
// A[v][w] * W[w][s[u]]. The neighbours' contributions are added in the same
// order (ascending t) in every mode.
template <bool UNIT, int MODE>
__device__ __forceinline__ void bc_push_range(const BcArgs& p, int32_t t0, int32_t t1, int32_t stride,
                                              const int (&s)[kBcPer], double (&acc)[kBcPer], BcRing& ring) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    // bulk form: the batch whose copies are in flight
    int pend_n = 0, pend_stage = 0, next_stage = 0;
    double pend_a[kBcHits];
    auto consume = [&](int stage, int n, const double (&as)[kBcHits]) {
        const bool ok = mbar_wait(ring.bar + stage, (ring.phase >> stage) & 1u, kBcWaitCycles);
        ring.phase ^= 1u << stage;
        if (!ok) {
            if (lane == 0) atomicExch(&p.st->stalled, 1);
            ring.ok = false;
            return;
        }
        const double* base = ring.rows + (size_t)stage * kBcHits * p.ns;
#pragma unroll
        for (int h = 0; h < kBcHits; ++h) {
            if (h >= n) break;
            const double* row = base + (size_t)h * p.ns;
#pragma unroll
            for (int u = 0; u < kBcPer; ++u)
                if (s[u] >= 0) acc[u] += as[h] * row[s[u]];
        }
    };
    for (int32_t g = t0; g < t1; g += stride) {
        const int32_t t = g + lane;
        int32_t w = -1;
        double a = 0.0;
        if (t < t1) {
            const int32_t x = __ldg(p.ac + t);
            if (__ldg(p.inlvl + (x >> 5)) & (1u << (x & 31))) {
                w = x;
                a = UNIT ? 1.0 : __ldg(p.av + t);
            }
        }
        unsigned hits = __ballot_sync(FULL, w >= 0);
        if (MODE == kBcBwdSingle || (MODE == kBcBwdBulk && !ring.ok)) {
            while (hits) {
                const int src = __ffs(hits) - 1;
                hits &= hits - 1;
                const int32_t ww = __shfl_sync(FULL, w, src);
                const double aa = __shfl_sync(FULL, a, src);
                const double* wrow = p.W + (size_t)ww * p.ns;
#pragma unroll
                for (int u = 0; u < kBcPer; ++u)
                    if (s[u] >= 0) acc[u] += aa * wrow[s[u]];
            }
        } else if (MODE == kBcBwdGather) {
            while (hits) {
                int32_t ws[kBcHits];
                double as[kBcHits];
                bc_take_hits(hits, w, a, ws, as);
                double x[kBcHits][kBcPer];
#pragma unroll
                for (int h = 0; h < kBcHits; ++h)
#pragma unroll
                    for (int u = 0; u < kBcPer; ++u)
                        x[h][u] = (ws[h] >= 0 && s[u] >= 0) ? p.W[(size_t)ws[h] * p.ns + s[u]] : 0.0;
#pragma unroll
                for (int h = 0; h < kBcHits; ++h)
                    if (ws[h] >= 0)
#pragma unroll
                        for (int u = 0; u < kBcPer; ++u)
                            if (s[u] >= 0) acc[u] += as[h] * x[h][u];
            }
        } else {
            while (hits) {
                int32_t ws[kBcHits];
                double as[kBcHits];
                const int n = bc_take_hits(hits, w, a, ws, as);
                // the stage is free once every lane has read its previous batch
                __syncwarp();
                if (lane == 0) {
                    const uint32_t bytes = (uint32_t)p.ns * sizeof(double);
                    double* base = ring.rows + (size_t)next_stage * kBcHits * p.ns;
                    fence_proxy_async_smem();
                    mbar_arrive_expect_tx(ring.bar + next_stage, bytes * (uint32_t)n);
#pragma unroll
                    for (int h = 0; h < kBcHits; ++h)
                        if (h < n)
                            bulk_copy_g2s(base + (size_t)h * p.ns, p.W + (size_t)ws[h] * p.ns, bytes,
                                          ring.bar + next_stage);
                }
                if (pend_n) consume(pend_stage, pend_n, pend_a);
                pend_n = n;
                pend_stage = next_stage;
#pragma unroll
                for (int h = 0; h < kBcHits; ++h) pend_a[h] = as[h];
                next_stage ^= 1;
                if (!ring.ok) break;
            }
        }
    }
    if (MODE == kBcBwdBulk && pend_n) {
        if (ring.ok) consume(pend_stage, pend_n, pend_a);
        else (void)mbar_wait(ring.bar + pend_stage, (ring.phase >> pend_stage) & 1u, kBcWaitCycles);
    }
}

// Rows of S[k-1]: acc_s = sum_w A[v][w] * W[w][s] over out-neighbours w that
// sit at level k; bcu += acc*sigma; bc[v] += sum_s acc*sigma. Rows of heavy
// vertices are shared by all warps of a CTA, the others take one warp.
template <bool UNIT, int MODE>
__global__ void __launch_bounds__(kBcThreads, 3) k_bc_backward(BcArgs p) {
    __shared__ double sacc[kBcMaxSources];
    __shared__ double s_vsum;
    extern __shared__ __align__(16) unsigned char bsmem[];
    const int k = p.st->k;
    if (k < 1) return;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int32_t r0 = p.level_rows[k - 1], r1 = p.level_rows[k];
    BcRing ring;
    ring.rows = nullptr;
    ring.bar = nullptr;
    ring.phase = 0;
    ring.ok = true;
    if (MODE == kBcBwdBulk) {
        ring.rows = reinterpret_cast<double*>(bsmem) + (size_t)wid * 2 * kBcHits * p.ns;
        ring.bar = reinterpret_cast<uint64_t*>(bsmem + (size_t)kBcWarps * 2 * kBcHits * p.ns * sizeof(double)) +
                   2 * wid;
        if (lane == 0) {
            mbar_init(ring.bar, 1);
            mbar_init(ring.bar + 1, 1);
            mbar_init_fence();
        }
        __syncwarp();
    }

    // heavy rows (listed by k_bc_set_w), one per CTA at a time: its warps
    // share the row, each warp taking every 8th group of 32 neighbours
    const int nh = p.st->nhrows;
    for (int hr = blockIdx.x; hr < nh; hr += gridDim.x) {
        const int32_t r = p.hrows[hr];
        const int32_t v = p.rv[r];
        const int32_t ab = p.ar[v], ae = p.ar[v + 1];
        const int32_t e0 = p.rs[r], n = p.rl[r];
        for (int e = threadIdx.x; e < n; e += blockDim.x) sacc[e] = 0.0;
        if (threadIdx.x == 0) s_vsum = 0.0;
        __syncthreads();
        for (int base = 0; base < n; base += 32 * kBcPer) {
            int s[kBcPer];
            double acc[kBcPer];
#pragma unroll
            for (int u = 0; u < kBcPer; ++u) {
                const int e = base + u * 32 + lane;
                s[u] = e < n ? p.es[e0 + e] : -1;
                acc[u] = 0.0;
            }
            bc_push_range<UNIT, MODE>(p, ab + wid * 32, ae, kBcWarps * 32, s, acc, ring);
#pragma unroll
            for (int u = 0; u < kBcPer; ++u) {
                const int e = base + u * 32 + lane;
                if (e < n && acc[u] != 0.0) atomicAdd(&sacc[e], acc[u]);
            }
        }
        __syncthreads();
        double part = 0.0;
        for (int e = threadIdx.x; e < n; e += blockDim.x) {
            const double c = sacc[e] * p.ev[e0 + e];
            p.ed[e0 + e] += c;
            part += c;
        }
        part = warp_sum<double>(part);
        if (lane == 0 && part != 0.0) atomicAdd(&s_vsum, part);
        __syncthreads();
        if (threadIdx.x == 0 && s_vsum != 0.0) atomicAdd(&p.bc[v], s_vsum);
        __syncthreads();
    }

    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t r = r0 + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); r < r1; r += warps) {
        const int32_t v = p.rv[r];
        const int32_t ab = p.ar[v], ae = p.ar[v + 1];
        if (ae - ab > kBcHeavyDeg) continue;  // done above
        const int32_t e0 = p.rs[r], n = p.rl[r];
        double vsum = 0.0;
        for (int base = 0; base < n; base += 32 * kBcPer) {
            int s[kBcPer];
            double acc[kBcPer];
#pragma unroll
            for (int u = 0; u < kBcPer; ++u) {
                const int e = base + u * 32 + lane;
                s[u] = e < n ? p.es[e0 + e] : -1;
                acc[u] = 0.0;
            }
            bc_push_range<UNIT, MODE>(p, ab, ae, 32, s, acc, ring);
#pragma unroll
            for (int u = 0; u < kBcPer; ++u) {
                const int e = base + u * 32 + lane;
                if (e < n) {
                    const double c = acc[u] * p.ev[e0 + e];
                    p.ed[e0 + e] += c;
                    vsum += c;
                }
            }
        }
        vsum = warp_sum<double>(vsum);
        if (lane == 0 && vsum != 0.0) atomicAdd(&p.bc[v], vsum);
    }
}

__global__ void k_bc_backward_finalize(BcArgs p, LoopCtl ctl) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    BcState* st = p.st;
    st->nhrows = 0;
    if (st->k >= 1) st->k -= 1;
    loop_continue(ctl, st->k >= 1);
}

// Per vertex (one thread): a self-loop (flags bit 1; rows are sorted, so a
// binary search finds it) and the list of vertices with more than
// kBcHeavyDeg in-neighbours (count in flags[1]).
__global__ void k_bc_scan_vertices(const int32_t* __restrict__ r, const int32_t* __restrict__ c,
                                   const int32_t* __restrict__ tr, int64_t m, int32_t* __restrict__ heavy,
                                   int* __restrict__ flags) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < m; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t b = r[v], n = r[v + 1] - b;
        const int pos = lower_bound_i32(c + b, n, (int32_t)v);
        if (pos < n && c[b + pos] == (int32_t)v) atomicOr(flags, 1);
        if (tr[v + 1] - tr[v] > kBcHeavyDeg) heavy[atomicAdd(flags + 1, 1)] = (int32_t)v;
    }
}

__global__ void k_bc_check_sources(const int32_t* __restrict__ src, int ns, int64_t m, int* __restrict__ mark,
                                   int* __restrict__ flags) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < ns; j += gridDim.x * blockDim.x) {
        int v = src[j];
        if (v < 0 || (int64_t)v >= m) { atomicOr(flags, 8); continue; }
        if (atomicAdd(&mark[v], 1) != 0) atomicOr(flags, 16);
    }
}

// Packed source columns of a batch over a block-diagonal union (device
// arrays): each source's column, the graphs' first rows (count + 1 of them)
// and their source counts; ncols = the largest source count.
struct BcPacking {
    const int32_t* scol = nullptr;
    const int64_t* voff = nullptr;
    const int32_t* gsrc = nullptr;
    int64_t count = 0;
    int ncols = 0;
};

// accumulate: add this batch's scores to d_bc instead of overwriting it.
static void bc_device(ga_ctx ctx, ga_csr A, const int32_t* d_sources, int64_t nsrc, double* d_bc,
                      bool accumulate = false, const BcPacking* pk = nullptr) {
    GA_REQUIRE(A->m == A->n, GA_ERR_SHAPE, "non-square matrix; BC is only for square matrices");
    GA_REQUIRE(nsrc >= 0 && (pk || nsrc <= kBcMaxSources), GA_ERR_INVALID_ARG,
               "BC: between 0 and 1024 sources per batch");
    GA_REQUIRE(!pk || (pk->ncols >= 1 && pk->ncols <= kBcMaxSources), GA_ERR_INVALID_ARG,
               "BC: between 1 and 1024 sources per graph of a batch");
    const int64_t m = A->m;
    if (!accumulate) GA_CUDA(cudaMemsetAsync(d_bc, 0, sizeof(double) * (m ? m : 1), ctx->stream));
    if (m == 0 || nsrc == 0) return;
    const int ns = pk ? pk->ncols : (int)nsrc;  // source columns
    const int words = (ns + 31) / 32;
    GA_REQUIRE(m * (int64_t)(ns + 1) + nsrc < INT32_MAX, GA_ERR_UNSUPPORTED,
               "BC: m x sources exceeds the int32 entry range");
    ProfScope whole(ctx, "bc");
    // Values enter the algebra as FP64. All-ones values are never read (the
    // unit kernels), so A's own arrays serve; otherwise an FP64 copy. A
    // symmetric A is its own transpose. Both properties are cached on the
    // handle after their first check.
    const bool unit = csr_unit_values(ctx, A);
    const bool symmetric = csr_is_symmetric(ctx, A);
    ga_csr Ad = unit ? nullptr : copy_csr(ctx, A, GA_FP64);
    ga_csr AT = nullptr;
    try {
        ga_csr Av = unit ? A : Ad;
        if (!symmetric) AT = transpose_csr(ctx, Av);
        ga_csr ATu = symmetric ? Av : AT;
        DBuf<int> flags(ctx, 2), mark(ctx, (size_t)m);
        DBuf<int32_t> heavy(ctx, (size_t)m + 1);
        GA_CUDA(cudaMemsetAsync(flags.p, 0, 2 * sizeof(int), ctx->stream));
        GA_CUDA(cudaMemsetAsync(mark.p, 0, sizeof(int) * m, ctx->stream));
        k_bc_scan_vertices<<<grid_for(m, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(Av->rst, Av->col, ATu->rst,
                                                                                        m, heavy.p, flags.p);
        post_launch("bc_scan_vertices");
        k_bc_check_sources<<<grid_for(nsrc, 256, 64), 256, 0, ctx->stream>>>(d_sources, (int)nsrc, m, mark.p,
                                                                            flags.p);
        post_launch("bc_check_sources");
        int hf[2];
        GA_CUDA(cudaMemcpyAsync(hf, flags.p, sizeof(hf), cudaMemcpyDeviceToHost, ctx->stream));
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
        const int f = hf[0];
        GA_REQUIRE(!(f & 1), GA_ERR_INVALID_ARG, "BC: the graph has self-loops");
        GA_REQUIRE(!(f & 8), GA_ERR_INVALID_ARG, "BC: source index out of range");
        GA_REQUIRE(!(f & 16), GA_ERR_INVALID_ARG, "BC: sources must be distinct");

        const int64_t cap_entries = m * (int64_t)ns + nsrc;
        const int64_t cap_rows = cap_entries;
        BcArgs p;
        p.atr = ATu->rst; p.atc = ATu->col; p.atv = unit ? nullptr : static_cast<const double*>(ATu->val);
        p.ar = Av->rst; p.ac = Av->col; p.av = unit ? nullptr : static_cast<const double*>(Av->val);
        p.m = m; p.ns = ns; p.words = words; p.sources = d_sources;
        p.nsrc = (int)nsrc; p.scol = pk ? pk->scol : nullptr;
        DBuf<BcState> st(ctx, 1);
        DBuf<int32_t> level_rows(ctx, (size_t)m + 2);
        DBuf<int32_t> cs0(ctx, m), cs1(ctx, m), cl0(ctx, m), cl1(ctx, m), vcnt(ctx, m);
        DBuf<uint32_t> vbits(ctx, (size_t)m * words), inlvl(ctx, (size_t)(m + 31) / 32);
        DBuf<int32_t> es(ctx, (size_t)cap_entries);
        DBuf<double> ev(ctx, (size_t)cap_entries), ed(ctx, (size_t)cap_entries);
        DBuf<int32_t> rv(ctx, (size_t)cap_rows), rs(ctx, (size_t)cap_rows), rl(ctx, (size_t)cap_rows);
        DBuf<double> W(ctx, (size_t)m * ns);
        GA_CUDA(cudaMemsetAsync(cl0.p, 0, sizeof(int32_t) * m, ctx->stream));
        GA_CUDA(cudaMemsetAsync(cl1.p, 0, sizeof(int32_t) * m, ctx->stream));
        GA_CUDA(cudaMemsetAsync(vcnt.p, 0, sizeof(int32_t) * m, ctx->stream));
        GA_CUDA(cudaMemsetAsync(vbits.p, 0, sizeof(uint32_t) * m * words, ctx->stream));
        GA_CUDA(cudaMemsetAsync(inlvl.p, 0, sizeof(uint32_t) * ((m + 31) / 32), ctx->stream));
        GA_CUDA(cudaMemsetAsync(W.p, 0, sizeof(double) * m * ns, ctx->stream));
        p.st = st.p; p.level_rows = level_rows.p;
        p.cur_start[0] = cs0.p; p.cur_start[1] = cs1.p; p.cur_len[0] = cl0.p; p.cur_len[1] = cl1.p;
        p.vbits = vbits.p; p.vcnt = vcnt.p;
        p.es = es.p; p.ev = ev.p; p.ed = ed.p;
        p.rv = rv.p; p.rs = rs.p; p.rl = rl.p;
        p.cap_entries = cap_entries; p.cap_rows = cap_rows;
        p.W = W.p; p.inlvl = inlvl.p; p.bc = d_bc;
        // vertices whose in-neighbour lists are split over a CTA
        p.heavy_in = heavy.p;
        p.nheavy_in = hf[1];

        // push-level state: touched bits, list of reached vertices, marks
        DBuf<uint32_t> tbits(ctx, (size_t)m * words);
        DBuf<int32_t> tlist(ctx, (size_t)m), tmark(ctx, (size_t)m), hrows(ctx, (size_t)m);
        GA_CUDA(cudaMemsetAsync(tbits.p, 0, sizeof(uint32_t) * m * words, ctx->stream));
        GA_CUDA(cudaMemsetAsync(tmark.p, 0, sizeof(int32_t) * m, ctx->stream));
        p.hrows = hrows.p; p.tbits = tbits.p; p.tlist = tlist.p; p.tmark = tmark.p;
        p.nnz = ATu->nnz;
        k_bc_state_init<<<1, 1, 0, ctx->stream>>>(p);
        post_launch("bc_state_init");
        if (pk) {
            k_bc_previsit<<<grid_for(m, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(p, pk->voff, pk->gsrc,
                                                                                       pk->count);
            post_launch("bc_previsit");
        }
        k_bc_init<<<grid_for(nsrc, 256, 64), 256, 0, ctx->stream>>>(p);
        post_launch("bc_init");

        const size_t per_warp = (size_t)ns * sizeof(double) + 2 * (size_t)words * sizeof(uint32_t) +
                                32 * (2 * sizeof(int) + sizeof(double));
        const size_t smem = kBcWarps * ((per_warp + 15) & ~(size_t)15);
        auto fwd = unit ? k_bc_forward<true> : k_bc_forward<false>;
        // The attribute is per kernel, not per call: calls with other source
        // counts may run concurrently (other contexts, other threads), so it
        // is always set to the largest size any call launches with.
        constexpr size_t kMaxWords = (kBcMaxSources + 31) / 32;
        constexpr size_t max_per_warp = (size_t)kBcMaxSources * sizeof(double) + 2 * kMaxWords * sizeof(uint32_t) +
                                        32 * (2 * sizeof(int) + sizeof(double));
        constexpr size_t max_smem = kBcWarps * ((max_per_warp + 15) & ~(size_t)15);
        GA_CUDA(cudaFuncSetAttribute(fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem));
        int per_sm = 1;
        GA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fwd, kBcThreads, smem));
        if (per_sm < 1) per_sm = 1;
        const int grid_fwd = ctx->num_sms * per_sm;
        const int grid_rows = ctx->num_sms * 8;
        {
            ProfScope ps(ctx, "bc_forward_loop");
            auto push = unit ? k_bc_push<true> : k_bc_push<false>;
            run_device_loop(ctx, [&](const LoopCtl& ctl) {
                k_bc_level_begin<<<1, 1, 0, ctx->stream>>>(p);
                post_launch("bc_level_begin");
                {
                    ProfScope pk(ctx, "bc_forward_pull");
                    fwd<<<grid_fwd, kBcThreads, smem, ctx->stream>>>(p);
                    post_launch("bc_forward");
                }
                {
                    ProfScope pk(ctx, "bc_forward_push");
                    push<<<grid_rows, kBcThreads, 0, ctx->stream>>>(p);
                    post_launch("bc_push");
                    k_bc_push_clear<<<grid_for(m, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(p);
                    post_launch("bc_push_clear");
                    k_bc_push_emit<<<grid_rows, kBcThreads, 0, ctx->stream>>>(p);
                    post_launch("bc_push_emit");
                }
                k_bc_forward_finalize<<<1, 32, 0, ctx->stream>>>(p, ctl);
                post_launch("bc_forward_finalize");
            }, m + 2);
        }
        {
            ProfScope ps(ctx, "bc_backward_loop");
            // the bulk form copies whole W rows: 16-byte aligned rows and at
            // most kBcBulkMaxCols columns (its shared-memory ring)
            int mode = ctx->bc_backward;
            if (mode == kBcBwdBulk &&
                (ns % 2 != 0 || ns > kBcBulkMaxCols || (reinterpret_cast<uintptr_t>(p.W) & 15u) != 0))
                mode = kBcBwdGather;
            void (*bwd)(BcArgs) = nullptr;
            size_t bsmem = 0;
            if (mode == kBcBwdBulk) {
                bwd = unit ? k_bc_backward<true, kBcBwdBulk> : k_bc_backward<false, kBcBwdBulk>;
                bsmem = (size_t)kBcWarps * 2 * kBcHits * ns * sizeof(double) + (size_t)kBcWarps * 2 * sizeof(uint64_t);
                constexpr size_t max_bsmem = (size_t)kBcWarps * 2 * kBcHits * kBcBulkMaxCols * sizeof(double) +
                                             (size_t)kBcWarps * 2 * sizeof(uint64_t);
                GA_CUDA(cudaFuncSetAttribute(bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_bsmem));
            } else if (mode == kBcBwdSingle) {
                bwd = unit ? k_bc_backward<true, kBcBwdSingle> : k_bc_backward<false, kBcBwdSingle>;
            } else {
                bwd = unit ? k_bc_backward<true, kBcBwdGather> : k_bc_backward<false, kBcBwdGather>;
            }
            run_device_loop(ctx, [&](const LoopCtl& ctl) {
                k_bc_set_w<<<grid_rows, 256, 0, ctx->stream>>>(p, true);
                post_launch("bc_set_w");
                {
                    ProfScope pk(ctx, "bc_backward");
                    bwd<<<grid_rows, kBcThreads, bsmem, ctx->stream>>>(p);
                    post_launch("bc_backward");
                }
                k_bc_set_w<<<grid_rows, 256, 0, ctx->stream>>>(p, false);
                post_launch("bc_clear_w");
                k_bc_backward_finalize<<<1, 32, 0, ctx->stream>>>(p, ctl);
                post_launch("bc_backward_finalize");
            }, m + 2);
        }
        BcState hs;
        GA_CUDA(cudaMemcpyAsync(&hs, st.p, sizeof(BcState), cudaMemcpyDeviceToHost, ctx->stream));
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
        GA_REQUIRE(!hs.overflow, GA_ERR_INVALID_ARG, "BC: entry store overflow");
        GA_REQUIRE(!hs.stalled, GA_ERR_TIMEOUT, "BC: a bulk copy of the backward sweep did not complete");
    } catch (...) {
        csr_destroy(ctx, AT);
        csr_destroy(ctx, Ad);
        throw;
    }
    csr_destroy(ctx, AT);
    csr_destroy(ctx, Ad);
}

__global__ void k_bc_iota(int32_t* __restrict__ out, int64_t first, int64_t n) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
        out[j] = (int32_t)(first + j);
}

// All-source BC (betweenness_centrality, include/betweenness_centrality.h:
// 5-123): sources 0..m-1 in blocks of `block`, every block's scores added
// into d_bc on the device. The reference adds each block's row sums minus
// the block's size (:103-111), which is the block's dependency sum, as
// bc_device computes it. A block larger than one device batch (1,024
// sources) runs as consecutive batches of at most 1,024: BC is a sum over
// sources, so the block size changes only the order of the additions.
static void bc_all_device(ga_ctx ctx, ga_csr A, int64_t block, double* d_bc) {
    GA_REQUIRE(A->m == A->n, GA_ERR_SHAPE, "non-square matrix; BC is only for square matrices");
    GA_REQUIRE(block >= 1, GA_ERR_INVALID_ARG, "BC: the block size must be at least 1");
    const int64_t m = A->m;
    GA_CUDA(cudaMemsetAsync(d_bc, 0, sizeof(double) * (m ? m : 1), ctx->stream));
    if (m == 0) return;
    const int64_t per = std::min<int64_t>(std::min<int64_t>(block, kBcMaxSources), m);
    DBuf<int32_t> src(ctx, (size_t)per);
    ProfScope ps(ctx, "bc_all");
    for (int64_t i = 0; i < m; i += block) {
        const int64_t n = std::min(block, m - i);
        for (int64_t j = 0; j < n; j += per) {
            const int64_t c = std::min(per, n - j);
            k_bc_iota<<<grid_for(c, 256, 64), 256, 0, ctx->stream>>>(src.p, i + j, c);
            post_launch("bc_iota");
            bc_device(ctx, A, src.p, c, d_bc, true);
        }
    }
}

void bc_union_device(ga_ctx ctx, ga_csr U, int64_t count, const int64_t* voff, const int64_t* soff,
                     const int32_t* sources, double* d_bc) {
    GA_REQUIRE(soff[0] == 0, GA_ERR_INVALID_ARG, "batched BC: source offsets must start at 0");
    const int64_t ns = soff[count];
    GA_REQUIRE(ns >= 0 && (ns == 0 || sources), GA_ERR_INVALID_ARG, "batched BC: sources missing");
    // graph g's sources, shifted to its rows of the union; source j of graph
    // g takes column j
    std::vector<int32_t> global((size_t)(ns > 0 ? ns : 1)), col((size_t)(ns > 0 ? ns : 1));
    std::vector<int32_t> gsrc((size_t)(count > 0 ? count : 1), 0);
    int64_t ncols = 0;
    for (int64_t g = 0; g < count; ++g) {
        GA_REQUIRE(soff[g] <= soff[g + 1], GA_ERR_INVALID_ARG, "batched BC: source offsets must not decrease");
        const int64_t mg = voff[g + 1] - voff[g];
        GA_REQUIRE(soff[g + 1] - soff[g] <= kBcMaxSources, GA_ERR_INVALID_ARG,
                   "batched BC: at most 1024 sources per graph");
        for (int64_t j = soff[g]; j < soff[g + 1]; ++j) {
            GA_REQUIRE(sources[j] >= 0 && sources[j] < mg, GA_ERR_INVALID_ARG, "batched BC: source out of range");
            global[(size_t)j] = (int32_t)(sources[j] + voff[g]);
            col[(size_t)j] = (int32_t)(j - soff[g]);
        }
        gsrc[(size_t)g] = (int32_t)(soff[g + 1] - soff[g]);
        ncols = std::max<int64_t>(ncols, soff[g + 1] - soff[g]);
    }
    if (ns == 0 || U->m == 0) {
        GA_CUDA(cudaMemsetAsync(d_bc, 0, sizeof(double) * (U->m ? U->m : 1), ctx->stream));
        return;
    }
    DBuf<int32_t> d_src(ctx, global.size()), d_col(ctx, col.size()), d_gsrc(ctx, gsrc.size());
    DBuf<int64_t> d_voff(ctx, (size_t)count + 1);
    GA_CUDA(cudaMemcpyAsync(d_src.p, global.data(), sizeof(int32_t) * global.size(), cudaMemcpyHostToDevice,
                            ctx->stream));
    GA_CUDA(cudaMemcpyAsync(d_col.p, col.data(), sizeof(int32_t) * col.size(), cudaMemcpyHostToDevice, ctx->stream));
    GA_CUDA(cudaMemcpyAsync(d_gsrc.p, gsrc.data(), sizeof(int32_t) * gsrc.size(), cudaMemcpyHostToDevice,
                            ctx->stream));
    GA_CUDA(cudaMemcpyAsync(d_voff.p, voff, sizeof(int64_t) * (count + 1), cudaMemcpyHostToDevice, ctx->stream));
    BcPacking pk;
    pk.scol = d_col.p;
    pk.voff = d_voff.p;
    pk.gsrc = d_gsrc.p;
    pk.count = count;
    pk.ncols = (int)ncols;
    bc_device(ctx, U, d_src.p, ns, d_bc, false, &pk);
    // the host vectors stay alive until the copies above are done
    GA_CUDA(cudaStreamSynchronize(ctx->stream));
}

}  // namespace ga

using namespace ga;

extern "C" {

int ga_bc_all(ga_ctx ctx, ga_csr A, int64_t block, double* bc) {
    if (!ctx || !A || !bc) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        DBuf<double> out(ctx, A->m > 0 ? (size_t)A->m : 1);
        bc_all_device(ctx, A, block, out.p);
        if (A->m)
            GA_CUDA(cudaMemcpyAsync(bc, out.p, sizeof(double) * A->m, cudaMemcpyDeviceToHost, ctx->stream));
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int ga_bc_all_device(ga_ctx ctx, ga_csr A, int64_t block, double* d_bc) {
    if (!ctx || !A || !d_bc) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, bc_all_device(ctx, A, block, d_bc));
}

int ga_bc_device(ga_ctx ctx, ga_csr A, const int32_t* d_sources, int64_t nsrc, double* d_bc) {
    if (!ctx || !A || !d_bc || (nsrc > 0 && !d_sources)) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, bc_device(ctx, A, d_sources, nsrc, d_bc));
}

int ga_bc(ga_ctx ctx, ga_csr A, const int32_t* sources, int64_t nsrc, double* bc) {
    if (!ctx || !A || !bc || (nsrc > 0 && !sources)) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        DBuf<int32_t> src(ctx, nsrc > 0 ? (size_t)nsrc : 1);
        DBuf<double> out(ctx, A->m > 0 ? (size_t)A->m : 1);
        if (nsrc > 0)
            GA_CUDA(cudaMemcpyAsync(src.p, sources, sizeof(int32_t) * nsrc, cudaMemcpyHostToDevice, ctx->stream));
        bc_device(ctx, A, src.p, nsrc, out.p);
        if (A->m)
            GA_CUDA(cudaMemcpyAsync(bc, out.p, sizeof(double) * A->m, cudaMemcpyDeviceToHost, ctx->stream));
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

}  // extern "C"
