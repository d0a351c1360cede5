// Triangle-listing form of the support product (GA_TRI): C<A> = A·A for a
// symmetric matrix A whose stored values are all 1 — the product the
// reference's k_truss evaluates every iteration (src/main.cpp:103,
// Tmp<C> = C·C) and whose row sums its triangle counts take.
//
// For such an A, C(i, j) = |N(i) ∩ N(j)| over vertices other than i and j
// (the triangles through edge {i, j}), plus 1 for each of i and j that holds
// a diagonal entry; C(i, i) = |N(i)| (the row's length, diagonal included).
// Every triangle is listed once: vertices get ranks 0..m-1 in order of
// degree (a counting sort, once per call; or their indices), each undirected
// edge is kept in the direction of increasing rank (the oriented list O_u of
// u holds the neighbours ranked above u, in column order), and a triangle
// u < v < w (by rank) is found as the wedge u -> v -> w with w in O_u. Its
// three edges' counts are raised: (u, v) by the entry's hit total, (u, w) in
// shared memory, (v, w) by a global atomic. Integer counts: the result is
// exact whatever the order, and whatever order ties of degree get.
//
// Lookups: each warp keeps a bitmap of O_u's members in a window of kTriWin
// ranks ending at O_u's highest rank, with per-word popcount prefixes giving
// a member's index in O(1); a w ranked below the window is binary-searched
// in O_u. Ranked by degree, almost every wedge of a power-law graph ends at
// a vertex of the top ranks (the hubs), inside the window. The ranks may
// also be the vertex indices (GA_OPT_TRI_ORDER): then the lists of a union
// of small graphs span fewer ranks than the window and no search is needed.
//
// A single evaluation (ga_mxm_masked, triangle counting, the autotuner) builds
// separate oriented lists; all launches read the current entry count on the
// device:
//   orient     rank flags per entry, diagonal flags, work counters
//   scan       flags -> positions in the oriented lists
//   scatter    oriented columns and their ranks, zeroed counts, oriented row
//              starts, tasks per row (kTriTask oriented entries each)
//   scan       tasks per row -> task starts; task list
//   support    one warp per task
//   writeback  counts (+ diagonal terms) to both mirror entries; C(i, i)
// The k-truss loop keeps the orientation in C itself instead (the `trikt`
// kernels at the end of this file): every row is stored as [oriented part |
// the rest] for the whole loop, so an iteration is task list, support, keep
// flags and the prune.
#include "ga_device.cuh"
#include "ga_loop.cuh"

#include <cstddef>

namespace ga {

constexpr int kTriThreads = 128;
constexpr int kTriTask = 16;                  // oriented entries per warp task (at most 32)
constexpr int kTriWin = 1 << 14;              // rank window of the member bitmaps
constexpr int kTriWinWords = kTriWin / 32;    // 512 bitmap words per warp
constexpr int kTriCntMax = 1024;              // longest O_u counted in shared memory
constexpr int kTriCntWords = kTriCntMax / 4;  // byte counters, four per word

// ------------------------------------------------------------------ ranks
// Degrees repeat a lot (a power-law graph has many vertices of degree 0, 1,
// 2, ...), so the lanes of a warp that share a degree are grouped
// (__match_any_sync) and one of them updates the bucket for the group.
__global__ void k_tri_deg_count(const int32_t* __restrict__ cr, int64_t m, int32_t* __restrict__ hist) {
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); b < m; b += stride) {
        const int64_t v = b + lane;
        const int32_t d = v < m ? cr[v + 1] - cr[v] : -1;
        const unsigned grp = __match_any_sync(0xffffffffu, d);
        if (d >= 0 && lane == __ffs(grp) - 1) atomicAdd(hist + d, __popc(grp));
    }
}

// After the scan of the degree histogram: rank = next free place of the
// vertex's degree bucket (a group of lanes with one degree reserves its
// places with one atomic).
__global__ void k_tri_rank(const int32_t* __restrict__ cr, int64_t m, int32_t* __restrict__ next,
                           int32_t* __restrict__ rank) {
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); b < m; b += stride) {
        const int64_t v = b + lane;
        const int32_t d = v < m ? cr[v + 1] - cr[v] : -1;
        const unsigned grp = __match_any_sync(0xffffffffu, d);
        const int leader = __ffs(grp) - 1;
        int32_t base = 0;
        if (d >= 0 && lane == leader) base = atomicAdd(next + d, __popc(grp));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (d >= 0) rank[v] = base + __popc(grp & ((1u << lane) - 1u));
    }
}

__global__ void k_tri_iota(int64_t m, int32_t* __restrict__ rank) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < m; v += (int64_t)gridDim.x * blockDim.x)
        rank[v] = (int32_t)v;
}

// Rank flag of every entry (column ranked above the row: kept in O_row),
// diagonal flags, and the Gustavson work counters the other forms report:
// counts 1, as for a k-truss support that evaluates the upper triangle
// (products of the rows whose upper part is not empty, upper entries); 2, as
// for the whole mask; 0, none (triangle counting).
__global__ void k_tri_orient(const int32_t* __restrict__ cr, const int32_t* __restrict__ cc,
                             const int32_t* __restrict__ row_of, const int32_t* __restrict__ rank, int64_t m,
                             int64_t cap, int32_t* __restrict__ flag, int32_t* __restrict__ diag,
                             unsigned long long* __restrict__ ctr, int counts) {
    const bool upper = counts == 1;
    const int64_t cur = cr[m];
    unsigned long long prod = 0, mask = 0;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < cap; q += (int64_t)gridDim.x * blockDim.x) {
        int32_t f = 0;
        if (q < cur) {
            const int32_t i = row_of[q], j = cc[q];
            if (i == j) diag[i] = 1;
            else f = rank[j] > rank[i];
            if (counts && (!upper || j >= i)) ++mask;
            if (counts && (!upper || cc[cr[i + 1] - 1] >= i)) prod += (unsigned long long)(cr[j + 1] - cr[j]);
        }
        flag[q] = f;
    }
    prod = warp_sum<unsigned long long>(prod);
    mask = warp_sum<unsigned long long>(mask);
    if ((threadIdx.x & 31) == 0) {
        if (prod) atomicAdd(&ctr[GA_CTR_PRODUCTS], prod);
        if (mask) atomicAdd(&ctr[GA_CTR_MASK_ENTRIES], mask);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(&ctr[GA_CTR_LAUNCHES], 1ull);
        atomicAdd(&ctr[GA_CTR_A_ENTRIES], (unsigned long long)cur);
        atomicAdd(&ctr[GA_CTR_ROWS], (unsigned long long)m);
    }
}

// After the scan `pos` of the flags: oriented columns, their ranks and
// zeroed counts at their positions, oriented row starts ost[i] = pos[cr[i]],
// and the number of warp tasks of each row.
__global__ void k_tri_scatter(const int32_t* __restrict__ cr, const int32_t* __restrict__ cc,
                              const int32_t* __restrict__ pos, const int32_t* __restrict__ rank, int64_t m,
                              int32_t* __restrict__ ocol, int32_t* __restrict__ orank, int32_t* __restrict__ sup_o,
                              int32_t* __restrict__ ost, int32_t* __restrict__ ntask) {
    const int64_t cur = cr[m];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < cur || q <= m; q += stride) {
        if (q <= m) {
            const int32_t s = pos[cr[q]];
            ost[q] = s;
            if (q < m) ntask[q] = (pos[cr[q + 1]] - s + kTriTask - 1) / kTriTask;
        }
        if (q < cur) {
            const int32_t d = pos[q];
            if (pos[q + 1] != d) {
                const int32_t j = cc[q];
                ocol[d] = j;
                orank[d] = rank[j];
                sup_o[d] = 0;
            }
        }
    }
}

// Row of every task (tasks of row u: tstart[u] .. tstart[u+1]-1).
__global__ void k_tri_tasklist(const int32_t* __restrict__ tstart, int64_t m, int32_t* __restrict__ task_row) {
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < m; u += (int64_t)gridDim.x * blockDim.x)
        for (int32_t t = tstart[u]; t < tstart[u + 1]; ++t) task_row[t] = (int32_t)u;
}

// One warp per task: up to kTriTask consecutive entries (u, v) of O_u
// (O_u = [ost[u], ost[u+1]), or [ost[u], ost[u] + ocnt[u]) with ocnt). The
// warp marks O_u's members of the rank window [win0, win0 + kTriWin) in its
// bitmap (an O_u longer than kTriCntMax uses 32 bucket splitters in
// registers and a short binary search instead). For each entry v in turn,
// the lanes take 32 entries w of O_v at a time: a member is the triangle
// (u, v, w). Its (u, v) count is the entry's ballot total (one atomic per
// entry), (u, w) a byte counter per member in shared memory (added to the
// oriented counts when the task ends; a task adds at most kTriTask to one
// member), (v, w) a global atomic.
//
// COUNT: triangle counting instead: no edge counts; each triangle adds 1 to
// the total and, with per_row, to the row of its largest vertex index (the
// row sums of C<L> = L·L over the strictly lower triangle L).
template <bool COUNT>
__global__ void __launch_bounds__(kTriThreads, 10) k_tri_support(const int32_t* __restrict__ ost,
                                                             const int32_t* __restrict__ ocnt,
                                                             const int32_t* __restrict__ ocol,
                                                             const int32_t* __restrict__ orank,
                                                             const int32_t* __restrict__ tstart,
                                                             const int32_t* __restrict__ task_row, int64_t m,
                                                             int32_t* __restrict__ sup_o,
                                                             unsigned long long* __restrict__ ctr,
                                                             unsigned long long* __restrict__ total,
                                                             unsigned long long* __restrict__ per_row) {
    // per bitmap word: its member bits (x) and the member index of its first
    // member (y), read together by one 64-bit shared load
    __shared__ uint2 words_s[kTriThreads / 32][kTriWinWords];
    __shared__ uint32_t cnt_s[kTriThreads / 32][kTriCntWords];
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    uint2* words = words_s[threadIdx.x >> 5];
    uint32_t* cnt = cnt_s[threadIdx.x >> 5];
    for (int s = lane; s < kTriWinWords; s += 32) words[s] = make_uint2(0u, 0u);
    for (int s = lane; s < kTriCntWords; s += 32) cnt[s] = 0;
    __syncwarp();
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t ntask = tstart[m];
    unsigned long long wedges = 0, tris = 0;
    for (int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < ntask; c += warps) {
        const int u = task_row[c];
        const int32_t ub = ost[u], un = ocnt ? ocnt[u] : ost[u + 1] - ub;
        const int32_t p0 = ub + (int32_t)(c - tstart[u]) * kTriTask;
        const int ne = min(kTriTask, ub + un - p0);
        const int32_t* Ou = ocol + ub;
        const bool counted = un <= kTriCntMax;
        // the task's entries (u, v) and v's lists, loaded before the bitmap
        // is built so the two chains of loads overlap
        int32_t v = 0, vs = 0, vn = 0;
        if (lane < ne) {
            v = __ldg(ocol + p0 + lane);
            vs = __ldg(ost + v);
            vn = ocnt ? __ldg(ocnt + v) : __ldg(ost + v + 1) - vs;
        }
        int32_t key = 0;
        int n_in = 0;
        // window: the kTriWin ranks up to O_u's highest (all of O_u when its
        // ranks span fewer); members below it are binary-searched
        int32_t win0 = 0;
        int nwords = 0;  // bitmap words the members span
        bool below = false;
        if (counted) {
            int32_t lo = INT32_MAX, hi = -1;
            for (int t = lane; t < un; t += 32) {
                const int32_t r = __ldg(orank + ub + t);
                lo = min(lo, r);
                hi = max(hi, r);
            }
            lo = __reduce_min_sync(FULL, lo);
            hi = __reduce_max_sync(FULL, hi);
            win0 = max(lo, hi - kTriWin + 1);
            below = lo < win0;
            nwords = ((hi - win0) >> 5) + 1;
            for (int t = lane; t < un; t += 32) {
                const int32_t b = __ldg(orank + ub + t) - win0;
                if (b >= 0) atomicOr(&words[b >> 5].x, 1u << (b & 31));
            }
            __syncwarp();
        }
        if (counted && !COUNT) {
            // member index of the first member of every bitmap word
            int run = 0;
            for (int k = 0; k < nwords; k += 32) {
                const int c1 = __popc(words[k + lane].x);
                const int incl = warp_incl_scan(c1);
                words[k + lane].y = (uint32_t)(run + incl - c1);
                run += __shfl_sync(FULL, incl, 31);
            }
            n_in = run;
            __syncwarp();
        } else if (!counted) {
            key = __ldg(Ou + (int)(((int64_t)(lane + 1) * un) >> 5) - 1);
        }
        for (int e = 0; e < ne; ++e) {
            const int32_t evs = __shfl_sync(FULL, vs, e);
            const int32_t evn = __shfl_sync(FULL, vn, e);
            const int32_t ev = __shfl_sync(FULL, v, e);
            uint32_t mine = 0;  // this lane's hits for the entry
            // one round of 32 wedges: the lane's wedge x of the entry, ld its
            // loaded rank (column when the list is not counted); INT32_MAX
            // past the list's end, which no lookup matches
            auto probe = [&](int32_t x, int32_t ld) {
                const int32_t wp = evs + x;
                bool hit = false;
                if (counted) {
                    // ranks above the window are above every member
                    const int32_t b = ld - win0;
                    if ((uint32_t)b < (uint32_t)kTriWin) {
                        const uint2 wd = words[b >> 5];
                        const uint32_t bit = 1u << (b & 31);
                        if (wd.x & bit) {
                            hit = true;
                            if (!COUNT) {
                                const int idx = (int)wd.y + __popc(wd.x & (bit - 1u));
                                atomicAdd(cnt + (idx >> 2), 1u << ((idx & 3) << 3));  // (u, w)
                            }
                        }
                    } else if (b < 0 && below) {
                        // below the window: binary search of O_u by column
                        const int32_t w = __ldg(ocol + wp);
                        const int t = lower_bound_i32(Ou, un, w);
                        if (t < un && __ldg(Ou + t) == w) {
                            hit = true;
                            if (!COUNT) atomicAdd(sup_o + ub + t, 1);  // (u, w)
                        }
                    }
                } else {
                    const int32_t w = ld;
                    const int bb = warp_lower_bound(key, w);
                    if (bb < 32) {
                        const int lo_b = (int)(((int64_t)bb * un) >> 5);
                        const int hi_b = (int)(((int64_t)(bb + 1) * un) >> 5);
                        const int t = lo_b + lower_bound_i32(Ou + lo_b, hi_b - lo_b, w);
                        if (t < hi_b && __ldg(Ou + t) == w) {
                            hit = true;
                            if (!COUNT) atomicAdd(sup_o + ub + t, 1);  // (u, w)
                        }
                    }
                }
                if (!COUNT && hit) atomicAdd(sup_o + wp, 1);  // (v, w)
                if (COUNT && hit && per_row) {
                    const int32_t w = __ldg(ocol + wp);
                    atomicAdd(per_row + max(max(u, ev), w), 1ull);
                }
                mine += hit ? 1u : 0u;
            };
            // two rounds per pass, both loads issued first
            const int32_t* src = counted ? orank : ocol;
            for (int32_t base = 0; base < evn; base += 64) {
                const int32_t x0 = base + lane, x1 = x0 + 32;
                const int32_t l0 = x0 < evn ? __ldg(src + evs + x0) : INT32_MAX;
                const int32_t l1 = x1 < evn ? __ldg(src + evs + x1) : INT32_MAX;
                probe(x0, l0);
                if (base + 32 < evn) probe(x1, l1);  // warp-uniform
            }
            const int32_t found = (int32_t)__reduce_add_sync(FULL, mine);
            if (lane == 0) {
                wedges += (unsigned long long)evn;
                tris += (unsigned long long)found;
                if (!COUNT && found) atomicAdd(sup_o + p0 + e, found);  // (u, v)
            }
        }
        if (counted && COUNT) {
            __syncwarp();
            for (int s = lane; s < nwords; s += 32) words[s] = make_uint2(0u, 0u);
            __syncwarp();
        } else if (counted) {
            __syncwarp();
            for (int t = lane; t < un; t += 32) {
                const int32_t b = __ldg(orank + ub + t) - win0;
                if (b >= 0) {
                    const uint2 wd = words[b >> 5];
                    const int idx = (int)wd.y + __popc(wd.x & ((1u << (b & 31)) - 1u));
                    const uint32_t n = (cnt[idx >> 2] >> ((idx & 3) * 8)) & 0xffu;
                    if (n) atomicAdd(sup_o + ub + t, (int32_t)n);
                }
            }
            __syncwarp();
            for (int s = lane; s < nwords; s += 32) words[s] = make_uint2(0u, 0u);
            for (int s = lane; s < ((n_in + 3) >> 2); s += 32) cnt[s] = 0;
            __syncwarp();
        }
    }
    if (lane == 0) {
        if (wedges) atomicAdd(&ctr[GA_CTR_WEDGES], wedges);
        if (tris) atomicAdd(&ctr[GA_CTR_TRIANGLES], tris);
        if (COUNT && tris) atomicAdd(total, tris);
    }
}

// Support of every entry of C: an oriented entry's count plus the diagonal
// terms goes to it and to its mirror; a diagonal entry gets its row length.
__global__ void k_tri_writeback(const int32_t* __restrict__ cr, const int32_t* __restrict__ cc,
                                const int32_t* __restrict__ row_of, const int32_t* __restrict__ mir,
                                const int32_t* __restrict__ pos, const int32_t* __restrict__ sup_o,
                                const int32_t* __restrict__ diag, int64_t m, int32_t* __restrict__ sup) {
    const int64_t cur = cr[m];
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < cur; q += (int64_t)gridDim.x * blockDim.x) {
        const int32_t i = row_of[q], j = cc[q];
        if (i == j) {
            sup[q] = cr[i + 1] - cr[i];
            continue;
        }
        const int32_t d = pos[q];
        if (pos[q + 1] != d) {
            const int32_t s = sup_o[d] + diag[i] + diag[j];
            sup[q] = s;
            sup[mir[q]] = s;
        }
    }
}

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

namespace {
struct TriScratch {
    int32_t *ocol, *orank, *sup_o, *task_row, *ost, *tstart, *diag, *rank;
    void* scan_scr;
};

size_t task_cap(int64_t m, int64_t cap) { return (size_t)(cap / kTriTask + m + 1); }

// Carves the buffers out of `scratch` (nullptr: only sizes them); returns
// the bytes used.
size_t carve(void* scratch, int64_t m, int64_t cap, TriScratch* t) {
    const size_t c = (size_t)(cap > 0 ? cap : 1), r = (size_t)m + 2;
    unsigned char* base = static_cast<unsigned char*>(scratch);
    size_t off = 0;
    auto take = [&](size_t count) {
        int32_t* p = base ? reinterpret_cast<int32_t*>(base + off) : nullptr;
        off += align256(sizeof(int32_t) * count);
        return p;
    };
    TriScratch s;
    s.ocol = take(c);
    s.orank = take(c);
    s.sup_o = take(c);
    s.task_row = take(task_cap(m, cap));
    s.ost = take(r);
    s.tstart = take(r);
    s.diag = take(r);
    s.rank = take(r);
    s.scan_scr = base ? base + off : nullptr;
    off += align256(scan_scratch_bytes((cap > m ? cap : m) + 2));
    if (t) *t = s;
    return off;
}
}  // namespace

size_t tri_scratch_bytes(int64_t m, int64_t cap) { return carve(nullptr, m, cap, nullptr); }

void tri_prepare(ga_ctx ctx, ga_csr C, void* scratch, int64_t cap) {
    const int64_t m = C->m;
    if (m == 0) return;
    TriScratch t;
    carve(scratch, m, cap, &t);
    const int grid = grid_for(m, 256, ctx->num_sms * 8);
    if (ctx->tune.tri_order == 1) {  // index order
        k_tri_iota<<<grid, 256, 0, ctx->stream>>>(m, t.rank);
        post_launch("tri_iota");
        return;
    }
    // ranks by degree: histogram of the degrees (0..m), its scan, then each
    // vertex takes the next place of its degree's bucket
    int32_t* hist = t.tstart;
    GA_CUDA(cudaMemsetAsync(hist, 0, sizeof(int32_t) * (size_t)(m + 2), ctx->stream));
    k_tri_deg_count<<<grid, 256, 0, ctx->stream>>>(C->rst, m, hist);
    post_launch("tri_deg_count");
    scan_exclusive_i32_scratch(ctx, hist, hist, m + 1, t.scan_scr);
    k_tri_rank<<<grid, 256, 0, ctx->stream>>>(C->rst, m, hist, t.rank);
    post_launch("tri_rank");
}

// Orientation, oriented lists and the task list of C's current pattern.
static void tri_lists(ga_ctx ctx, ga_csr C, const int32_t* row_of, int32_t* pos, const TriScratch& t, int64_t cap,
                      int counts) {
    const int64_t m = C->m;
    const int grid_ent = grid_for(cap, 256, ctx->num_sms * 16);
    const int grid_copy = grid_for(m + cap, 256, ctx->num_sms * 8);
    const int grid_rows = grid_for(m, 256, ctx->num_sms * 8);
    ProfScope ps(ctx, "tri_orient");
    GA_CUDA(cudaMemsetAsync(t.diag, 0, sizeof(int32_t) * (size_t)m, ctx->stream));
    k_tri_orient<<<grid_ent, 256, 0, ctx->stream>>>(C->rst, C->col, row_of, t.rank, m, cap, pos, t.diag,
                                                    ctx->d_counters, counts);
    post_launch("tri_orient");
    scan_exclusive_i32_scratch(ctx, pos, pos, cap, t.scan_scr);
    k_tri_scatter<<<grid_copy, 256, 0, ctx->stream>>>(C->rst, C->col, pos, t.rank, m, t.ocol, t.orank, t.sup_o,
                                                      t.ost, t.tstart);
    post_launch("tri_scatter");
    scan_exclusive_i32_scratch(ctx, t.tstart, t.tstart, m, t.scan_scr);
    k_tri_tasklist<<<grid_rows, 256, 0, ctx->stream>>>(t.tstart, m, t.task_row);
    post_launch("tri_tasklist");
}

// Persistent grid: as many blocks as are resident at once.
template <bool COUNT>
static int tri_blocks_per_sm() {
    static const int per_sm = [] {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_tri_support<COUNT>, kTriThreads, 0) != cudaSuccess ||
            b < 1)
            b = 1;
        return b;
    }();
    return per_sm;
}

void tri_support_launch(ga_ctx ctx, ga_csr C, const int32_t* row_of, const int32_t* mir, int32_t* pos,
                        int32_t* sup, void* scratch, int64_t cap, bool upper_counts) {
    const int64_t m = C->m;
    if (m == 0) return;
    TriScratch t;
    carve(scratch, m, cap, &t);
    tri_lists(ctx, C, row_of, pos, t, cap, upper_counts ? 1 : 2);
    {
        ProfScope ps(ctx, "tri_support");
        k_tri_support<false><<<ctx->num_sms * tri_blocks_per_sm<false>(), kTriThreads, 0, ctx->stream>>>(
            t.ost, nullptr, t.ocol, t.orank, t.tstart, t.task_row, m, t.sup_o, ctx->d_counters, nullptr, nullptr);
        post_launch("tri_support");
    }
    ProfScope ps(ctx, "tri_writeback");
    k_tri_writeback<<<grid_for(cap, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(C->rst, C->col, row_of, mir,
                                                                                   pos, t.sup_o, t.diag, m, sup);
    post_launch("tri_writeback");
}

void tri_count(ga_ctx ctx, ga_csr A, unsigned long long* d_total, unsigned long long* d_per_row) {
    const int64_t m = A->m, cap = A->nnz;
    if (d_per_row) GA_CUDA(cudaMemsetAsync(d_per_row, 0, sizeof(int64_t) * (size_t)m, ctx->stream));
    if (m == 0 || cap == 0) return;
    DBuf<int32_t> row_of(ctx, (size_t)cap), pos(ctx, (size_t)cap + 1);
    DBuf<unsigned char> scr(ctx, tri_scratch_bytes(m, cap));
    TriScratch t;
    carve(scr.p, m, cap, &t);
    expand_rows(ctx, A, row_of.p);
    tri_prepare(ctx, A, scr.p, cap);
    tri_lists(ctx, A, row_of.p, pos.p, t, cap, 0);
    ProfScope ps(ctx, "tri_count");
    k_tri_support<true><<<ctx->num_sms * tri_blocks_per_sm<true>(), kTriThreads, 0, ctx->stream>>>(
        t.ost, nullptr, t.ocol, t.orank, t.tstart, t.task_row, m, nullptr, ctx->d_counters, d_total, d_per_row);
    post_launch("tri_count");
}

bool tri_applies(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr M) {
    const bool same = (A == B || (A->rst == B->rst && A->col == B->col && A->val == B->val)) &&
                      (A == M || (A->rst == M->rst && A->col == M->col));
    return same && A->dtype == GA_INT32 && csr_is_symmetric(ctx, A) && csr_unit_values(ctx, A);
}

// C<A> = A·A by triangle listing into values aligned with A's pattern.
void tri_masked_into(ga_ctx ctx, ga_csr A, int32_t* sup) {
    const int64_t m = A->m, cap = A->nnz;
    if (m == 0 || cap == 0) return;
    DBuf<int32_t> row_of(ctx, (size_t)cap), mir(ctx, (size_t)cap), pos(ctx, (size_t)cap + 1);
    DBuf<unsigned char> scr(ctx, tri_scratch_bytes(m, cap));
    expand_rows(ctx, A, row_of.p);
    mirror_index(ctx, A, row_of.p, mir.p);
    tri_prepare(ctx, A, scr.p, cap);
    tri_support_launch(ctx, A, row_of.p, mir.p, pos.p, sup, scr.p, cap, false);
}

// =============================================== resident orientation (k-truss)
// Entry q of the unpartitioned C (column order) goes to the oriented part of
// its row when its column is ranked above the row.
__global__ void k_trikt_part_flags(const int32_t* __restrict__ cr, const int32_t* __restrict__ cc,
                                   const int32_t* __restrict__ row_of, const int32_t* __restrict__ rank, int64_t m,
                                   int64_t cap, int32_t* __restrict__ flag) {
    const int64_t cur = cr[m];
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < cap; q += (int64_t)gridDim.x * blockDim.x) {
        int32_t f = 0;
        if (q < cur) {
            const int32_t i = row_of[q], j = cc[q];
            f = i != j && rank[j] > rank[i];
        }
        flag[q] = f;
    }
}

// After the flags' scan: stable partition of every row (oriented part, then
// the rest), the rank of every placed column, and per row its oriented count
// and tasks.
__global__ void k_trikt_part_place(const int32_t* __restrict__ cr, const int32_t* __restrict__ cc,
                                   const int32_t* __restrict__ row_of, const int32_t* __restrict__ rank,
                                   const int32_t* __restrict__ pos, int64_t m, int32_t* __restrict__ out_col,
                                   int32_t* __restrict__ crank, int32_t* __restrict__ ocount,
                                   int32_t* __restrict__ ntask) {
    const int64_t cur = cr[m];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < cur || q < m; q += stride) {
        if (q < m) {
            const int32_t oc = pos[cr[q + 1]] - pos[cr[q]];
            ocount[q] = oc;
            ntask[q] = (oc + kTriTask - 1) / kTriTask;
        }
        if (q < cur) {
            const int32_t i = row_of[q], rb = cr[i];
            const int32_t before = pos[q] - pos[rb];            // oriented entries before q in its row
            const int32_t oc = pos[cr[i + 1]] - pos[rb];
            const bool o = pos[q + 1] != pos[q];
            const int32_t np = o ? rb + before : rb + oc + (int32_t)(q - rb) - before;
            const int32_t j = cc[q];
            out_col[np] = j;
            crank[np] = rank[j];
        }
    }
}

// Mirror of every entry and each row's diagonal position in the partitioned
// layout: (j, i) lies in the oriented part of row j when i is ranked above j.
__global__ void k_trikt_part_mirror(const int32_t* __restrict__ cr, const int32_t* __restrict__ cc,
                                    const int32_t* __restrict__ row_of, const int32_t* __restrict__ crank,
                                    const int32_t* __restrict__ ocount, int64_t nnz, int32_t* __restrict__ mir,
                                    int32_t* __restrict__ dpos) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x) {
        const int32_t i = row_of[q], j = cc[q];
        if (i == j) {
            dpos[i] = (int32_t)q;
            mir[q] = (int32_t)q;
            continue;
        }
        // rank of i: the mirror's rank; q is oriented in row i iff rank(j) > rank(i)
        const bool q_oriented = (int64_t)q - cr[i] < ocount[i];
        const int32_t b = q_oriented ? cr[j] + ocount[j] : cr[j];  // i ranks below j: the rest of row j
        const int32_t e = q_oriented ? cr[j + 1] : cr[j] + ocount[j];
        mir[q] = b + lower_bound_i32(cc + b, e - b, i);
    }
}

// Keep flags: an oriented entry's support is its count, another entry's the
// count of its mirror (plus one per diagonal entry of its two rows); a
// diagonal entry's support is its row's length. Work counters as for an
// upper-triangle support product.
__global__ void k_trikt_flags(const int32_t* __restrict__ cr, const int32_t* __restrict__ cc,
                              const int32_t* __restrict__ row_of, const int32_t* __restrict__ mir,
                              const int32_t* __restrict__ ocount, const int32_t* __restrict__ dpos,
                              const int32_t* __restrict__ sup, int64_t m, int64_t cap, int k,
                              const int32_t* __restrict__ gid, const int32_t* __restrict__ done_g,
                              const int32_t* __restrict__ kg, int32_t* __restrict__ flag,
                              unsigned long long* __restrict__ ctr) {
    const int64_t cur = cr[m];
    unsigned long long prod = 0, mask = 0;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < cap; q += (int64_t)gridDim.x * blockDim.x) {
        int32_t keep = 0;
        if (q < cur) {
            const int32_t i = row_of[q], j = cc[q];
            const int32_t rb = cr[i], re = cr[i + 1], oc = ocount[i];
            int32_t s;
            if (i == j) s = re - rb;
            else s = sup[q - rb < oc ? q : mir[q]] + (dpos[i] >= 0) + (dpos[j] >= 0);
            if (kg) {
                const int g = gid[i];
                keep = done_g[g] != 0 || s >= kg[g] - 2;
            } else {
                keep = s >= k - 2;
                if (!keep && gid) keep = done_g[gid[i]] != 0;
            }
            // the row's largest column: the last of either part
            const int32_t cmax = max(oc > 0 ? cc[rb + oc - 1] : -1, re > rb + oc ? cc[re - 1] : -1);
            if (j >= i) ++mask;
            if (cmax >= i) prod += (unsigned long long)(cr[j + 1] - cr[j]);
        }
        flag[q] = keep;
    }
    prod = warp_sum<unsigned long long>(prod);
    mask = warp_sum<unsigned long long>(mask);
    if ((threadIdx.x & 31) == 0) {
        if (prod) atomicAdd(&ctr[GA_CTR_PRODUCTS], prod);
        if (mask) atomicAdd(&ctr[GA_CTR_MASK_ENTRIES], mask);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(&ctr[GA_CTR_LAUNCHES], 1ull);
        atomicAdd(&ctr[GA_CTR_A_ENTRIES], (unsigned long long)cur);
        atomicAdd(&ctr[GA_CTR_ROWS], (unsigned long long)m);
    }
}

// After the flags' scan: kept entries move to pos[q] (columns, rows, column
// ranks), pos_new[q] is the new position or -1, the new row starts are
// tr[i] = pos[cr[i]]; per row the oriented count shrinks to the kept
// oriented entries (updated in place: unchanged when nothing was pruned) and
// the next iteration's task count follows.
__global__ void k_trikt_scatter(const int32_t* __restrict__ cr, const int32_t* __restrict__ cc,
                                const int32_t* __restrict__ pos, const int32_t* __restrict__ row_of,
                                const int32_t* __restrict__ crank, int64_t m, int32_t* __restrict__ ocount,
                                int32_t* __restrict__ ntask, int32_t* __restrict__ tc, int32_t* __restrict__ tr,
                                int32_t* __restrict__ pos_new, int32_t* __restrict__ trow,
                                int32_t* __restrict__ tcrank, const int32_t* __restrict__ gid,
                                const int32_t* __restrict__ done_g) {
    const int64_t cur = cr[m];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < cur || q <= m; q += stride) {
        if (q <= m) {
            tr[q] = pos[cr[q]];
            if (q < m) {
                const int32_t rb = cr[q];
                const int32_t oc = pos[rb + ocount[q]] - pos[rb];
                ocount[q] = oc;
                // rows of finished graphs (batches) need no more support
                ntask[q] = gid && done_g[gid[q]] ? 0 : (oc + kTriTask - 1) / kTriTask;
            }
        }
        if (q < cur) {
            const int32_t d = pos[q];
            const bool keep = pos[q + 1] != d;
            if (keep) {
                tc[d] = cc[q];
                trow[d] = row_of[q];
                tcrank[d] = crank[q];
            }
            pos_new[q] = keep ? d : -1;
        }
    }
}

// When the iteration swapped: C <- the pruned matrix (row starts, columns,
// values 1), and the per-entry arrays (rows, mirrors, column ranks) and the
// diagonal positions follow it; one launch for all of them.
__global__ void k_trikt_copyback(const KtState* st, int64_t m, const int32_t* __restrict__ tr,
                                 const int32_t* __restrict__ tc, const int32_t* __restrict__ trow,
                                 const int32_t* __restrict__ mir_new, const int32_t* __restrict__ pos_new,
                                 const int32_t* __restrict__ tcrank, int32_t* __restrict__ cr,
                                 int32_t* __restrict__ cc, int32_t* __restrict__ cv, int32_t* __restrict__ row_of,
                                 int32_t* __restrict__ mir, int32_t* __restrict__ crank,
                                 int32_t* __restrict__ dpos) {
    if (!st->swapped) return;
    const int64_t nnz = st->nnz;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nnz || q <= m; q += stride) {
        if (q <= m) cr[q] = tr[q];
        if (q < m && dpos[q] >= 0) dpos[q] = pos_new[dpos[q]];
        if (q < nnz) {
            cc[q] = tc[q];
            cv[q] = 1;
            row_of[q] = trow[q];
            mir[q] = mir_new[q];
            crank[q] = tcrank[q];
        }
    }
}

// Rows back in column order: an entry's place in its row is its index in its
// part plus the entries of the other part with smaller columns.
__global__ void k_trikt_unpart(const int32_t* __restrict__ cr, const int32_t* __restrict__ cc,
                               const int32_t* __restrict__ row_of, const int32_t* __restrict__ ocount, int64_t nnz,
                               int32_t* __restrict__ out_col) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x) {
        const int32_t i = row_of[q], rb = cr[i], re = cr[i + 1], oc = ocount[i];
        const int32_t k = (int32_t)(q - rb);
        const bool o = k < oc;
        const int32_t ob = o ? rb + oc : rb, oe = o ? re : rb + oc;
        const int32_t j = cc[q];
        out_col[rb + (o ? k : k - oc) + lower_bound_i32(cc + ob, oe - ob, j)] = j;
    }
}

namespace {
size_t trikt_carve(void* scratch, int64_t m, int64_t cap, TriKt* t) {
    const size_t c = (size_t)(cap > 0 ? cap : 1), r = (size_t)m + 2;
    unsigned char* base = static_cast<unsigned char*>(scratch);
    size_t off = 0;
    auto take = [&](size_t count) {
        int32_t* p = base ? reinterpret_cast<int32_t*>(base + off) : nullptr;
        off += align256(sizeof(int32_t) * count);
        return p;
    };
    TriKt s;
    s.crank = take(c);
    s.tcrank = take(c);
    s.ocount = take(r);
    s.tstart = take(r);
    s.task_row = take(task_cap(m, cap));
    s.dpos = take(r);
    s.scan_scr = base ? base + off : nullptr;
    off += align256(scan_scratch_bytes((cap > m ? cap : m) + 2));
    if (t) *t = s;
    return off;
}
}  // namespace

size_t tri_kt_bytes(int64_t m, int64_t cap) { return trikt_carve(nullptr, m, cap, nullptr); }

void tri_kt_carve(void* scratch, int64_t m, int64_t cap, TriKt* t) { trikt_carve(scratch, m, cap, t); }

void tri_kt_setup(ga_ctx ctx, ga_csr C, const int32_t* row_of, int32_t* mir, int32_t* tmp_col, int32_t* tmp_flag,
                  const TriKt& t, int64_t cap) {
    const int64_t m = C->m, nnz = C->nnz;
    // ranks by degree (or index) into task_row, which the loop fills later
    int32_t* rank = t.task_row;
    const int grid_v = grid_for(m, 256, ctx->num_sms * 8);
    if (ctx->tune.tri_order == 1) {
        k_tri_iota<<<grid_v, 256, 0, ctx->stream>>>(m, rank);
        post_launch("tri_iota");
    } else {
        GA_CUDA(cudaMemsetAsync(t.tstart, 0, sizeof(int32_t) * (size_t)(m + 2), ctx->stream));
        k_tri_deg_count<<<grid_v, 256, 0, ctx->stream>>>(C->rst, m, t.tstart);
        post_launch("tri_deg_count");
        scan_exclusive_i32_scratch(ctx, t.tstart, t.tstart, m + 1, t.scan_scr);
        k_tri_rank<<<grid_v, 256, 0, ctx->stream>>>(C->rst, m, t.tstart, rank);
        post_launch("tri_rank");
    }
    const int grid_ent = grid_for(cap, 256, ctx->num_sms * 16);
    k_trikt_part_flags<<<grid_ent, 256, 0, ctx->stream>>>(C->rst, C->col, row_of, rank, m, cap, tmp_flag);
    post_launch("trikt_part_flags");
    scan_exclusive_i32_scratch(ctx, tmp_flag, tmp_flag, cap, t.scan_scr);
    k_trikt_part_place<<<grid_for(m + cap, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(
        C->rst, C->col, row_of, rank, tmp_flag, m, tmp_col, t.crank, t.ocount, t.tstart);
    post_launch("trikt_part_place");
    if (nnz) GA_CUDA(cudaMemcpyAsync(C->col, tmp_col, sizeof(int32_t) * (size_t)nnz, cudaMemcpyDeviceToDevice,
                                     ctx->stream));
    GA_CUDA(cudaMemsetAsync(t.dpos, 0xff, sizeof(int32_t) * (size_t)m, ctx->stream));
    if (nnz) {
        k_trikt_part_mirror<<<grid_for(nnz, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(
            C->rst, C->col, row_of, t.crank, t.ocount, nnz, mir, t.dpos);
        post_launch("trikt_part_mirror");
    }
}

void tri_kt_support(ga_ctx ctx, ga_csr C, int32_t* sup, const TriKt& t, int64_t cap) {
    const int64_t m = C->m;
    {
        ProfScope ps(ctx, "tri_orient");
        GA_CUDA(cudaMemsetAsync(sup, 0, sizeof(int32_t) * (size_t)cap, ctx->stream));
        scan_exclusive_i32_scratch(ctx, t.tstart, t.tstart, m, t.scan_scr);
        k_tri_tasklist<<<grid_for(m, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(t.tstart, m, t.task_row);
        post_launch("tri_tasklist");
    }
    ProfScope ps(ctx, "tri_support");
    k_tri_support<false><<<ctx->num_sms * tri_blocks_per_sm<false>(), kTriThreads, 0, ctx->stream>>>(
        C->rst, t.ocount, C->col, t.crank, t.tstart, t.task_row, m, sup, ctx->d_counters, nullptr, nullptr);
    post_launch("tri_support");
}

void tri_kt_flags(ga_ctx ctx, ga_csr C, const int32_t* row_of, const int32_t* mir, const int32_t* sup,
                  const TriKt& t, int64_t cap, int k, const KtBatch* batch, int32_t* flag) {
    k_trikt_flags<<<grid_for(cap, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(
        C->rst, C->col, row_of, mir, t.ocount, t.dpos, sup, C->m, cap, k, batch ? batch->gid : nullptr,
        batch ? batch->done_g : nullptr, batch ? batch->kg : nullptr, flag, ctx->d_counters);
    post_launch("trikt_flags");
}

void tri_kt_scatter(ga_ctx ctx, ga_csr C, const int32_t* pos, const int32_t* row_of, const TriKt& t, int64_t cap,
                    int32_t* tc, int32_t* tr, int32_t* pos_new, int32_t* trow, const KtBatch* batch) {
    k_trikt_scatter<<<grid_for(C->m + cap, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(
        C->rst, C->col, pos, row_of, t.crank, C->m, t.ocount, t.tstart, tc, tr, pos_new, trow, t.tcrank,
        batch ? batch->gid : nullptr, batch ? batch->done_g : nullptr);
    post_launch("trikt_scatter");
}

void tri_kt_copyback(ga_ctx ctx, ga_csr C, const KtState* st, const int32_t* tr, const int32_t* tc,
                     const int32_t* trow, const int32_t* mir_new, const int32_t* pos_new, int32_t* row_of,
                     int32_t* mir, const TriKt& t, int64_t cap) {
    k_trikt_copyback<<<grid_for(C->m + cap, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(
        st, C->m, tr, tc, trow, mir_new, pos_new, t.tcrank, C->rst, C->col, static_cast<int32_t*>(C->val), row_of,
        mir, t.crank, t.dpos);
    post_launch("trikt_copyback");
}

void tri_kt_finish(ga_ctx ctx, ga_csr C, const int32_t* row_of, const TriKt& t, int32_t* tmp_col) {
    const int64_t nnz = C->nnz;
    if (nnz == 0) return;
    k_trikt_unpart<<<grid_for(nnz, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(C->rst, C->col, row_of, t.ocount,
                                                                                   nnz, tmp_col);
    post_launch("trikt_unpart");
    GA_CUDA(cudaMemcpyAsync(C->col, tmp_col, sizeof(int32_t) * (size_t)nnz, cudaMemcpyDeviceToDevice, ctx->stream));
}

// ======================================== frontier k-truss (one matrix)
// The reference's k_truss recomputes the whole support every iteration
// (src/main.cpp:100-127). Between iterations only the triangles that lose
// an edge change, so after one listing the loop keeps the supports and, per
// iteration t with C_t its edges and s_t their exact supports:
//   F_t  = edges of C_t with s_t < k - 2 (iteration 0: found by one pass over
//          the entries; later: the edges whose support crossed below k - 2
//          in iteration t - 1, which are exactly the ones below it);
//   every triangle of C_t with an edge in F_t is destroyed: each of its edges
//          outside F_t loses 1, counted once by the triangle's F_t edge with
//          the smallest id (the position of its oriented entry); an entry
//          (i, i) in F_t lowers every edge of row i by 1 instead, and an edge
//          in F_t shortens its two rows, which lowers their diagonal entries;
//   C_{t+1} = C_t minus F_t; stop when F_t is empty (iteration count t + 1)
//          or after m iterations (count 0), as the reference does.
// Entries never move during the loop: an edge lives at its oriented entry
// (state alive / in F_t / gone, support), the other entry points to it
// (oid); one compaction at the end writes the kept entries in column order.
// A pruned edge's triangles are found by walking the shorter of its two rows
// and binary-searching the other (in the part its rank selects), stopping
// once its support's worth of triangles is found.
//
// Work counters: iteration t adds the Gustavson products of the reference's
// Tmp<C> = C_t*C_t over the rows with an upper part, P_t = sum over entries
// (i, j) of C_t of h(i) deg(j) (h(i): row i has a column >= i; deg: row
// lengths) = sum_j deg(j) H(j), H(j) = entries (i, j) with h(i) = 1. P is
// kept as a running total: an iteration changes deg and H only at the
// endpoints of its pruned edges and, when a row loses its last upper entry
// (once per row and call), at that row's remaining neighbours; those
// vertices' terms are recomputed, so no iteration passes over all entries.
namespace {

enum : uint8_t { kAlive = 0, kDying = 1, kGone = 2 };

struct TriFrontState {
    int32_t cnt[2];              // frontier sizes; the current one is cnt[t & 1]
    int32_t t;                   // iteration
    int32_t iters;               // reported iteration count
    int32_t done;
    int32_t ntouch;              // vertices whose terms of P change this iteration
    int32_t nflip;               // rows that lost their last upper entry
    int32_t nseg;                // segments of long rows listed this iteration
    uint32_t blocks_done;        // delta kernel: blocks finished
    uint32_t blocks_done_g;      // graph kernel (batches): blocks finished
    int32_t live;                // batches: graphs still iterating
    unsigned long long prod;     // P_t (batches: summed over the live graphs)
    unsigned long long mask;     // entries (i, j) of C_t with j >= i
    unsigned long long ent;      // entries of C_t
};

struct TriFrontArgs {
    const int32_t* cr;      // row starts (fixed during the loop)
    const int32_t* cc;      // columns, every row as [oriented part | rest]
    const int32_t* row_of;
    const int32_t* mir;
    const int32_t* crank;   // rank of each entry's column
    const int32_t* ocount;
    const int32_t* dpos;    // position of each row's diagonal entry, -1 if none
    int32_t* oid;           // entry -> position of its edge's record
    int32_t* sup;           // supports at the records
    uint8_t* state;         // states at the records
    int32_t* deg;           // entries of each row still in C
    int32_t* upc;           // of those, the ones with column >= row
    uint8_t* h;             // upc > 0, as of the iteration's start
    int32_t* H;             // per vertex: entries (i, j) of C with h(i) = 1
    int32_t* rd;            // per vertex: entries its row lost this iteration
    int32_t* rh;            // per vertex: what H lost this iteration
    int32_t* mark;          // per vertex: listed in touched
    int32_t* touched;
    int32_t* flip;
    int32_t* f0;
    int32_t* f1;
    int2* seg;              // segments of long rows: (frontier slot, segment)
    int32_t* efound;        // per frontier slot: triangles its segments found
    int64_t segcap;
    TriFrontState* st;
    unsigned long long* ctr;
    int64_t m;
    int64_t nnz;
    int k;
    // batches of graphs (block-diagonal union; gid == nullptr: one matrix)
    const int32_t* gid;     // graph of each row
    const int32_t* kg;      // per-graph k (nullptr: k for every graph)
    const int32_t* nvert;   // vertices per graph
    int32_t* done_g;        // graph finished (converged, or stopped after n_g iterations)
    int32_t* iters_g;       // reported iteration count per graph
    int32_t* cntg;          // 2 x ngraphs: frontier elements per graph, by iteration parity
    long long* pg;          // P per graph
    int64_t ngraphs;
};

__device__ __forceinline__ void front_push(int32_t* buf, int32_t* cnt, int32_t x) { buf[atomicAdd(cnt, 1)] = x; }

// k - 2 for the graph of row i
__device__ __forceinline__ int kt_thr(const TriFrontArgs& a, int32_t i) {
    return (a.kg ? a.kg[a.gid[i]] : a.k) - 2;
}

// A frontier element of row i for iteration parity par (batches also count
// it for the row's graph).
__device__ __forceinline__ void front_add(const TriFrontArgs& a, int32_t* buf, int32_t* cnt, int32_t x, int32_t i,
                                          int par) {
    front_push(buf, cnt, x);
    if (a.gid) atomicAdd(a.cntg + par * a.ngraphs + a.gid[i], 1);
}

// Batches: the element's graph finished (a graph stopped by its iteration
// bound keeps its edges; its queued elements are dropped).
__device__ __forceinline__ bool kt_frozen(const TriFrontArgs& a, int32_t i) {
    return a.gid && a.done_g[a.gid[i]];
}

// One support unit less; the edge joins the next frontier when it drops below k - 2.
__device__ __forceinline__ void lower_support(const TriFrontArgs& a, int32_t f, int32_t* fn, int32_t* cn, int par) {
    const int32_t i = a.row_of[f];
    if (atomicSub(a.sup + f, 1) == kt_thr(a, i)) front_add(a, fn, cn, f, i, par);
}

__device__ __forceinline__ void touch(const TriFrontArgs& a, int32_t x) {
    if (atomicExch(a.mark + x, 1) == 0) front_push(a.touched, &a.st->ntouch, x);
}

__global__ void k_trif_init_rows(TriFrontArgs a) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.m; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t b = a.cr[i], e = a.cr[i + 1], oc = a.ocount[i];
        const int32_t up = (oc - lower_bound_i32(a.cc + b, oc, (int32_t)i)) +
                           (e - b - oc - lower_bound_i32(a.cc + b + oc, e - b - oc, (int32_t)i));
        a.deg[i] = e - b;
        a.upc[i] = up;
        a.h[i] = up > 0;
        a.rd[i] = 0;
        a.rh[i] = 0;
        a.mark[i] = 0;
    }
}

// Records of the edges (the oriented entry; a diagonal entry is its own),
// states, the diagonal terms of the listed supports, and the first frontier.
__global__ void k_trif_seed(TriFrontArgs a) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < a.nnz; q += (int64_t)gridDim.x * blockDim.x) {
        const int32_t i = a.row_of[q], j = a.cc[q];
        const bool rec = i == j || (int64_t)q - a.cr[i] < a.ocount[i];
        a.oid[q] = rec ? (int32_t)q : a.mir[q];
        a.state[q] = kAlive;
        // one matrix: a record of the first frontier is marked at once
        // (batches mark theirs in k_trif_mark)
        if (i == j) {
            if (a.deg[i] < kt_thr(a, i)) {
                front_add(a, a.f0, &a.st->cnt[0], (int32_t)q, i, 0);
                if (!a.gid) a.state[q] = kDying;
            }
        } else if (rec) {
            const int32_t s = a.sup[q] + (a.dpos[i] >= 0) + (a.dpos[j] >= 0);
            a.sup[q] = s;
            if (s < kt_thr(a, i)) {
                front_add(a, a.f0, &a.st->cnt[0], (int32_t)q, i, 0);
                if (!a.gid) a.state[q] = kDying;
            }
        }
    }
}

// A later k of a sweep (one matrix): the edges left by the previous k have
// exact supports in C, so the first frontier of the new k is the live
// records below the new k - 2 (a diagonal record: its row's length).
__global__ void k_trif_reseed(TriFrontArgs a) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < a.nnz; q += (int64_t)gridDim.x * blockDim.x) {
        if (a.oid[q] != (int32_t)q || a.state[q] != kAlive) continue;
        const int32_t i = a.row_of[q];
        const int32_t s = a.cc[q] == i ? a.deg[i] : a.sup[q];
        if (s < kt_thr(a, i)) {
            front_push(a.f0, &a.st->cnt[0], (int32_t)q);
            a.state[q] = kDying;
        }
    }
}

// H, and P_0, the upper entries and the entries of C_0; one warp per row.
__global__ void k_trif_init_counts(TriFrontArgs a) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    unsigned long long prod = 0, mask = 0, ent = 0;
    for (int64_t j = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < a.m; j += warps) {
        int hs = 0;
        for (int32_t p = a.cr[j] + lane; p < a.cr[j + 1]; p += 32) hs += a.h[a.cc[p]];
        hs = warp_sum<int>(hs);
        if (lane == 0) {
            a.H[j] = hs;
            const unsigned long long pj = (unsigned long long)a.deg[j] * (unsigned long long)hs;
            prod += pj;
            if (a.gid && pj) atomicAdd(reinterpret_cast<unsigned long long*>(a.pg + a.gid[j]), pj);
            mask += (unsigned long long)a.upc[j];
            ent += (unsigned long long)a.deg[j];
        }
    }
    if (lane == 0) {
        if (prod) atomicAdd(&a.st->prod, prod);
        if (mask) atomicAdd(&a.st->mask, mask);
        if (ent) atomicAdd(&a.st->ent, ent);
    }
    // batches: the graphs still to iterate
    if (a.gid)
        for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < a.ngraphs;
             g += (int64_t)gridDim.x * blockDim.x)
            if (!a.done_g[g]) atomicAdd(&a.st->live, 1);
}

// The reference's work for one iteration's support product C_t * C_t (its
// Gustavson products, mask and stored entries), added to the context's
// counters by one thread.
__device__ __forceinline__ void trif_count_iteration(const TriFrontArgs& a) {
    atomicAdd(&a.ctr[GA_CTR_PRODUCTS], a.st->prod);
    atomicAdd(&a.ctr[GA_CTR_MASK_ENTRIES], a.st->mask);
    atomicAdd(&a.ctr[GA_CTR_A_ENTRIES], a.st->ent);
    atomicAdd(&a.ctr[GA_CTR_LAUNCHES], 1ull);
    atomicAdd(&a.ctr[GA_CTR_ROWS], (unsigned long long)a.m);
}

// One matrix, before a k's first iteration (whose frontier the seed marked):
// that iteration's counters. Later iterations are counted by k_trif_delta.
__global__ void k_trif_begin(TriFrontArgs a) {
    if (blockIdx.x == 0 && threadIdx.x == 0) trif_count_iteration(a);
}

// Batches, start of iteration t: the work counters of its support product,
// and the frontier marked.
__global__ void k_trif_mark(const TriFrontArgs* __restrict__ ap) {
    const TriFrontArgs a = *ap;
    const int t = a.st->t;
    const int32_t n = a.st->cnt[t & 1];
    const int32_t* F = (t & 1) ? a.f1 : a.f0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(&a.ctr[GA_CTR_PRODUCTS], a.st->prod);
        atomicAdd(&a.ctr[GA_CTR_MASK_ENTRIES], a.st->mask);
        atomicAdd(&a.ctr[GA_CTR_A_ENTRIES], a.st->ent);
        atomicAdd(&a.ctr[GA_CTR_LAUNCHES], 1ull);
        atomicAdd(&a.ctr[GA_CTR_ROWS], (unsigned long long)a.m);
    }
    for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
        const int32_t q = F[x];
        if (!kt_frozen(a, a.row_of[q])) a.state[q] = kDying;
    }
}

// Rows of at most this many entries are staged in shared memory (columns
// and record positions) before the probes search them.
constexpr int kTrifStage = 512;
// An edge whose shorter row has more than kTrifSplit entries is walked in
// segments of kTrifSeg entries by separate warps (k_trif_lower_seg).
constexpr int kTrifSplit = 128;
constexpr int kTrifSeg = 64;
// Grids of the loop's kernels, per SM: the pruning kernels (128 threads)
// and the passes over the frontier (256 threads).
constexpr int kTrifLowerCtas = 8;
constexpr int kTrifPassCtas = 2;

// A frontier edge (u, v) to walk: the shorter row x, the other row y with
// its oriented part [yb, yo) and the rest [yo, ye), y's rank, and the
// triangles the edge is in (its support without the diagonal terms).
struct TrifEdge {
    int32_t q, u, v, xb, xe, yb, yo, ye, ry;
    int target;
};

__device__ __forceinline__ TrifEdge trif_edge(const TriFrontArgs& a, int32_t q, int32_t u, int32_t v) {
    TrifEdge e;
    e.q = q;
    e.u = u;
    e.v = v;
    const int32_t du = a.dpos[u], dv = a.dpos[v];
    e.target = a.sup[q] - (du >= 0 && a.state[du] != kGone) - (dv >= 0 && a.state[dv] != kGone);
    const int32_t ub = a.cr[u], ue = a.cr[u + 1], vb = a.cr[v], ve = a.cr[v + 1];
    const bool xu = ue - ub <= ve - vb;  // walk the shorter row
    e.xb = xu ? ub : vb;
    e.xe = xu ? ue : ve;
    const int32_t y = xu ? v : u;
    e.yb = xu ? vb : ub;
    e.ye = xu ? ve : ue;
    e.yo = e.yb + a.ocount[y];
    // rank of y: the entry (u, v) holds rank(v), its mirror rank(u)
    e.ry = xu ? a.crank[q] : a.crank[a.mir[q]];
    return e;
}

// Entry p of row x looked up in row y (scol / soid: y's columns and record
// positions indexed from yb); loads only, so that a lane's lookups of
// several entries overlap. A hit is the triangle (u, v, w): f and g are the
// records of its other two edges (u or v, w) and (y, w), with their states.
struct TrifHit {
    int32_t f, g;
    uint8_t sf, sg;
    bool hit;
};

__device__ __forceinline__ TrifHit trif_find(const TriFrontArgs& a, const TrifEdge& e, int32_t p, const int32_t* scol,
                                             const int32_t* soid) {
    TrifHit h;
    h.hit = false;
    h.f = h.g = 0;
    h.sf = h.sg = kGone;
    const int32_t w = a.cc[p];
    if (w == e.u || w == e.v) return h;
    h.f = a.oid[p];
    h.sf = a.state[h.f];
    if (h.sf == kGone) return h;
    // w ranked above y: (y, w) is in y's oriented part
    const bool above = a.crank[p] > e.ry;
    const int32_t sb = above ? 0 : e.yo - e.yb, se = above ? e.yo - e.yb : e.ye - e.yb;
    const int32_t r = sb + lower_bound_i32(scol + sb, se - sb, w);
    if (r >= se || scol[r] != w) return h;
    h.g = soid[r];
    h.sg = a.state[h.g];
    h.hit = h.sg != kGone;
    return h;
}

// A hit lowers the supports of the triangle's other two edges, each once
// (the frontier edge with the smallest record position owns a triangle with
// two frontier edges).
__device__ __forceinline__ void trif_apply_hit(const TriFrontArgs& a, const TrifEdge& e, const TrifHit& h, int32_t* fn,
                                               int32_t* cn, int np) {
    if (!h.hit) return;
    if (h.sf == kAlive && (h.sg == kAlive || e.q < h.g)) lower_support(a, h.f, fn, cn, np);
    if (h.sg == kAlive && (h.sf == kAlive || e.q < h.f)) lower_support(a, h.g, fn, cn, np);
}

// One warp per frontier edge: its triangles in C_t, the supports they lower.
// The warp walks the shorter row x of the edge and looks each entry up in
// the other row y: in y's part that the entry's rank selects, binary-searched
// in shared memory when y has at most kTrifStage entries (its columns and
// record positions copied there first, coalesced), else in global memory.
// A row x longer than kTrifSplit is listed as segments for
// k_trif_lower_seg instead (while the segment list has room).
__global__ void __launch_bounds__(128, 8) k_trif_lower(const TriFrontArgs* __restrict__ ap) {
    __shared__ int32_t s_col[4][kTrifStage];
    __shared__ int32_t s_oid[4][kTrifStage];
    const TriFrontArgs a = *ap;
    const int lane = threadIdx.x & 31;
    int32_t* ycol = s_col[threadIdx.x >> 5];
    int32_t* yoid = s_oid[threadIdx.x >> 5];
    const int t = a.st->t;
    const int32_t n = a.st->cnt[t & 1];
    const int32_t* F = (t & 1) ? a.f1 : a.f0;
    int32_t* fn = (t & 1) ? a.f0 : a.f1;
    int32_t* cn = &a.st->cnt[(t + 1) & 1];
    const int np = (t + 1) & 1;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    unsigned long long probes = 0, tris = 0, edges = 0;
    for (int64_t x = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; x < n; x += warps) {
        const int32_t q = F[x];
        const int32_t u = a.row_of[q], v = a.cc[q];
        if (kt_frozen(a, u)) continue;
        if (lane == 0) ++edges;
        if (u == v) {
            // a diagonal entry leaves: every other edge of its row loses 1
            for (int32_t p = a.cr[u] + lane; p < a.cr[u + 1]; p += 32) {
                if (a.cc[p] == u) continue;
                const int32_t f = a.oid[p];
                if (a.state[f] == kAlive) lower_support(a, f, fn, cn, np);
            }
            continue;
        }
        const TrifEdge e = trif_edge(a, q, u, v);
        if (e.target <= 0) continue;
        if (e.xe - e.xb > kTrifSplit) {
            // segments for k_trif_lower_seg: (frontier slot, segment)
            const int nseg = (e.xe - e.xb + kTrifSeg - 1) / kTrifSeg;
            int base = 0;
            if (lane == 0) base = atomicAdd(&a.st->nseg, nseg);
            base = __shfl_sync(0xffffffffu, base, 0);
            if ((int64_t)base + nseg <= a.segcap) {
                if (lane == 0) a.efound[x] = 0;
                for (int j = lane; j < nseg; j += 32) a.seg[base + j] = make_int2((int32_t)x, j);
                continue;
            }
            // no room: holes in the list are marked, the warp walks the row
            for (int64_t j = base + lane; j < a.segcap && j < (int64_t)base + nseg; j += 32)
                a.seg[j] = make_int2(-1, 0);
        }
        const bool staged = e.ye - e.yb <= kTrifStage;
        if (staged) {
            __syncwarp();  // the previous edge's lookups are done
            for (int32_t i = lane; i < e.ye - e.yb; i += 32) {
                ycol[i] = a.cc[e.yb + i];
                yoid[i] = a.oid[e.yb + i];
            }
            __syncwarp();
        }
        const int32_t* scol = staged ? ycol : a.cc + e.yb;
        const int32_t* soid = staged ? yoid : a.oid + e.yb;
        // 32 entries per pass, stopping once the edge's triangles are found
        // (two entries per lane per pass were slower: the later stop wastes
        // more lookups than the overlap gains)
        int found = 0;
        for (int32_t base = e.xb; base < e.xe; base += 32) {
            const int32_t p = base + lane;
            TrifHit h;
            h.hit = false;
            if (p < e.xe) {
                ++probes;
                h = trif_find(a, e, p, scol, soid);
                trif_apply_hit(a, e, h, fn, cn, np);
            }
            const int hcount = __popc(__ballot_sync(0xffffffffu, h.hit));
            found += hcount;
            if (lane == 0) tris += (unsigned long long)hcount;
            if (found >= e.target) break;
        }
    }
    probes = warp_sum<unsigned long long>(probes);
    if (lane == 0) {
        if (edges) atomicAdd(&a.ctr[GA_CTR_FRONT_EDGES], edges);
        if (probes) atomicAdd(&a.ctr[GA_CTR_FRONT_PROBES], probes);
        if (tris) atomicAdd(&a.ctr[GA_CTR_FRONT_TRIANGLES], tris);
    }
}

// The segments k_trif_lower listed, one warp each: kTrifSeg entries of a
// long row x looked up in y in global memory. The edge's triangles found so
// far are counted in efound (per frontier slot); a segment stops once they
// reach the edge's total.
__global__ void __launch_bounds__(128, 8) k_trif_lower_seg(const TriFrontArgs* __restrict__ ap) {
    const TriFrontArgs a = *ap;
    const int lane = threadIdx.x & 31;
    const int t = a.st->t;
    const int32_t* F = (t & 1) ? a.f1 : a.f0;
    int32_t* fn = (t & 1) ? a.f0 : a.f1;
    int32_t* cn = &a.st->cnt[(t + 1) & 1];
    const int np = (t + 1) & 1;
    const int64_t ns = min((int64_t)a.st->nseg, a.segcap);
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    unsigned long long probes = 0, tris = 0;
    for (int64_t sx = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; sx < ns; sx += warps) {
        const int2 sg = a.seg[sx];
        if (sg.x < 0) continue;
        const int32_t q = F[sg.x];
        const TrifEdge e = trif_edge(a, q, a.row_of[q], a.cc[q]);
        if (*(volatile int32_t*)(a.efound + sg.x) >= e.target) continue;
        const int32_t s0 = e.xb + sg.y * kTrifSeg, s1 = min(e.xe, s0 + kTrifSeg);
        const int32_t* scol = a.cc + e.yb;
        const int32_t* soid = a.oid + e.yb;
        for (int32_t base = s0; base < s1; base += 32) {
            const int32_t p = base + lane;
            TrifHit h;
            h.hit = false;
            if (p < s1) {
                ++probes;
                h = trif_find(a, e, p, scol, soid);
                trif_apply_hit(a, e, h, fn, cn, np);
            }
            const int hcount = __popc(__ballot_sync(0xffffffffu, h.hit));
            int before = 0;
            if (lane == 0) {
                tris += (unsigned long long)hcount;
                before = hcount ? atomicAdd(a.efound + sg.x, hcount) : *(volatile int32_t*)(a.efound + sg.x);
            }
            before = __shfl_sync(0xffffffffu, before, 0);
            if (before + hcount >= e.target) break;
        }
    }
    probes = warp_sum<unsigned long long>(probes);
    if (lane == 0) {
        if (probes) atomicAdd(&a.ctr[GA_CTR_FRONT_PROBES], probes);
        if (tris) atomicAdd(&a.ctr[GA_CTR_FRONT_TRIANGLES], tris);
    }
}

// The frontier's edges leave C_t: rows shorten (diagonal entries whose row
// length drops below k - 2 join the next frontier), the terms of P at their
// endpoints change, rows that lose their last upper entry are listed.
__global__ void k_trif_apply(const TriFrontArgs* __restrict__ ap) {
    const TriFrontArgs a = *ap;
    const int t = a.st->t;
    const int32_t n = a.st->cnt[t & 1];
    const int32_t* F = (t & 1) ? a.f1 : a.f0;
    int32_t* fn = (t & 1) ? a.f0 : a.f1;
    int32_t* cn = &a.st->cnt[(t + 1) & 1];
    const int np = (t + 1) & 1;
    unsigned long long mask = 0, ent = 0;
    for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
        const int32_t q = F[x];
        const int32_t u = a.row_of[q], v = a.cc[q];
        if (kt_frozen(a, u)) continue;
        a.state[q] = kGone;
        ++mask;
        // deg and H keep their values from the iteration's start; the losses
        // are counted in rd and rh and applied by k_trif_delta
        if (u == v) {
            ++ent;
            atomicAdd(a.rd + u, 1);
            atomicAdd(a.rh + u, 1);  // h(u) = 1 while its diagonal entry is there
            touch(a, u);
            if (atomicSub(a.upc + u, 1) == 1) front_push(a.flip, &a.st->nflip, u);
            continue;
        }
        ent += 2;
        // the row lengths before this entry left
        const int32_t ou = a.deg[u] - atomicAdd(a.rd + u, 1), ov = a.deg[v] - atomicAdd(a.rd + v, 1);
        if (a.h[u]) atomicAdd(a.rh + v, 1);
        if (a.h[v]) atomicAdd(a.rh + u, 1);
        touch(a, u);
        touch(a, v);
        const int32_t lo = min(u, v);
        if (atomicSub(a.upc + lo, 1) == 1) front_push(a.flip, &a.st->nflip, lo);
        // a diagonal entry's support is its row's length
        if (ou == kt_thr(a, u)) {
            const int32_t d = a.dpos[u];
            if (d >= 0 && a.state[d] == kAlive) front_add(a, fn, cn, d, u, np);
        }
        if (ov == kt_thr(a, v)) {
            const int32_t d = a.dpos[v];
            if (d >= 0 && a.state[d] == kAlive) front_add(a, fn, cn, d, v, np);
        }
    }
    mask = warp_sum<unsigned long long>(mask);
    ent = warp_sum<unsigned long long>(ent);
    if ((threadIdx.x & 31) == 0 && mask) {
        atomicAdd(&a.st->mask, (unsigned long long)(-(long long)mask));
        atomicAdd(&a.st->ent, (unsigned long long)(-(long long)ent));
    }
}

// Rows that lost their last upper entry: h drops to 0, so every remaining
// neighbour's H loses 1. One warp per row.
// H(j) loses 1 here directly, and P loses deg(j) (the row length at the
// iteration's start): k_trif_delta's term for a touched j, computed from
// this H, then misses exactly that; a j that nothing else touched changes
// by exactly that. So the flipped rows' neighbours are neither touched nor
// counted in rh.
__global__ void k_trif_flip(const TriFrontArgs* __restrict__ ap) {
    const TriFrontArgs a = *ap;
    const int lane = threadIdx.x & 31;
    const int32_t n = a.st->nflip;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    long long d = 0;  // this lane's part of the change of P
    for (int64_t x = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; x < n; x += warps) {
        const int32_t i = a.flip[x];
        if (lane == 0) a.h[i] = 0;
        long long di = 0;
        for (int32_t p = a.cr[i] + lane; p < a.cr[i + 1]; p += 32) {
            if (a.state[a.oid[p]] == kGone) continue;
            const int32_t j = a.cc[p];
            atomicSub(a.H + j, 1);
            di -= a.deg[j];
        }
        if (a.gid) {
            // the neighbours of row i are in i's graph
            const long long gi = warp_sum<long long>(di);
            if (lane == 0 && gi) atomicAdd(reinterpret_cast<unsigned long long*>(a.pg + a.gid[i]), (unsigned long long)gi);
        }
        d += di;
    }
    d = warp_sum<long long>(d);
    if (lane == 0 && d) atomicAdd(&a.st->prod, (unsigned long long)d);
}

// P_{t+1} = P_t + the change of deg(j) H(j) at every touched vertex (for a
// batch also per graph). For one matrix, the last block to finish ends the
// iteration (stop when F_t was empty, or after m iterations) and tells the
// loop whether to go on; batches end it in k_trif_graphs.
__global__ void __launch_bounds__(256) k_trif_delta(const TriFrontArgs* __restrict__ ap, LoopCtl ctl) {
    const TriFrontArgs a = *ap;
    __shared__ long long part[8];
    __shared__ bool last;
    const int32_t n = a.st->ntouch;
    if (!a.gid) {
        // one matrix: the next frontier is complete, so its edges are marked
        // here instead of by a marking kernel at the next iteration's start
        const int t = a.st->t;
        const int32_t nn = a.st->cnt[(t + 1) & 1];
        const int32_t* Fn = (t & 1) ? a.f0 : a.f1;
        for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < nn; x += (int64_t)gridDim.x * blockDim.x)
            a.state[Fn[x]] = kDying;
    }
    long long d = 0;
    for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
        const int32_t j = a.touched[x];
        const long long od = a.deg[j], oh = a.H[j];
        const long long nd = od - a.rd[j], nh = oh - a.rh[j];
        const long long dj = nd * nh - od * oh;
        d += dj;
        if (a.gid && dj) atomicAdd(reinterpret_cast<unsigned long long*>(a.pg + a.gid[j]), (unsigned long long)dj);
        a.deg[j] = (int32_t)nd;
        a.H[j] = (int32_t)nh;
        a.rd[j] = 0;
        a.rh[j] = 0;
        a.mark[j] = 0;
    }
    d = warp_sum<long long>(d);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = d;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += part[w];
        if (s) atomicAdd(&a.st->prod, (unsigned long long)s);
        __threadfence();
        last = atomicAdd(&a.st->blocks_done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    TriFrontState* st = a.st;
    st->blocks_done = 0;
    st->ntouch = 0;
    st->nflip = 0;
    st->nseg = 0;
    if (a.gid) return;
    const int t = st->t;
    if (st->cnt[t & 1] == 0) {
        st->iters = t + 1;
        st->done = 1;
    } else {
        st->cnt[t & 1] = 0;
        st->t = t + 1;
        if ((int64_t)(t + 1) >= a.m) {
            st->iters = 0;
            st->done = 1;
        }
    }
    if (!st->done) trif_count_iteration(a);
    loop_continue(ctl, st->done == 0);
}

// Batches, end of iteration t, one thread per graph: a live graph without
// frontier elements in this iteration has converged (iteration count t + 1),
// one that reached its bound stops with count 0 (n_g iterations, as the
// reference's loop); both leave the live set and their P leaves the work
// total. The last block ends the iteration; the loop goes on while a graph
// is live.
__global__ void __launch_bounds__(256) k_trif_graphs(const TriFrontArgs* __restrict__ ap, LoopCtl ctl) {
    const TriFrontArgs a = *ap;
    __shared__ long long part[8];
    __shared__ int lpart[8];
    __shared__ bool last;
    const int t = a.st->t;
    int32_t* cnt = a.cntg + (t & 1) * a.ngraphs;
    long long dp = 0;
    int dl = 0;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < a.ngraphs;
         g += (int64_t)gridDim.x * blockDim.x) {
        const int32_t c = cnt[g];
        cnt[g] = 0;
        if (a.done_g[g]) continue;
        if (c == 0 || (int64_t)(t + 1) >= a.nvert[g]) {
            a.iters_g[g] = c == 0 ? t + 1 : 0;
            a.done_g[g] = 1;
            dp -= a.pg[g];
            ++dl;
        }
    }
    dp = warp_sum<long long>(dp);
    dl = warp_sum<int>(dl);
    if ((threadIdx.x & 31) == 0) {
        part[threadIdx.x >> 5] = dp;
        lpart[threadIdx.x >> 5] = dl;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long s = 0;
        int l = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            s += part[w];
            l += lpart[w];
        }
        if (s) atomicAdd(&a.st->prod, (unsigned long long)s);
        if (l) atomicSub(&a.st->live, l);
        __threadfence();
        last = atomicAdd(&a.st->blocks_done_g, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    TriFrontState* st = a.st;
    st->blocks_done_g = 0;
    st->cnt[t & 1] = 0;
    st->t = t + 1;
    if (st->live <= 0) st->done = 1;
    loop_continue(ctl, st->done == 0);
}

__global__ void k_trif_keep(TriFrontArgs a, int64_t cap, int32_t* __restrict__ flag) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < cap; q += (int64_t)gridDim.x * blockDim.x)
        flag[q] = q < a.nnz && a.state[a.oid[q]] != kGone;
}

// After the keep flags' scan (pos): kept entries written in column order (an
// entry's place: kept entries before it in its part, plus kept entries of
// the other part with smaller columns), new row starts.
__global__ void k_trif_out(TriFrontArgs a, const int32_t* __restrict__ pos, int32_t* __restrict__ tc,
                           int32_t* __restrict__ tr) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < a.nnz || q <= a.m; q += stride) {
        if (q <= a.m) tr[q] = pos[a.cr[q]];
        if (q < a.nnz && pos[q + 1] != pos[q]) {
            const int32_t i = a.row_of[q], rb = a.cr[i], re = a.cr[i + 1], ro = rb + a.ocount[i];
            const bool o = q < ro;
            const int32_t pb = o ? rb : ro;
            const int32_t ob = o ? ro : rb, oe = o ? re : ro;
            const int32_t j = a.cc[q];
            const int32_t t = ob + lower_bound_i32(a.cc + ob, oe - ob, j);
            tc[pos[rb] + (pos[q] - pos[pb]) + (pos[t] - pos[ob])] = j;
        }
    }
}

}  // namespace

struct TriFront::Impl {
    ga_ctx ctx;
    ga_csr C;
    TriKt t;
    int64_t cap;
    TriFrontBufs b;
    const KtBatch* batch;
    int64_t ng;
    DBuf<int32_t> deg, upc, H, rd, rh, mark, touched, flip;
    DBuf<uint8_t> h;
    DBuf<TriFrontState> st;
    DBuf<int32_t> cntg;
    DBuf<long long> pg;
    DBuf<int2> seg;
    DBuf<int32_t> efound;
    TriFrontArgs a;
    bool first = true;

    Impl(ga_ctx ctx_, ga_csr C_, const int32_t* row_of, const int32_t* mir, const TriKt& t_, int64_t cap_,
         const TriFrontBufs& b_, const KtBatch* batch_)
        : ctx(ctx_), C(C_), t(t_), cap(cap_), b(b_), batch(batch_), ng(batch_ ? batch_->ngraphs : 0),
          deg(ctx_, (size_t)C_->m + 1), upc(ctx_, (size_t)C_->m + 1), H(ctx_, (size_t)C_->m + 1),
          rd(ctx_, (size_t)C_->m + 1), rh(ctx_, (size_t)C_->m + 1), mark(ctx_, (size_t)C_->m + 1),
          touched(ctx_, (size_t)C_->m + 1), flip(ctx_, (size_t)C_->m + 1), h(ctx_, (size_t)C_->m + 1),
          st(ctx_, 1), cntg(ctx_, batch_ ? (size_t)(2 * batch_->ngraphs) : 1),
          pg(ctx_, batch_ ? (size_t)batch_->ngraphs : 1),
          seg(ctx_, (size_t)std::max<int64_t>(cap_ / 8, 4096)), efound(ctx_, (size_t)cap_) {
        GA_CUDA(cudaMemsetAsync(st.p, 0, sizeof(TriFrontState), ctx->stream));
        if (batch) {
            GA_CUDA(cudaMemsetAsync(cntg.p, 0, sizeof(int32_t) * (size_t)(2 * ng), ctx->stream));
            GA_CUDA(cudaMemsetAsync(pg.p, 0, sizeof(long long) * (size_t)ng, ctx->stream));
        }
        a.cr = C->rst;
        a.cc = C->col;
        a.row_of = row_of;
        a.mir = mir;
        a.crank = t.crank;
        a.ocount = t.ocount;
        a.dpos = t.dpos;
        a.oid = b.oid;
        a.sup = b.sup;
        a.state = b.state;
        a.deg = deg.p;
        a.upc = upc.p;
        a.h = h.p;
        a.H = H.p;
        a.rd = rd.p;
        a.rh = rh.p;
        a.mark = mark.p;
        a.touched = touched.p;
        a.flip = flip.p;
        a.f0 = b.f0;
        a.f1 = b.f1;
        a.seg = seg.p;
        a.efound = efound.p;
        a.segcap = (int64_t)seg.count;
        a.st = st.p;
        a.ctr = ctx->d_counters;
        a.m = C->m;
        a.nnz = C->nnz;
        a.k = 0;
        a.gid = batch ? batch->gid : nullptr;
        a.kg = batch ? batch->kg : nullptr;
        a.nvert = batch ? batch->nvert : nullptr;
        a.done_g = batch ? batch->done_g : nullptr;
        a.iters_g = batch ? batch->iters_g : nullptr;
        a.cntg = batch ? cntg.p : nullptr;
        a.pg = batch ? pg.p : nullptr;
        a.ngraphs = ng;
    }

    void run(int k) {
        const int64_t m = a.m, nnz = a.nnz;
        a.k = k;
        const int grid_ent = grid_for(nnz > 0 ? nnz : 1, 256, ctx->num_sms * 16);
        if (first) {
            first = false;
            // iteration 0's supports: one listing of every triangle
            tri_kt_support(ctx, C, b.sup, t, cap);
            ProfScope ps(ctx, "trif_seed");
            k_trif_init_rows<<<grid_for(m, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(a);
            post_launch("trif_init_rows");
            if (nnz) {
                k_trif_seed<<<grid_ent, 256, 0, ctx->stream>>>(a);
                post_launch("trif_seed");
            }
            k_trif_init_counts<<<grid_for(std::max<int64_t>(m * 32, ng), 256, ctx->num_sms * 16), 256, 0,
                                 ctx->stream>>>(a);
            post_launch("trif_init_counts");
        } else {
            GA_REQUIRE(!batch, GA_ERR_INVALID_ARG, "a batched frontier k-truss runs one k");
            // a new k: the loop state restarts (the running work totals stay)
            ProfScope ps(ctx, "trif_seed");
            GA_CUDA(cudaMemsetAsync(st.p, 0, offsetof(TriFrontState, live), ctx->stream));
            if (nnz) {
                k_trif_reseed<<<grid_ent, 256, 0, ctx->stream>>>(a);
                post_launch("trif_reseed");
            }
        }
        if (!batch) {
            k_trif_begin<<<1, 32, 0, ctx->stream>>>(a);
            post_launch("trif_begin");
        }
        // The loop's kernels read the call's parameters from a device copy and
        // have fixed grids, so the context captures the loop once per slot and
        // relaunches it on later calls.
        const int slot = batch ? kLoopSlotTriFrontBatch : kLoopSlotTriFront;
        TriFrontArgs* dargs = static_cast<TriFrontArgs*>(cached_loop_args(ctx, slot, sizeof(TriFrontArgs)));
        GA_CUDA(cudaMemcpyAsync(dargs, &a, sizeof(TriFrontArgs), cudaMemcpyHostToDevice, ctx->stream));
        const int sms = ctx->num_sms;
        const bool batched = batch != nullptr;
        ga_ctx c = ctx;
        auto body = [c, dargs, sms, batched](const LoopCtl& ctl) {
            if (batched) {
                ProfScope ps(c, "trif_mark");
                k_trif_mark<<<sms * 4, 256, 0, c->stream>>>(dargs);
                post_launch("trif_mark");
            }
            {
                ProfScope ps(c, "trif_lower");
                k_trif_lower<<<sms * kTrifLowerCtas, 128, 0, c->stream>>>(dargs);
                post_launch("trif_lower");
                k_trif_lower_seg<<<sms * kTrifLowerCtas, 128, 0, c->stream>>>(dargs);
                post_launch("trif_lower_seg");
            }
            {
                ProfScope ps(c, "trif_apply");
                k_trif_apply<<<sms * kTrifPassCtas, 256, 0, c->stream>>>(dargs);
                post_launch("trif_apply");
            }
            {
                ProfScope ps(c, "trif_flip");
                k_trif_flip<<<sms * kTrifPassCtas, 256, 0, c->stream>>>(dargs);
                post_launch("trif_flip");
            }
            ProfScope ps(c, "trif_delta");
            k_trif_delta<<<sms * 2, 256, 0, c->stream>>>(dargs, ctl);
            post_launch("trif_delta");
            if (batched) {
                k_trif_graphs<<<sms * 2, 256, 0, c->stream>>>(dargs, ctl);
                post_launch("trif_graphs");
            }
        };
        ProfScope ps(ctx, "ktruss_loop");
        run_cached_loop(ctx, slot, body, m + 1);
    }

    int64_t compact(int* iters) {
        const int64_t m = a.m, nnz = a.nnz;
        ProfScope ps(ctx, "trif_compact");
        k_trif_keep<<<grid_for(cap, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(a, cap, b.flag);
        post_launch("trif_keep");
        scan_exclusive_i32_scratch(ctx, b.flag, b.flag, cap, b.scan_scr);
        k_trif_out<<<grid_for(nnz > m ? nnz : m + 1, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(a, b.flag, b.tc,
                                                                                                 b.tr);
        post_launch("trif_out");
        TriFrontState hs;
        int32_t kept = 0;
        GA_CUDA(cudaMemcpyAsync(&hs, st.p, sizeof(TriFrontState), cudaMemcpyDeviceToHost, ctx->stream));
        GA_CUDA(cudaMemcpyAsync(&kept, b.tr + m, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
        if (iters) *iters = hs.iters;
        return kept;
    }
};

TriFront::TriFront(ga_ctx ctx, ga_csr C, const int32_t* row_of, const int32_t* mir, const TriKt& t, int64_t cap,
                   const TriFrontBufs& b, const KtBatch* batch)
    : impl_(new Impl(ctx, C, row_of, mir, t, cap, b, batch)) {}

TriFront::~TriFront() { delete impl_; }

void TriFront::run(int k) { impl_->run(k); }

int64_t TriFront::compact(int* iters) { return impl_->compact(iters); }

int tri_kt_frontier(ga_ctx ctx, ga_csr C, int k, const int32_t* row_of, const int32_t* mir, const TriKt& t,
                    int64_t cap, const TriFrontBufs& b, const KtBatch* batch) {
    TriFront f(ctx, C, row_of, mir, t, cap, b, batch);
    f.run(k);
    int iters = 0;
    const int64_t kept = f.compact(&iters);
    const int64_t m = C->m;
    GA_CUDA(cudaMemcpyAsync(C->rst, b.tr, sizeof(int32_t) * (size_t)(m + 1), cudaMemcpyDeviceToDevice, ctx->stream));
    if (kept) GA_CUDA(cudaMemcpyAsync(C->col, b.tc, sizeof(int32_t) * (size_t)kept, cudaMemcpyDeviceToDevice,
                                      ctx->stream));
    C->nnz = kept;
    return iters;
}

}  // namespace ga
