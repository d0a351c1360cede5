// Masked SpGEMM C<M> = A*B (structural mask, C has M's pattern).
//
// Design (one pass, no symbolic phase: the output pattern is M's):
//  1. k_row_bin: one warp per output row computes the mask length m_i and the
//     Gustavson product count P_i = sum_{k in A_i} nnz(B_k). Rows with an
//     empty mask are skipped, rows without products get explicit zeros, short
//     light rows (m_i <= kWarpSlots, P_i <= warp_max_flops) go to a warp
//     queue, all others to a CTA queue as windows of at most kCtaSlots mask
//     slots spanning fewer than kWinCols columns (heavy rows first).
//  2. k_mxm_masked: a persistent kernel (one wave of CTAs sized by occupancy)
//     drains the CTA queue, then every warp drains the warp queue. The
//     accumulator is indexed by mask slot and lives in shared memory.
//     Column -> slot lookup per variant:
//       GA_MSA  : a dense bitmap of the window's mask columns in shared memory
//                 (the reference MSA keeps a dense state array over the
//                 columns, matrix_la.h:681-749); a set bit is resolved to its
//                 slot as the word's first slot plus a popcount (the
//                 slot base is kept per 32-column word). Warp rows use a
//                 4096-bit hashed filter and a 512-entry hash table.
//       GA_MCA  : binary search of the sorted mask row in shared memory (the
//                 reference MCA walks the mask row, matrix_la.h:625-632),
//                 after a membership test that rejects the columns outside
//                 the mask (most products of a k-truss support miss it): a
//                 bitmap over the window (CTA items) or the 4096-bit hashed
//                 filter (warp rows);
//       GA_HEAP : sorted merge of each B row against the mask row
//                 (replaces the priority-queue merge,
//                 matrix_la.h:1030-1084): lanes take 32 A entries; a B row
//                 with few entries inside the window is merged by its lane,
//                 a longer one is cut into 32 slices merged by one lane
//                 each (the mask side gallops), and a B row far longer
//                 than the mask row is merged by the whole warp, 32
//                 columns against 32, galloping over the B runs that
//                 cannot meet the mask.
//     Work distribution inside a CTA item: warps take the row's A entries 32
//     at a time; B rows of up to kLongSeg entries (32 when the A row is too
//     short to occupy every warp) are flattened over the
//     warp's lanes (warp scan of the lengths, lanes walk the flattened index);
//     longer B rows (hubs) go to a shared list and are cut into kChunk-entry
//     pieces that all warps of the CTA stream coalesced.
// Integer results are exact and equal across variants; floating-point sums
// are accumulated with shared-memory atomics (order not fixed).
#include "ga_device.cuh"

#include <type_traits>

namespace ga {

constexpr int kMxmThreads = 512;
constexpr int kMxmWarps = kMxmThreads / 32;
constexpr int kCtaSlots = 4096;            // mask slots per CTA work item
constexpr int kWinCols = 1 << 17;          // column span of a CTA work item
constexpr int kWinWords = kWinCols / 32;   // dense bitmap words
constexpr int kWarpSlots = 256;            // mask slots per warp row
constexpr int kWarpTblBits = 9;            // warp-row hash table: 512 entries
constexpr int kFilterBits = 12;            // warp-row filter: 4096 bits
constexpr int kDotTask = 8;                // hybrid form: mask entries per inner-product task
// Bin thresholds (rows above warp_max_flops products go to a CTA; CTA items
// of rows with at least heavy_flops products are scheduled first) and the
// persistent grid size are runtime parameters (ga_ctx tune, set by options
// or the autotuner).
constexpr int kLongSeg = 256;              // B rows longer than this are shared by the CTA
constexpr int kShortARow = kMxmThreads;    // A rows with fewer entries leave warps idle in phase A:
constexpr int kLongSegShort = 32;          // their B rows longer than this are shared instead
constexpr int kLongCap = 1024;             // long B rows listed per item
constexpr int kChunk = 1024;               // entries per long-row piece

struct MxmQueue {
    int32_t warp_count;
    int32_t heavy_count;   // CTA items at the front of the item array
    int32_t normal_count;  // CTA items at the back
    int32_t warp_next;
    int32_t cta_next;
    int32_t dot_count;     // hybrid form: inner-product tasks listed
    unsigned long long flops;
};

template <typename T, typename A>
struct MxmArgs {
    const int32_t* ar; const int32_t* ac; const T* av;
    const int32_t* br; const int32_t* bc; const T* bv;
    const int32_t* mr; const int32_t* mc;
    const int32_t* mre;  // optional mask row ends (row i's mask is [mr[i], mre[i])); nullptr: mr[i+1]
    T* cv;
    int64_t m;
    MxmQueue* q;
    int32_t* warp_rows;
    int4* cta_items;          // (row, first slot, end slot, unused)
    int32_t cta_cap;
    unsigned long long* ctr;  // context work counters (GA_CTR_*)
    int64_t warp_max_flops, heavy_flops;
    // hybrid form: rows whose inner-product work (sum over mask entries of
    // min(|A_i|, |B^T_j|)) times hybrid_ratio is below their Gustavson work
    // are listed in dot_tasks (row, first mask entry; count in the queue),
    // kDotTask mask entries per task, for the inner-product kernel
    const int32_t* btr;  // B^T row starts (nullptr: no hybrid)
    int2* dot_tasks;
    int64_t hybrid_ratio;
};

__global__ void k_reset_queue(MxmQueue* q) {
    if (threadIdx.x == 0) {
        q->warp_count = 0; q->heavy_count = 0; q->normal_count = 0;
        q->warp_next = 0; q->cta_next = 0; q->dot_count = 0; q->flops = 0ull;
    }
}

// ------------------------------------------------------------------ binning
template <typename T, typename A>
__global__ void k_row_bin(MxmArgs<T, A> p) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    unsigned long long my_flops = 0, my_mask = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(&p.ctr[GA_CTR_LAUNCHES], 1ull);
        atomicAdd(&p.ctr[GA_CTR_A_ENTRIES], (unsigned long long)(p.ar[p.m] - p.ar[0]));
        atomicAdd(&p.ctr[GA_CTR_ROWS], (unsigned long long)p.m);
    }
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < p.m; i += warps) {
        const int32_t mb = p.mr[i], me = p.mre ? p.mre[i] : p.mr[i + 1];
        const int32_t mi = me - mb;
        if (mi == 0) continue;
        if (lane == 0) my_mask += (unsigned long long)mi;
        const int32_t ab = p.ar[i], ae = p.ar[i + 1];
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
        if (p.btr) {
            // inner-product work of the row; the cheaper form takes it
            const int32_t an = ae - ab;
            long long dsum = 0;
            for (int32_t q = mb + lane; q < me; q += 32) {
                const int32_t j = p.mc[q];
                const int32_t bn = p.btr[j + 1] - p.btr[j];
                dsum += an < bn ? an : bn;
            }
            dsum = warp_sum<long long>(dsum);
            if (dsum * p.hybrid_ratio < f) {
                const int ntask = (mi + kDotTask - 1) / kDotTask;
                int first = 0;
                if (lane == 0) {
                    my_flops += (unsigned long long)f;
                    first = atomicAdd(&p.q->dot_count, ntask);
                }
                first = __shfl_sync(0xffffffffu, first, 0);
                for (int t = lane; t < ntask; t += 32) p.dot_tasks[first + t] = make_int2((int)i, mb + t * kDotTask);
                continue;
            }
        }
        if (lane == 0) {
            my_flops += (unsigned long long)f;
            if (mi <= kWarpSlots && f <= p.warp_max_flops) {
                int pos = atomicAdd(&p.q->warp_count, 1);
                p.warp_rows[pos] = (int32_t)i;
            } else {
                const int32_t* mcol = p.mc + mb;
                const bool heavy = f >= p.heavy_flops;
                int s0 = 0;
                while (s0 < mi) {
                    int s1 = min(mi, s0 + kCtaSlots);
                    const int32_t c0 = mcol[s0];
                    if (mcol[s1 - 1] - c0 >= kWinCols) {
                        const int64_t lim = (int64_t)c0 + (kWinCols - 1);
                        s1 = s0 + upper_bound_i32(mcol + s0, s1 - s0, (int32_t)(lim < INT32_MAX ? lim : INT32_MAX));
                    }
                    int pos;
                    if (heavy) pos = atomicAdd(&p.q->heavy_count, 1);
                    else pos = p.cta_cap - 1 - atomicAdd(&p.q->normal_count, 1);
                    p.cta_items[pos] = make_int4((int)i, s0, s1, 0);
                    s0 = s1;
                }
            }
        }
    }
    if (lane == 0 && my_flops) {
        atomicAdd(&p.q->flops, my_flops);
        atomicAdd(&p.ctr[GA_CTR_PRODUCTS], my_flops);
    }
    if (lane == 0 && my_mask) atomicAdd(&p.ctr[GA_CTR_MASK_ENTRIES], my_mask);
}

// ------------------------------------------------------------------ lookups
// MODE: how a product's column finds its mask slot.
// MD_BSEARCH: CTA items (window bitmap, then search); MD_BSEARCH_F: warp
// rows (hashed filter, then search).
enum { MD_DENSE = 0, MD_HASHED = 1, MD_BSEARCH = 2, MD_MERGE = 3, MD_BSEARCH_F = 4 };

// The mask columns of one work item, staged in shared memory.
struct SlotView {
    const int32_t* mcol;    // MD_BSEARCH(_F) / MD_MERGE: sorted mask columns
    const uint32_t* bits;   // MD_DENSE, MD_BSEARCH: bitmap over [lo, lo + kWinCols)
    const uint16_t* wbase;  // MD_DENSE: slot of the first mask column of each bitmap word
    const uint32_t* filt;   // MD_HASHED, MD_BSEARCH_F: 4096-bit filter of hashed columns
    const int32_t* hkeys;   // MD_HASHED: open-addressing table (2^kWarpTblBits)
    const uint8_t* hslot;
    int ns;
    int32_t lo, hi;
};

template <int MD>
__device__ __forceinline__ int slot_of(const SlotView& v, int32_t c) {
    if (MD == MD_DENSE) {
        // dense state over the window: a set bit is a mask column, and its
        // slot is the word's first slot plus the set bits below it
        const uint32_t d = (uint32_t)(c - v.lo);
        if (d > (uint32_t)(v.hi - v.lo)) return -1;
        const uint32_t w = v.bits[d >> 5];
        const uint32_t b = d & 31;
        if (!((w >> b) & 1u)) return -1;
        return (int)v.wbase[d >> 5] + __popc(w & ((1u << b) - 1u));
    } else if (MD == MD_HASHED) {
        const uint32_t h = hash_col(c);
        const uint32_t f = h >> (32 - kFilterBits);
        if (!((v.filt[f >> 5] >> (f & 31)) & 1u)) return -1;
        const uint32_t mask = (1u << kWarpTblBits) - 1u;
        uint32_t pos = h >> (32 - kWarpTblBits);
        while (true) {
            const int32_t key = v.hkeys[pos];
            if (key == c) return (int)v.hslot[pos];
            if (key == kEmpty) return -1;
            pos = (pos + 1) & mask;
        }
    } else {
        if (c < v.lo || c > v.hi) return -1;
        if (MD == MD_BSEARCH) {
            const uint32_t d = (uint32_t)(c - v.lo);
            if (!((v.bits[d >> 5] >> (d & 31)) & 1u)) return -1;
        } else if (MD == MD_BSEARCH_F) {
            const uint32_t f = hash_col(c) >> (32 - kFilterBits);
            if (!((v.filt[f >> 5] >> (f & 31)) & 1u)) return -1;
        }
        const int pos = lower_bound_i32(v.mcol, v.ns, c);
        return (pos < v.ns && v.mcol[pos] == c) ? pos : -1;
    }
}

// Value modes: VM 0 general, 1 B's values are all ones (no B value loads),
// 2 A's and B's values are all ones (every product is 1: no value loads or
// multiplies at all; int32 only).
// B value of entry j in the accumulator type.
template <int VM, typename T, typename A>
__device__ __forceinline__ A bval(const MxmArgs<T, A>& p, int32_t j) {
    return VM >= 1 ? (A)1 : to_acc<T, A>(__ldg(p.bv + j));
}

// Product of the A value staged for segment q and a B value.
template <int VM, typename A>
__device__ __forceinline__ A seg_product(const A* s_a, int q, A b) {
    return VM == 2 ? (A)1 : s_a[q] * b;
}

template <int MD, typename A>
__device__ __forceinline__ void add_product(const SlotView& v, A* acc, int32_t c, A prod) {
    const int slot = slot_of<MD>(v, c);
    if (slot >= 0) atomic_add_acc<A>(&acc[slot], prod);
}

// Four consecutive values starting at a 16-byte aligned index.
template <typename T> struct Vec4 { T x, y, z, w; };
template <typename T>
__device__ __forceinline__ Vec4<T> load4(const T* ptr) {
    Vec4<T> r;
    if (sizeof(T) == 4) {
        const int4 t = __ldg(reinterpret_cast<const int4*>(ptr));
        memcpy(&r, &t, 16);
    } else if (sizeof(T) == 8) {
        const int4 a = __ldg(reinterpret_cast<const int4*>(ptr));
        const int4 b = __ldg(reinterpret_cast<const int4*>(ptr) + 1);
        memcpy(&r, &a, 16);
        memcpy(reinterpret_cast<char*>(&r) + 16, &b, 16);
    } else {
        r.x = __ldg(ptr); r.y = __ldg(ptr + 1); r.z = __ldg(ptr + 2); r.w = __ldg(ptr + 3);
    }
    return r;
}

// B-row range of A entry t, optionally clipped to the item's column window.
template <typename T, typename A>
__device__ __forceinline__ void b_range(const MxmArgs<T, A>& p, int32_t t, bool clip, int32_t lo, int32_t hi,
                                        int32_t& bs, int32_t& be) {
    const int32_t k = __ldg(p.ac + t);
    bs = __ldg(p.br + k);
    be = __ldg(p.br + k + 1);
    if (clip) {
        const int n = be - bs;
        const int l = lower_bound_i32(p.bc + bs, n, lo);
        const int h = upper_bound_i32(p.bc + bs, n, hi);
        be = bs + h;
        bs = bs + l;
    }
}

// Flattened products of the 32 A entries starting at t_first (one per lane).
// Non-empty B rows are compacted; for each window of 32 consecutive product
// indices the segment ends falling inside it form one 32-bit mask (a warp OR
// reduction), so every lane finds its B row with a popcount - no per-lane
// search loop. Lanes whose B row is long may hand it to the CTA's long list.
// Returns the number of products it processed (warp-uniform).
template <int MD, int VM, typename T, typename A, bool PUSH>
__device__ __forceinline__ int group_products(const MxmArgs<T, A>& p, int32_t t_first, int32_t t_end, bool clip,
                                              const SlotView& v, A* acc, int* s_incl, int* s_off, A* s_a,
                                              int* s_nlong, int32_t* s_lbs, int32_t* s_lend, A* s_la,
                                              int long_seg = kLongSeg) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int32_t t = t_first + lane;
    int len = 0;
    int32_t bs = 0;
    A av = (A)0;
    if (t < t_end) {
        int32_t be;
        b_range(p, t, clip, v.lo, v.hi, bs, be);
        av = VM == 2 ? (A)1 : to_acc<T, A>(__ldg(p.av + t));
        len = be - bs;
        if (PUSH && len > long_seg) {
            const int slot = atomicAdd(s_nlong, 1);
            if (slot < kLongCap) {
                s_lbs[slot] = bs;
                s_lend[slot] = be;
                s_la[slot] = av;
                len = 0;
            }
        }
    }
    const unsigned nz = __ballot_sync(FULL, len > 0);
    if (nz == 0) return 0;
    const int nseg = __popc(nz);
    const int incl = warp_incl_scan(len);
    const int total = __shfl_sync(FULL, incl, 31);
    if (len > 0) {
        const int rank = __popc(nz & ((1u << lane) - 1u));
        s_incl[rank] = incl;
        s_off[rank] = bs - (incl - len);
        if (VM != 2) s_a[rank] = av;
    }
    __syncwarp();
    const int my_end = lane < nseg ? s_incl[lane] - 1 : INT32_MAX;  // last product of segment `lane`
    const unsigned lt = (1u << lane) - 1u;
    int q_base = 0;
    int base = 0;
    for (; base + 32 < total; base += 64) {
        const int e0 = my_end - base, e1 = my_end - base - 32;
        const unsigned bm0 = __reduce_or_sync(FULL, (e0 >= 0 && e0 < 32) ? (1u << e0) : 0u);
        const unsigned bm1 = __reduce_or_sync(FULL, (e1 >= 0 && e1 < 32) ? (1u << e1) : 0u);
        const int q0 = q_base + __popc(bm0 & lt);
        const int q1 = q_base + __popc(bm0) + __popc(bm1 & lt);
        const int x1 = base + 32 + lane;
        const int32_t j0 = base + lane + s_off[q0];
        const int32_t c0 = __ldg(p.bc + j0);
        const A b0 = bval<VM, T, A>(p, j0);
        int32_t c1 = 0;
        A b1 = (A)0;
        if (x1 < total) {
            const int32_t j1 = x1 + s_off[q1];
            c1 = __ldg(p.bc + j1);
            b1 = bval<VM, T, A>(p, j1);
        }
        add_product<MD, A>(v, acc, c0, seg_product<VM, A>(s_a, q0, b0));
        if (x1 < total) add_product<MD, A>(v, acc, c1, seg_product<VM, A>(s_a, q1, b1));
        q_base += __popc(bm0) + __popc(bm1);
    }
    if (base < total) {
        const int e0 = my_end - base;
        const unsigned bm0 = __reduce_or_sync(FULL, (e0 >= 0 && e0 < 32) ? (1u << e0) : 0u);
        const int x = base + lane;
        if (x < total) {
            const int q = q_base + __popc(bm0 & lt);
            const int32_t j = x + s_off[q];
            add_product<MD, A>(v, acc, __ldg(p.bc + j), seg_product<VM, A>(s_a, q, bval<VM, T, A>(p, j)));
        }
    }
    __syncwarp();
    return total;
}

// Stream B entries [j0, j1) of one row with scalar head/tail and a
// 16-byte vector body (columns, and values unless they are all ones).
template <int MD, int VM, typename T, typename A>
__device__ __forceinline__ void stream_row(const MxmArgs<T, A>& p, const SlotView& v, A* acc, int32_t j0,
                                           int32_t j1, A a) {
    const int lane = threadIdx.x & 31;
    int32_t ja = (j0 + 3) & ~3;
    if (ja > j1) ja = j1;
    if (j0 + lane < ja) add_product<MD, A>(v, acc, __ldg(p.bc + j0 + lane), a * bval<VM, T, A>(p, j0 + lane));
    const int32_t groups = (j1 - ja) >> 2;
    int32_t g = lane;
    for (; g + 32 < groups; g += 64) {
        const int32_t j = ja + 4 * g, jy = j + 128;
        const Vec4<int32_t> x = load4<int32_t>(p.bc + j);
        const Vec4<int32_t> y = load4<int32_t>(p.bc + jy);
        if (VM >= 1) {
            add_product<MD, A>(v, acc, x.x, a); add_product<MD, A>(v, acc, x.y, a);
            add_product<MD, A>(v, acc, x.z, a); add_product<MD, A>(v, acc, x.w, a);
            add_product<MD, A>(v, acc, y.x, a); add_product<MD, A>(v, acc, y.y, a);
            add_product<MD, A>(v, acc, y.z, a); add_product<MD, A>(v, acc, y.w, a);
        } else {
            const Vec4<T> bx = load4<T>(p.bv + j);
            const Vec4<T> by = load4<T>(p.bv + jy);
            add_product<MD, A>(v, acc, x.x, a * to_acc<T, A>(bx.x));
            add_product<MD, A>(v, acc, x.y, a * to_acc<T, A>(bx.y));
            add_product<MD, A>(v, acc, x.z, a * to_acc<T, A>(bx.z));
            add_product<MD, A>(v, acc, x.w, a * to_acc<T, A>(bx.w));
            add_product<MD, A>(v, acc, y.x, a * to_acc<T, A>(by.x));
            add_product<MD, A>(v, acc, y.y, a * to_acc<T, A>(by.y));
            add_product<MD, A>(v, acc, y.z, a * to_acc<T, A>(by.z));
            add_product<MD, A>(v, acc, y.w, a * to_acc<T, A>(by.w));
        }
    }
    if (g < groups) {
        const int32_t j = ja + 4 * g;
        const Vec4<int32_t> x = load4<int32_t>(p.bc + j);
        if (VM >= 1) {
            add_product<MD, A>(v, acc, x.x, a); add_product<MD, A>(v, acc, x.y, a);
            add_product<MD, A>(v, acc, x.z, a); add_product<MD, A>(v, acc, x.w, a);
        } else {
            const Vec4<T> bx = load4<T>(p.bv + j);
            add_product<MD, A>(v, acc, x.x, a * to_acc<T, A>(bx.x));
            add_product<MD, A>(v, acc, x.y, a * to_acc<T, A>(bx.y));
            add_product<MD, A>(v, acc, x.z, a * to_acc<T, A>(bx.z));
            add_product<MD, A>(v, acc, x.w, a * to_acc<T, A>(bx.w));
        }
    }
    const int32_t jt = ja + 4 * groups;
    if (jt + lane < j1) add_product<MD, A>(v, acc, __ldg(p.bc + jt + lane), a * bval<VM, T, A>(p, jt + lane));
}

// First index in [lo, hi) of a sorted array whose value is >= key (hi if
// none), found by the whole warp with 32 probes per step: the first step
// probes the ends of the next 32 runs of 32 entries (a short skip costs two
// steps), later steps split what is left 32 ways. GLOBAL: the array is in
// global memory (read-only path), else in shared memory. Warp-uniform
// arguments and result.
template <bool GLOBAL>
__device__ __forceinline__ int32_t warp_lower_bound(const int32_t* a, int32_t lo, int32_t hi, int32_t key) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int64_t step = 32;
    // the answer lies in [lo, hi]; hi itself when every entry below it is < key
    while (hi - lo > 32) {
        const int64_t idx = (int64_t)lo + (int64_t)(lane + 1) * step - 1;
        const bool lt = idx < hi && (GLOBAL ? __ldg(a + idx) : a[idx]) < key;
        const int cnt = __popc(__ballot_sync(FULL, lt));
        if (cnt == 32) {
            lo = (int32_t)min((int64_t)hi, (int64_t)lo + 32 * step);
        } else {
            lo = (int32_t)((int64_t)lo + cnt * step);
            hi = (int32_t)min((int64_t)hi, (int64_t)lo + step - 1);
        }
        step = ((int64_t)(hi - lo) + 31) >> 5;
    }
    const bool lt = lo + lane < hi && (GLOBAL ? __ldg(a + lo + lane) : a[lo + lane]) < key;
    return lo + __popc(__ballot_sync(FULL, lt));
}

// Warp-cooperative sorted merge of B row [bs, be) against the item's sorted
// mask columns; matches add a*b into the slot accumulator. Each step ranks
// 32 B entries against 32 mask columns; the side whose run ends first moves
// past what it resolved, and when the entry 64 ahead on that side is still
// below the other side's first unresolved value, it gallops there by a warp
// search instead of walking (a hub B row against a short mask row costs a
// few searches per mask column, not a pass over the hub). Returns the B
// entries it compared.
template <typename T, typename A>
__device__ __forceinline__ int32_t merge_row(const MxmArgs<T, A>& p, int32_t bs, int32_t be, A av,
                                             const SlotView& v, A* acc) {
    const int lane = threadIdx.x & 31;
    const unsigned FULL = 0xffffffffu;
    if (bs >= be) return 0;
    int32_t yc = warp_lower_bound<false>(v.mcol, 0, v.ns, __ldg(p.bc + bs));
    int32_t xb = bs, seen = 0;
    while (xb < be && yc < v.ns) {
        const int32_t x = (xb + lane < be) ? __ldg(p.bc + xb + lane) : INT32_MAX;
        const int32_t xp = (xb + 63 < be) ? __ldg(p.bc + xb + 63) : INT32_MAX;  // end of the next B run
        const int32_t y = (yc + lane < v.ns) ? v.mcol[yc + lane] : INT32_MAX;
        const int32_t yp = (yc + 63 < v.ns) ? v.mcol[yc + 63] : INT32_MAX;  // end of the next mask run
        seen += min(32, be - xb);
        int r = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            const int32_t yy = __shfl_sync(FULL, y, r + step - 1);
            if (yy < x) r += step;
        }
        const int32_t y31 = __shfl_sync(FULL, y, 31);
        if (r == 31 && y31 < x) r = 32;
        const int32_t yr = __shfl_sync(FULL, y, r & 31);
        if (r < 32 && yr == x && x != INT32_MAX)
            atomic_add_acc<A>(&acc[yc + r], av * to_acc<T, A>(__ldg(p.bv + xb + lane)));
        // the run whose last element is smaller is resolved; for B that is
        // its last stored element (past the row's end the lanes hold INT32_MAX)
        const int32_t xl = __shfl_sync(FULL, x, min(31, be - 1 - xb));
        if (xl <= y31) {
            // mask columns <= xl are resolved too; yu: the first one above
            const unsigned gt = __ballot_sync(FULL, y > xl);
            if (gt == 0u) {
                xb += 32;
                yc += 32;
            } else {
                const int f = __ffs(gt) - 1;
                const int32_t yu = __shfl_sync(FULL, y, f);
                yc += f;
                xb = xp < yu ? warp_lower_bound<true>(p.bc, xb + 64, be, yu) : xb + 32;
            }
        } else {
            // B entries <= y31 are resolved; xu: the first one above
            const int g = __ffs(__ballot_sync(FULL, x > y31)) - 1;
            const int32_t xu = __shfl_sync(FULL, x, g);
            xb += g;
            yc = yp < xu ? warp_lower_bound<false>(v.mcol, yc + 64, v.ns, xu) : yc + 32;
        }
    }
    return seen;
}

// One lane's sorted merge of B row [bs, be) against the mask columns: a
// binary search places the first B column, then the mask position gallops
// (doubling steps, then a binary search) to the first column >= each next
// B column. B columns are loaded four at a time, the next four while the
// current ones are merged.
template <typename T, typename A>
__device__ __forceinline__ void lane_merge(const MxmArgs<T, A>& p, int32_t bs, int32_t be, A av, const SlotView& v,
                                           A* acc) {
    const int32_t* mc = v.mcol;
    const int32_t ns = v.ns;
    int32_t xn[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) xn[q] = bs + q < be ? __ldg(p.bc + bs + q) : INT32_MAX;
    int32_t yc = lower_bound_i32(mc, ns, xn[0]);
    if (yc >= ns) return;
    for (int32_t j = bs; j < be; j += 4) {
        int32_t x[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            x[q] = xn[q];
            xn[q] = j + 4 + q < be ? __ldg(p.bc + j + 4 + q) : INT32_MAX;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (j + q >= be) break;
            if (mc[yc] < x[q]) {
                int32_t b = 1;
                while (yc + b < ns && mc[yc + b] < x[q]) b <<= 1;
                // mc[yc + b/2] < x; mc[yc + b] >= x unless past the end
                int32_t lo = yc + (b >> 1) + 1, hi = min(ns, yc + b);
                while (lo < hi) {
                    const int32_t mid = (lo + hi) >> 1;
                    if (mc[mid] < x[q]) lo = mid + 1; else hi = mid;
                }
                yc = lo;
                if (yc >= ns) return;
            }
            if (mc[yc] == x[q]) atomic_add_acc<A>(&acc[yc], av * to_acc<T, A>(__ldg(p.bv + j + q)));
        }
    }
}

// The lane's share of B entries [j0, j1) cut into 32 contiguous slices,
// merged against the mask by one lane each.
template <typename T, typename A>
__device__ __forceinline__ void merge_slices(const MxmArgs<T, A>& p, int32_t j0, int32_t j1, A av, const SlotView& v,
                                             A* acc) {
    const int32_t per = (j1 - j0 + 31) >> 5;
    const int32_t s0 = j0 + (threadIdx.x & 31) * per, s1 = min(j1, s0 + per);
    if (s0 < s1) lane_merge<T, A>(p, s0, s1, av, v, acc);
}

// Merge variant, 32 A entries at a time (lane l takes entry t0 + l). A B
// row whose part inside [lo, hi] has at most kLaneMerge entries is merged by
// its own lane. In a CTA item (PUSH) one with more than kMergePiece entries
// is listed for the CTA, which cuts it into pieces that all warps share.
// The others are merged by the whole warp afterwards, one at a time: cut
// into 32 slices (merge_slices); or, when a B row is more than kMergeRatio
// times longer than the mask row, by the warp-cooperative merge (which
// gallops over the long B row). Returns the B entries compared
// (warp-uniform; listed rows are counted where their pieces are merged).
constexpr int kLaneMerge = 8;
constexpr int kMergeRatio = 8;
constexpr int kMergePiece = 256;
template <typename T, typename A, bool PUSH>
__device__ __forceinline__ int64_t merge_group(const MxmArgs<T, A>& p, int32_t t0, int32_t ae, bool clip,
                                               const SlotView& v, A* acc, int* s_nlong, int32_t* s_lbs,
                                               int32_t* s_lend, A* s_la) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int32_t t = t0 + lane;
    int32_t bs = 0, be = 0;
    A av = (A)0;
    if (t < ae) {
        b_range(p, t, clip, v.lo, v.hi, bs, be);
        av = to_acc<T, A>(__ldg(p.av + t));
        if (PUSH && be - bs > kMergePiece) {
            const int slot = atomicAdd(s_nlong, 1);
            if (slot < kLongCap) {
                s_lbs[slot] = bs;
                s_lend[slot] = be;
                s_la[slot] = av;
                be = bs;
            }
        }
    }
    const bool wide = be - bs > kLaneMerge;
    if (!wide && bs < be) lane_merge<T, A>(p, bs, be, av, v, acc);
    int64_t seen = warp_sum<int64_t>(wide ? 0 : be - bs);
    for (unsigned w = __ballot_sync(FULL, wide); w; w &= w - 1) {
        const int l = __ffs(w) - 1;
        const int32_t s = __shfl_sync(FULL, bs, l), e = __shfl_sync(FULL, be, l);
        const A a = __shfl_sync(FULL, av, l);
        if ((int64_t)v.ns * kMergeRatio < (int64_t)(e - s)) {
            seen += merge_row<T, A>(p, s, e, a, v, acc);
        } else {
            merge_slices<T, A>(p, s, e, a, v, acc);
            seen += e - s;
        }
    }
    return seen;
}

// Shared-memory layout per variant (MD of the CTA phase: MD_DENSE for MSA).
template <int MD, typename A>
struct MxmSmem {
    static constexpr bool dense = MD == MD_DENSE;
    static constexpr bool filt = MD == MD_BSEARCH;  // bitmap / hashed filter in front of the search
    // CTA phase
    static constexpr size_t off_acc = 0;
    static constexpr size_t off_lbs = off_acc + (size_t)kCtaSlots * sizeof(A);
    static constexpr size_t off_lend = off_lbs + (size_t)kLongCap * 4;
    static constexpr size_t off_lchunk = off_lend + (size_t)kLongCap * 4;
    static constexpr size_t off_la = off_lchunk + (size_t)(kLongCap + 8) * 4;
    static constexpr size_t off_key = off_la + (size_t)kLongCap * sizeof(A);  // bits+wbase, bits+mcol or mcol
    static constexpr size_t off_wbase = off_key + (size_t)kWinWords * 4;
    static constexpr size_t off_fcol = off_key + (size_t)kWinWords * 4;  // MCA: mcol after the bitmap
    static constexpr size_t cta_bytes = dense  ? off_wbase + (size_t)kWinWords * 2
                                        : filt ? off_fcol + (size_t)kCtaSlots * 4
                                               : off_key + (size_t)kCtaSlots * 4;
    // warp phase (per warp): acc, hashed filter + table (MSA) or mcol (others)
    static constexpr size_t w_acc = 0;
    static constexpr size_t w_filt = w_acc + (size_t)kWarpSlots * sizeof(A);
    static constexpr size_t w_hkeys = w_filt + (size_t)(1 << kFilterBits) / 8;
    static constexpr size_t w_hslot = w_hkeys + (size_t)(1 << kWarpTblBits) * 4;
    static constexpr size_t w_mcol = filt ? w_filt + (size_t)(1 << kFilterBits) / 8 : w_filt;
    static constexpr size_t warp_one =
        dense ? w_hslot + (size_t)(1 << kWarpTblBits) : w_mcol + (size_t)kWarpSlots * 4;
    static constexpr size_t warp_bytes = warp_one * kMxmWarps;
    static constexpr size_t region = cta_bytes > warp_bytes ? cta_bytes : warp_bytes;
    // per-warp flattening scratch (both phases)
    static constexpr size_t scratch_bytes = (size_t)kMxmWarps * 32 * (2 * sizeof(int) + sizeof(A));
    static constexpr size_t total = region + scratch_bytes;
};

template <int MD, int VM, typename T, typename A>
__global__ void __launch_bounds__(kMxmThreads, 3) k_mxm_masked(MxmArgs<T, A> p) {
    extern __shared__ __align__(16) unsigned char smem[];
    using SM = MxmSmem<MD, A>;
    constexpr bool DENSE = MD == MD_DENSE;
    constexpr bool FILT = MD == MD_BSEARCH;   // MCA: membership filters in front of the search
    constexpr bool BITS = DENSE || FILT;      // CTA items keep a window bitmap
    constexpr int WMD = DENSE ? MD_HASHED : FILT ? MD_BSEARCH_F : MD;  // warp-row lookup
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned char* scr = smem + SM::region;
    int* s_incl = reinterpret_cast<int*>(scr) + wid * 32;
    int* s_off = reinterpret_cast<int*>(scr) + kMxmWarps * 32 + wid * 32;
    A* s_a = reinterpret_cast<A*>(scr + (size_t)kMxmWarps * 32 * 2 * sizeof(int)) + wid * 32;
    __shared__ int s_item, s_nlong, s_nchunks, s_chunk_next;
    unsigned long long executed = 0;  // products this warp processed (warp-uniform)

    // ------------------------------------------------------------ CTA items
    {
        A* acc = reinterpret_cast<A*>(smem + SM::off_acc);
        int32_t* lbs = reinterpret_cast<int32_t*>(smem + SM::off_lbs);
        int32_t* lend = reinterpret_cast<int32_t*>(smem + SM::off_lend);
        int32_t* lchunk = reinterpret_cast<int32_t*>(smem + SM::off_lchunk);
        A* la = reinterpret_cast<A*>(smem + SM::off_la);
        uint32_t* bits = reinterpret_cast<uint32_t*>(smem + SM::off_key);
        uint16_t* wbase = reinterpret_cast<uint16_t*>(smem + SM::off_wbase);
        int32_t* mcol = reinterpret_cast<int32_t*>(smem + (FILT ? SM::off_fcol : SM::off_key));
        if (BITS)
            for (int t = threadIdx.x; t < kWinWords; t += blockDim.x) bits[t] = 0u;
        const int nheavy = p.q->heavy_count;
        const int ncta = nheavy + p.q->normal_count;
        while (true) {
            if (threadIdx.x == 0) {
                s_item = atomicAdd(&p.q->cta_next, 1);
                s_nlong = 0;
            }
            __syncthreads();
            const int it = s_item;
            if (it >= ncta) break;
            const int4 item = p.cta_items[it < nheavy ? it : p.cta_cap - 1 - (it - nheavy)];
            const int64_t i = item.x;
            const int32_t mb = p.mr[i], mi = (p.mre ? p.mre[i] : p.mr[i + 1]) - mb;
            const int s0 = item.y, ns = item.z - item.y;
            const int32_t* gcol = p.mc + mb + s0;
            SlotView v;
            v.mcol = mcol; v.bits = bits; v.wbase = wbase; v.filt = nullptr; v.hkeys = nullptr; v.hslot = nullptr;
            v.ns = ns;
            v.lo = __ldg(gcol); v.hi = __ldg(gcol + ns - 1);
            for (int s = threadIdx.x; s < ns; s += blockDim.x) {
                const int32_t c = __ldg(gcol + s);
                acc[s] = (A)0;
                if (DENSE) {
                    const uint32_t d = (uint32_t)(c - v.lo);
                    atomicOr(&bits[d >> 5], 1u << (d & 31));
                    if (s == 0 || ((uint32_t)(__ldg(gcol + s - 1) - v.lo) >> 5) != (d >> 5)) wbase[d >> 5] = (uint16_t)s;
                } else {
                    mcol[s] = c;
                    if (FILT) {
                        const uint32_t d = (uint32_t)(c - v.lo);
                        atomicOr(&bits[d >> 5], 1u << (d & 31));
                    }
                }
            }
            __syncthreads();
            // a window that does not span the whole row, or a mask restricted
            // to part of the row, only meets B entries inside [lo, hi]
            const bool clip = ns < mi || p.mre != nullptr;
            const int32_t ab = p.ar[i], ae = p.ar[i + 1];
            if (MD == MD_MERGE) {
                // phase A: groups of up to 32 A entries, small enough that
                // every warp gets one when the row is short; B rows longer
                // than kMergePiece listed
                const int32_t gsz = min(32, (ae - ab + kMxmWarps - 1) / kMxmWarps);
                for (int32_t g = ab + wid * gsz; g < ae; g += kMxmWarps * gsz)
                    executed += (unsigned long long)merge_group<T, A, true>(p, g, min(ae, g + gsz), clip, v, acc,
                                                                            &s_nlong, lbs, lend, la);
            } else {
                // phase A: short B rows flattened per warp, long ones listed
                // (an A row too short to give every warp 32 entries lists
                // its B rows from 32 entries up, so all warps share them)
                const int long_seg = ae - ab < kShortARow ? kLongSegShort : kLongSeg;
                for (int32_t g = ab + wid * 32; g < ae; g += kMxmWarps * 32)
                    executed += (unsigned long long)group_products<MD, VM, T, A, true>(
                        p, g, ae, clip, v, acc, s_incl, s_off, s_a, &s_nlong, lbs, lend, la, long_seg);
            }
            __syncthreads();
            {
                // phase B: long B rows cut into kChunk pieces shared by all warps
                const int nlong = min(s_nlong, kLongCap);
                if (nlong > 0) {
                    if (wid == 0) {
                        int running = 0;
                        for (int base = 0; base < nlong; base += 32) {
                            const int x = base + lane;
                            const int c = x < nlong ? (lend[x] - lbs[x] + kChunk - 1) / kChunk : 0;
                            const int incl = warp_incl_scan(c);
                            if (x < nlong) lchunk[x + 1] = running + incl;
                            running += __shfl_sync(FULL, incl, 31);
                        }
                        if (lane == 0) {
                            lchunk[0] = 0;
                            s_nchunks = running;
                            s_chunk_next = 0;
                        }
                    }
                    __syncthreads();
                    const int nch = s_nchunks;
                    while (true) {
                        int c = 0;
                        if (lane == 0) c = atomicAdd(&s_chunk_next, 1);
                        c = __shfl_sync(FULL, c, 0);
                        if (c >= nch) break;
                        const int seg = upper_bound_i32(lchunk + 1, nlong, c);
                        const int32_t j0 = lbs[seg] + (c - lchunk[seg]) * kChunk;
                        const int32_t j1 = min(lend[seg], j0 + kChunk);
                        if (MD == MD_MERGE) merge_slices<T, A>(p, j0, j1, la[seg], v, acc);
                        else stream_row<MD, VM, T, A>(p, v, acc, j0, j1, la[seg]);
                        executed += (unsigned long long)(j1 - j0);
                    }
                }
            }
            __syncthreads();
            for (int s = threadIdx.x; s < ns; s += blockDim.x) {
                p.cv[mb + s0 + s] = from_acc<T, A>(acc[s]);
                if (BITS) bits[(uint32_t)(__ldg(gcol + s) - v.lo) >> 5] = 0u;
            }
            __syncthreads();
        }
    }

    // ----------------------------------------------------------- warp rows
    {
        unsigned char* base = smem + wid * SM::warp_one;
        A* acc = reinterpret_cast<A*>(base + SM::w_acc);
        uint32_t* filt = reinterpret_cast<uint32_t*>(base + SM::w_filt);
        int32_t* hkeys = reinterpret_cast<int32_t*>(base + SM::w_hkeys);
        uint8_t* hslot = reinterpret_cast<uint8_t*>(base + SM::w_hslot);
        int32_t* mcol = reinterpret_cast<int32_t*>(base + SM::w_mcol);
        constexpr int FW = (1 << kFilterBits) / 32;
        constexpr int TBL = 1 << kWarpTblBits;
        if (DENSE || FILT)
            for (int t = lane; t < FW; t += 32) filt[t] = 0u;
        if (DENSE)
            for (int t = lane; t < TBL; t += 32) hkeys[t] = kEmpty;
        __syncwarp();
        const int nwarp = p.q->warp_count;
        while (true) {
            int r = 0;
            if (lane == 0) r = atomicAdd(&p.q->warp_next, 1);
            r = __shfl_sync(FULL, r, 0);
            if (r >= nwarp) break;
            const int64_t i = p.warp_rows[r];
            const int32_t mb = p.mr[i], mi = (p.mre ? p.mre[i] : p.mr[i + 1]) - mb;
            const bool clip = p.mre != nullptr;
            const int32_t* gcol = p.mc + mb;
            SlotView v;
            v.mcol = mcol; v.bits = nullptr; v.wbase = nullptr; v.filt = filt; v.hkeys = hkeys; v.hslot = hslot;
            v.ns = mi;
            v.lo = __ldg(gcol); v.hi = __ldg(gcol + mi - 1);
            for (int s = lane; s < mi; s += 32) {
                const int32_t c = __ldg(gcol + s);
                acc[s] = (A)0;
                if (DENSE) {
                    const uint32_t h = hash_col(c);
                    const uint32_t f = h >> (32 - kFilterBits);
                    atomicOr(&filt[f >> 5], 1u << (f & 31));
                    hash_insert<uint8_t>(hkeys, hslot, kWarpTblBits, c, (uint8_t)s);
                } else {
                    mcol[s] = c;
                    if (FILT) {
                        const uint32_t f = hash_col(c) >> (32 - kFilterBits);
                        atomicOr(&filt[f >> 5], 1u << (f & 31));
                    }
                }
            }
            __syncwarp();
            const int32_t ab = p.ar[i], ae = p.ar[i + 1];
            if (MD == MD_MERGE) {
                for (int32_t g = ab; g < ae; g += 32)
                    executed += (unsigned long long)merge_group<T, A, false>(p, g, ae, clip, v, acc, nullptr,
                                                                             nullptr, nullptr, nullptr);
            } else {
                for (int32_t g = ab; g < ae; g += 32)
                    executed += (unsigned long long)group_products<WMD, VM, T, A, false>(
                        p, g, ae, clip, v, acc, s_incl, s_off, s_a, nullptr, nullptr, nullptr, nullptr);
            }
            __syncwarp();
            for (int s = lane; s < mi; s += 32) p.cv[mb + s] = from_acc<T, A>(acc[s]);
            if (DENSE || FILT)
                for (int t = lane; t < FW; t += 32) filt[t] = 0u;
            if (DENSE)
                for (int t = lane; t < TBL; t += 32) hkeys[t] = kEmpty;
            __syncwarp();
        }
    }
    if (lane == 0 && executed) atomicAdd(&p.ctr[GA_CTR_EXECUTED], executed);
}

static int64_t cta_item_cap(int64_t m, int64_t n, int64_t mask_nnz) {
    // windows per row <= ceil(m_i / kCtaSlots) + ceil(n / kWinCols), and <= m_i
    const int64_t per_row = 1 + (n + kWinCols - 1) / kWinCols;
    int64_t cap = m * per_row + mask_nnz / kCtaSlots + 1;
    if (cap > mask_nnz + 1) cap = mask_nnz + 1;
    return cap;
}

// Launch the masked product for one value type and lookup variant.
template <int LK, int VM, typename T>
static void launch_masked(ga_ctx ctx, ga_csr A_, ga_csr B_, ga_csr M_, T* cv, MxmQueue* q, int32_t* warp_rows,
                          int4* cta_items, int32_t cta_cap, const int32_t* mre, const int32_t* btr = nullptr,
                          int2* dot_tasks = nullptr) {
    using Ac = typename Acc<T>::type;
    MxmArgs<T, Ac> p;
    p.ar = A_->rst; p.ac = A_->col; p.av = static_cast<const T*>(A_->val);
    p.br = B_->rst; p.bc = B_->col; p.bv = static_cast<const T*>(B_->val);
    p.mr = M_->rst; p.mc = M_->col; p.mre = mre;
    p.cv = cv; p.m = M_->m; p.q = q; p.warp_rows = warp_rows; p.cta_items = cta_items; p.cta_cap = cta_cap;
    p.ctr = ctx->d_counters;
    p.warp_max_flops = ctx->tune.warp_max_flops;
    p.heavy_flops = ctx->tune.heavy_flops;
    p.btr = btr;
    p.dot_tasks = dot_tasks;
    p.hybrid_ratio = ctx->tune.hybrid_ratio;
    {
        ProfScope ps(ctx, "mxm_row_bin");
        int grid = grid_for(p.m * 32, 256, ctx->num_sms * 16);
        k_row_bin<T, Ac><<<grid, 256, 0, ctx->stream>>>(p);
        post_launch("mxm_row_bin");
    }
    const size_t smem = MxmSmem<LK, Ac>::total;
    auto kern = k_mxm_masked<LK, VM, T, Ac>;
    GA_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    GA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kMxmThreads, smem));
    if (per_sm < 1) per_sm = 1;
    if (ctx->tune.ctas_per_sm > 0 && ctx->tune.ctas_per_sm < per_sm) per_sm = ctx->tune.ctas_per_sm;
    const char* name = LK == MD_DENSE ? "mxm_msa" : LK == MD_BSEARCH ? "mxm_mca" : "mxm_heap_merge";
    ProfScope ps(ctx, name);
    kern<<<ctx->num_sms * per_sm, kMxmThreads, smem, ctx->stream>>>(p);
    post_launch(name);
}

// ------------------------------------------------------- inner-product form
// C<M>(i, j) = sum over k in A_i ∩ (B^T)_j of A(i, k) * B(k, j): one warp per
// mask entry, the shorter of the two sorted lists walked 32 entries at a
// time (one per lane), each lane binary-searching the longer one. Warps take
// `chunk` consecutive mask entries; a chunk finds its row by a binary
// search of the row partition `seg`. Row i's mask is [lo[i], hi[i]) within
// the partition [seg[i], seg[i+1]) (the k-truss support evaluates only the
// upper part of each row). No shared memory and no atomics: each mask entry
// is written by one warp.
constexpr int kDotThreads = 256;

template <typename T>
struct DotArgs {
    const int32_t* ar; const int32_t* ac; const T* av;
    const int32_t* tr; const int32_t* tc; const T* tv;  // B^T
    const int32_t* br;                                  // B row starts (product count)
    const int32_t* seg; const int32_t* lo; const int32_t* hi;
    const int32_t* mc;
    T* cv;
    int64_t m, total;
    int chunk;  // mask entries per warp task
    unsigned long long* ctr;
};

// Gustavson products of the masked rows (the work every other variant does),
// mask entries and launch counters, as k_row_bin counts them.
template <typename T>
__global__ void k_dot_count(DotArgs<T> p) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    unsigned long long my_flops = 0, my_mask = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(&p.ctr[GA_CTR_LAUNCHES], 1ull);
        atomicAdd(&p.ctr[GA_CTR_A_ENTRIES], (unsigned long long)(p.ar[p.m] - p.ar[0]));
        atomicAdd(&p.ctr[GA_CTR_ROWS], (unsigned long long)p.m);
    }
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < p.m; i += warps) {
        const int32_t mi = p.hi[i] - p.lo[i];
        if (mi <= 0) continue;
        long long f = 0;
        for (int32_t t = p.ar[i] + lane; t < p.ar[i + 1]; t += 32) {
            const int32_t k = p.ac[t];
            f += p.br[k + 1] - p.br[k];
        }
        f = warp_sum<long long>(f);
        if (lane == 0) {
            my_flops += (unsigned long long)f;
            my_mask += (unsigned long long)mi;
        }
    }
    if (lane == 0 && my_flops) atomicAdd(&p.ctr[GA_CTR_PRODUCTS], my_flops);
    if (lane == 0 && my_mask) atomicAdd(&p.ctr[GA_CTR_MASK_ENTRIES], my_mask);
}

template <typename T, bool UNIT>
__global__ void __launch_bounds__(kDotThreads) k_mxm_dot(DotArgs<T> p) {
    using Ac = typename Acc<T>::type;
    const int lane = threadIdx.x & 31;
    const unsigned FULL = 0xffffffffu;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    unsigned long long executed = 0;
    // entries of the partition as the device holds it now (inside a captured
    // k-truss loop, p.total is only the launch-time upper bound)
    const int64_t total = p.seg[p.m];
    for (int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; c * p.chunk < total; c += warps) {
        const int32_t q0 = (int32_t)(c * p.chunk);
        const int32_t q1 = (int32_t)min((int64_t)q0 + p.chunk, total);
        int i = upper_bound_i32(p.seg, (int)p.m + 1, q0) - 1;
        for (int32_t q = q0; q < q1; ++q) {
            while (q >= p.seg[i + 1]) ++i;
            if (q < p.lo[i] || q >= p.hi[i]) continue;
            const int32_t j = p.mc[q];
            const int32_t ab = p.ar[i], an = p.ar[i + 1] - ab;
            const int32_t tb = p.tr[j], tn = p.tr[j + 1] - tb;
            Ac s = 0;
            if (an > 0 && tn > 0) {
                const bool walk_a = an <= tn;  // walk the shorter list, search the longer
                const int32_t* Wc = walk_a ? p.ac + ab : p.tc + tb;
                const int32_t* Sc = walk_a ? p.tc + tb : p.ac + ab;
                const int wn = walk_a ? an : tn, sn = walk_a ? tn : an;
                if (lane == 0) executed += (unsigned long long)wn;
                // The searched list in registers: up to 32 entries one per
                // lane (searched by shuffles, no memory access), else, when
                // 32 or more entries are walked, the last entry of each of 32
                // equal buckets (the shuffle search picks the bucket, a
                // binary search in memory finishes); else a plain binary
                // search.
                // bucket splitters pay off only when at least 32 entries are walked
                const bool small = sn <= 32, bucketed = !small && wn >= 32;
                int32_t key = INT32_MAX;
                if (small) {
                    key = lane < sn ? __ldg(Sc + lane) : INT32_MAX;
                } else if (bucketed) {
                    const int hi_b = (int)(((int64_t)(lane + 1) * sn) >> 5);
                    key = __ldg(Sc + hi_b - 1);
                }
                for (int base = 0; base < wn; base += 32) {
                    const int e = base + lane;
                    const int32_t x = e < wn ? __ldg(Wc + e) : INT32_MAX;
                    // first register entry >= x (32: none)
                    const int b = (small || bucketed) ? warp_lower_bound(key, x) : 0;
                    bool hit = false;
                    int pos = 0;
                    if (small) {
                        const int32_t y = __shfl_sync(FULL, key, b & 31);
                        pos = b;
                        hit = e < wn && b < sn && y == x;
                    } else if (bucketed) {
                        if (e < wn && b < 32) {
                            const int lo_b = (int)(((int64_t)b * sn) >> 5);
                            const int hi_b = (int)(((int64_t)(b + 1) * sn) >> 5);
                            pos = lo_b + lower_bound_i32(Sc + lo_b, hi_b - lo_b, x);
                            hit = pos < hi_b && __ldg(Sc + pos) == x;
                        }
                    } else if (e < wn) {
                        pos = lower_bound_i32(Sc, sn, x);
                        hit = pos < sn && __ldg(Sc + pos) == x;
                    }
                    if (UNIT) {
                        s += (Ac)__popc(__ballot_sync(FULL, hit));
                    } else if (hit) {
                        const T va = walk_a ? p.av[ab + e] : p.av[ab + pos];
                        const T vb = walk_a ? p.tv[tb + pos] : p.tv[tb + e];
                        s += (Ac)va * (Ac)vb;
                    }
                }
                if (!UNIT) s = warp_sum<Ac>(s);
            }
            if (lane == 0) p.cv[q] = (T)s;
        }
    }
    if (lane == 0 && executed) atomicAdd(&p.ctr[GA_CTR_EXECUTED_DOT], executed);
}

// Hybrid form, inner-product rows: one warp per listed task (a row and up
// to kDotTask of its mask entries), each entry an intersection as in k_mxm_dot.
template <typename T, bool UNIT>
__global__ void __launch_bounds__(kDotThreads) k_mxm_dot_rows(DotArgs<T> p, const int2* __restrict__ tasks,
                                                              const MxmQueue* __restrict__ q) {
    using Ac = typename Acc<T>::type;
    const int lane = threadIdx.x & 31;
    const unsigned FULL = 0xffffffffu;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int n = q->dot_count;
    unsigned long long executed = 0;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
        const int2 task = tasks[r];
        const int32_t i = task.x;
        const int32_t ab = p.ar[i], an = p.ar[i + 1] - ab;
        const int32_t q_end = min(p.hi[i], task.y + kDotTask);
        for (int32_t qq = task.y; qq < q_end; ++qq) {
            const int32_t j = p.mc[qq];
            const int32_t tb = p.tr[j], tn = p.tr[j + 1] - tb;
            Ac s = 0;
            if (an > 0 && tn > 0) {
                const bool walk_a = an <= tn;
                const int32_t* Wc = walk_a ? p.ac + ab : p.tc + tb;
                const int32_t* Sc = walk_a ? p.tc + tb : p.ac + ab;
                const int wn = walk_a ? an : tn, sn = walk_a ? tn : an;
                if (lane == 0) executed += (unsigned long long)wn;
                const bool small = sn <= 32, bucketed = !small && wn >= 32;
                int32_t key = INT32_MAX;
                if (small) {
                    key = lane < sn ? __ldg(Sc + lane) : INT32_MAX;
                } else if (bucketed) {
                    const int hi_b = (int)(((int64_t)(lane + 1) * sn) >> 5);
                    key = __ldg(Sc + hi_b - 1);
                }
                for (int base = 0; base < wn; base += 32) {
                    const int e = base + lane;
                    const int32_t x = e < wn ? __ldg(Wc + e) : INT32_MAX;
                    const int b = (small || bucketed) ? warp_lower_bound(key, x) : 0;
                    bool hit = false;
                    int pos = 0;
                    if (small) {
                        const int32_t y = __shfl_sync(FULL, key, b & 31);
                        pos = b;
                        hit = e < wn && b < sn && y == x;
                    } else if (bucketed) {
                        if (e < wn && b < 32) {
                            const int lo_b = (int)(((int64_t)b * sn) >> 5);
                            const int hi_b = (int)(((int64_t)(b + 1) * sn) >> 5);
                            pos = lo_b + lower_bound_i32(Sc + lo_b, hi_b - lo_b, x);
                            hit = pos < hi_b && __ldg(Sc + pos) == x;
                        }
                    } else if (e < wn) {
                        pos = lower_bound_i32(Sc, sn, x);
                        hit = pos < sn && __ldg(Sc + pos) == x;
                    }
                    if (UNIT) {
                        s += (Ac)__popc(__ballot_sync(FULL, hit));
                    } else if (hit) {
                        const T va = walk_a ? p.av[ab + e] : p.av[ab + pos];
                        const T vb = walk_a ? p.tv[tb + pos] : p.tv[tb + e];
                        s += (Ac)va * (Ac)vb;
                    }
                }
                if (!UNIT) s = warp_sum<Ac>(s);
            }
            if (lane == 0) p.cv[qq] = (T)s;
        }
    }
    if (lane == 0 && executed) atomicAdd(&p.ctr[GA_CTR_EXECUTED_DOT], executed);
}

template <typename T>
static void launch_dot_t(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr Bt, ga_csr M, T* cv, bool unit,
                         const int32_t* mre, const int2* dot_tasks = nullptr, const MxmQueue* q = nullptr) {
    DotArgs<T> p;
    p.ar = A->rst; p.ac = A->col; p.av = static_cast<const T*>(A->val);
    p.tr = Bt->rst; p.tc = Bt->col; p.tv = static_cast<const T*>(Bt->val);
    p.br = B->rst;
    // with mask row ends, M's columns are those of the CSR whose row starts
    // are mre - 1 (the partition of the entries); else M's own rows
    p.seg = mre ? mre - 1 : M->rst;
    p.lo = M->rst;
    p.hi = mre ? mre : M->rst + 1;
    p.mc = M->col;
    p.cv = cv; p.m = M->m; p.ctr = ctx->d_counters;
    p.total = M->nnz;
    p.chunk = ctx->tune.dot_chunk > 0 ? ctx->tune.dot_chunk : 8;
    if (dot_tasks) {  // hybrid form: the tasks binning listed (it also counted the work)
        ProfScope ps(ctx, "mxm_dot_rows");
        const int grid = ctx->num_sms * (2048 / kDotThreads);
        if (unit) k_mxm_dot_rows<T, true><<<grid, kDotThreads, 0, ctx->stream>>>(p, dot_tasks, q);
        else k_mxm_dot_rows<T, false><<<grid, kDotThreads, 0, ctx->stream>>>(p, dot_tasks, q);
        post_launch("mxm_dot_rows");
        return;
    }
    {
        ProfScope ps(ctx, "mxm_dot_count");
        k_dot_count<T><<<grid_for(p.m * 32, 256, ctx->num_sms * 16), 256, 0, ctx->stream>>>(p);
        post_launch("mxm_dot_count");
    }
    if (p.total == 0) return;
    const int grid = grid_for((p.total + p.chunk - 1) / p.chunk * 32, kDotThreads, ctx->num_sms * 16);
    ProfScope ps(ctx, "mxm_dot");
    if (unit) k_mxm_dot<T, true><<<grid, kDotThreads, 0, ctx->stream>>>(p);
    else k_mxm_dot<T, false><<<grid, kDotThreads, 0, ctx->stream>>>(p);
    post_launch("mxm_dot");
}

// Inner-product launch: Bt holds B^T (B itself when B is symmetric); unit:
// A's and B's values are all ones. Allocates nothing (capturable). With
// mask_row_end, M->nnz must be the entry count of the full partition.
void mxm_dot_launch(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr Bt, ga_csr M, void* d_cvals, bool unit,
                    const int32_t* mask_row_end) {
    GA_DISPATCH_DTYPE(A->dtype, T, { launch_dot_t<T>(ctx, A, B, Bt, M, static_cast<T*>(d_cvals), unit, mask_row_end); });
}

void naive_masked_into(ga_ctx ctx, ga_csr A, ga_csr B, ga_csr M, void* d_cvals);

// Hybrid form: inner-product tasks, at most one per kDotTask mask entries of a row.
static int64_t dot_task_cap(int64_t m, int64_t mask_nnz) { return mask_nnz / kDotTask + m + 1; }

size_t mxm_scratch_bytes(int64_t m, int64_t n, int64_t mask_nnz, bool hybrid) {
    // queue header, warp rows, CTA items, hybrid inner-product tasks
    return 256 + sizeof(int32_t) * (size_t)(m + 1) + 16 + sizeof(int4) * (size_t)cta_item_cap(m, n, mask_nnz) +
           (hybrid ? sizeof(int2) * (size_t)dot_task_cap(m, mask_nnz) : 0);
}

// Non-allocating launch (usable inside captured loops): `scratch` holds
// mxm_scratch_bytes(M->m, M->n, max nnz(M)) bytes; `cap_nnz` is that max.
// unit_b: B's values are all ones (no value loads). mask_row_end (optional):
// row i's mask is [M->rst[i], mask_row_end[i]) instead of the whole row.
void mxm_masked_launch(ga_ctx ctx, ga_algo algo, ga_csr A, ga_csr B, ga_csr M, void* d_cvals, void* scratch,
                       int64_t cap_nnz, bool unit_b, const int32_t* mask_row_end, bool unit_a, ga_csr Bt) {
    GA_REQUIRE(algo == GA_MSA || algo == GA_MCA || algo == GA_HEAP || algo == GA_HYBRID, GA_ERR_INVALID_ARG,
               "mxm: unknown algorithm");
    GA_REQUIRE(algo != GA_HYBRID || Bt != nullptr, GA_ERR_INVALID_ARG, "mxm: the hybrid form needs B^T");
    unsigned char* s = static_cast<unsigned char*>(scratch);
    MxmQueue* q = reinterpret_cast<MxmQueue*>(s);
    int32_t* warp_rows = reinterpret_cast<int32_t*>(s + 256);
    size_t off = 256 + sizeof(int32_t) * (size_t)(M->m + 1);
    off = (off + 15) & ~(size_t)15;
    int4* cta_items = reinterpret_cast<int4*>(s + off);
    const int64_t cap = cta_item_cap(M->m, M->n, cap_nnz);
    int2* dot_tasks = algo == GA_HYBRID ? reinterpret_cast<int2*>(s + off + sizeof(int4) * (size_t)cap) : nullptr;
    GA_REQUIRE(cap < INT32_MAX, GA_ERR_UNSUPPORTED, "mxm: too many work items");
    k_reset_queue<<<1, 32, 0, ctx->stream>>>(q);
    post_launch("mxm_reset_queue");
    GA_DISPATCH_DTYPE(A->dtype, T, {
        T* cv = static_cast<T*>(d_cvals);
        const int32_t c32 = (int32_t)cap;
        // value mode 2 (every product is 1) only for int32, the k-truss / TC type
        const bool ones = unit_a && unit_b && std::is_same<T, int32_t>::value;
        if (algo == GA_HYBRID) {
            // Gustavson (MSA) rows, then the inner-product rows flagged while binning
            const int32_t* btr = Bt->rst;
            if (ones)
                launch_masked<MD_DENSE, 2, T>(ctx, A, B, M, cv, q, warp_rows, cta_items, c32, mask_row_end, btr,
                                              dot_tasks);
            else if (unit_b)
                launch_masked<MD_DENSE, 1, T>(ctx, A, B, M, cv, q, warp_rows, cta_items, c32, mask_row_end, btr,
                                              dot_tasks);
            else
                launch_masked<MD_DENSE, 0, T>(ctx, A, B, M, cv, q, warp_rows, cta_items, c32, mask_row_end, btr,
                                              dot_tasks);
            launch_dot_t<T>(ctx, A, B, Bt, M, cv, unit_a && unit_b, mask_row_end, dot_tasks, q);
        } else if (algo == GA_MSA) {
            if (ones) launch_masked<MD_DENSE, 2, T>(ctx, A, B, M, cv, q, warp_rows, cta_items, c32, mask_row_end);
            else if (unit_b) launch_masked<MD_DENSE, 1, T>(ctx, A, B, M, cv, q, warp_rows, cta_items, c32, mask_row_end);
            else launch_masked<MD_DENSE, 0, T>(ctx, A, B, M, cv, q, warp_rows, cta_items, c32, mask_row_end);
        } else if (algo == GA_MCA) {
            if (unit_b) launch_masked<MD_BSEARCH, 1, T>(ctx, A, B, M, cv, q, warp_rows, cta_items, c32, mask_row_end);
            else launch_masked<MD_BSEARCH, 0, T>(ctx, A, B, M, cv, q, warp_rows, cta_items, c32, mask_row_end);
        } else {
            launch_masked<MD_MERGE, 0, T>(ctx, A, B, M, cv, q, warp_rows, cta_items, c32, mask_row_end);
        }
    });
}

void mxm_masked_into(ga_ctx ctx, ga_algo algo, ga_csr A, ga_csr B, ga_csr M, void* d_cvals) {
    GA_REQUIRE(A->n == B->m, GA_ERR_SHAPE, "mxm: A.n != B.m");
    GA_REQUIRE(M->m == A->m && M->n == B->n, GA_ERR_SHAPE, "mxm: mask shape differs from A*B");
    GA_REQUIRE(A->dtype == B->dtype, GA_ERR_DTYPE, "mxm: A and B dtypes differ");
    if (M->nnz == 0 || M->m == 0) return;
    TuneScope tscope(ctx);
    algo = resolve_mxm_algo(ctx, algo, A, B, M);
    if (algo == GA_TRI) {
        if (tri_applies(ctx, A, B, M)) {
            tri_masked_into(ctx, A, static_cast<int32_t*>(d_cvals));
            return;
        }
        algo = GA_HYBRID;
    }
    if (algo == GA_NAIVE) {
        naive_masked_into(ctx, A, B, M, d_cvals);
        return;
    }
    if (algo == GA_DOT || algo == GA_HYBRID) {
        const bool unit_b = csr_unit_values(ctx, B);
        const bool unit_a = csr_unit_values(ctx, A);
        const bool sym = csr_is_symmetric(ctx, B);
        ga_csr Bt = sym ? B : transpose_csr(ctx, B);
        try {
            if (algo == GA_DOT) {
                mxm_dot_launch(ctx, A, B, Bt, M, d_cvals, unit_a && unit_b, nullptr);
            } else {
                DBuf<unsigned char> scratch(ctx, mxm_scratch_bytes(M->m, M->n, M->nnz));
                mxm_masked_launch(ctx, GA_HYBRID, A, B, M, d_cvals, scratch.p, M->nnz, unit_b, nullptr,
                                  unit_a && A->dtype == GA_INT32, Bt);
            }
        } catch (...) {
            if (!sym) csr_destroy(ctx, Bt);
            throw;
        }
        if (!sym) csr_destroy(ctx, Bt);
        return;
    }
    const bool unit_b = csr_unit_values(ctx, B);
    const bool unit_a = unit_b && A->dtype == GA_INT32 && csr_unit_values(ctx, A);
    DBuf<unsigned char> scratch(ctx, mxm_scratch_bytes(M->m, M->n, M->nnz));
    mxm_masked_launch(ctx, algo, A, B, M, d_cvals, scratch.p, M->nnz, unit_b, nullptr, unit_a);
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
