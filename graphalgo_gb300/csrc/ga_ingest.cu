// Graph ingestion on the device: edge lists to CSR (the reference CLI's
// preparation steps as flags, rows sorted, duplicates merged), Matrix Market
// coordinate files parsed on the device (read_mtx_to_crs semantics,
// include/matrix.h:280-417), and the reference's binary CSR layout
// (write_crs_to_bin / read_bin_to_crs, include/matrix.h:259-277, 441-482).
//
// Edge list to CSR, in six launches plus the row sort:
//   check     endpoints inside the matrix
//   count     entries per row after the flags' expansion (atomics)
//   fill      each entry at an atomically reserved slot of its row, with its
//             edge index as the payload
//   sort      rows by column (sort_rows_by_key)
//   heads     first entry of every run of equal (row, column)
//   compact   one entry per run, value of the run's smallest edge index
// Matrix Market bodies are tokenised on the device: a token starts at a
// non-space byte after a space; token positions come from a block count, a
// scan and a block-local recount; then one thread parses one entry.
#include "ga_device.cuh"

#include <clocale>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <locale.h>
#include <string>
#include <vector>

namespace ga {

// ================================================================ edge lists
struct EdgeRule {
    bool mirror_in;   // each edge also as its reverse (symmetric files)
    bool drop_loops;  // drop (i, i)
    bool lower;       // keep i > j only, and each kept entry's mirror
};

// Entries that edge (s, d) stands for under `r`, in the reference's order.
__device__ __forceinline__ int edge_entries(int32_t s, int32_t d, EdgeRule r, int32_t* er, int32_t* ec) {
    int n = 0;
    for (int t = 0; t < (r.mirror_in ? 2 : 1); ++t) {
        const int32_t a = t ? d : s, b = t ? s : d;
        if ((r.drop_loops || r.lower) && a == b) continue;
        if (r.lower && a < b) continue;
        er[n] = a; ec[n] = b; ++n;
        if (r.lower) { er[n] = b; ec[n] = a; ++n; }
    }
    return n;
}

__global__ void k_edges_check(const int32_t* __restrict__ src, const int32_t* __restrict__ dst, int64_t ne,
                              int64_t m, int64_t n, int* __restrict__ flag) {
    bool bad = false;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x)
        bad |= src[e] < 0 || src[e] >= m || dst[e] < 0 || dst[e] >= n;
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

__global__ void k_edges_count(const int32_t* __restrict__ src, const int32_t* __restrict__ dst, int64_t ne,
                              EdgeRule r, int32_t* __restrict__ cnt) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
        int32_t er[4], ec[4];
        const int k = edge_entries(src[e], dst[e], r, er, ec);
        for (int t = 0; t < k; ++t) atomicAdd(&cnt[er[t]], 1);
    }
}

__global__ void k_edges_fill(const int32_t* __restrict__ src, const int32_t* __restrict__ dst, int64_t ne,
                             EdgeRule r, int32_t* __restrict__ cursor, int32_t* __restrict__ col,
                             int32_t* __restrict__ pay) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
        int32_t er[4], ec[4];
        const int k = edge_entries(src[e], dst[e], r, er, ec);
        for (int t = 0; t < k; ++t) {
            const int32_t p = atomicAdd(&cursor[er[t]], 1);
            col[p] = ec[t];
            pay[p] = (int32_t)e;
        }
    }
}

// head[q] = 1 when entry q starts a run of equal columns in its row.
__global__ void k_run_heads(const int32_t* __restrict__ col, int64_t nnz, int32_t* __restrict__ head) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x)
        head[q] = q == 0 || col[q] != col[q - 1];
}

__global__ void k_row_heads(const int32_t* __restrict__ rst, int64_t m, int32_t* __restrict__ head) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        if (rst[i] < rst[i + 1]) head[rst[i]] = 1;
}

// One output entry per run; `hs` is the exclusive scan of the heads.
template <typename T>
__global__ void k_runs_compact(const int32_t* __restrict__ col, const int32_t* __restrict__ pay,
                               const int32_t* __restrict__ head, const int32_t* __restrict__ hs, int64_t nnz,
                               const T* __restrict__ val, int32_t* __restrict__ ocol, T* __restrict__ oval) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x) {
        if (!head[q]) continue;
        int32_t best = pay[q];
        for (int64_t t = q + 1; t < nnz && !head[t]; ++t) best = min(best, pay[t]);
        const int32_t o = hs[q];
        ocol[o] = col[q];
        oval[o] = val ? val[best] : (T)1;
    }
}

__global__ void k_runs_rst(const int32_t* __restrict__ rst, const int32_t* __restrict__ hs, int64_t m,
                           int32_t* __restrict__ orst) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= m; i += (int64_t)gridDim.x * blockDim.x)
        orst[i] = hs[rst[i]];
}

static EdgeRule rule_of(int flags) {
    EdgeRule r;
    r.mirror_in = (flags & GA_EDGES_MIRROR) != 0;
    r.drop_loops = (flags & GA_EDGES_DROP_LOOPS) != 0;
    r.lower = (flags & GA_EDGES_LOWER_SYMM) != 0;
    return r;
}

static constexpr int kEdgeFlags = GA_EDGES_MIRROR | GA_EDGES_DROP_LOOPS | GA_EDGES_LOWER_SYMM | GA_EDGES_UNIT;

// Device edge arrays to a CSR; val (device, `dt`) may be null for all-1
// values. With GA_EDGES_UNIT the values are int32 ones.
static ga_csr edges_to_csr(ga_ctx ctx, int64_t m, int64_t n, int64_t ne, const int32_t* src, const int32_t* dst,
                           const void* val, ga_dtype dt, int flags) {
    GA_REQUIRE((flags & ~kEdgeFlags) == 0, GA_ERR_INVALID_ARG, "edges: unknown flag");
    const EdgeRule r = rule_of(flags);
    GA_REQUIRE(!(r.mirror_in || r.lower) || m == n, GA_ERR_SHAPE, "edges: mirroring needs a square matrix");
    GA_REQUIRE(m < INT32_MAX && n < INT32_MAX && ne < INT32_MAX, GA_ERR_INVALID_ARG,
               "edges: beyond the int32 index range");
    if (flags & GA_EDGES_UNIT) {
        val = nullptr;
        dt = GA_INT32;
    }
    ProfScope ps(ctx, "edges_to_csr");
    const int grid_e = grid_for(ne, 256, ctx->num_sms * 8);
    if (ne) {
        DBuf<int> flag(ctx, 1);
        GA_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), ctx->stream));
        k_edges_check<<<grid_e, 256, 0, ctx->stream>>>(src, dst, ne, m, n, flag.p);
        post_launch("edges_check");
        GA_REQUIRE(read_i32(ctx, flag.p) == 0, GA_ERR_INVALID_ARG, "edges: an endpoint is outside the matrix");
    }
    // up to four entries per edge: the total must stay in int32
    GA_REQUIRE(ne < INT32_MAX / ((r.mirror_in ? 2 : 1) * (r.lower ? 2 : 1)), GA_ERR_INVALID_ARG,
               "edges: the expanded entry count is beyond the int32 index range");
    DBuf<int32_t> rst(ctx, (size_t)m + 1);
    GA_CUDA(cudaMemsetAsync(rst.p, 0, sizeof(int32_t) * (m + 1), ctx->stream));
    int prof = prof_begin(ctx, "edges_count");
    if (ne) {
        k_edges_count<<<grid_e, 256, 0, ctx->stream>>>(src, dst, ne, r, rst.p);
        post_launch("edges_count");
    }
    prof_end(ctx, prof);
    scan_exclusive_i32(ctx, rst.p, rst.p, m);
    const int64_t kept = m ? read_i32(ctx, rst.p + m) : 0;
    DBuf<int32_t> col(ctx, (size_t)kept + 1), pay(ctx, (size_t)kept + 1);
    if (kept) {
        DBuf<int32_t> cursor(ctx, (size_t)m + 1);
        GA_CUDA(cudaMemcpyAsync(cursor.p, rst.p, sizeof(int32_t) * (m + 1), cudaMemcpyDeviceToDevice, ctx->stream));
        prof = prof_begin(ctx, "edges_fill");
        k_edges_fill<<<grid_e, 256, 0, ctx->stream>>>(src, dst, ne, r, cursor.p, col.p, pay.p);
        post_launch("edges_fill");
        prof_end(ctx, prof);
        sort_rows_by_key(ctx, rst.p, m, col.p, pay.p, kept);
    }
    prof = prof_begin(ctx, "edges_runs");
    DBuf<int32_t> head(ctx, (size_t)kept + 1), hs(ctx, (size_t)kept + 1);
    const int grid_q = grid_for(kept, 256, ctx->num_sms * 8);
    if (kept) {
        k_run_heads<<<grid_q, 256, 0, ctx->stream>>>(col.p, kept, head.p);
        post_launch("run_heads");
        k_row_heads<<<grid_for(m, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(rst.p, m, head.p);
        post_launch("row_heads");
    }
    scan_exclusive_i32(ctx, head.p, hs.p, kept);
    const int64_t nnz = kept ? read_i32(ctx, hs.p + kept) : 0;
    ga_csr A = csr_alloc(ctx, m, n, nnz, dt);
    try {
        k_runs_rst<<<grid_for(m + 1, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(rst.p, hs.p, m, A->rst);
        post_launch("runs_rst");
        if (kept) {
            GA_DISPATCH_DTYPE(dt, T, {
                k_runs_compact<T><<<grid_q, 256, 0, ctx->stream>>>(col.p, pay.p, head.p, hs.p, kept,
                                                                   static_cast<const T*>(val), A->col,
                                                                   static_cast<T*>(A->val));
            });
            post_launch("runs_compact");
        }
        prof_end(ctx, prof);
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
    } catch (...) {
        csr_destroy(ctx, A);
        throw;
    }
    if (!val) A->unit = 1;
    return A;
}

// ================================================================ R-MAT
// The host generator's random streams (ga_gen.cpp): xoshiro256** seeded by
// splitmix64 per chunk of 2^16 edges; one thread walks one chunk, so every
// edge gets the same bits as on the host.
__device__ __forceinline__ uint64_t dev_splitmix64(uint64_t& x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct DevXoshiro {
    uint64_t s0, s1, s2, s3;
    __device__ explicit DevXoshiro(uint64_t seed) {
        uint64_t x = seed;
        s0 = dev_splitmix64(x);
        s1 = dev_splitmix64(x);
        s2 = dev_splitmix64(x);
        s3 = dev_splitmix64(x);
    }
    __device__ static uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
    __device__ uint64_t next() {
        const uint64_t r = rotl(s1 * 5, 7) * 9;
        const uint64_t t = s1 << 17;
        s2 ^= s0; s3 ^= s1; s1 ^= s2; s0 ^= s3;
        s2 ^= t;
        s3 = rotl(s3, 45);
        return r;
    }
    __device__ double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

constexpr int64_t kRmatChunk = 1 << 16;

__global__ void k_rmat_edges(int scale, int64_t edges, double a, double ab, double abc, uint64_t seed,
                             int32_t* __restrict__ src, int32_t* __restrict__ dst) {
    const int64_t ch = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t e0 = ch * kRmatChunk;
    if (e0 >= edges) return;
    const int64_t e1 = min(edges, e0 + kRmatChunk);
    uint64_t x = seed ^ (0xD1B54A32D192ED03ull * ((uint64_t)ch + 1));
    DevXoshiro rng(dev_splitmix64(x));
    for (int64_t e = e0; e < e1; ++e) {
        uint32_t u = 0, v = 0;
        for (int l = 0; l < scale; ++l) {
            const double r = rng.uniform();
            const uint32_t bu = r >= ab, bv = (r >= a && r < ab) || r >= abc;
            u = (u << 1) | bu;
            v = (v << 1) | bv;
        }
        src[e] = (int32_t)u;
        dst[e] = (int32_t)v;
    }
}

static ga_csr gen_rmat_device(ga_ctx ctx, int scale, int edge_factor, double a, double b, double c, uint64_t seed) {
    GA_REQUIRE(scale >= 1 && scale <= 26 && edge_factor >= 1, GA_ERR_INVALID_ARG, "rmat: scale or edge factor");
    GA_REQUIRE(a >= 0 && b >= 0 && c >= 0 && a + b + c <= 1.0, GA_ERR_INVALID_ARG, "rmat: quadrant probabilities");
    const int64_t n = 1ll << scale, edges = n * edge_factor;
    GA_REQUIRE(edges < INT32_MAX / 2, GA_ERR_INVALID_ARG, "rmat: too many edges for int32 entries");
    DBuf<int32_t> src(ctx, (size_t)edges), dst(ctx, (size_t)edges);
    const int64_t nch = (edges + kRmatChunk - 1) / kRmatChunk;
    {
        ProfScope ps(ctx, "rmat_edges");
        k_rmat_edges<<<(unsigned)((nch + 63) / 64), 64, 0, ctx->stream>>>(scale, edges, a, a + b, a + b + c, seed,
                                                                          src.p, dst.p);
        post_launch("rmat_edges");
    }
    return edges_to_csr(ctx, n, n, edges, src.p, dst.p, nullptr, GA_INT32,
                        GA_EDGES_MIRROR | GA_EDGES_DROP_LOOPS | GA_EDGES_UNIT);
}

// ============================================================ file staging
struct File {
    FILE* f = nullptr;
    File(const char* path, const char* mode) : f(fopen(path, mode)) {}
    ~File() {
        if (f) fclose(f);
    }
};

// Copies `bytes` from the file's current position to device memory at `dst`
// through two pinned staging buffers, so reading chunk k+1 overlaps the copy
// of chunk k.
static void file_to_device(ga_ctx ctx, FILE* f, void* dst, int64_t bytes, const char* what) {
    if (bytes <= 0) return;
    const int64_t chunk = bytes < (32 << 20) ? bytes : (32 << 20);
    char* stage[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    auto release = [&]() {
        for (int b = 0; b < 2; ++b) {
            if (done[b]) cudaEventDestroy(done[b]);
            if (stage[b]) cudaFreeHost(stage[b]);
        }
    };
    try {
        for (int b = 0; b < 2; ++b) {
            GA_CUDA(cudaMallocHost((void**)&stage[b], (size_t)chunk));
            GA_CUDA(cudaEventCreateWithFlags(&done[b], cudaEventDisableTiming));
        }
        int64_t off = 0;
        for (int k = 0; off < bytes; ++k) {
            const int b = k & 1;
            const int64_t len = bytes - off < chunk ? bytes - off : chunk;
            GA_CUDA(cudaEventSynchronize(done[b]));
            if ((int64_t)fread(stage[b], 1, (size_t)len, f) != len)
                fail(GA_ERR_INVALID_ARG, std::string(what) + ": truncated file");
            GA_CUDA(cudaMemcpyAsync(static_cast<char*>(dst) + off, stage[b], (size_t)len, cudaMemcpyHostToDevice,
                                    ctx->stream));
            GA_CUDA(cudaEventRecord(done[b], ctx->stream));
            off += len;
        }
        for (int b = 0; b < 2; ++b) GA_CUDA(cudaEventSynchronize(done[b]));
    } catch (...) {
        cudaStreamSynchronize(ctx->stream);
        release();
        throw;
    }
    release();
}

// ============================================================ Matrix Market
constexpr int kTokThreads = 256;
constexpr int kTokBytes = 64;  // bytes per thread
constexpr int64_t kTokBlockBytes = (int64_t)kTokThreads * kTokBytes;

__device__ __forceinline__ bool is_space(unsigned c) { return c == ' ' || (c >= 9 && c <= 13); }

// Token starts among this thread's kTokBytes bytes (bit b: byte base + b);
// `text` is padded with spaces to a whole number of blocks.
__device__ __forceinline__ uint64_t token_start_mask(const unsigned char* __restrict__ text, int64_t base) {
    unsigned prev = base ? text[base - 1] : ' ';
    uint64_t mask = 0;
    const uint4* p = reinterpret_cast<const uint4*>(text + base);
#pragma unroll
    for (int v = 0; v < kTokBytes / 16; ++v) {
        const uint4 w = p[v];
        const uint32_t words[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int b = 0; b < 16; ++b) {
            const unsigned c = (words[b >> 2] >> (8 * (b & 3))) & 0xffu;
            if (!is_space(c) && is_space(prev)) mask |= 1ull << (v * 16 + b);
            prev = c;
        }
    }
    return mask;
}

__global__ void __launch_bounds__(kTokThreads) k_tok_count(const unsigned char* __restrict__ text,
                                                           int64_t* __restrict__ block_count) {
    __shared__ int warp_sum[kTokThreads / 32];
    const int64_t base = ((int64_t)blockIdx.x * kTokThreads + threadIdx.x) * kTokBytes;
    int c = __popcll(token_start_mask(text, base));
    c = __reduce_add_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t t = 0;
        for (int w = 0; w < kTokThreads / 32; ++w) t += warp_sum[w];
        block_count[blockIdx.x] = t;
    }
}

// Writes the byte offset of every token with index < need.
__global__ void __launch_bounds__(kTokThreads) k_tok_emit(const unsigned char* __restrict__ text,
                                                          const int64_t* __restrict__ block_off, int64_t need,
                                                          int64_t* __restrict__ tokpos) {
    __shared__ int warp_sum[kTokThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t base = ((int64_t)blockIdx.x * kTokThreads + threadIdx.x) * kTokBytes;
    uint64_t mask = token_start_mask(text, base);
    const int c = __popcll(mask);
    int incl = c;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int x = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += x;
    }
    if (lane == 31) warp_sum[warp] = incl;
    __syncthreads();
    int64_t idx = block_off[blockIdx.x] + incl - c;
    for (int w = 0; w < warp; ++w) idx += warp_sum[w];
    while (mask && idx < need) {
        const int b = __ffsll((long long)mask) - 1;
        mask &= mask - 1;
        tokpos[idx++] = base + b;
    }
}

enum : int {
    kBadIndex = 1,    // row or column token is not an integer
    kIndexRange = 2,  // row or column outside 1..m / 1..n
    kBadValue = 4,    // integer value token malformed or beyond int32
};

// Decimal integer with an optional sign, ending at a space; false on
// anything else.
__device__ bool parse_int(const unsigned char* __restrict__ s, int64_t& out) {
    int i = 0;
    bool neg = false;
    if (s[0] == '+' || s[0] == '-') {
        neg = s[0] == '-';
        i = 1;
    }
    int64_t v = 0;
    int nd = 0;
    for (; s[i] >= '0' && s[i] <= '9'; ++i, ++nd) {
        if (nd >= 18) return false;
        v = v * 10 + (s[i] - '0');
    }
    if (nd == 0 || !is_space(s[i])) return false;
    out = neg ? -v : v;
    return true;
}

// Correct rounding (to nearest, ties to even) of an exact positive rational
// to a double, by integer arithmetic from the definition of IEEE rounding:
// the value is m * 2^x with m the 53 leading bits of the exact quotient
// (or product), incremented when the dropped part exceeds half an ulp or
// equals it with m odd. Results here are always in the normal range.
__device__ __forceinline__ int msb128(unsigned __int128 v) {
    const uint64_t hi = (uint64_t)(v >> 64);
    return hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)(uint64_t)v);
}

// m in [2^52, 2^53] (2^53 after a rounding carry) times 2^x as a double.
__device__ __forceinline__ double make_double(uint64_t m, int x) {
    if (m == (1ull << 53)) {
        m >>= 1;
        ++x;
    }
    const uint64_t bits = ((uint64_t)(1075 + x) << 52) | (m & ((1ull << 52) - 1));
    return __longlong_as_double((long long)bits);
}

// N > 0, exact integer.
__device__ double round_u128(unsigned __int128 N) {
    const int p = msb128(N);
    if (p <= 52) return (double)(uint64_t)N;  // exactly representable
    const int sh = p - 52;
    uint64_t m = (uint64_t)(N >> sh);
    const unsigned __int128 rem = N & ((((unsigned __int128)1) << sh) - 1);
    const unsigned __int128 half = ((unsigned __int128)1) << (sh - 1);
    if (rem > half || (rem == half && (m & 1))) ++m;
    return make_double(m, sh);
}

// w / 10^k for w >= 1 and 1 <= k <= 22: the integer quotient q of
// w * 2^s / 10^k, with s >= 0 the least shift that makes q exceed 2^53
// (the numerator stays below 2^(54 + bits(10^k)) <= 2^128); the remainder
// is the sticky bit.
__device__ double round_div_pow10(uint64_t w, int k) {
    unsigned __int128 D = 1;
    for (int t = 0; t < k; ++t) D *= 10u;
    const int bw = 64 - __clzll((long long)w), bd = msb128(D) + 1;
    const int s = 54 + bd - bw > 0 ? 54 + bd - bw : 0;
    const unsigned __int128 N = ((unsigned __int128)w) << s;
    const unsigned __int128 q = N / D;  // 2^53 <= q < 2^64
    const bool sticky = (N - q * D) != 0;
    const int sh = msb128(q) - 52;  // 1 to 11
    uint64_t m = (uint64_t)(q >> sh);
    const uint64_t rem = (uint64_t)q & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (sticky || (m & 1)))) ++m;
    return make_double(m, sh - s);
}

// Decimal real [+-] digits [. digits] [(e|E) [+-] digits] with at most 19
// significant digits W and a decimal exponent e (value W * 10^e) such that
// -22 <= e and W * 10^e < 2^128: correctly rounded, so equal to strtod.
// Anything else (more digits, other exponents, inf/nan/hex forms) returns
// false and is converted on the host.
__device__ bool parse_real(const unsigned char* __restrict__ s, double& out) {
    int i = 0;
    bool neg = false;
    if (s[0] == '+' || s[0] == '-') {
        neg = s[0] == '-';
        i = 1;
    }
    uint64_t w = 0;
    int nd = 0, e10 = 0;
    bool any = false;
    for (; s[i] >= '0' && s[i] <= '9'; ++i) {
        any = true;
        if (w == 0 && s[i] == '0') continue;
        if (nd >= 19) return false;
        w = w * 10 + (s[i] - '0');
        ++nd;
    }
    if (s[i] == '.') {
        for (++i; s[i] >= '0' && s[i] <= '9'; ++i) {
            any = true;
            if (w == 0 && s[i] == '0') {
                --e10;
                continue;
            }
            if (nd >= 19) return false;
            w = w * 10 + (s[i] - '0');
            ++nd;
            --e10;
        }
    }
    if (!any) return false;
    if (s[i] == 'e' || s[i] == 'E') {
        ++i;
        bool eneg = false;
        if (s[i] == '+' || s[i] == '-') {
            eneg = s[i] == '-';
            ++i;
        }
        int ex = 0, ed = 0;
        for (; s[i] >= '0' && s[i] <= '9'; ++i, ++ed) {
            if (ex > 100000) return false;
            ex = ex * 10 + (s[i] - '0');
        }
        if (ed == 0) return false;
        e10 += eneg ? -ex : ex;
    }
    if (!is_space(s[i])) return false;
    double v;
    if (w == 0) {
        v = 0.0;
    } else if (e10 < 0) {
        if (e10 < -22) return false;
        v = round_div_pow10(w, -e10);
    } else {
        if (e10 > 38) return false;
        unsigned __int128 P = 1;
        for (int t = 0; t < e10; ++t) P *= 10u;
        if (64 - __clzll((long long)w) + msb128(P) + 1 > 128) return false;  // product could pass 2^128
        v = round_u128((unsigned __int128)w * P);
    }
    out = neg ? -v : v;
    return true;
}

// value_kind: 0 none (pattern, or values not wanted), 1 int32, 2 double.
__global__ void k_mtx_entries(const unsigned char* __restrict__ text, const int64_t* __restrict__ tokpos,
                              int64_t nz, int per, int value_kind, int64_t m, int64_t n,
                              int32_t* __restrict__ src, int32_t* __restrict__ dst, void* __restrict__ val,
                              int* __restrict__ err, int64_t* __restrict__ slow, int64_t* __restrict__ nslow) {
    int bad = 0;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nz; e += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = 0, j = 0;
        src[e] = dst[e] = 0;
        if (!parse_int(text + tokpos[per * e], i) || !parse_int(text + tokpos[per * e + 1], j)) {
            bad |= kBadIndex;
            continue;
        }
        if (i < 1 || i > m || j < 1 || j > n) {
            bad |= kIndexRange;
            continue;
        }
        src[e] = (int32_t)(i - 1);
        dst[e] = (int32_t)(j - 1);
        if (value_kind == 1) {
            int64_t v = 0;
            if (!parse_int(text + tokpos[per * e + 2], v) || v < INT32_MIN || v > INT32_MAX) {
                bad |= kBadValue;
                v = 0;
            }
            static_cast<int32_t*>(val)[e] = (int32_t)v;
        } else if (value_kind == 2) {
            double v = 0.0;
            if (!parse_real(text + tokpos[per * e + 2], v))
                slow[atomicAdd(reinterpret_cast<unsigned long long*>(nslow), 1ull)] = e;
            static_cast<double*>(val)[e] = v;
        }
    }
    if (bad) atomicOr(err, bad);
}

__global__ void k_gather_slow_pos(const int64_t* __restrict__ slow, int64_t count,
                                  const int64_t* __restrict__ tokpos, int per, int64_t* __restrict__ pos) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += (int64_t)gridDim.x * blockDim.x)
        pos[t] = tokpos[per * slow[t] + 2];
}

__global__ void k_scatter_f64(const int64_t* __restrict__ idx, const double* __restrict__ v, int64_t count,
                              double* __restrict__ out) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += (int64_t)gridDim.x * blockDim.x)
        out[idx[t]] = v[t];
}

struct MtxHeader {
    char code[4] = {'M', 'C', 'R', 'G'};
    int64_t m = 0, n = 0, nz = 0;
    long body = 0;  // byte offset of the first entry
};

static bool read_line(FILE* f, std::string& line) {
    line.clear();
    int c;
    while ((c = fgetc(f)) != EOF) {
        if (c == '\n') return true;
        line.push_back((char)c);
    }
    return !line.empty();
}

static std::string lower(std::string s) {
    for (auto& c : s) c = (char)((c >= 'A' && c <= 'Z') ? c - 'A' + 'a' : c);
    return s;
}

// Banner "%%MatrixMarket matrix <coordinate|array> <field> <symmetry>" (the
// fields of src/mmio.cpp mm_read_banner), comment and blank lines, "m n nz".
static MtxHeader mtx_header(FILE* f) {
    MtxHeader h;
    std::string line;
    if (!read_line(f, line)) fail(GA_ERR_INVALID_ARG, "mtx: empty file");
    char w[5][64] = {};
    if (sscanf(line.c_str(), "%63s %63s %63s %63s %63s", w[0], w[1], w[2], w[3], w[4]) != 5)
        fail(GA_ERR_INVALID_ARG, "mtx: malformed banner");
    if (std::string(w[0]) != "%%MatrixMarket" || lower(w[1]) != "matrix")
        fail(GA_ERR_INVALID_ARG, "mtx: not a Matrix Market file");
    const std::string fmt = lower(w[2]), field = lower(w[3]), sym = lower(w[4]);
    if (fmt == "coordinate") h.code[1] = 'C';
    else if (fmt == "array") h.code[1] = 'A';
    else fail(GA_ERR_INVALID_ARG, "mtx: unknown storage format");
    if (field == "real") h.code[2] = 'R';
    else if (field == "integer") h.code[2] = 'I';
    else if (field == "pattern") h.code[2] = 'P';
    else if (field == "complex") h.code[2] = 'C';
    else fail(GA_ERR_INVALID_ARG, "mtx: unknown value field");
    if (sym == "general") h.code[3] = 'G';
    else if (sym == "symmetric") h.code[3] = 'S';
    else if (sym == "skew-symmetric") h.code[3] = 'K';
    else if (sym == "hermitian") h.code[3] = 'H';
    else fail(GA_ERR_INVALID_ARG, "mtx: unknown symmetry");
    if (h.code[1] != 'C' || h.code[2] == 'C') fail(GA_ERR_UNSUPPORTED, "mtx: complex and array files are not read");
    for (;;) {
        if (!read_line(f, line)) fail(GA_ERR_INVALID_ARG, "mtx: no size line");
        if (line.empty() || line[0] == '%') continue;
        long long m, n, nz;
        if (sscanf(line.c_str(), "%lld %lld %lld", &m, &n, &nz) != 3) {
            bool blank = true;
            for (char c : line) blank &= (c == ' ' || (c >= 9 && c <= 13));
            if (blank) continue;
            fail(GA_ERR_INVALID_ARG, "mtx: malformed size line");
        }
        if (m < 0 || n < 0 || nz < 0 || m >= INT32_MAX || n >= INT32_MAX || nz >= INT32_MAX)
            fail(GA_ERR_INVALID_ARG, "mtx: sizes beyond the int32 index range");
        h.m = m;
        h.n = n;
        h.nz = nz;
        break;
    }
    if (h.m != h.n) fail(GA_ERR_SHAPE, "mtx: the matrix is not square");
    h.body = ftell(f);
    return h;
}

// Host conversion of the value tokens the device parser leaves: strtod
// in the "C" locale over the whole token.
static void mtx_slow_values(ga_ctx ctx, FILE* f, const MtxHeader& h, const int64_t* tokpos, int per, int64_t count,
                            const int64_t* slow, double* dval) {
    DBuf<int64_t> dpos(ctx, (size_t)count);
    k_gather_slow_pos<<<grid_for(count, 256, ctx->num_sms * 4), 256, 0, ctx->stream>>>(slow, count, tokpos, per,
                                                                                       dpos.p);
    post_launch("mtx_slow_pos");
    std::vector<int64_t> pos((size_t)count), idx((size_t)count);
    GA_CUDA(cudaMemcpyAsync(pos.data(), dpos.p, sizeof(int64_t) * count, cudaMemcpyDeviceToHost, ctx->stream));
    GA_CUDA(cudaStreamSynchronize(ctx->stream));
    locale_t cl = newlocale(LC_ALL_MASK, "C", (locale_t)0);
    if (!cl) fail(GA_ERR_INVALID_ARG, "mtx: no C locale");
    std::vector<double> v((size_t)count);
    char buf[512];
    bool ok = true;
    for (int64_t t = 0; t < count && ok; ++t) {
        ok = fseek(f, h.body + (long)pos[(size_t)t], SEEK_SET) == 0;
        const size_t len = ok ? fread(buf, 1, sizeof buf - 1, f) : 0;
        size_t e = 0;
        while (e < len && !(buf[e] == ' ' || (buf[e] >= 9 && buf[e] <= 13))) ++e;
        buf[e] = 0;
        char* end = nullptr;
        v[(size_t)t] = strtod_l(buf, &end, cl);
        ok = ok && e > 0 && e < sizeof buf - 1 && end == buf + e;
    }
    freelocale(cl);
    if (!ok) fail(GA_ERR_INVALID_ARG, "mtx: malformed real value");
    DBuf<double> dv(ctx, (size_t)count);
    GA_CUDA(cudaMemcpyAsync(dv.p, v.data(), sizeof(double) * count, cudaMemcpyHostToDevice, ctx->stream));
    k_scatter_f64<<<grid_for(count, 256, ctx->num_sms * 4), 256, 0, ctx->stream>>>(slow, dv.p, count, dval);
    post_launch("mtx_slow_scatter");
    GA_CUDA(cudaStreamSynchronize(ctx->stream));
}

static ga_csr read_mtx(ga_ctx ctx, const char* path, int flags, char* matcode) {
    GA_REQUIRE((flags & ~(GA_EDGES_LOWER_SYMM | GA_EDGES_UNIT)) == 0, GA_ERR_INVALID_ARG,
               "mtx: only GA_EDGES_LOWER_SYMM and GA_EDGES_UNIT apply");
    File file(path, "rb");
    if (!file.f) fail(GA_ERR_INVALID_ARG, std::string("mtx: cannot open ") + path);
    const MtxHeader h = mtx_header(file.f);
    if (matcode) memcpy(matcode, h.code, 4);
    GA_REQUIRE(fseek(file.f, 0, SEEK_END) == 0, GA_ERR_INVALID_ARG, "mtx: cannot seek");
    const int64_t body = (int64_t)ftell(file.f) - h.body;
    GA_REQUIRE(fseek(file.f, h.body, SEEK_SET) == 0, GA_ERR_INVALID_ARG, "mtx: cannot seek");
    const int per = h.code[2] == 'P' ? 2 : 3;
    const int64_t need = per * h.nz;
    // text padded with spaces to whole tokenizer blocks, at least one byte of
    // padding, so every token is followed by a space
    const int64_t nblk = body / kTokBlockBytes + 1;
    DBuf<unsigned char> text(ctx, (size_t)(nblk * kTokBlockBytes));
    GA_CUDA(cudaMemsetAsync(text.p + body, ' ', (size_t)(nblk * kTokBlockBytes - body), ctx->stream));
    file_to_device(ctx, file.f, text.p, body, "mtx");
    DBuf<int64_t> bcount(ctx, (size_t)nblk + 1);
    int prof = prof_begin(ctx, "mtx_tokenize");
    k_tok_count<<<(unsigned)nblk, kTokThreads, 0, ctx->stream>>>(text.p, bcount.p);
    post_launch("mtx_tok_count");
    scan_exclusive_i64(ctx, bcount.p, bcount.p, nblk);
    const int64_t ntok = read_i64(ctx, bcount.p + nblk);
    GA_REQUIRE(ntok >= need, GA_ERR_INVALID_ARG, "mtx: fewer entries than the size line states");
    DBuf<int64_t> tokpos(ctx, (size_t)need + 1);
    k_tok_emit<<<(unsigned)nblk, kTokThreads, 0, ctx->stream>>>(text.p, bcount.p, need, tokpos.p);
    post_launch("mtx_tok_emit");
    prof_end(ctx, prof);

    const bool want_vals = per == 3 && !(flags & GA_EDGES_UNIT);
    const int value_kind = want_vals ? (h.code[2] == 'R' ? 2 : 1) : 0;
    const ga_dtype dt = value_kind == 2 ? GA_FP64 : GA_INT32;
    DBuf<int32_t> src(ctx, (size_t)h.nz + 1), dst(ctx, (size_t)h.nz + 1);
    DBuf<unsigned char> val(ctx, value_kind ? (size_t)h.nz * dtype_size(dt) + 8 : 8);
    DBuf<int64_t> slow(ctx, value_kind == 2 ? (size_t)h.nz + 1 : 1), nslow(ctx, 1);
    DBuf<int> err(ctx, 1);
    GA_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), ctx->stream));
    GA_CUDA(cudaMemsetAsync(nslow.p, 0, sizeof(int64_t), ctx->stream));
    prof = prof_begin(ctx, "mtx_parse");
    if (h.nz) {
        k_mtx_entries<<<grid_for(h.nz, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(
            text.p, tokpos.p, h.nz, per, value_kind, h.m, h.n, src.p, dst.p, val.p, err.p, slow.p, nslow.p);
        post_launch("mtx_entries");
    }
    prof_end(ctx, prof);
    const int e = read_i32(ctx, err.p);
    if (e & kBadIndex) fail(GA_ERR_INVALID_ARG, "mtx: a row or column index is not an integer");
    if (e & kIndexRange) fail(GA_ERR_INVALID_ARG, "mtx: an entry lies outside the matrix");
    if (e & kBadValue) fail(GA_ERR_INVALID_ARG, "mtx: an integer value is malformed or beyond int32");
    const int64_t ns = read_i64(ctx, nslow.p);
    if (ns) mtx_slow_values(ctx, file.f, h, tokpos.p, per, ns, slow.p, reinterpret_cast<double*>(val.p));
    text = DBuf<unsigned char>();
    tokpos = DBuf<int64_t>();
    int eflags = flags | GA_EDGES_DROP_LOOPS | (h.code[3] == 'S' ? GA_EDGES_MIRROR : 0);
    if (!value_kind) eflags |= GA_EDGES_UNIT;
    return edges_to_csr(ctx, h.m, h.n, h.nz, src.p, dst.p, value_kind ? val.p : nullptr, dt, eflags);
}

// ============================================================ binary CSR
// Row of every entry (the last i with rst[i] <= q); rst is checked monotone.
__global__ void k_rows_of_entries(const int32_t* __restrict__ rst, int64_t m, int64_t nnz,
                                  int32_t* __restrict__ row) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x) {
        int64_t lo = 0, hi = m;
        while (hi - lo > 1) {
            const int64_t mid = (lo + hi) >> 1;
            if (rst[mid] <= q) lo = mid;
            else hi = mid;
        }
        row[q] = (int32_t)lo;
    }
}

static ga_csr read_bin(ga_ctx ctx, const char* path, int flags, char* matcode) {
    GA_REQUIRE((flags & ~(GA_EDGES_LOWER_SYMM | GA_EDGES_UNIT)) == 0, GA_ERR_INVALID_ARG,
               "bin: only GA_EDGES_LOWER_SYMM and GA_EDGES_UNIT apply");
    File file(path, "rb");
    if (!file.f) fail(GA_ERR_INVALID_ARG, std::string("bin: cannot open ") + path);
    char code[4];
    uint64_t m = 0, n = 0, nz = 0;
    if (fread(code, 1, 4, file.f) != 4 || fread(&m, 8, 1, file.f) != 1 || fread(&n, 8, 1, file.f) != 1 ||
        fread(&nz, 8, 1, file.f) != 1)
        fail(GA_ERR_INVALID_ARG, "bin: truncated header");
    if (matcode) memcpy(matcode, code, 4);
    if (m >= (uint64_t)INT32_MAX || n >= (uint64_t)INT32_MAX || nz >= (uint64_t)INT32_MAX)
        fail(GA_ERR_INVALID_ARG, "bin: sizes beyond the int32 index range");
    // the value type the reference CLI reads for a binary file (src/main.cpp:279-292)
    if (!(code[2] == 'R' || code[2] == 'I' || code[2] == 'P')) fail(GA_ERR_DTYPE, "bin: unknown value type");
    const ga_dtype dt = code[2] == 'R' ? GA_FP64 : GA_INT32;
    const int64_t es = (int64_t)dtype_size(dt);
    GA_REQUIRE(fseek(file.f, 0, SEEK_END) == 0, GA_ERR_INVALID_ARG, "bin: cannot seek");
    const int64_t size = (int64_t)ftell(file.f);
    GA_REQUIRE(size >= 28 + 4 * (int64_t)(m + 1) + (4 + es) * (int64_t)nz, GA_ERR_INVALID_ARG,
               "bin: truncated file");
    GA_REQUIRE(fseek(file.f, 28, SEEK_SET) == 0, GA_ERR_INVALID_ARG, "bin: cannot seek");
    ga_csr A = csr_alloc(ctx, (int64_t)m, (int64_t)n, (int64_t)nz, dt);
    try {
        file_to_device(ctx, file.f, A->rst, 4 * (int64_t)(m + 1), "bin");
        file_to_device(ctx, file.f, A->col, 4 * (int64_t)nz, "bin");
        file_to_device(ctx, file.f, A->val, es * (int64_t)nz, "bin");
        const int bits = csr_check_bits(ctx, A->rst, A->col, (int64_t)m, (int64_t)n, (int64_t)nz);
        if (bits & 1) fail(GA_ERR_INVALID_CSR, "bin: row starts are not a monotone 0..nz sequence");
        if (bits & 2) fail(GA_ERR_INVALID_CSR, "bin: column index out of range");
        if (bits == 0 && flags == 0) return A;  // rows already sorted and duplicate-free
        DBuf<int32_t> row(ctx, (size_t)nz + 1);
        if (nz) {
            k_rows_of_entries<<<grid_for((int64_t)nz, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(
                A->rst, (int64_t)m, (int64_t)nz, row.p);
            post_launch("bin_rows");
        }
        ga_csr B = edges_to_csr(ctx, (int64_t)m, (int64_t)n, (int64_t)nz, row.p, A->col, A->val, dt, flags);
        csr_destroy(ctx, A);
        return B;
    } catch (...) {
        csr_destroy(ctx, A);
        throw;
    }
}

static void write_bin(ga_ctx ctx, ga_csr A, const char* matcode, const char* path) {
    GA_REQUIRE(A->dtype == GA_INT32 || A->dtype == GA_FP64, GA_ERR_DTYPE,
               "bin: the layout holds int32 or double values");
    std::vector<int32_t> rst((size_t)A->m + 1), col((size_t)A->nnz + 1);
    std::vector<unsigned char> val((size_t)A->nnz * dtype_size(A->dtype) + 8);
    GA_CUDA(cudaMemcpyAsync(rst.data(), A->rst, sizeof(int32_t) * (A->m + 1), cudaMemcpyDeviceToHost, ctx->stream));
    if (A->nnz) {
        GA_CUDA(cudaMemcpyAsync(col.data(), A->col, sizeof(int32_t) * A->nnz, cudaMemcpyDeviceToHost, ctx->stream));
        GA_CUDA(cudaMemcpyAsync(val.data(), A->val, dtype_size(A->dtype) * A->nnz, cudaMemcpyDeviceToHost,
                                ctx->stream));
    }
    GA_CUDA(cudaStreamSynchronize(ctx->stream));
    char code[4] = {'M', 'C', A->dtype == GA_FP64 ? 'R' : 'I', 'G'};
    if (matcode) memcpy(code, matcode, 4);
    File file(path, "wb");
    if (!file.f) fail(GA_ERR_INVALID_ARG, std::string("bin: cannot create ") + path);
    const uint64_t m = (uint64_t)A->m, n = (uint64_t)A->n, nz = (uint64_t)A->nnz;
    const bool ok = fwrite(code, 1, 4, file.f) == 4 && fwrite(&m, 8, 1, file.f) == 1 &&
                    fwrite(&n, 8, 1, file.f) == 1 && fwrite(&nz, 8, 1, file.f) == 1 &&
                    fwrite(rst.data(), 4, m + 1, file.f) == m + 1 &&
                    (nz == 0 || fwrite(col.data(), 4, nz, file.f) == nz) &&
                    (nz == 0 || fwrite(val.data(), dtype_size(A->dtype), nz, file.f) == nz);
    if (!ok || fflush(file.f) != 0) fail(GA_ERR_INVALID_ARG, std::string("bin: write failed: ") + path);
}

}  // namespace ga

using namespace ga;

extern "C" {

int ga_csr_from_edges(ga_ctx ctx, int64_t m, int64_t n, int64_t ne, const int32_t* src, const int32_t* dst,
                      const void* val, ga_dtype dtype, int flags, ga_csr* out) {
    if (!ctx || !out || m < 0 || n < 0 || ne < 0 || (ne > 0 && (!src || !dst)) || !dtype_valid(dtype))
        return GA_ERR_INVALID_ARG;
    *out = nullptr;
    GA_API_BODY(ctx, {
        GA_REQUIRE(ne < INT32_MAX, GA_ERR_INVALID_ARG, "edges: beyond the int32 index range");
        const size_t es = dtype_size(dtype);
        DBuf<int32_t> ds(ctx, (size_t)ne + 1), dd(ctx, (size_t)ne + 1);
        DBuf<unsigned char> dv(ctx, val ? es * (size_t)ne + 8 : 8);
        if (ne) {
            GA_CUDA(cudaMemcpyAsync(ds.p, src, sizeof(int32_t) * ne, cudaMemcpyHostToDevice, ctx->stream));
            GA_CUDA(cudaMemcpyAsync(dd.p, dst, sizeof(int32_t) * ne, cudaMemcpyHostToDevice, ctx->stream));
            if (val) GA_CUDA(cudaMemcpyAsync(dv.p, val, es * ne, cudaMemcpyHostToDevice, ctx->stream));
        }
        *out = edges_to_csr(ctx, m, n, ne, ds.p, dd.p, val ? dv.p : nullptr, dtype, flags);
    });
}

int ga_csr_from_device_edges(ga_ctx ctx, int64_t m, int64_t n, int64_t ne, const int32_t* src, const int32_t* dst,
                             const void* val, ga_dtype dtype, int flags, ga_csr* out) {
    if (!ctx || !out || m < 0 || n < 0 || ne < 0 || (ne > 0 && (!src || !dst)) || !dtype_valid(dtype))
        return GA_ERR_INVALID_ARG;
    *out = nullptr;
    GA_API_BODY(ctx, *out = edges_to_csr(ctx, m, n, ne, src, dst, val, dtype, flags));
}

int ga_gen_rmat_device(ga_ctx ctx, int scale, int edge_factor, double a, double b, double c, uint64_t seed,
                       ga_csr* out) {
    if (!ctx || !out) return GA_ERR_INVALID_ARG;
    *out = nullptr;
    GA_API_BODY(ctx, {
        *out = gen_rmat_device(ctx, scale, edge_factor, a, b, c, seed);
        (*out)->sym = 1;
    });
}

int ga_read_mtx(ga_ctx ctx, const char* path, int flags, char* matcode, ga_csr* out) {
    if (!ctx || !path || !out) return GA_ERR_INVALID_ARG;
    *out = nullptr;
    GA_API_BODY(ctx, *out = read_mtx(ctx, path, flags, matcode));
}

int ga_read_bin(ga_ctx ctx, const char* path, int flags, char* matcode, ga_csr* out) {
    if (!ctx || !path || !out) return GA_ERR_INVALID_ARG;
    *out = nullptr;
    GA_API_BODY(ctx, *out = read_bin(ctx, path, flags, matcode));
}

int ga_write_bin(ga_ctx ctx, ga_csr A, const char* matcode, const char* path) {
    if (!ctx || !A || !path) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, write_bin(ctx, A, matcode, path));
}

}  // extern "C"
