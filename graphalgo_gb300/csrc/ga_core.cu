// Context, memory, handles, validation, profiling and timing.
#include "ga_internal.cuh"

#include <atomic>
#include <cstdio>
#include <cstring>
#include <cstdlib>

namespace ga {

void fail(int code, const std::string& msg) { throw Error{code, msg}; }

void check_cuda(cudaError_t e, const char* what, const char* file, int line) {
    if (e == cudaSuccess) return;
    char buf[512];
    const char* base = strrchr(file, '/');
    snprintf(buf, sizeof(buf), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), base ? base + 1 : file,
             line);
    int code = (e == cudaErrorMemoryAllocation) ? GA_ERR_OOM
               : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ||
                  e == cudaErrorNoKernelImageForDevice || e == cudaErrorInvalidDevice)
                   ? GA_ERR_NO_DEVICE
                   : GA_ERR_CUDA;
    fail(code, buf);
}

static std::atomic<int64_t> g_launches{0};

void post_launch(const char* name) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        char buf[256];
        snprintf(buf, sizeof(buf), "kernel %s launch failed: %s", name, cudaGetErrorString(e));
        fail(e == cudaErrorNoKernelImageForDevice ? GA_ERR_NO_DEVICE : GA_ERR_CUDA, buf);
    }
}

size_t dtype_size(ga_dtype t) {
    switch (t) {
    case GA_INT32: return 4;
    case GA_INT64: return 8;
    case GA_FP32: return 4;
    case GA_FP64: return 8;
    case GA_UINT8: return 1;
    }
    return 0;
}

bool dtype_valid(int t) { return t >= GA_INT32 && t <= GA_UINT8; }

void* dalloc(ga_ctx ctx, size_t bytes) {
    if (ctx->fail_alloc_after >= 0) {
        if (ctx->fail_alloc_after == 0) {
            ctx->fail_alloc_after = -1;
            fail(GA_ERR_OOM, "device allocation failed (injected)");
        }
        --ctx->fail_alloc_after;
    }
    void* p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMallocFromPoolAsync(&p, bytes, ctx->pool, ctx->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        char buf[128];
        snprintf(buf, sizeof(buf), "device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        fail(e == cudaErrorMemoryAllocation ? GA_ERR_OOM : GA_ERR_CUDA, buf);
    }
    ctx->live[p] = bytes;
    ctx->bytes_in_use += (int64_t)bytes;
    if (ctx->bytes_in_use > ctx->bytes_peak) ctx->bytes_peak = ctx->bytes_in_use;
    return p;
}

void dfree(ga_ctx ctx, void* p) {
    if (!p) return;
    auto it = ctx->live.find(p);
    if (it != ctx->live.end()) {  // memory of another context is freed without accounting
        ctx->bytes_in_use -= (int64_t)it->second;
        ctx->live.erase(it);
    }
    cudaFreeAsync(p, ctx->stream);
}

ga_csr csr_alloc(ga_ctx ctx, int64_t m, int64_t n, int64_t nnz, ga_dtype dt) {
    GA_REQUIRE(m >= 0 && n >= 0 && nnz >= 0, GA_ERR_INVALID_ARG, "negative CSR dimension");
    GA_REQUIRE(m < INT32_MAX && n <= INT32_MAX && nnz <= INT32_MAX, GA_ERR_INVALID_ARG,
               "CSR dimensions exceed the int32 index range of spMtx");
    ga_csr A = new ga_csr_s;
    A->m = m; A->n = n; A->nnz = nnz; A->dtype = dt; A->cap = (size_t)nnz;
    try {
        A->rst = dalloc_t<int32_t>(ctx, (size_t)m + 1);
        A->col = dalloc_t<int32_t>(ctx, nnz ? (size_t)nnz : 1);
        A->val = dalloc(ctx, (nnz ? (size_t)nnz : 1) * dtype_size(dt));
    } catch (...) {
        csr_destroy(ctx, A);
        throw;
    }
    return A;
}

void csr_destroy(ga_ctx ctx, ga_csr A) {
    if (!A) return;
    if (A->copied) cudaEventDestroy(A->copied);
    dfree(ctx, A->rst);
    dfree(ctx, A->col);
    dfree(ctx, A->val);
    delete A;
}

// ---------------------------------------------------------------- profiling
int prof_begin(ga_ctx ctx, const char* name) {
    if (!ctx->profile || ctx->capturing) return -1;
    cudaEvent_t a, b;
    if (ctx->event_pool.size() >= 2) {
        a = ctx->event_pool.back(); ctx->event_pool.pop_back();
        b = ctx->event_pool.back(); ctx->event_pool.pop_back();
    } else {
        GA_CUDA(cudaEventCreate(&a));
        GA_CUDA(cudaEventCreate(&b));
    }
    GA_CUDA(cudaEventRecord(a, ctx->stream));
    ctx->pending.push_back(PendingTiming{name, a, b});
    return (int)ctx->pending.size() - 1;
}

void prof_end(ga_ctx ctx, int token) {
    if (token < 0 || token >= (int)ctx->pending.size()) return;
    cudaEventRecord(ctx->pending[token].stop, ctx->stream);
}

static void prof_collect(ga_ctx ctx) {
    if (ctx->pending.empty()) return;
    GA_CUDA(cudaStreamSynchronize(ctx->stream));
    for (auto& p : ctx->pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.start, p.stop) == cudaSuccess) {
            KStat& s = ctx->kstats[p.name];
            s.launches += 1;
            s.total_ms += ms;
        } else {
            cudaGetLastError();
        }
        ctx->event_pool.push_back(p.start);
        ctx->event_pool.push_back(p.stop);
    }
    ctx->pending.clear();
}

int64_t read_i64(ga_ctx ctx, const int64_t* d) {
    GA_CUDA(cudaMemcpyAsync(ctx->h_pinned, d, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    GA_CUDA(cudaStreamSynchronize(ctx->stream));
    return *ctx->h_pinned;
}

int32_t read_i32(ga_ctx ctx, const int32_t* d) {
    int32_t* h = reinterpret_cast<int32_t*>(ctx->h_pinned);
    GA_CUDA(cudaMemcpyAsync(h, d, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    GA_CUDA(cudaStreamSynchronize(ctx->stream));
    return *h;
}

int grid_for(int64_t work, int block, int max_blocks) {
    int64_t g = (work + block - 1) / block;
    if (g < 1) g = 1;
    if (g > max_blocks) g = max_blocks;
    return (int)g;
}

// ---------------------------------------------------------------- validation
// One warp per row: row starts monotone, columns in [0, n) and strictly
// ascending. Bit 0: bad row starts, bit 1: column out of range, bit 2:
// unsorted or duplicate columns.
__global__ void k_validate_csr(const int32_t* __restrict__ rst, const int32_t* __restrict__ col, int64_t m,
                               int64_t n, int64_t nnz, int* __restrict__ err) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w == 0 && lane == 0) {
        if (rst[0] != 0 || (int64_t)rst[m] != nnz) atomicOr(err, 1);
    }
    for (int64_t i = w; i < m; i += warps) {
        int32_t b = rst[i], e = rst[i + 1];
        if (e < b || b < 0 || (int64_t)e > nnz) {
            if (lane == 0) atomicOr(err, 1);
            continue;
        }
        int bad = 0;
        for (int32_t q = b + lane; q < e; q += 32) {
            int32_t c = col[q];
            if (c < 0 || (int64_t)c >= n) bad |= 2;
            if (q + 1 < e && col[q + 1] <= c) bad |= 4;
        }
        bad = __reduce_or_sync(0xffffffffu, bad);
        if (bad && lane == 0) atomicOr(err, bad);
    }
}

int csr_check_bits(ga_ctx ctx, const int32_t* rst, const int32_t* col, int64_t m, int64_t n, int64_t nnz) {
    DBuf<int> err(ctx, 1);
    GA_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), ctx->stream));
    int block = 256;
    int grid = grid_for(m * 32, block, ctx->num_sms * 16);
    k_validate_csr<<<grid, block, 0, ctx->stream>>>(rst, col, m, n, nnz, err.p);
    post_launch("validate_csr");
    return read_i32(ctx, err.p);
}

void validate_csr(ga_ctx ctx, const int32_t* rst, const int32_t* col, int64_t m, int64_t n, int64_t nnz) {
    const int e = csr_check_bits(ctx, rst, col, m, n, nnz);
    if (e & 1) fail(GA_ERR_INVALID_CSR, "invalid CSR: row starts are not a monotone 0..nnz sequence");
    if (e & 2) fail(GA_ERR_INVALID_CSR, "invalid CSR: column index out of range");
    if (e & 4) fail(GA_ERR_INVALID_CSR, "invalid CSR: columns not strictly ascending within a row");
}

}  // namespace ga

using namespace ga;

// ====================================================================== ABI
extern "C" {

const char* ga_status_string(int s) {
    switch (s) {
    case GA_OK: return "ok";
    case GA_ERR_INVALID_ARG: return "invalid argument";
    case GA_ERR_INVALID_CSR: return "invalid CSR";
    case GA_ERR_SHAPE: return "shape mismatch";
    case GA_ERR_DTYPE: return "dtype mismatch";
    case GA_ERR_CUDA: return "CUDA error";
    case GA_ERR_OOM: return "out of device memory";
    case GA_ERR_NO_DEVICE: return "no usable CUDA device";
    case GA_ERR_TIMEOUT: return "device wait timed out";
    case GA_ERR_UNSUPPORTED: return "unsupported";
    case GA_ERR_ADMISSION: return "admission refused";
    case GA_ERR_CANCELLED: return "cancelled";
    }
    return "unknown status";
}

int ga_version(int* major, int* minor) {
    if (major) *major = 1;
    if (minor) *minor = 0;
    return GA_OK;
}

int ga_device_count(int* count) {
    int c = 0;
    cudaError_t e = cudaGetDeviceCount(&c);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (count) *count = 0;
        return GA_ERR_NO_DEVICE;
    }
    if (count) *count = c;
    return GA_OK;
}

int ga_ctx_create(int device, void* stream, ga_ctx* out) {
    if (!out) return GA_ERR_INVALID_ARG;
    *out = nullptr;
    ga_ctx ctx = new ga_ctx_s;
    try {
        int count = 0;
        cudaError_t e = cudaGetDeviceCount(&count);
        if (e != cudaSuccess || count == 0) {
            cudaGetLastError();
            fail(GA_ERR_NO_DEVICE, "no CUDA device available");
        }
        GA_REQUIRE(device >= 0 && device < count, GA_ERR_INVALID_ARG, "device index out of range");
        ctx->device = device;
        GA_CUDA(cudaSetDevice(device));
        cudaDeviceProp prop;
        GA_CUDA(cudaGetDeviceProperties(&prop, device));
        ctx->num_sms = prop.multiProcessorCount;
        ctx->cc_major = prop.major;
        ctx->cc_minor = prop.minor;
        ctx->smem_optin = prop.sharedMemPerBlockOptin;
        if (stream) {
            ctx->stream = (cudaStream_t)stream;
        } else {
            GA_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
            ctx->own_stream = true;
        }
        GA_CUDA(cudaDeviceGetDefaultMemPool(&ctx->pool, device));
        uint64_t threshold = UINT64_MAX;  // keep freed blocks cached in the pool
        GA_CUDA(cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &threshold));
        GA_CUDA(cudaMallocHost((void**)&ctx->h_pinned, 64));
        GA_CUDA(cudaMalloc((void**)&ctx->d_counters, sizeof(unsigned long long) * GA_CTR_COUNT));
        GA_CUDA(cudaMemsetAsync(ctx->d_counters, 0, sizeof(unsigned long long) * GA_CTR_COUNT, ctx->stream));
        GA_CUDA(cudaEventCreate(&ctx->timer_start));
        GA_CUDA(cudaEventCreate(&ctx->timer_stop));
        *out = ctx;
        return GA_OK;
    } catch (const Error& e) {
        int code = e.code;
        // the caller has no context to query; keep the message on stderr
        fprintf(stderr, "graphalgo_gb300: ga_ctx_create: %s\n", e.msg.c_str());
        if (ctx->d_counters) cudaFree(ctx->d_counters);
        if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
        if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
        delete ctx;
        return code;
    }
}

int ga_ctx_destroy(ga_ctx ctx) {
    if (!ctx) return GA_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto& p : ctx->pending) {
        cudaEventDestroy(p.start);
        cudaEventDestroy(p.stop);
    }
    for (auto ev : ctx->event_pool) cudaEventDestroy(ev);
    ga::destroy_loop_caches(ctx);
    if (ctx->timer_start) cudaEventDestroy(ctx->timer_start);
    if (ctx->timer_stop) cudaEventDestroy(ctx->timer_stop);
    if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
    if (ctx->d_counters) cudaFree(ctx->d_counters);
    if (ctx->l2_flush) cudaFree(ctx->l2_flush);
    if (ctx->copy_stream) {
        cudaStreamSynchronize(ctx->copy_stream);
        cudaStreamDestroy(ctx->copy_stream);
        cudaEventDestroy(ctx->copy_ready);
        cudaEventDestroy(ctx->copy_done);
    }
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GA_OK;
}

int64_t ga_kernel_launches(void) { return ga::g_launches.load(std::memory_order_relaxed); }

int ga_ctx_work_counters(ga_ctx ctx, int64_t* out, int reset) {
    if (!ctx || !out) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        unsigned long long h[GA_CTR_COUNT];
        GA_CUDA(cudaMemcpyAsync(h, ctx->d_counters, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
        for (int i = 0; i < GA_CTR_COUNT; ++i) out[i] = (int64_t)h[i];
        if (reset) GA_CUDA(cudaMemsetAsync(ctx->d_counters, 0, sizeof(h), ctx->stream));
    });
}

int ga_ctx_flush_l2(ga_ctx ctx) {
    if (!ctx) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        if (!ctx->l2_flush) {
            ctx->l2_flush_bytes = (size_t)256 << 20;
            GA_CUDA(cudaMalloc(&ctx->l2_flush, ctx->l2_flush_bytes));
        }
        GA_CUDA(cudaMemsetAsync(ctx->l2_flush, ctx->l2_flush_bytes & 0xff, ctx->l2_flush_bytes, ctx->stream));
    });
}

int ga_host_register(void* ptr, size_t bytes) {
    if (!ptr || !bytes) return GA_ERR_INVALID_ARG;
    cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return GA_ERR_CUDA;
    }
    return GA_OK;
}

int ga_host_unregister(void* ptr) {
    if (!ptr) return GA_ERR_INVALID_ARG;
    cudaError_t e = cudaHostUnregister(ptr);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return GA_ERR_CUDA;
    }
    return GA_OK;
}

const char* ga_last_error(ga_ctx ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

int ga_ctx_sync(ga_ctx ctx) {
    if (!ctx) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, GA_CUDA(cudaStreamSynchronize(ctx->stream)));
}

int ga_ctx_stream(ga_ctx ctx, void** stream) {
    if (!ctx || !stream) return GA_ERR_INVALID_ARG;
    *stream = (void*)ctx->stream;
    return GA_OK;
}

int ga_ctx_set_option(ga_ctx ctx, int option, int64_t value) {
    if (!ctx) return GA_ERR_INVALID_ARG;
    switch (option) {
    case GA_OPT_DEVICE_LOOPS: ctx->device_loops = value != 0; return GA_OK;
    case GA_OPT_PROFILE: ctx->profile = value != 0; return GA_OK;
    case GA_OPT_FAIL_ALLOC_AFTER: ctx->fail_alloc_after = value; return GA_OK;
    case GA_OPT_KNN_TILED: ctx->knn_tiled = value != 0; return GA_OK;
    case GA_OPT_MXM_WARP_FLOPS: ctx->tune.warp_max_flops = value; return GA_OK;
    case GA_OPT_MXM_HEAVY_FLOPS: ctx->tune.heavy_flops = value; return GA_OK;
    case GA_OPT_MXM_CTAS_PER_SM:
        if (value < 0) break;
        ctx->tune.ctas_per_sm = (int)value;
        return GA_OK;
    case GA_OPT_DOT_CHUNK:
        if (value < 1 || value > 4096) break;
        ctx->tune.dot_chunk = (int)value;
        return GA_OK;
    case GA_OPT_HYBRID_RATIO:
        if (value < 0 || value > (1 << 20)) break;
        ctx->tune.hybrid_ratio = value;
        return GA_OK;
    case GA_OPT_TRI_ORDER:
        if (value != 0 && value != 1) break;
        ctx->tune.tri_order = (int)value;
        return GA_OK;
    case GA_OPT_KT_FRONTIER: ctx->kt_frontier = value != 0; return GA_OK;
    case GA_OPT_BC_BACKWARD:
        if (value < 0 || value > 2) break;
        ctx->bc_backward = (int)value;
        return GA_OK;
    }
    ctx->last_error = "unknown option";
    return GA_ERR_INVALID_ARG;
}

int ga_ctx_kernel_stats(ga_ctx ctx, ga_kernel_stat* out, int cap, int* count) {
    if (!ctx) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        prof_collect(ctx);
        int i = 0;
        for (auto& kv : ctx->kstats) {
            if (out && i < cap) {
                memset(out[i].name, 0, sizeof(out[i].name));
                strncpy(out[i].name, kv.first.c_str(), sizeof(out[i].name) - 1);
                out[i].launches = kv.second.launches;
                out[i].total_ms = kv.second.total_ms;
            }
            ++i;
        }
        if (count) *count = i;
    });
}

int ga_ctx_reset_kernel_stats(ga_ctx ctx) {
    if (!ctx) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        prof_collect(ctx);
        ctx->kstats.clear();
    });
}

int ga_timer_start(ga_ctx ctx) {
    if (!ctx) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, GA_CUDA(cudaEventRecord(ctx->timer_start, ctx->stream)));
}

int ga_timer_stop(ga_ctx ctx, double* ms) {
    if (!ctx) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        GA_CUDA(cudaEventRecord(ctx->timer_stop, ctx->stream));
        GA_CUDA(cudaEventSynchronize(ctx->timer_stop));
        float f = 0.f;
        GA_CUDA(cudaEventElapsedTime(&f, ctx->timer_start, ctx->timer_stop));
        if (ms) *ms = (double)f;
    });
}

int ga_mem_info(ga_ctx ctx, int64_t* free_bytes, int64_t* total_bytes) {
    if (!ctx) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        size_t f = 0, t = 0;
        GA_CUDA(cudaMemGetInfo(&f, &t));
        if (free_bytes) *free_bytes = (int64_t)f;
        if (total_bytes) *total_bytes = (int64_t)t;
    });
}

int ga_ctx_mem_stats(ga_ctx ctx, int64_t* in_use, int64_t* peak, int reset_peak) {
    if (!ctx) return GA_ERR_INVALID_ARG;
    if (in_use) *in_use = ctx->bytes_in_use;
    if (peak) *peak = ctx->bytes_peak;
    if (reset_peak) ctx->bytes_peak = ctx->bytes_in_use;
    return GA_OK;
}

// ---------------------------------------------------------------- CSR handle
static int upload_impl(ga_ctx ctx, int64_t m, int64_t n, int64_t nnz, const int32_t* rst, const int32_t* col,
                       const void* val, ga_dtype dtype, ga_csr* out, cudaMemcpyKind kind) {
    if (!ctx || !out) return GA_ERR_INVALID_ARG;
    *out = nullptr;
    GA_API_BODY(ctx, {
        GA_REQUIRE(dtype_valid(dtype), GA_ERR_DTYPE, "unknown dtype");
        GA_REQUIRE(rst != nullptr, GA_ERR_INVALID_ARG, "rst is NULL");
        GA_REQUIRE(nnz == 0 || col != nullptr, GA_ERR_INVALID_ARG, "col is NULL");
        ga_csr A = csr_alloc(ctx, m, n, nnz, dtype);
        try {
            size_t es = dtype_size(dtype);
            GA_CUDA(cudaMemcpyAsync(A->rst, rst, sizeof(int32_t) * (m + 1), kind, ctx->stream));
            if (nnz) {
                GA_CUDA(cudaMemcpyAsync(A->col, col, sizeof(int32_t) * nnz, kind, ctx->stream));
                if (val) {
                    GA_CUDA(cudaMemcpyAsync(A->val, val, es * nnz, kind, ctx->stream));
                } else {
                    fill_ones(ctx, A->val, nnz, dtype);
                    A->unit = 1;
                }
            }
            validate_csr(ctx, A->rst, A->col, m, n, nnz);
        } catch (...) {
            csr_destroy(ctx, A);
            throw;
        }
        *out = A;
    });
}

int ga_csr_upload(ga_ctx ctx, int64_t m, int64_t n, int64_t nnz, const int32_t* rst, const int32_t* col,
                  const void* val, ga_dtype dtype, ga_csr* out) {
    return upload_impl(ctx, m, n, nnz, rst, col, val, dtype, out, cudaMemcpyHostToDevice);
}

int ga_csr_from_device(ga_ctx ctx, int64_t m, int64_t n, int64_t nnz, const int32_t* rst, const int32_t* col,
                       const void* val, ga_dtype dtype, ga_csr* out) {
    return upload_impl(ctx, m, n, nnz, rst, col, val, dtype, out, cudaMemcpyDeviceToDevice);
}

int ga_csr_info(ga_csr A, int64_t* m, int64_t* n, int64_t* nnz, int* dtype) {
    if (!A) return GA_ERR_INVALID_ARG;
    if (m) *m = A->m;
    if (n) *n = A->n;
    if (nnz) *nnz = A->nnz;
    if (dtype) *dtype = (int)A->dtype;
    return GA_OK;
}

int ga_csr_download(ga_ctx ctx, ga_csr A, int32_t* rst, int32_t* col, void* val) {
    if (!ctx || !A) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        if (rst)
            GA_CUDA(cudaMemcpyAsync(rst, A->rst, sizeof(int32_t) * (A->m + 1), cudaMemcpyDeviceToHost,
                                    ctx->stream));
        if (col && A->nnz)
            GA_CUDA(cudaMemcpyAsync(col, A->col, sizeof(int32_t) * A->nnz, cudaMemcpyDeviceToHost, ctx->stream));
        if (val && A->nnz)
            GA_CUDA(cudaMemcpyAsync(val, A->val, dtype_size(A->dtype) * A->nnz, cudaMemcpyDeviceToHost,
                                    ctx->stream));
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int ga_csr_device_ptrs(ga_csr A, void** rst, void** col, void** val) {
    if (!A) return GA_ERR_INVALID_ARG;
    if (rst) *rst = A->rst;
    if (col) *col = A->col;
    if (val) *val = A->val;
    return GA_OK;
}

int ga_csr_set_symmetric(ga_ctx ctx, ga_csr A, int symmetric) {
    if (!ctx || !A || symmetric < -1 || symmetric > 1) return GA_ERR_INVALID_ARG;
    if (symmetric == 1 && A->m != A->n) {
        ctx->last_error = "a symmetric matrix is square";
        return GA_ERR_SHAPE;
    }
    A->sym = symmetric;
    return GA_OK;
}

int ga_csr_free(ga_ctx ctx, ga_csr A) {
    if (!ctx) return GA_ERR_INVALID_ARG;
    if (!A) return GA_OK;
    GA_API_BODY(ctx, {
        // a download of this handle still in flight on the copy stream
        // finishes before the stream-ordered free
        if (A->copied) GA_CUDA(cudaStreamWaitEvent(ctx->stream, A->copied, 0));
        csr_destroy(ctx, A);
    });
}

int ga_csr_download_async(ga_ctx ctx, ga_csr A, int32_t* rst, int32_t* col, void* val) {
    if (!ctx || !A) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        if (!ctx->copy_stream) {
            GA_CUDA(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
            GA_CUDA(cudaEventCreateWithFlags(&ctx->copy_ready, cudaEventDisableTiming));
            GA_CUDA(cudaEventCreateWithFlags(&ctx->copy_done, cudaEventDisableTiming));
        }
        GA_CUDA(cudaEventRecord(ctx->copy_ready, ctx->stream));
        GA_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ctx->copy_ready, 0));
        if (rst)
            GA_CUDA(cudaMemcpyAsync(rst, A->rst, sizeof(int32_t) * (A->m + 1), cudaMemcpyDeviceToHost,
                                    ctx->copy_stream));
        if (col && A->nnz)
            GA_CUDA(cudaMemcpyAsync(col, A->col, sizeof(int32_t) * A->nnz, cudaMemcpyDeviceToHost, ctx->copy_stream));
        if (val && A->nnz)
            GA_CUDA(cudaMemcpyAsync(val, A->val, dtype_size(A->dtype) * A->nnz, cudaMemcpyDeviceToHost,
                                    ctx->copy_stream));
        GA_CUDA(cudaEventRecord(ctx->copy_done, ctx->copy_stream));
        if (!A->copied) GA_CUDA(cudaEventCreateWithFlags(&A->copied, cudaEventDisableTiming));
        GA_CUDA(cudaEventRecord(A->copied, ctx->copy_stream));
    });
}

int ga_ctx_copy_sync(ga_ctx ctx) {
    if (!ctx) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        if (ctx->copy_stream) GA_CUDA(cudaStreamSynchronize(ctx->copy_stream));
    });
}

int ga_csr_convert(ga_ctx ctx, ga_csr A, ga_dtype dtype, ga_csr* out) {
    if (!ctx || !A || !out) return GA_ERR_INVALID_ARG;
    *out = nullptr;
    GA_API_BODY(ctx, {
        GA_REQUIRE(dtype_valid(dtype), GA_ERR_DTYPE, "unknown dtype");
        *out = copy_csr(ctx, A, dtype);
    });
}

// ---------------------------------------------------------------- dense
int ga_dense_create(ga_ctx ctx, int64_t m, int64_t n, ga_dtype dtype, const void* host_vals, ga_dense* out) {
    if (!ctx || !out) return GA_ERR_INVALID_ARG;
    *out = nullptr;
    GA_API_BODY(ctx, {
        GA_REQUIRE(dtype_valid(dtype), GA_ERR_DTYPE, "unknown dtype");
        GA_REQUIRE(m >= 0 && n >= 0, GA_ERR_INVALID_ARG, "negative dense dimension");
        ga_dense D = new ga_dense_s;
        D->m = m; D->n = n; D->dtype = dtype;
        size_t bytes = (size_t)m * (size_t)n * dtype_size(dtype);
        try {
            D->val = dalloc(ctx, bytes);
            if (host_vals)
                GA_CUDA(cudaMemcpyAsync(D->val, host_vals, bytes, cudaMemcpyHostToDevice, ctx->stream));
            else
                GA_CUDA(cudaMemsetAsync(D->val, 0, bytes, ctx->stream));
        } catch (...) {
            dfree(ctx, D->val);
            delete D;
            throw;
        }
        *out = D;
    });
}

int ga_dense_download(ga_ctx ctx, ga_dense D, void* host_vals) {
    if (!ctx || !D || !host_vals) return GA_ERR_INVALID_ARG;
    GA_API_BODY(ctx, {
        size_t bytes = (size_t)D->m * (size_t)D->n * dtype_size(D->dtype);
        GA_CUDA(cudaMemcpyAsync(host_vals, D->val, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        GA_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int ga_dense_info(ga_dense D, int64_t* m, int64_t* n, int* dtype) {
    if (!D) return GA_ERR_INVALID_ARG;
    if (m) *m = D->m;
    if (n) *n = D->n;
    if (dtype) *dtype = (int)D->dtype;
    return GA_OK;
}

int ga_dense_device_ptr(ga_dense D, void** vals) {
    if (!D || !vals) return GA_ERR_INVALID_ARG;
    *vals = D->val;
    return GA_OK;
}

int ga_dense_free(ga_ctx ctx, ga_dense D) {
    if (!ctx) return GA_ERR_INVALID_ARG;
    if (!D) return GA_OK;
    GA_API_BODY(ctx, {
        dfree(ctx, D->val);
        delete D;
    });
}

}  // extern "C"
