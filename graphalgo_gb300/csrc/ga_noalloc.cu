// Allocation-free masked SpGEMM entry point.
//
// Some callers cannot allocate device memory at the moment they need the
// product: host applications that hand the whole device-memory budget to
// their own arena at start-up and do not let libraries allocate, and
// latency-critical callers that cannot accept the device-wide
// synchronisation cudaMalloc and cudaFree may cause. This entry point takes
// the caller's device buffers for every input and output, creates no
// context, and keeps the kernel's scratch (work queue, row lists, CTA work
// items) in one file-scope device array of fixed size. Every GPU that loads
// this library holds that array until the process exits. The schedule is the
// default one (bin thresholds and grid size); tuned schedules belong to
// contexts, which this entry point does not have.
#include "ga_device.cuh"

#include <mutex>

namespace ga {
namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)16 << 20;  // 16 MiB

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
__device__ unsigned long long g_noalloc_counters[GA_CTR_COUNT];

struct NoAllocDevice {
    bool ready = false;
    void* scratch = nullptr;               // device address of g_noalloc_scratch
    unsigned long long* counters = nullptr;
    int num_sms = 0;
};

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
NoAllocDevice g_noalloc_dev[kMaxDevices];

// Resolves the device addresses of the file-scope arrays for the current
// device, once per device (the host-side names are not device addresses).
const NoAllocDevice& noalloc_setup() {
    int dev = 0;
    GA_CUDA(cudaGetDevice(&dev));
    GA_REQUIRE(dev >= 0 && dev < kMaxDevices, GA_ERR_UNSUPPORTED, "noalloc: device index too large");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoAllocDevice& d = g_noalloc_dev[dev];
    if (!d.ready) {
        void* s = nullptr;
        void* c = nullptr;
        GA_CUDA(cudaGetSymbolAddress(&s, g_noalloc_scratch));
        GA_CUDA(cudaGetSymbolAddress(&c, g_noalloc_counters));
        int sms = 0;
        GA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        d.scratch = s;
        d.counters = static_cast<unsigned long long*>(c);
        d.num_sms = sms;
        d.ready = true;
    }
    return d;
}

}  // namespace
}  // namespace ga

using namespace ga;

extern "C" int ga_mxm_masked_noalloc(void* stream, ga_algo algo, int64_t m, int64_t k, int64_t n,
                                     const int32_t* a_rst, const int32_t* a_col, const void* a_val,
                                     const int32_t* b_rst, const int32_t* b_col, const void* b_val,
                                     const int32_t* m_rst, const int32_t* m_col, int64_t mask_nnz, ga_dtype dtype,
                                     int b_unit, void* c_val) {
    if (m < 0 || k < 0 || n < 0 || mask_nnz < 0) return GA_ERR_INVALID_ARG;
    if (algo != GA_MSA && algo != GA_MCA && algo != GA_HEAP) return GA_ERR_UNSUPPORTED;
    if (!dtype_valid(dtype)) return GA_ERR_DTYPE;
    if (m == 0 || mask_nnz == 0) return GA_OK;
    if (m >= INT32_MAX || n > INT32_MAX || k > INT32_MAX || mask_nnz > INT32_MAX) return GA_ERR_INVALID_ARG;
    if (!a_rst || !a_col || !a_val || !b_rst || !b_col || !m_rst || !m_col || !c_val) return GA_ERR_INVALID_ARG;
    // the sorted merge (GA_HEAP) always reads B's values
    if ((!b_unit || algo == GA_HEAP) && !b_val) return GA_ERR_INVALID_ARG;
    // the scratch needed for this shape must fit the fixed array
    if (mxm_scratch_bytes(m, n, mask_nnz, false) > kNoAllocScratchBytes) return GA_ERR_INVALID_ARG;
    try {
        const NoAllocDevice& d = noalloc_setup();
        ga_ctx_s ctx;  // stack-only view: stream and device facts, no allocations
        GA_CUDA(cudaGetDevice(&ctx.device));
        ctx.stream = static_cast<cudaStream_t>(stream);
        ctx.num_sms = d.num_sms;
        ctx.d_counters = d.counters;
        ctx.profile = false;
        ga_csr_s A, B, M;
        A.m = m; A.n = k; A.dtype = dtype; A.rst = const_cast<int32_t*>(a_rst);
        A.col = const_cast<int32_t*>(a_col); A.val = const_cast<void*>(a_val);
        B.m = k; B.n = n; B.dtype = dtype; B.rst = const_cast<int32_t*>(b_rst);
        B.col = const_cast<int32_t*>(b_col); B.val = const_cast<void*>(b_val);
        M.m = m; M.n = n; M.nnz = mask_nnz; M.dtype = dtype; M.rst = const_cast<int32_t*>(m_rst);
        M.col = const_cast<int32_t*>(m_col);
        mxm_masked_launch(&ctx, algo, &A, &B, &M, c_val, d.scratch, mask_nnz, b_unit != 0 && algo != GA_HEAP);
        return GA_OK;
    } catch (const Error& e) {
        return e.code;
    } catch (...) {
        return GA_ERR_CUDA;
    }
}
