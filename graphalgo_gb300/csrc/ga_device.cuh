// Device-side helpers shared by the kernels: value-type traits, warp scans,
// shared-memory hash tables.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "ga_internal.cuh"

namespace ga {

// Accumulator type per value type. Sums are taken in the accumulator type and
// stored back in the value type: for uint8 this is addition modulo 256, the
// same result the reference's `T += a*b` on unsigned char gives.
template <typename T> struct Acc { using type = T; };
template <> struct Acc<uint8_t> { using type = uint32_t; };
template <> struct Acc<int32_t> { using type = int32_t; };
template <> struct Acc<int64_t> { using type = unsigned long long; };

template <typename A>
__device__ __forceinline__ void atomic_add_acc(A* p, A v) {
    atomicAdd(p, v);
}
template <>
__device__ __forceinline__ void atomic_add_acc<int32_t>(int32_t* p, int32_t v) {
    atomicAdd(p, v);
}

template <typename T, typename A>
__device__ __forceinline__ A to_acc(T v) {
    return (A)v;
}
template <>
__device__ __forceinline__ unsigned long long to_acc<int64_t, unsigned long long>(int64_t v) {
    return (unsigned long long)v;
}

template <typename T, typename A>
__device__ __forceinline__ T from_acc(A v) {
    return (T)v;
}

// products in the accumulator type (two's-complement wrap for integers)
template <typename T, typename A>
__device__ __forceinline__ A mul_acc(T a, T b) {
    return to_acc<T, A>(a) * to_acc<T, A>(b);
}
template <>
__device__ __forceinline__ int32_t mul_acc<int32_t, int32_t>(int32_t a, int32_t b) {
    return (int32_t)((uint32_t)a * (uint32_t)b);
}

// acc + a*b rounded as two separate operations (no fused multiply-add), the
// evaluation the reference's host loops get from a compiler that does not
// contract; integers are unaffected.
template <typename T>
__device__ __forceinline__ T mul_add_separate(T acc, T a, T b) {
    return acc + a * b;
}
template <>
__device__ __forceinline__ double mul_add_separate<double>(double acc, double a, double b) {
    return __dadd_rn(acc, __dmul_rn(a, b));
}
template <>
__device__ __forceinline__ float mul_add_separate<float>(float acc, float a, float b) {
    return __fadd_rn(acc, __fmul_rn(a, b));
}

// ---------------------------------------------------------------- warp scans
__device__ __forceinline__ int warp_incl_scan(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += t;
    }
    return v;
}

__device__ __forceinline__ long long warp_incl_scan_ll(long long v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        long long t = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += t;
    }
    return v;
}

template <typename V>
__device__ __forceinline__ V warp_sum(V v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
    return v;
}

// --------------------------------------------------------------- hashing
__device__ __forceinline__ uint32_t hash_col(int32_t c) { return (uint32_t)c * 0x9E3779B1u; }

// Insert distinct key `k` with payload `slot` into an open-addressing table of
// 2^bits entries (keys initialised to kEmpty). Linear probing.
template <typename S>
__device__ __forceinline__ void hash_insert(int32_t* keys, S* slots, int bits, int32_t k, S slot) {
    const uint32_t mask = (1u << bits) - 1u;
    uint32_t h = hash_col(k) >> (32 - bits);
    while (true) {
        int32_t prev = atomicCAS(&keys[h], kEmpty, k);
        if (prev == kEmpty || prev == k) {
            slots[h] = slot;
            return;
        }
        h = (h + 1) & mask;
    }
}

// Returns the payload for key `k`, or -1 when absent.
template <typename S>
__device__ __forceinline__ int hash_find(const int32_t* keys, const S* slots, int bits, int32_t k) {
    const uint32_t mask = (1u << bits) - 1u;
    uint32_t h = hash_col(k) >> (32 - bits);
    while (true) {
        int32_t cur = keys[h];
        if (cur == k) return (int)slots[h];
        if (cur == kEmpty) return -1;
        h = (h + 1) & mask;
    }
}

// lower_bound over a sorted int32 array
__device__ __forceinline__ int lower_bound_i32(const int32_t* a, int n, int32_t x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] < x) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ int upper_bound_i32(const int32_t* a, int n, int32_t x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] <= x) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Lower bound of x among 32 ascending values held one per lane (`key`):
// the first lane whose value is >= x, 32 if none. Six shuffle steps; every
// lane searches for its own x.
__device__ __forceinline__ int warp_lower_bound(int32_t key, int32_t x) {
    int lo = 0, hi = 32;
#pragma unroll
    for (int step = 0; step < 6; ++step) {
        const int mid = (lo + hi) >> 1;
        const int32_t v = __shfl_sync(0xffffffffu, key, mid & 31);
        if (lo < hi) {
            if (v < x) lo = mid + 1;
            else hi = mid;
        }
    }
    return lo;
}

// ------------------------------------------------ bulk copies (sm_90 and up)
// One thread copies a contiguous global range into shared memory with the
// tensor memory accelerator's untiled bulk copy; the bytes complete a
// transaction count on a shared-memory barrier that the consumers wait on.
// Both addresses must be 16-byte aligned and the size a multiple of 16.
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t arrivals) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(arrivals) : "memory");
}

// Makes barrier initialisation visible to the bulk-copy unit.
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One arrival that also announces `bytes` of bulk copies to come.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Orders this thread's earlier shared-memory accesses before later bulk
// copies into the same memory.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Waits until the barrier's phase of parity `parity` has completed, for at
// most `max_cycles` SM clock cycles; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long max_cycles) {
    const long long t0 = clock64();
    while (true) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > max_cycles) return false;
    }
}

}  // namespace ga

// value-type dispatch over a ga_dtype
#define GA_DISPATCH_DTYPE(dt, T, ...)                                  \
    switch (dt) {                                                      \
    case GA_INT32: { using T = int32_t; __VA_ARGS__; break; }          \
    case GA_INT64: { using T = int64_t; __VA_ARGS__; break; }          \
    case GA_FP32: { using T = float; __VA_ARGS__; break; }             \
    case GA_FP64: { using T = double; __VA_ARGS__; break; }            \
    case GA_UINT8: { using T = uint8_t; __VA_ARGS__; break; }          \
    default: ::ga::fail(GA_ERR_DTYPE, "unsupported dtype");            \
    }
