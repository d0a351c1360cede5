// Device-resident iteration loops.
//
// A loop body is a host function that enqueues kernels on the context
// stream and never synchronises. Its last kernel calls loop_continue() with
// the device-side decision. With GA_OPT_DEVICE_LOOPS the body is captured
// once into the body graph of a CUDA-graph WHILE conditional node and the
// whole loop runs from one graph launch: no host round trip per iteration.
// Otherwise the same body is enqueued from a host loop that reads the
// decision back after every iteration.
#pragma once

#include "ga_internal.cuh"

#include <functional>

namespace ga {

struct LoopCtl {
    cudaGraphConditionalHandle handle;  // valid when use_handle != 0
    int use_handle;
    int* cont;                          // device flag (host-loop mode)
};

// Called by exactly one thread of the body's final kernel.
__device__ __forceinline__ void loop_continue(const LoopCtl& c, bool more) {
    if (c.use_handle) cudaGraphSetConditional(c.handle, more ? 1u : 0u);
    *c.cont = more ? 1 : 0;
}

// Runs body(ctl) until the device says stop. max_host_iters bounds the host
// loop (the device-side bodies also carry their own iteration caps).
void run_device_loop(ga_ctx ctx, const std::function<void(const LoopCtl&)>& body, int64_t max_host_iters);

// The same for a body whose kernels take nothing that changes from call to
// call except through device memory (cached_loop_args): its graph is
// captured and instantiated on the context's first call for `slot` and only
// relaunched afterwards. The kernel grid sizes must not depend on the call.
void run_cached_loop(ga_ctx ctx, int slot, const std::function<void(const LoopCtl&)>& body, int64_t max_host_iters);
// A device buffer of `bytes` kept with the slot's loop for the context's
// lifetime: where the host writes the call's parameters before the launch.
void* cached_loop_args(ga_ctx ctx, int slot, size_t bytes);
enum { kLoopSlotTriFront = 0, kLoopSlotTriFrontBatch = 1 };

}  // namespace ga
