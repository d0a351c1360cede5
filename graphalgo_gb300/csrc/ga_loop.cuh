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

}  // namespace ga
