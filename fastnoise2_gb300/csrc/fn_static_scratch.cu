// fn_static_scratch.cu -- an allocation-free launch of the interpreter.
//
// The ordinary device entry points keep their scratch (the tree's program blob
// and the min/max reduction workspace) in memory that the library obtains with
// cudaMalloc on first use.  Some callers cannot let a library allocate:
//   * applications that hand all device memory to their own pool allocator at
//     start-up, so a later cudaMalloc from a library fails or evicts their pool;
//   * frame loops with a fixed time budget, where cudaFree synchronises the
//     whole device and an allocation can stall for milliseconds.
// For them, this file keeps the scratch in one statically sized __device__
// array that is part of the loaded module, so no call ever allocates device
// memory.  The price: every call shares that one array.
#include <cuda_runtime.h>

#include <cstddef>
#include <cstring>
#include <mutex>

#include "fn_kernels.cuh"
#include "fn_static_scratch.h"

namespace fn {

namespace {

struct StaticScratch {
    MinMaxWork work;                                         // reduction workspace; counter and keys must start at zero
    alignas(256) unsigned char prog[kStaticProgramBytes];     // the tree's program blob
};

// The shared scratch: one per device, sized at compile time (about 17 KB).
static __device__ __align__(256) unsigned char g_scratch[sizeof(StaticScratch)];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
StaticScratch* g_scratch_ptr[kMaxDevices] = {};

// One-time set-up per device, done with that device current: look up the
// device address of g_scratch.
cudaError_t scratch_for_current_device(StaticScratch** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = static_cast<StaticScratch*>(p);
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

}  // namespace

cudaError_t launch_interpreter_static(const void* blob, uint32_t blob_bytes, const PointArgs& args, float* out,
                                      float* dminmax, cudaStream_t stream)
{
    if (blob_bytes > kStaticProgramBytes || (blob_bytes & 15)) return cudaErrorInvalidValue;
    StaticScratch* s = nullptr;
    cudaError_t e = scratch_for_current_device(&s);
    if (e != cudaSuccess) return e;
    // Both copies are stream-ordered: they land after any earlier call on this
    // stream has finished with the array, and before this call's kernel reads it.
    e = cudaMemcpyAsync(s->prog, blob, blob_bytes, cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(&s->work, 0, offsetof(MinMaxWork, result), stream);   // counter and min/max keys
    if (e != cudaSuccess) return e;
    return launch_interpreter(reinterpret_cast<const FnProgramHeader*>(s->prog), blob_bytes, args, out, &s->work, dminmax,
                              stream);
}

}  // namespace fn
