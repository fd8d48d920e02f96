// fn_static_scratch.h -- allocation-free interpreter launch (fn_static_scratch.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fn_types.h"

namespace fn {

// Largest program blob the static scratch holds (header + instructions +
// parameters, bytes).  16 KiB covers trees of several hundred nodes.
constexpr uint32_t kStaticProgramBytes = 16 * 1024;

// Copy `blob` (host memory, a compiled program) into the per-device static
// scratch on `stream`, clear the reduction counter and launch the interpreter.
// Never allocates device memory.  The first call on a device looks up the
// scratch address for that device.  Calls that overlap on the GPU (different
// streams, no ordering between them) share the scratch and race.
// cudaErrorInvalidValue when blob_bytes exceeds kStaticProgramBytes.
cudaError_t launch_interpreter_static(const void* blob, uint32_t blob_bytes, const PointArgs& args, float* out,
                                      float* dminmax, cudaStream_t stream);

}  // namespace fn
