// fn_kernels.cuh -- host-visible declarations of the compiled kernels' launchers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fn_program.h"
#include "fn_types.h"

namespace fn {

// Launch the interpreter over `args.total` points of `prog` (a device pointer
// to a program blob of `prog_bytes`).  Writes out[i] and the min/max to
// work->result (and to dminmax when not null).  Returns a cudaError_t.
cudaError_t launch_interpreter(const FnProgramHeader* prog, uint32_t prog_bytes, const PointArgs& args, float* out,
                               MinMaxWork* work, float* dminmax, cudaStream_t stream);

int num_sms();

// Batched persistent launch of the interpreter (see fn_types.h).
// items[i] = (request index, tile index within the request).
cudaError_t launch_batch(BatchHeader* hdr, const BatchRequest* reqs, BatchState* states, const uint2* items,
                         uint32_t max_prog_bytes, int grid, int block, cudaStream_t stream);

// CTAs per SM the batch kernel can keep resident for `block` threads and `smem` bytes.
int batch_occupancy(int block, uint32_t smem);

}  // namespace fn
