// fn_kernels.cuh -- host-visible declarations of the interpreter launchers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fn_program.h"

namespace fn {

// How points are generated (reference batch drivers, Generator.inl:79-433).
enum PointSource : int {
    kSrcGrid = 0,      // GenUniformGrid{2,3,4}D: pos_k = fma(float(i_k), step_k, offset_k)
    kSrcTileable = 1,  // GenTileable2D: 4D torus from cos/sin of the 2D index
    kSrcPositions = 2, // GenPositionArray{2,3,4}D: pos_k = offset_k + array_k[i]
};

struct PointArgs {
    int src;              // PointSource
    int dim;              // dimensionality of the root position
    int seed;
    long long total;      // number of points
    int count[4];         // grid counts (x fastest)
    float offset[4];
    float step[4];
    float tmul[2], tfreq[2];   // tileable constants
    const float* pos[4];  // position arrays (device)
};

// Per-launch reduction workspace.  `counter` must be zero before the first
// launch; the last block to finish resets it, so a workspace can be reused by
// consecutive launches on one stream (never by overlapping launches).
struct MinMaxWork {
    unsigned int counter;
    unsigned int pad[3];
    float result[2];
    float pad2[2];
    float partial[2 * 4096];
};

constexpr int kMaxReduceBlocks = 4096;

// Launch the interpreter over `args.total` points of `prog` (a device pointer
// to a program blob of `prog_bytes`).  Writes out[i] and the min/max to
// work->result (and to dminmax when not null).  Returns a cudaError_t.
cudaError_t launch_interpreter(const FnProgramHeader* prog, uint32_t prog_bytes, const PointArgs& args, float* out,
                               MinMaxWork* work, float* dminmax, cudaStream_t stream);

int num_sms();

}  // namespace fn
