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

// ---------------------------------------------------------------- batched persistent launch
//
// A batch is N requests (each: one tree program, one point source, one output
// array) cut into tiles of `tile_points` points.  Work items (request, tile)
// are listed in `items`; persistent CTAs pull the next item index from
// `hdr->head` with one atomicAdd, so CTAs that draw cheap tiles simply take
// more of them.  Each request's min/max is folded with order-preserving
// integer atomics; the CTA that finishes a request's last tile decodes it,
// writes it to `minmax` (device) and to `host_minmax` / `host_done` (mapped
// pinned memory, visible to the host as soon as the request is done).

struct BatchRequest {
    PointArgs args;
    const FnProgramHeader* prog;
    float* out;
    float* minmax;               // device float[2] or null
    float* host_minmax;          // mapped pinned float[2] or null
    unsigned int* host_done;     // mapped pinned flag or null (set to 1 on completion)
    uint32_t prog_bytes;
    uint32_t n_tiles;
    uint32_t pad[4];
};

struct BatchState {              // per-request mutable state, zeroed by the host upload
    unsigned int mn_enc;         // order-preserving encodings (host sets 0xFFFFFFFF / 0)
    unsigned int mx_enc;
    unsigned int tiles_done;
    unsigned int pad;
};

struct BatchHeader {
    unsigned int n_req;
    unsigned int n_items;
    unsigned int tile_points;
    unsigned int head;           // next work item (host uploads 0)
    unsigned int requests_done;
    unsigned int max_prog_bytes;
    unsigned int pad[2];
};

// items[i] = (request index, tile index within the request)
cudaError_t launch_batch(BatchHeader* hdr, const BatchRequest* reqs, BatchState* states, const uint2* items,
                         uint32_t max_prog_bytes, int grid, int block, cudaStream_t stream);

// CTAs per SM the batch kernel can keep resident for `block` threads and `smem` bytes.
int batch_occupancy(int block, uint32_t smem);
cudaError_t batch_kernel_node_params(void** func);

}  // namespace fn
