// fn_types.h -- plain-data launch types shared by the host runtime, the
// compiled kernels and the run-time specialised kernels (no includes, so the
// header can also be handed to NVRTC as source).
#pragma once

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
    // Division of a point index by count[k] (k < 3) as a multiply-high and shifts:
    // q = (t + ((n - t) >> 1)) >> (divs[k] - 1), t = umulhi(n, divm[k]); divs = 0 means count 1.
    unsigned int divm[3];
    unsigned int divs[3];
    // Index of this launch's first point in the whole request (0 unless a large grid is
    // generated slab by slab): positions come from base + i, output and min/max cover i only.
    unsigned int base;
};

// Per-launch reduction workspace.  Every block folds its min/max into the two
// keys with order-preserving atomics (mn_key holds the complement of the encoded
// minimum, so that zero means "nothing folded" for both keys), then counts itself
// in `counter`; the last block decodes the keys into `result` and clears
// counter and keys.  The first 16 bytes must be zero before the first launch;
// a workspace can then be reused by consecutive launches on one stream (never
// by overlapping launches).
struct MinMaxWork {
    unsigned int counter;
    unsigned int mn_key;
    unsigned int mx_key;
    unsigned int pad;
    float result[2];
    float pad2[2];
};

constexpr int kMaxReduceBlocks = 4096;

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
    const void* prog;            // FnProgramHeader* of the interpreter program
    float* out;
    float* minmax;               // device float[2] or null
    float* host_minmax;          // mapped pinned float[2] or null
    unsigned int* host_done;     // mapped pinned flag or null (set to 1 on completion)
    unsigned int prog_bytes;
    unsigned int n_tiles;
    int jit_slot;                // index of this tree in a specialised batch kernel, or -1
    unsigned int pad;
    unsigned long long* host_time;   // mapped pinned or null: device clock (ns) when the request completed
};

struct BatchState {              // per-request mutable state, zeroed by the host upload
    unsigned int mn_enc;         // order-preserving encodings (host sets 0xFFFFFFFF / 0)
    unsigned int mx_enc;
    unsigned int tiles_done;
    unsigned int pad;
};

struct BatchGroup {               // the work items of one tree (specialised batch kernels)
    unsigned int item_begin;
    unsigned int item_end;
    unsigned int head;           // next item offset (host uploads 0)
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

}  // namespace fn
