// fn_mesh.h -- chunk meshers (fn_mesh.cu) and their host driver (fn_mesh.cpp).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

namespace fn {

struct MeshVertex {         // the Node Editor's VertexData: position and light
    float x, y, z, light;
};

// Per-thread device scratch of the bloxel mesher.
struct MeshScratch {
    unsigned* counts = nullptr;        // faces per voxel
    unsigned* offsets = nullptr;       // exclusive scan of counts
    unsigned* block_totals = nullptr;  // per 1024-voxel block, scanned in place
    unsigned* total = nullptr;         // faces in the chunk
    unsigned* airsolid = nullptr;      // order-preserving min air y / max solid y
    size_t cap_voxels = 0;
};

// Per-thread device scratch of the dual marching cubes mesher.
struct DmcScratch {
    uint2* offsets = nullptr;          // per cell: first vertex it creates, first quad it emits (tiles that hold quads)
    uint2* tile_sums = nullptr;        // per 2048 cells: vertices, quads; then scanned into tile offsets
    uint2* total = nullptr;            // vertices, quads in the chunk
    unsigned* masks = nullptr;         // per cell: which of its 12 quad slots create a vertex
    unsigned* airsolid = nullptr;      // order-preserving min air y / max solid y
    unsigned* counters = nullptr;      // work items listed: vertices, quads
    unsigned* vert_items = nullptr;    // 4 (size+1)^3: every (vertex cell, piece) at most once
    unsigned* quad_items = nullptr;    // 3 size^3: every cut edge at most once
    unsigned char* cases = nullptr;    // (size+1)^3 marching-cubes cases
    size_t cap_cells = 0;
};

// The sparse density form of a chunk (no density array): two classification bitmasks of
// every density (bit i of word i / 32), written by the tree's fnjit_solid kernel; the needed
// densities marked in `need`, their ranks per word, their index list and their values
// (written by the tree's fnjit_list kernel from idx and total).
struct SparseScratch {
    unsigned* above = nullptr;         // density > iso
    unsigned* solid = nullptr;         // density <= iso
    unsigned* need = nullptr;
    unsigned* cells = nullptr;         // dual marching cubes: base corners of the created vertices' cells
    unsigned* counts = nullptr;        // set bits per word of need
    unsigned* rank = nullptr;          // exclusive scan of counts
    uint2* stored = nullptr;           // per word of need: (rank, bits), for value lookups
    unsigned* block_totals = nullptr;
    unsigned* total = nullptr;         // needed densities
    unsigned* idx = nullptr;           // their density indices, ascending
    float* vals = nullptr;             // their values
    size_t cap_densities = 0;
};

// Mesh the density array of a bloxel chunk (size^3 voxels, (size+2)^3 densities
// with a one-voxel apron; `up_axis_z` = the densities were generated with y and z
// swapped).  Writes at most vcap vertices / icap indices; the face total and the
// min air / max solid heights land in `s`.  Asynchronous on `stream`.
cudaError_t launch_bloxel(const float* dens, int size, bool up_axis_z, float px, float py, float pz, float iso,
                          const float* dminmax, MeshScratch& s, MeshVertex* verts, unsigned vcap, unsigned* idx,
                          unsigned icap, cudaStream_t stream);

// The bloxel mesher on the sparse form, in two parts around the evaluation of the needed
// densities: prepare (faces, the face scan, the needed list: every voxel with a face), then
// emit.  The bitmasks and OutputMinMax must be in place first.
cudaError_t launch_bloxel_sparse_prepare(SparseScratch& sp, int size, bool up_axis_z, float px, float py, float pz, float iso,
                                         const float* dminmax, MeshScratch& s, cudaStream_t stream);
cudaError_t launch_bloxel_sparse_emit(const SparseScratch& sp, int size, bool up_axis_z, float px, float py, float pz, float iso,
                                      const float* dminmax, MeshScratch& s, MeshVertex* verts, unsigned vcap, unsigned* idx,
                                      unsigned icap, cudaStream_t stream);

// Heightmap chunk: size^2 quads over (size+1)^2 densities.
cudaError_t launch_heightmap(const float* dens, int size, float px, float pz, float mul, MeshVertex* verts, unsigned vcap,
                             unsigned* idx, unsigned icap, cudaStream_t stream);

// Dual marching cubes chunk: size^3 cells over (size+4)^3 densities (a two-voxel
// apron).  Vertices and indices are written only when both fit (vcap / icap);
// the vertex and quad totals land in s.total either way.
cudaError_t launch_dmc(const float* dens, int size, bool up_axis_z, int px, int py, int pz, float iso, const float* dminmax,
                       DmcScratch& s, MeshVertex* verts, unsigned vcap, unsigned* idx, unsigned icap, cudaStream_t stream);

// Dual marching cubes on the sparse form: prepare (cases, quads, vertices, scans, the needed
// list: the densities around every created vertex's cell), then the vertex and quad passes.
cudaError_t launch_dmc_sparse_prepare(SparseScratch& sp, int size, bool up_axis_z, float iso, const float* dminmax, DmcScratch& s,
                                      cudaStream_t stream);
cudaError_t launch_dmc_sparse_finish(const SparseScratch& sp, int size, bool up_axis_z, int px, int py, int pz, float iso,
                                     DmcScratch& s, MeshVertex* verts, unsigned vcap, unsigned* idx, unsigned icap,
                                     cudaStream_t stream);

}  // namespace fn
