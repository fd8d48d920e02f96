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

// Mesh the density array of a bloxel chunk (size^3 voxels, (size+2)^3 densities
// with a one-voxel apron; `up_axis_z` = the densities were generated with y and z
// swapped).  Writes at most vcap vertices / icap indices; the face total and the
// min air / max solid heights land in `s`.  Asynchronous on `stream`.
cudaError_t launch_bloxel(const float* dens, int size, bool up_axis_z, float px, float py, float pz, float iso,
                          const float* dminmax, MeshScratch& s, MeshVertex* verts, unsigned vcap, unsigned* idx,
                          unsigned icap, cudaStream_t stream);

// Heightmap chunk: size^2 quads over (size+1)^2 densities.
cudaError_t launch_heightmap(const float* dens, int size, float px, float pz, float mul, MeshVertex* verts, unsigned vcap,
                             unsigned* idx, unsigned icap, cudaStream_t stream);

}  // namespace fn
