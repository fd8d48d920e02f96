// fn_capi_mesh.cpp -- the chunk-meshing entry points of include/FastNoise/FastNoise_C.h
// (fnBuildChunkMesh*, fnBuildChunkMeshes*): per-thread device scratch, the lanes of the
// multi-chunk calls, and the host side of the meshers in fn_mesh.cu.  They restate the Node
// Editor's chunk meshers (reference tools/NodeEditor/MeshNoisePreview.cpp) on the GPU.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>

#include "../../include/FastNoise/FastNoise_C.h"
#include "fn_capi_internal.h"
#include "fn_jit.h"
#include "fn_mesh.h"

using namespace fn;
using namespace fn::capi;

// ---------------------------------------------------------------- chunk meshing
namespace {

// Device scratch of one mesher lane: densities, their min/max, the bloxel scan buffers
// and the dual marching cubes buffers, plus a pinned read-back area for single calls.
// Single-chunk calls use the thread's lane on the caller's stream; multi-chunk calls
// spread their chunks over kMeshLanes lanes with their own streams.
struct MeshCtx {
    float* dens = nullptr;
    size_t dens_cap = 0;
    float* dminmax = nullptr;
    MeshScratch scratch;
    DmcScratch dmc;
    SparseScratch sp;                  // the sparse density form (trees with specialised kernels)
    unsigned* host = nullptr;          // pinned read-back of one chunk (see enqueue_chunk)
    ~MeshCtx()
    {
        if (dens) cudaFree(dens);
        if (dminmax) cudaFree(dminmax);
        if (scratch.counts) cudaFree(scratch.counts);
        if (dmc.offsets) cudaFree(dmc.offsets);
        if (sp.stored) cudaFree(sp.stored);
        if (host) cudaFreeHost(host);
    }

    // Bitmasks, ranks and the needed list for `densities` densities.  The index list and the
    // value array are sized for every density, though a chunk stores only the few near its
    // surface.
    bool reserve_sparse(size_t densities)
    {
        if (densities <= sp.cap_densities) return true;
        if (sp.stored) cudaFree(sp.stored);
        sp = SparseScratch();
        const size_t words = (densities + 31) / 32, nb = (words + 1023) / 1024;
        char* block = nullptr;
        // stored (uint2) | above | solid | need | cells | counts | rank | block totals | total | idx | vals
        const size_t uwords = 6 * words + nb + 1 + densities;
        if (!cuda_ok(cudaMalloc(&block, words * sizeof(uint2) + uwords * sizeof(unsigned) + densities * sizeof(float)),
                     "cudaMalloc(mesh sparse densities)"))
            return false;
        sp.stored = reinterpret_cast<uint2*>(block);
        unsigned* w = reinterpret_cast<unsigned*>(block + words * sizeof(uint2));
        sp.above = w;
        sp.solid = w + words;
        sp.need = w + 2 * words;
        sp.cells = w + 3 * words;
        sp.counts = w + 4 * words;
        sp.rank = w + 5 * words;
        sp.block_totals = w + 6 * words;
        sp.total = w + 6 * words + nb;
        sp.idx = w + 6 * words + nb + 1;
        sp.vals = reinterpret_cast<float*>(w + 6 * words + nb + 1 + densities);
        sp.cap_densities = densities;
        return true;
    }

    bool reserve(size_t densities, size_t voxels)
    {
        if (!dminmax && !cuda_ok(cudaMalloc(&dminmax, 2 * sizeof(float)), "cudaMalloc(mesh minmax)")) return false;
        if (!host && !cuda_ok(cudaMallocHost(&host, 8 * sizeof(unsigned)), "cudaMallocHost(mesh read-back)")) return false;
        if (densities > dens_cap) {
            if (dens) cudaFree(dens);
            dens = nullptr; dens_cap = 0;
            if (!cuda_ok(cudaMalloc(&dens, densities * sizeof(float)), "cudaMalloc(mesh densities)")) return false;
            dens_cap = densities;
        }
        if (voxels > scratch.cap_voxels) {
            if (scratch.counts) cudaFree(scratch.counts);
            scratch = MeshScratch();
            const size_t nb = (voxels + 1023) / 1024;
            unsigned* block = nullptr;                  // counts | offsets | block totals | total | air, solid
            if (!cuda_ok(cudaMalloc(&block, (2 * voxels + nb + 4) * sizeof(unsigned)), "cudaMalloc(mesh scan)")) return false;
            scratch.counts = block;
            scratch.offsets = block + voxels;
            scratch.block_totals = block + 2 * voxels;
            scratch.total = block + 2 * voxels + nb;
            scratch.airsolid = block + 2 * voxels + nb + 1;
            scratch.cap_voxels = voxels;
        }
        return true;
    }

    bool reserve_dmc(int size)
    {
        const size_t cells = (size_t)size * size * size, vcells = (size_t)(size + 1) * (size + 1) * (size + 1);
        if (cells <= dmc.cap_cells) return true;
        if (dmc.offsets) cudaFree(dmc.offsets);
        dmc = DmcScratch();
        const size_t tiles = (cells + 2047) / 2048;
        // uint2: offsets | tile sums | total; uint32: masks | air, solid | list counters |
        // vertex items | quad items; then cases (uint8)
        const size_t pairs = cells + tiles + 1, words = cells + 4 + 4 * vcells + 3 * cells;
        char* block = nullptr;
        if (!cuda_ok(cudaMalloc(&block, pairs * sizeof(uint2) + words * sizeof(unsigned) + vcells), "cudaMalloc(dmc scratch)"))
            return false;
        uint2* p = reinterpret_cast<uint2*>(block);
        dmc.offsets = p;
        dmc.tile_sums = p + cells;
        dmc.total = p + cells + tiles;
        unsigned* w = reinterpret_cast<unsigned*>(p + pairs);
        dmc.masks = w;
        dmc.airsolid = w + cells;
        dmc.counters = w + cells + 2;
        dmc.vert_items = w + cells + 4;
        dmc.quad_items = w + cells + 4 + 4 * vcells;
        dmc.cases = reinterpret_cast<unsigned char*>(w + words);
        dmc.cap_cells = cells;
        return true;
    }
};
thread_local MeshCtx t_mesh;

// FN_MESH_DENSITY_ARRAY (default) or FN_MESH_DENSITY_SPARSE (fnSetMeshDensityForm).
std::atomic<int> g_mesh_form{FN_MESH_DENSITY_ARRAY};

constexpr int kMeshLanes = 4;

struct MeshLanes {
    MeshCtx lane[kMeshLanes];
    cudaStream_t stream[kMeshLanes] = {};
    cudaEvent_t fork = nullptr, join[kMeshLanes] = {};
    unsigned* host = nullptr;          // pinned read-back, 8 words per chunk
    size_t host_cap = 0;               // chunks
    ~MeshLanes()
    {
        for (int k = 0; k < kMeshLanes; ++k) {
            if (join[k]) cudaEventDestroy(join[k]);
            if (stream[k]) cudaStreamDestroy(stream[k]);
        }
        if (fork) cudaEventDestroy(fork);
        if (host) cudaFreeHost(host);
    }
};
thread_local MeshLanes* t_mesh_lanes = nullptr;

MeshLanes* mesh_lanes(size_t chunks)
{
    if (!t_mesh_lanes) {
        MeshLanes* l = new MeshLanes();
        bool ok = cuda_ok(cudaEventCreateWithFlags(&l->fork, cudaEventDisableTiming), "event");
        for (int k = 0; ok && k < kMeshLanes; ++k)
            ok = cuda_ok(cudaStreamCreateWithFlags(&l->stream[k], cudaStreamNonBlocking), "stream") &&
                 cuda_ok(cudaEventCreateWithFlags(&l->join[k], cudaEventDisableTiming), "event");
        if (!ok) { delete l; return nullptr; }
        t_mesh_lanes = l;
    }
    MeshLanes* l = t_mesh_lanes;
    if (chunks > l->host_cap) {
        if (l->host) cudaFreeHost(l->host);
        l->host = nullptr;
        l->host_cap = 0;
        if (!cuda_ok(cudaMallocHost(&l->host, chunks * 8 * sizeof(unsigned)), "cudaMallocHost(mesh read-back)")) return nullptr;
        l->host_cap = chunks;
    }
    return l;
}

float decode_ordered(unsigned u) { return f_of((int32_t)((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u)); }

enum MeshKind { kBloxel = 0, kDmc = 1 };

bool mesh_args_ok(int size, const fnChunkMesh* mesh)
{
    return mesh && size >= 1 && size <= 256 && mesh->vertexCapacity >= 0 && mesh->indexCapacity >= 0;
}

// Queue one chunk on `s` with lane `m`: its densities (GenPositionArray3D over the editor's
// grid positions offset by the chunk position -- MeshNoisePreview.cpp:447-455 bloxel, -1 ..
// size; :594-603 DMC, -2 .. size+1 -- as a grid of the same exact integer-valued floats; with
// the z axis up, y and z swap roles), the mesher, and the read-back into host8: bloxel
// [faces, air, solid], DMC [vertices, quads, air, solid]; [4..5] OutputMinMax.
bool enqueue_chunk(MeshKind kind, const DeviceProgram& prog, MeshCtx& m, cudaStream_t s, int size, int px, int py, int pz,
                   int seed, float iso, int upAxisZ, const fnChunkMesh* mesh, unsigned* host8)
{
    const int apron = kind == kDmc ? 2 : 1;
    const int sg = size + 2 * apron;
    const size_t n_dens = (size_t)sg * sg * sg;
    MinMaxWork* work = work_for_stream(s);
    if (!work) return false;
    const float off[3] = {(float)(px - apron), (float)((upAxisZ ? pz : py) - apron), (float)((upAxisZ ? py : pz) - apron)};
    const int cnt[3] = {sg, sg, sg};
    const float step[3] = {1, 1, 1};
    const PointArgs args = grid_args(3, off, cnt, step, seed);
    // The density array (default): the tree's kernel writes every density of the chunk (9 MB
    // for the editor's 128^3, which stays in L2 between generation and meshing).  The sparse
    // form (fnSetMeshDensityForm, trees with specialised kernels): the densities stay in
    // registers, only their classification against the iso level is stored, and the exact
    // values the passes read are evaluated again at those voxels only.
    bool sparse = false;
    if (g_mesh_form.load(std::memory_order_relaxed) == FN_MESH_DENSITY_SPARSE && jit_enabled()) {
        if (!m.reserve(0, kind == kBloxel ? (size_t)size * size * size : 0) || (kind == kDmc && !m.reserve_dmc(size)) ||
            !m.reserve_sparse(n_dens))
            return false;
        cudaError_t err = cudaSuccess;
        sparse = jit_launch_solid(prog.hash, args, m.sp.above, m.sp.solid, work, m.dminmax, iso, s, err);
        if (sparse && !cuda_ok(err, "densities (classification)")) return false;
    }
    if (!sparse) {
        if (!m.reserve(n_dens, kind == kBloxel ? (size_t)size * size * size : 0) || (kind == kDmc && !m.reserve_dmc(size)))
            return false;
        if (!cuda_ok(launch_points(prog, args, m.dens, work, m.dminmax, s), "densities")) return false;
    }
    MeshVertex* verts = reinterpret_cast<MeshVertex*>(mesh->vertices);
    auto needed_values = [&]() {
        cudaError_t err = cudaSuccess;
        return jit_launch_list(prog.hash, args, m.sp.idx, m.sp.total, (unsigned)n_dens, m.sp.vals, s, err) &&
               cuda_ok(err, "needed densities");
    };
    if (kind == kBloxel) {
        const bool queued =
            sparse ? cuda_ok(launch_bloxel_sparse_prepare(m.sp, size, upAxisZ != 0, (float)px, (float)py, (float)pz, iso, m.dminmax,
                                                          m.scratch, s), "bloxel mesher") &&
                         needed_values() &&
                         cuda_ok(launch_bloxel_sparse_emit(m.sp, size, upAxisZ != 0, (float)px, (float)py, (float)pz, iso, m.dminmax,
                                                           m.scratch, verts, (unsigned)mesh->vertexCapacity, mesh->indices,
                                                           (unsigned)mesh->indexCapacity, s), "bloxel mesher")
                   : cuda_ok(launch_bloxel(m.dens, size, upAxisZ != 0, (float)px, (float)py, (float)pz, iso, m.dminmax, m.scratch,
                                           verts, (unsigned)mesh->vertexCapacity, mesh->indices, (unsigned)mesh->indexCapacity, s),
                             "bloxel mesher");
        if (!queued || !cuda_ok(cudaMemcpyAsync(host8, m.scratch.total, 3 * sizeof(unsigned), cudaMemcpyDeviceToHost, s), "read back"))
            return false;
    } else {
        const bool queued =
            sparse ? cuda_ok(launch_dmc_sparse_prepare(m.sp, size, upAxisZ != 0, iso, m.dminmax, m.dmc, s), "dual marching cubes mesher") &&
                         needed_values() &&
                         cuda_ok(launch_dmc_sparse_finish(m.sp, size, upAxisZ != 0, px, py, pz, iso, m.dmc, verts,
                                                          (unsigned)mesh->vertexCapacity, mesh->indices, (unsigned)mesh->indexCapacity, s),
                                 "dual marching cubes mesher")
                   : cuda_ok(launch_dmc(m.dens, size, upAxisZ != 0, px, py, pz, iso, m.dminmax, m.dmc, verts,
                                        (unsigned)mesh->vertexCapacity, mesh->indices, (unsigned)mesh->indexCapacity, s),
                             "dual marching cubes mesher");
        if (!queued ||
            !cuda_ok(cudaMemcpyAsync(host8, m.dmc.total, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, s), "read back") ||
            !cuda_ok(cudaMemcpyAsync(host8 + 2, m.dmc.airsolid, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, s), "read back"))
            return false;
    }
    return cuda_ok(cudaMemcpyAsync(host8 + 4, m.dminmax, 2 * sizeof(float), cudaMemcpyDeviceToHost, s), "read back");
}

// Fill a chunk's results from its read-back (after the stream has finished); FN_OK or
// FN_ERR_CAPACITY (counts filled) when its buffers were too small.
int finish_chunk(MeshKind kind, int size, int posY, float iso, const unsigned* host8, fnChunkMesh* mesh)
{
    const unsigned air = kind == kBloxel ? host8[1] : host8[2], solid = kind == kBloxel ? host8[2] : host8[3];
    float minAir = air == 0xFFFFFFFFu ? INFINITY : decode_ordered(air);
    float maxSolid = solid == 0u ? -INFINITY : decode_ordered(solid);
    std::memcpy(mesh->minMax, host8 + 4, 2 * sizeof(float));
    if (mesh->minMax[0] > iso) minAir = (float)posY;                                   // all air (:459-461, :610-613)
    else if (mesh->minMax[1] < iso) maxSolid = (float)posY - 1.0f + (float)size;       // all solid (:463-465, :614-617)
    mesh->minAirY = minAir;
    mesh->maxSolidY = maxSolid;
    const long long nv = kind == kBloxel ? (long long)host8[0] * 4 : (long long)host8[0];
    const long long ni = kind == kBloxel ? (long long)host8[0] * 6 : (long long)host8[1] * 6;
    mesh->vertexCount = nv > INT32_MAX ? INT32_MAX : (int)nv;
    mesh->indexCount = ni > INT32_MAX ? INT32_MAX : (int)ni;
    if (nv > mesh->vertexCapacity || ni > mesh->indexCapacity) {
        set_error(FN_ERR_CAPACITY, "mesh needs " + std::to_string(nv) + " vertices and " + std::to_string(ni) + " indices");
        return FN_ERR_CAPACITY;
    }
    return FN_OK;
}

int build_chunk_mesh(MeshKind kind, const void* node, int size, int px, int py, int pz, int seed, float iso, int upAxisZ,
                     fnChunkMesh* mesh, void* stream)
{
    clear_error();
    if (!node || !mesh_args_ok(size, mesh)) { set_error(FN_ERR_ARG, "invalid arguments"); return FN_ERR_ARG; }
    if (!thread_ctx()) return FN_ERR_CUDA;
    DeviceProgram prog;
    if (!get_program(N(node), 3, prog)) return last_error();
    if (!ensure_runnable(prog)) return FN_ERR_COMPILE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    MeshCtx& m = t_mesh;
    if (!m.reserve(0, 0)) return FN_ERR_CUDA;
    if (!enqueue_chunk(kind, prog, m, s, size, px, py, pz, seed, iso, upAxisZ, mesh, m.host) ||
        !cuda_ok(cudaStreamSynchronize(s), "synchronize"))
        return FN_ERR_CUDA;
    return finish_chunk(kind, size, py, iso, m.host, mesh);
}

// Many chunks: chunk i runs on lane i % kMeshLanes, so the short, latency-bound mesher
// kernels of neighbouring chunks overlap; the caller's stream orders the whole call.
int build_chunk_meshes(MeshKind kind, const void* node, int size, int count, const int* positions, int seed, float iso,
                       int upAxisZ, fnChunkMesh* meshes, void* stream)
{
    clear_error();
    if (!node || count < 0 || (count > 0 && (!positions || !meshes))) { set_error(FN_ERR_ARG, "invalid arguments"); return FN_ERR_ARG; }
    for (int i = 0; i < count; ++i)
        if (!mesh_args_ok(size, meshes + i)) { set_error(FN_ERR_ARG, "invalid mesh " + std::to_string(i)); return FN_ERR_ARG; }
    if (count == 0) return FN_OK;
    if (!thread_ctx()) return FN_ERR_CUDA;
    DeviceProgram prog;
    if (!get_program(N(node), 3, prog)) return last_error();
    if (!ensure_runnable(prog)) return FN_ERR_COMPILE;
    MeshLanes* l = mesh_lanes((size_t)count);
    if (!l) return FN_ERR_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!cuda_ok(cudaEventRecord(l->fork, s), "record")) return FN_ERR_CUDA;
    const int lanes = std::min(count, kMeshLanes);
    for (int k = 0; k < lanes; ++k)
        if (!cuda_ok(cudaStreamWaitEvent(l->stream[k], l->fork, 0), "wait")) return FN_ERR_CUDA;
    for (int i = 0; i < count; ++i) {
        const int k = i % kMeshLanes;
        const int* p = positions + 3 * (size_t)i;
        if (!enqueue_chunk(kind, prog, l->lane[k], l->stream[k], size, p[0], p[1], p[2], seed, iso, upAxisZ, meshes + i,
                           l->host + 8 * (size_t)i))
            return FN_ERR_CUDA;
    }
    for (int k = 0; k < lanes; ++k)
        if (!cuda_ok(cudaEventRecord(l->join[k], l->stream[k]), "record") || !cuda_ok(cudaStreamWaitEvent(s, l->join[k], 0), "wait"))
            return FN_ERR_CUDA;
    if (!cuda_ok(cudaStreamSynchronize(s), "synchronize")) return FN_ERR_CUDA;
    int rc = FN_OK;
    for (int i = 0; i < count; ++i) {
        const int r = finish_chunk(kind, size, positions[3 * (size_t)i + 1], iso, l->host + 8 * (size_t)i, meshes + i);
        if (r != FN_OK && rc == FN_OK) rc = r;
    }
    if (rc != FN_OK) set_error(rc, "at least one chunk's mesh did not fit its buffers (see its counts)");
    return rc;
}

}  // namespace

extern "C" {

int fnSetMeshDensityForm(int form)
{
    if (form != FN_MESH_DENSITY_ARRAY && form != FN_MESH_DENSITY_SPARSE) return FN_ERR_ARG;
    return g_mesh_form.exchange(form);
}

int fnBuildChunkMeshBloxel(const void* node, int size, int posX, int posY, int posZ, int seed, float isoSurface, int upAxisZ,
                           fnChunkMesh* mesh, void* stream)
{
    return build_chunk_mesh(kBloxel, node, size, posX, posY, posZ, seed, isoSurface, upAxisZ, mesh, stream);
}

int fnBuildChunkMeshDmc(const void* node, int size, int posX, int posY, int posZ, int seed, float isoSurface, int upAxisZ,
                        fnChunkMesh* mesh, void* stream)
{
    return build_chunk_mesh(kDmc, node, size, posX, posY, posZ, seed, isoSurface, upAxisZ, mesh, stream);
}

int fnBuildChunkMeshesBloxel(const void* node, int size, int count, const int* positions, int seed, float isoSurface,
                             int upAxisZ, fnChunkMesh* meshes, void* stream)
{
    return build_chunk_meshes(kBloxel, node, size, count, positions, seed, isoSurface, upAxisZ, meshes, stream);
}

int fnBuildChunkMeshesDmc(const void* node, int size, int count, const int* positions, int seed, float isoSurface, int upAxisZ,
                          fnChunkMesh* meshes, void* stream)
{
    return build_chunk_meshes(kDmc, node, size, count, positions, seed, isoSurface, upAxisZ, meshes, stream);
}

int fnBuildChunkMeshHeightmap(const void* node, int size, int posX, int posZ, int seed, float heightMultiplier, fnChunkMesh* mesh,
                              void* stream)
{
    clear_error();
    if (!node || !mesh || size < 1 || size > 8192 || mesh->vertexCapacity < 0 || mesh->indexCapacity < 0) {
        set_error(FN_ERR_ARG, "invalid arguments");
        return FN_ERR_ARG;
    }
    if (!thread_ctx()) return FN_ERR_CUDA;
    DeviceProgram prog;
    if (!get_program(N(node), 2, prog)) return last_error();
    if (!ensure_runnable(prog)) return FN_ERR_COMPILE;
    const int sg = size + 1;
    MeshCtx& m = t_mesh;
    if (!m.reserve((size_t)sg * sg, 0)) return FN_ERR_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    MinMaxWork* work = work_for_stream(s);
    if (!work) return FN_ERR_CUDA;
    // GenPositionArray2D over 0 .. size, offset (pos.x, pos.z) (MeshNoisePreview.cpp:958-962)
    const float off[2] = {(float)posX, (float)posZ};
    const int cnt[2] = {sg, sg};
    const float step[2] = {1, 1};
    if (!cuda_ok(launch_points(prog, grid_args(2, off, cnt, step, seed), m.dens, work, m.dminmax, s), "densities")) return FN_ERR_CUDA;
    if (!cuda_ok(launch_heightmap(m.dens, size, (float)posX, (float)posZ, heightMultiplier, reinterpret_cast<MeshVertex*>(mesh->vertices),
                                  (unsigned)mesh->vertexCapacity, mesh->indices, (unsigned)mesh->indexCapacity, s),
                 "heightmap mesher"))
        return FN_ERR_CUDA;
    if (!cuda_ok(cudaMemcpyAsync(m.host + 4, m.dminmax, 2 * sizeof(float), cudaMemcpyDeviceToHost, s), "read back") ||
        !cuda_ok(cudaStreamSynchronize(s), "synchronize"))
        return FN_ERR_CUDA;
    std::memcpy(mesh->minMax, m.host + 4, 2 * sizeof(float));
    mesh->minAirY = INFINITY;
    mesh->maxSolidY = -INFINITY;
    const long long quads = (long long)size * size;
    mesh->vertexCount = (int)(quads * 4);
    mesh->indexCount = (int)(quads * 6);
    if (mesh->vertexCount > mesh->vertexCapacity || mesh->indexCount > mesh->indexCapacity) {
        set_error(FN_ERR_CAPACITY, "mesh needs " + std::to_string(mesh->vertexCount) + " vertices and " +
                                       std::to_string(mesh->indexCount) + " indices");
        return FN_ERR_CAPACITY;
    }
    return FN_OK;
}

}  // extern "C"
