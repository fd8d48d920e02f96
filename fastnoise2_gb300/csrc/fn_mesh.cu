// fn_mesh.cu -- chunk meshing on the GPU, after the noise.
//
// Restates the Node Editor's chunk meshers (reference
// tools/NodeEditor/MeshNoisePreview.cpp): the bloxel (block) mesher with ambient
// occlusion (BuildBloxel3DMesh :443-540, BloxelAddQuadAO :542-590) and the
// heightmap mesher (BuildHeightMap2DMesh :956-1004).  The density array the
// reference fills with GenPositionArray3D/2D is produced by the tree's own
// generation kernel into a scratch buffer that stays in L2 for editor-size
// chunks; the meshers then run as
//   count  -- faces per voxel (and the min air / max solid heights),
//   scan   -- exclusive prefix sum of the face counts (three small kernels),
//   emit   -- 4 vertices + 6 indices per face at the scanned offset,
// so vertices and indices come out in exactly the reference's sequential order.
// The OutputMinMax early-out (:457-467) skips all voxels when the chunk is all
// air or all solid.
#include <cuda_runtime.h>

#include "fn_mesh.h"

namespace fn {

namespace {

constexpr float kLightX = 0.6f, kLightY = 1.0f, kLightZ = 0.4f;   // MeshNoisePreview.h:158
constexpr float kAmbient = 0.3f;                                   // :159
constexpr float kAoStrength = 0.9f;                                // :160

__device__ __forceinline__ unsigned enc(float f)
{
    const unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

struct Vox {
    const float* d;
    int sx, sy, sz;    // density strides of the mesher's x / y / z axes
};

// BuildBloxel3DMesh's early-out: densities all above (air) or all at/below (solid) the iso level
__device__ __forceinline__ bool early_out(const float* minmax, float iso)
{
    return minmax[0] > iso || minmax[1] < iso;
}

// bit k set = face k (Right, Left, Up, Down, Forward, Back) is emitted
__device__ __forceinline__ unsigned face_mask(const Vox& v, int i, float iso)
{
    if (!(v.d[i] <= iso)) return 0u;
    unsigned m = 0;
    m |= (v.d[i + v.sx] > iso) ? 1u : 0u;
    m |= (v.d[i - v.sx] > iso) ? 2u : 0u;
    m |= (v.d[i + v.sy] > iso) ? 4u : 0u;
    m |= (v.d[i - v.sy] > iso) ? 8u : 0u;
    m |= (v.d[i + v.sz] > iso) ? 16u : 0u;
    m |= (v.d[i - v.sz] > iso) ? 32u : 0u;
    return m;
}

__global__ void bloxel_count(Vox v, int size, float3 pos, float iso, const float* minmax, unsigned* counts,
                             unsigned* airsolid)
{
    const unsigned n = (unsigned)size * size * size;
    const bool skip = early_out(minmax, iso);
    unsigned air = 0xFFFFFFFFu, solid = 0u;        // encoded min air y / max solid y
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int x = t % size, y = (t / size) % size, z = t / ((unsigned)size * size);
        const int i = (x + 1) * v.sx + (y + 1) * v.sy + (z + 1) * v.sz;
        unsigned c = 0;
        if (!skip) {
            const float yf = (float)y + pos.y;
            if (v.d[i] <= iso) {
                c = __popc(face_mask(v, i, iso));
                solid = max(solid, enc(yf));
            } else {
                air = min(air, enc(yf));
            }
        }
        counts[t] = c;
    }
    // one pair of atomics per block: warp shuffles, then the block's warps in shared memory
    __shared__ unsigned s_air[8], s_solid[8];
    for (int o = 16; o > 0; o >>= 1) {
        air = min(air, __shfl_xor_sync(0xffffffffu, air, o));
        solid = max(solid, __shfl_xor_sync(0xffffffffu, solid, o));
    }
    if ((threadIdx.x & 31) == 0) { s_air[threadIdx.x >> 5] = air; s_solid[threadIdx.x >> 5] = solid; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) { air = min(air, s_air[w]); solid = max(solid, s_solid[w]); }
        if (air != 0xFFFFFFFFu) atomicMin(&airsolid[0], air);
        if (solid != 0u) atomicMax(&airsolid[1], solid);
    }
}

// ---- exclusive scan of n uint32 (1024 per block), block totals scanned by one block

constexpr int kScanBlock = 1024;

__device__ __forceinline__ unsigned block_exclusive_scan(unsigned v, unsigned* warp_sums, unsigned& total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned w = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_sums[lane] = w;                       // inclusive over warps
    }
    __syncthreads();
    const unsigned before = warp ? warp_sums[warp - 1] : 0u;
    total = warp_sums[(blockDim.x >> 5) - 1];
    return before + x - v;
}

__global__ void __launch_bounds__(kScanBlock) scan_blocks(const unsigned* in, unsigned* out, unsigned* block_totals, unsigned n)
{
    __shared__ unsigned ws[32];
    const unsigned i = blockIdx.x * kScanBlock + threadIdx.x;
    const unsigned v = i < n ? in[i] : 0u;
    unsigned total;
    const unsigned ex = block_exclusive_scan(v, ws, total);
    if (i < n) out[i] = ex;
    if (threadIdx.x == 0) block_totals[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanBlock) scan_totals(unsigned* totals, unsigned nb, unsigned* grand_total)
{
    __shared__ unsigned ws[32];
    unsigned carry = 0;
    for (unsigned base = 0; base < nb; base += kScanBlock) {
        const unsigned i = base + threadIdx.x;
        const unsigned v = i < nb ? totals[i] : 0u;
        unsigned total;
        const unsigned ex = block_exclusive_scan(v, ws, total);
        if (i < nb) totals[i] = carry + ex;
        carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) *grand_total = carry;
}

__global__ void __launch_bounds__(kScanBlock) scan_add(unsigned* out, const unsigned* totals, unsigned n)
{
    const unsigned i = blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) out[i] += totals[blockIdx.x];
}

// ---- bloxel emit: BloxelAddQuadAO for every face of every solid voxel

struct Quad {
    int facing, oa, ob;
    float light;
    float3 p00, p01, p11, p10;
};

__device__ __forceinline__ void emit_quad(const Vox& v, int i, float iso, const Quad& q, unsigned face, MeshVertex* verts,
                                          unsigned* idx, unsigned vcap, unsigned icap)
{
    const int f = i + q.facing;
    const unsigned sa0 = v.d[f - q.oa] <= iso, sa1 = v.d[f + q.oa] <= iso;
    const unsigned sb0 = v.d[f - q.ob] <= iso, sb1 = v.d[f + q.ob] <= iso;
    const unsigned c00 = (sa0 & sb0) || v.d[f - q.oa - q.ob] <= iso;
    const unsigned c01 = (sa0 & sb1) || v.d[f - q.oa + q.ob] <= iso;
    const unsigned c10 = (sa1 & sb0) || v.d[f + q.oa - q.ob] <= iso;
    const unsigned c11 = (sa1 & sb1) || v.d[f + q.oa + q.ob] <= iso;
    constexpr float aoAdjust = kAoStrength / 3.0f;
    const float ao00 = (float)(sa0 + sb0 + c00) * aoAdjust;
    const float ao01 = (float)(sa1 + sb0 + c10) * aoAdjust;
    const float ao10 = (float)(sa0 + sb1 + c01) * aoAdjust;
    const float ao11 = (float)(sa1 + sb1 + c11) * aoAdjust;
    float light = q.light - (iso - v.d[i]) * 4.0f;
    light = light * fabsf(light);
    light = kAmbient < light ? light : kAmbient;              // std::max(AMBIENT_LIGHT, light)
    const unsigned base = face * 4u;
    if (base + 3u < vcap) {
        verts[base + 0] = MeshVertex{q.p00.x, q.p00.y, q.p00.z, (1.0f - ao00) * light};
        verts[base + 1] = MeshVertex{q.p01.x, q.p01.y, q.p01.z, (1.0f - ao01) * light};
        verts[base + 2] = MeshVertex{q.p10.x, q.p10.y, q.p10.z, (1.0f - ao10) * light};
        verts[base + 3] = MeshVertex{q.p11.x, q.p11.y, q.p11.z, (1.0f - ao11) * light};
    }
    const unsigned rot = (ao00 + ao11 > ao01 + ao10) ? 2u : 0u;
    const unsigned k = face * 6u;
    if (k + 5u < icap) {
        idx[k + 0] = base;
        idx[k + 1] = base + 3u - rot;
        idx[k + 2] = base + 2u;
        idx[k + 3] = base + 3u;
        idx[k + 4] = base + rot;
        idx[k + 5] = base + 1u;
    }
}

__global__ void bloxel_emit(Vox v, int size, float3 pos, float iso, const float* minmax, const unsigned* offsets,
                            MeshVertex* verts, unsigned* idx, unsigned vcap, unsigned icap)
{
    if (early_out(minmax, iso)) return;
    const unsigned n = (unsigned)size * size * size;
    constexpr float sunX = kLightX * (1.0f - kAmbient), sunY = kLightY * (1.0f - kAmbient), sunZ = kLightZ * (1.0f - kAmbient);
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int x = t % size, y = (t / size) % size, z = t / ((unsigned)size * size);
        const int i = (x + 1) * v.sx + (y + 1) * v.sy + (z + 1) * v.sz;
        const unsigned m = face_mask(v, i, iso);
        if (!m) continue;
        const float xf = (float)x + pos.x, yf = (float)y + pos.y, zf = (float)z + pos.z;
        const float x1 = xf + 1.0f, y1 = yf + 1.0f, z1 = zf + 1.0f;
        unsigned face = offsets[t];
        if (m & 1u) emit_quad(v, i, iso, Quad{v.sx, v.sy, v.sz, sunX + kAmbient, {x1, yf, zf}, {x1, y1, zf}, {x1, y1, z1}, {x1, yf, z1}},
                              face++, verts, idx, vcap, icap);
        if (m & 2u) emit_quad(v, i, iso, Quad{-v.sx, -v.sy, v.sz, 1.0f - sunX, {xf, y1, zf}, {xf, yf, zf}, {xf, yf, z1}, {xf, y1, z1}},
                              face++, verts, idx, vcap, icap);
        if (m & 4u) emit_quad(v, i, iso, Quad{v.sy, v.sz, v.sx, sunY + kAmbient, {xf, y1, zf}, {xf, y1, z1}, {x1, y1, z1}, {x1, y1, zf}},
                              face++, verts, idx, vcap, icap);
        if (m & 8u) emit_quad(v, i, iso, Quad{-v.sy, -v.sz, v.sx, 1.0f - sunY, {xf, yf, z1}, {xf, yf, zf}, {x1, yf, zf}, {x1, yf, z1}},
                              face++, verts, idx, vcap, icap);
        if (m & 16u) emit_quad(v, i, iso, Quad{v.sz, v.sx, v.sy, sunZ + kAmbient, {xf, yf, z1}, {x1, yf, z1}, {x1, y1, z1}, {xf, y1, z1}},
                               face++, verts, idx, vcap, icap);
        if (m & 32u) emit_quad(v, i, iso, Quad{-v.sz, -v.sx, v.sy, 1.0f - sunZ, {x1, yf, zf}, {xf, yf, zf}, {xf, y1, zf}, {x1, y1, zf}},
                               face++, verts, idx, vcap, icap);
    }
}

// ---- heightmap: every quad emits 4 vertices and 6 indices (Magnum vector forms restated)

__device__ __forceinline__ float3 sub3(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 add3(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float dot3(float3 a, float3 b)
{
    float acc = 0.0f;
    acc = acc + a.x * b.x;
    acc = acc + a.y * b.y;
    acc = acc + a.z * b.z;
    return acc;
}
__device__ __forceinline__ float3 cross3(float3 a, float3 b)
{
    return make_float3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
__device__ __forceinline__ float3 normalized3(float3 v)
{
    const float inv = 1.0f / sqrtf(dot3(v, v));
    return make_float3(v.x * inv, v.y * inv, v.z * inv);
}

__global__ void heightmap_emit(const float* d, int size, float2 pos, float mul, MeshVertex* verts, unsigned* idx, unsigned vcap,
                               unsigned icap)
{
    const unsigned n = (unsigned)size * size;
    const int sg = size + 1;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int x = t % size, y = t / size;
        const int i = y * sg + x;
        const float xf = (float)x + pos.x, yf = (float)y + pos.y;
        const float x1 = xf + 1.0f, y1 = yf + 1.0f;
        const float3 v00 = make_float3(xf, d[i] * mul, yf);
        const float3 v01 = make_float3(xf, d[i + sg] * mul, y1);
        const float3 v10 = make_float3(x1, d[i + 1] * mul, yf);
        const float3 v11 = make_float3(x1, d[i + 1 + sg] * mul, y1);
        const float3 nrm = normalized3(add3(normalized3(cross3(sub3(v10, v11), sub3(v00, v11))),
                                            normalized3(cross3(sub3(v01, v00), sub3(v11, v00)))));
        const float3 ln = make_float3(kLightX * nrm.x, kLightY * nrm.y, kLightZ * nrm.z);
        const float light = dot3(ln, ln);
        const unsigned base = t * 4u;
        if (base + 3u < vcap) {
            verts[base + 0] = MeshVertex{v00.x, v00.y, v00.z, light};
            verts[base + 1] = MeshVertex{v01.x, v01.y, v01.z, light};
            verts[base + 2] = MeshVertex{v10.x, v10.y, v10.z, light};
            verts[base + 3] = MeshVertex{v11.x, v11.y, v11.z, light};
        }
        const float3 s0 = add3(v00, v11), s1 = add3(v01, v10);
        const unsigned rot = dot3(s0, s0) < dot3(s1, s1) ? 2u : 0u;
        const unsigned k = t * 6u;
        if (k + 5u < icap) {
            idx[k + 0] = base;
            idx[k + 1] = base + 3u - rot;
            idx[k + 2] = base + 2u;
            idx[k + 3] = base + 3u;
            idx[k + 4] = base + rot;
            idx[k + 5] = base + 1u;
        }
    }
}

// Grid-stride launches: one thread per element up to 8 waves of 256-thread blocks per SM.
int grid_for(unsigned n, int block)
{
    static int cap = 0;
    if (!cap) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cap = (sms > 0 ? sms : 1) * 8;
    }
    long long g = ((long long)n + block - 1) / block;
    return (int)(g < 1 ? 1 : g > cap ? cap : g);
}

}  // namespace

cudaError_t launch_bloxel(const float* dens, int size, bool up_axis_z, float px, float py, float pz, float iso, const float* dminmax,
                          MeshScratch& s, MeshVertex* verts, unsigned vcap, unsigned* idx, unsigned icap, cudaStream_t stream)
{
    const int sg = size + 2;
    Vox v{dens, 1, up_axis_z ? sg * sg : sg, up_axis_z ? sg : sg * sg};
    const unsigned n = (unsigned)size * size * size;
    const unsigned nb = (n + kScanBlock - 1) / kScanBlock;
    cudaError_t e = cudaMemsetAsync(s.airsolid, 0, 2 * sizeof(unsigned), stream);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(s.airsolid, 0xFF, sizeof(unsigned), stream);           // min air starts at "none"
    if (e != cudaSuccess) return e;
    const float3 pos = make_float3(px, py, pz);
    bloxel_count<<<grid_for(n, 256), 256, 0, stream>>>(v, size, pos, iso, dminmax, s.counts, s.airsolid);
    scan_blocks<<<nb, kScanBlock, 0, stream>>>(s.counts, s.offsets, s.block_totals, n);
    scan_totals<<<1, kScanBlock, 0, stream>>>(s.block_totals, nb, s.total);
    scan_add<<<nb, kScanBlock, 0, stream>>>(s.offsets, s.block_totals, n);
    bloxel_emit<<<grid_for(n, 256), 256, 0, stream>>>(v, size, pos, iso, dminmax, s.offsets, verts, idx, vcap, icap);
    return cudaGetLastError();
}

cudaError_t launch_heightmap(const float* dens, int size, float px, float pz, float mul, MeshVertex* verts, unsigned vcap,
                             unsigned* idx, unsigned icap, cudaStream_t stream)
{
    const unsigned n = (unsigned)size * size;
    heightmap_emit<<<grid_for(n, 256), 256, 0, stream>>>(dens, size, make_float2(px, pz), mul, verts, idx, vcap, icap);
    return cudaGetLastError();
}

}  // namespace fn
