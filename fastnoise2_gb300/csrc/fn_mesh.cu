// fn_mesh.cu -- chunk meshing on the GPU, after the noise.
//
// Restates the Node Editor's chunk meshers (reference
// tools/NodeEditor/MeshNoisePreview.cpp): the bloxel (block) mesher with ambient
// occlusion (BuildBloxel3DMesh :443-540, BloxelAddQuadAO :542-590) and the
// heightmap mesher (BuildHeightMap2DMesh :956-1004), and the dual marching cubes
// mesher (BuildDmc3DMesh :592-769, DmcGetVertIndex :771-953).  The density array the
// reference fills with GenPositionArray3D/2D is produced by the tree's own
// generation kernel into a scratch buffer that stays in L2 for editor-size
// chunks; the meshers then run as
//   count  -- faces per voxel (and the min air / max solid heights),
//   scan   -- exclusive prefix sum of the face counts (three small kernels),
//   emit   -- 4 vertices + 6 indices per face at the scanned offset,
// so vertices and indices come out in exactly the reference's sequential order.
// The OutputMinMax early-out (:457-467) skips all voxels when the chunk is all
// air or all solid.  Dual marching cubes shares a vertex between the quads of up
// to twelve cut edges, numbered in the order the reference's hash map first sees
// it; here every reference to a vertex finds its first use directly (the lowest
// cell / axis / slot among the quads that use it), so the count pass marks the
// creating references, a scan numbers them, and the quads look their vertices up
// without a map.
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

// Where a mesher reads the chunk's densities.  DenseSrc: the density array.  SparseSrc: no
// density array -- two classification bitmasks of every density (computed where the tree is
// evaluated) and exact values only at the voxels a pass needs them (marked in `need`, stored
// in index order; `rank` = values stored before each 32-bit word of `need`).  NaN densities are
// neither above nor at-or-below the iso level in both forms.
struct DenseSrc {
    const float* d;
    __device__ __forceinline__ bool above(int i, float iso) const { return d[i] > iso; }
    __device__ __forceinline__ bool solid(int i, float iso) const { return d[i] <= iso; }
    __device__ __forceinline__ float value(int i) const { return d[i]; }
};

struct SparseSrc {
    const unsigned* gt;      // bit i: density i > iso
    const unsigned* le;      // bit i: density i <= iso
    const uint2* stored;     // per 32 densities: (values stored before them, bit k: density 32w + k is stored)
    const float* vals;
    __device__ __forceinline__ bool above(int i, float) const { return (__ldg(&gt[i >> 5]) >> (i & 31)) & 1u; }
    __device__ __forceinline__ bool solid(int i, float) const { return (__ldg(&le[i >> 5]) >> (i & 31)) & 1u; }
    __device__ __forceinline__ float value(int i) const
    {
        const uint2 w = stored[(unsigned)i >> 5];
        return vals[w.x + __popc(w.y & ((1u << (i & 31)) - 1u))];
    }
};

template <class S>
struct Vox {
    S src;
    int sx, sy, sz;    // density strides of the mesher's x / y / z axes
};

// BuildBloxel3DMesh's early-out: densities all above (air) or all at/below (solid) the iso level
__device__ __forceinline__ bool early_out(const float* minmax, float iso)
{
    return minmax[0] > iso || minmax[1] < iso;
}

// bit k set = face k (Right, Left, Up, Down, Forward, Back) is emitted
template <class S>
__device__ __forceinline__ unsigned face_mask(const Vox<S>& v, int i, float iso)
{
    if (!v.src.solid(i, iso)) return 0u;
    unsigned m = 0;
    m |= v.src.above(i + v.sx, iso) ? 1u : 0u;
    m |= v.src.above(i - v.sx, iso) ? 2u : 0u;
    m |= v.src.above(i + v.sy, iso) ? 4u : 0u;
    m |= v.src.above(i - v.sy, iso) ? 8u : 0u;
    m |= v.src.above(i + v.sz, iso) ? 16u : 0u;
    m |= v.src.above(i - v.sz, iso) ? 32u : 0u;
    return m;
}

// Faces per voxel and the min air / max solid heights.  `need` (sparse form, else null):
// every voxel with a face is marked, since emitting its faces reads its density.
template <class S>
__global__ void bloxel_count(Vox<S> v, int size, float3 pos, float iso, const float* minmax, unsigned* counts,
                             unsigned* airsolid, unsigned* need)
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
            if (v.src.solid(i, iso)) {
                c = __popc(face_mask(v, i, iso));
                solid = max(solid, enc(yf));
                if (c && need) atomicOr(&need[i >> 5], 1u << (i & 31));
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

// ---- exclusive scan of n counts (1024 per block), block totals scanned by one block.
// T = unsigned (bloxel faces) or uint2 (dual marching cubes: vertices, quads).

__device__ __forceinline__ unsigned shfl_up(unsigned v, int o) { return __shfl_up_sync(0xffffffffu, v, o); }
__device__ __forceinline__ uint2 shfl_up(uint2 v, int o)
{
    return make_uint2(__shfl_up_sync(0xffffffffu, v.x, o), __shfl_up_sync(0xffffffffu, v.y, o));
}
__device__ __forceinline__ unsigned plus(unsigned a, unsigned b) { return a + b; }
__device__ __forceinline__ uint2 plus(uint2 a, uint2 b) { return make_uint2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ unsigned minus(unsigned a, unsigned b) { return a - b; }
__device__ __forceinline__ uint2 minus(uint2 a, uint2 b) { return make_uint2(a.x - b.x, a.y - b.y); }
template <class T> __device__ __forceinline__ T zero() { return T{}; }

constexpr int kScanBlock = 1024;

template <class T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* warp_sums, T& total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const T y = shfl_up(x, o);
        if (lane >= o) x = plus(x, y);
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        T w = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : zero<T>();
        for (int o = 1; o < 32; o <<= 1) {
            const T y = shfl_up(w, o);
            if (lane >= o) w = plus(w, y);
        }
        warp_sums[lane] = w;                       // inclusive over warps
    }
    __syncthreads();
    const T before = warp ? warp_sums[warp - 1] : zero<T>();
    total = warp_sums[(blockDim.x >> 5) - 1];
    return plus(before, minus(x, v));
}

template <class T>
__global__ void __launch_bounds__(kScanBlock) scan_blocks(const T* in, T* out, T* block_totals, unsigned n)
{
    __shared__ T ws[32];
    const unsigned i = blockIdx.x * kScanBlock + threadIdx.x;
    const T v = i < n ? in[i] : zero<T>();
    T total;
    const T ex = block_exclusive_scan(v, ws, total);
    if (i < n) out[i] = ex;
    if (threadIdx.x == 0) block_totals[blockIdx.x] = total;
}

template <class T>
__global__ void __launch_bounds__(kScanBlock) scan_totals(T* totals, unsigned nb, T* grand_total)
{
    __shared__ T ws[32];
    T carry = zero<T>();
    for (unsigned base = 0; base < nb; base += kScanBlock) {
        const unsigned i = base + threadIdx.x;
        const T v = i < nb ? totals[i] : zero<T>();
        T total;
        const T ex = block_exclusive_scan(v, ws, total);
        if (i < nb) totals[i] = plus(carry, ex);
        carry = plus(carry, total);
        __syncthreads();
    }
    if (threadIdx.x == 0) *grand_total = carry;
}

template <class T>
__global__ void __launch_bounds__(kScanBlock) scan_add(T* out, const T* totals, unsigned n)
{
    const unsigned i = blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) out[i] = plus(out[i], totals[blockIdx.x]);
}

// Exclusive scan of n counts into `out`; the grand total lands in `total`.
template <class T>
void exclusive_scan(const T* in, T* out, T* block_totals, T* total, unsigned n, cudaStream_t stream)
{
    const unsigned nb = (n + kScanBlock - 1) / kScanBlock;
    scan_blocks<T><<<nb, kScanBlock, 0, stream>>>(in, out, block_totals, n);
    scan_totals<T><<<1, kScanBlock, 0, stream>>>(block_totals, nb, total);
    scan_add<T><<<nb, kScanBlock, 0, stream>>>(out, block_totals, n);
}

// ---- bloxel emit: BloxelAddQuadAO for every face of every solid voxel

struct Quad {
    int facing, oa, ob;
    float light;
    float3 p00, p01, p11, p10;
};

template <class S>
__device__ __forceinline__ void emit_quad(const Vox<S>& v, int i, float iso, float density, const Quad& q, unsigned face,
                                          MeshVertex* verts, unsigned* idx, unsigned vcap, unsigned icap)
{
    const int f = i + q.facing;
    const unsigned sa0 = v.src.solid(f - q.oa, iso), sa1 = v.src.solid(f + q.oa, iso);
    const unsigned sb0 = v.src.solid(f - q.ob, iso), sb1 = v.src.solid(f + q.ob, iso);
    const unsigned c00 = (sa0 & sb0) || v.src.solid(f - q.oa - q.ob, iso);
    const unsigned c01 = (sa0 & sb1) || v.src.solid(f - q.oa + q.ob, iso);
    const unsigned c10 = (sa1 & sb0) || v.src.solid(f + q.oa - q.ob, iso);
    const unsigned c11 = (sa1 & sb1) || v.src.solid(f + q.oa + q.ob, iso);
    constexpr float aoAdjust = kAoStrength / 3.0f;
    const float ao00 = (float)(sa0 + sb0 + c00) * aoAdjust;
    const float ao01 = (float)(sa1 + sb0 + c10) * aoAdjust;
    const float ao10 = (float)(sa0 + sb1 + c01) * aoAdjust;
    const float ao11 = (float)(sa1 + sb1 + c11) * aoAdjust;
    float light = q.light - (iso - density) * 4.0f;
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

template <class S>
__global__ void bloxel_emit(Vox<S> v, int size, float3 pos, float iso, const float* minmax, const unsigned* offsets,
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
        const float dens = v.src.value(i);
        unsigned face = offsets[t];
        if (m & 1u) emit_quad(v, i, iso, dens, Quad{v.sx, v.sy, v.sz, sunX + kAmbient, {x1, yf, zf}, {x1, y1, zf}, {x1, y1, z1}, {x1, yf, z1}},
                              face++, verts, idx, vcap, icap);
        if (m & 2u) emit_quad(v, i, iso, dens, Quad{-v.sx, -v.sy, v.sz, 1.0f - sunX, {xf, y1, zf}, {xf, yf, zf}, {xf, yf, z1}, {xf, y1, z1}},
                              face++, verts, idx, vcap, icap);
        if (m & 4u) emit_quad(v, i, iso, dens, Quad{v.sy, v.sz, v.sx, sunY + kAmbient, {xf, y1, zf}, {xf, y1, z1}, {x1, y1, z1}, {x1, y1, zf}},
                              face++, verts, idx, vcap, icap);
        if (m & 8u) emit_quad(v, i, iso, dens, Quad{-v.sy, -v.sz, v.sx, 1.0f - sunY, {xf, yf, z1}, {xf, yf, zf}, {x1, yf, zf}, {x1, yf, z1}},
                              face++, verts, idx, vcap, icap);
        if (m & 16u) emit_quad(v, i, iso, dens, Quad{v.sz, v.sx, v.sy, sunZ + kAmbient, {xf, yf, z1}, {x1, yf, z1}, {x1, y1, z1}, {xf, y1, z1}},
                               face++, verts, idx, vcap, icap);
        if (m & 32u) emit_quad(v, i, iso, dens, Quad{-v.sz, -v.sx, v.sy, 1.0f - sunZ, {x1, yf, zf}, {xf, yf, zf}, {xf, y1, zf}, {x1, y1, zf}},
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

// ---- dual marching cubes (BuildDmc3DMesh :592-769, DmcGetVertIndex :771-953)
//
// Cell corners are numbered x + 2y + 4z; edge k joins kDmcEdgeCorner[k].  A
// marching-cubes case (bit k = corner k above the iso level) has one dual point
// per connected piece of its surface; each piece is the set of cut edges that
// the face contours join.  On a face with two cut edges they are joined; on an
// ambiguous face (diagonal corners, four cut edges) each corner above the iso
// level is cut off on its own.  The table is derived here at compile time from
// that rule; it equals the reference's kDualPointsList (DmcTable.inl) case for
// case, piece order aside (the mesher only asks which piece holds an edge).
//
// Quads: the edge of axis a (x, y, z) from a cell's base corner is cut; its four
// dual vertices sit in cells base + dmc_slot_off(a, s, .), on edge dmc_slot_edge(a, s)
// (slot s = 0..3; slot bit 0 steps back along axis (a + 2) % 3, bit 1 along (a + 1) % 3).
// The reference numbers a vertex when its first quad (cell-major, then axis, then
// slot) asks for it; `dmc_first_use` finds that quad from the vertex's side.

__host__ __device__ constexpr int dmc_slot_off(int a, int s, int k)
{
    return -((k == (a + 2) % 3 ? (s & 1) : 0) + (k == (a + 1) % 3 ? (s >> 1) & 1 : 0));
}
__host__ __device__ constexpr int dmc_slot_edge(int a, int s)
{
    constexpr int t[3][4] = {{0, 2, 4, 6}, {8, 9, 11, 10}, {3, 7, 1, 5}};
    return t[a][s];
}
// Inverse: edge e of a vertex cell is used by the quad of cell + dmc_use_off(e, .),
// at slot dmc_use_slot(e) = axis * 4 + slot.
__host__ __device__ constexpr int dmc_use_off(int e, int k)
{
    for (int a = 0; a < 3; ++a)
        for (int s = 0; s < 4; ++s)
            if (dmc_slot_edge(a, s) == e) return -dmc_slot_off(a, s, k);
    return 0;
}
__host__ __device__ constexpr int dmc_use_slot(int e)
{
    for (int a = 0; a < 3; ++a)
        for (int s = 0; s < 4; ++s)
            if (dmc_slot_edge(a, s) == e) return a * 4 + s;
    return 0;
}
// Order of edge e's quad among the quads around one vertex cell when all of them lie
// inside the chunk: cell-major (z, y, x of the using cell), then slot.
__host__ __device__ constexpr int dmc_use_rank(int e)
{
    return ((dmc_use_off(e, 2) * 2 + dmc_use_off(e, 1)) * 2 + dmc_use_off(e, 0)) * 12 + dmc_use_slot(e);
}

struct DmcTable {
    unsigned long long edge_piece[256];   // 4 bits per edge: its piece, 0xF = edge not cut
    unsigned short code[256][4];          // cut-edge bit set of each piece
    unsigned char first[256][4];          // each piece's edge whose quad comes first (all quads in the chunk)
};

constexpr int kDmcEdgeCorner[12][2] = {{0, 1}, {1, 5}, {4, 5}, {0, 4}, {2, 3}, {3, 7},
                                       {6, 7}, {2, 6}, {0, 2}, {1, 3}, {5, 7}, {4, 6}};
// the six faces: corners in cyclic order, edge k joins corner k and corner k+1
constexpr int kDmcFaceCorner[6][4] = {{0, 2, 6, 4}, {1, 3, 7, 5}, {0, 1, 5, 4}, {2, 3, 7, 6}, {0, 1, 3, 2}, {4, 5, 7, 6}};
constexpr int kDmcFaceEdge[6][4] = {{8, 7, 11, 3}, {9, 5, 10, 1}, {0, 1, 2, 3}, {4, 5, 6, 7}, {0, 9, 4, 8}, {2, 10, 6, 11}};

constexpr int dmc_root(const int* label, int e)
{
    while (label[e] != e) e = label[e];
    return e;
}

constexpr DmcTable make_dmc_table()
{
    DmcTable t{};
    for (int c = 0; c < 256; ++c) {
        int label[12] = {};
        bool cut[12] = {};
        for (int e = 0; e < 12; ++e) {
            label[e] = e;
            cut[e] = ((c >> kDmcEdgeCorner[e][0]) & 1) != ((c >> kDmcEdgeCorner[e][1]) & 1);
        }
        for (int f = 0; f < 6; ++f) {
            int n = 0, first = -1, last = -1;
            for (int k = 0; k < 4; ++k) {
                const int e = kDmcFaceEdge[f][k];
                if (!cut[e]) continue;
                ++n;
                if (first < 0) first = e;
                last = e;
            }
            int pairs[2][2] = {{-1, -1}, {-1, -1}};
            int np = 0;
            if (n == 2) {
                pairs[np][0] = first; pairs[np][1] = last; ++np;
            } else if (n == 4) {
                for (int k = 0; k < 4; ++k)
                    if ((c >> kDmcFaceCorner[f][k]) & 1) { pairs[np][0] = kDmcFaceEdge[f][(k + 3) & 3]; pairs[np][1] = kDmcFaceEdge[f][k]; ++np; }
            }
            for (int p = 0; p < np; ++p) {
                const int ra = dmc_root(label, pairs[p][0]), rb = dmc_root(label, pairs[p][1]);
                if (ra < rb) label[rb] = ra; else label[ra] = rb;
            }
        }
        int piece_of_root[12] = {};
        for (int e = 0; e < 12; ++e) piece_of_root[e] = -1;
        int pieces = 0;
        unsigned long long ep = ~0ull;
        for (int e = 0; e < 12; ++e) {
            if (!cut[e]) continue;
            const int r = dmc_root(label, e);
            if (piece_of_root[r] < 0) piece_of_root[r] = pieces++;
            const int p = piece_of_root[r];
            ep &= ~(0xFull << (4 * e));
            ep |= (unsigned long long)p << (4 * e);
            t.code[c][p] = (unsigned short)(t.code[c][p] | (1u << e));
            if (t.code[c][p] == (1u << e) || dmc_use_rank(e) < dmc_use_rank(t.first[c][p])) t.first[c][p] = (unsigned char)e;
        }
        t.edge_piece[c] = ep;
    }
    return t;
}

__device__ const DmcTable kDmc = make_dmc_table();

// The slot tables packed into integers for run-time lookup: 4 bits per slot for the
// slot edges, 4 bits per edge for the use slot, 3 bits (x, y, z) per edge for the use offset.
constexpr unsigned long long pack_slot_edges()
{
    unsigned long long v = 0;
    for (int b = 0; b < 12; ++b) v |= (unsigned long long)dmc_slot_edge(b / 4, b % 4) << (4 * b);
    return v;
}
constexpr unsigned long long pack_use_slots()
{
    unsigned long long v = 0;
    for (int e = 0; e < 12; ++e) v |= (unsigned long long)dmc_use_slot(e) << (4 * e);
    return v;
}
constexpr unsigned long long pack_use_offs()
{
    unsigned long long v = 0;
    for (int e = 0; e < 12; ++e)
        v |= (unsigned long long)(dmc_use_off(e, 0) | dmc_use_off(e, 1) << 1 | dmc_use_off(e, 2) << 2) << (3 * e);
    return v;
}
constexpr unsigned long long kDmcSlotEdges = pack_slot_edges();
constexpr unsigned long long kDmcUseSlots = pack_use_slots();
constexpr unsigned long long kDmcUseOffs = pack_use_offs();
static_assert(dmc_use_slot(1) == 10 && dmc_use_off(10, 0) == 1 && dmc_use_off(10, 2) == 1 && dmc_use_off(6, 1) == 1,
              "quad slot tables");
static_assert(make_dmc_table().first[1][0] == 0 && make_dmc_table().first[255 - 64][0] == 7, "first-use edges");

template <class S>
struct DmcGrid {
    S src;                        // the densities (DenseSrc or SparseSrc)
    int sx, sy, sz;               // density strides of the mesher's x / y / z axes
    int size;                     // cells per axis
    unsigned char* cases;         // marching-cubes case of each vertex cell, (size + 1)^3, from -1
};

template <class S>
__device__ __forceinline__ int dmc_index(const DmcGrid<S>& g, int x, int y, int z)
{
    return (x + 2) * g.sx + (y + 2) * g.sy + (z + 2) * g.sz;
}

template <class S>
__device__ __forceinline__ unsigned dmc_case_at(const DmcGrid<S>& g, int x, int y, int z)
{
    const unsigned s1 = (unsigned)g.size + 1u;
    return g.cases[((unsigned)(z + 1) * s1 + (unsigned)(y + 1)) * s1 + (unsigned)(x + 1)];
}

// DmcGetVertIndex's cell code (:774-790)
template <class S>
__device__ __forceinline__ unsigned dmc_case(const DmcGrid<S>& g, int i, float iso)
{
    unsigned c = 0;
    c |= g.src.above(i, iso) ? 1u : 0u;
    c |= g.src.above(i + g.sx, iso) ? 2u : 0u;
    c |= g.src.above(i + g.sy, iso) ? 4u : 0u;
    c |= g.src.above(i + g.sx + g.sy, iso) ? 8u : 0u;
    c |= g.src.above(i + g.sz, iso) ? 16u : 0u;
    c |= g.src.above(i + g.sx + g.sz, iso) ? 32u : 0u;
    c |= g.src.above(i + g.sy + g.sz, iso) ? 64u : 0u;
    c |= g.src.above(i + g.sx + g.sy + g.sz, iso) ? 128u : 0u;
    return c;
}

// cut edges from a cell's base corner: bit 0 x (corners 0-1), bit 1 y (0-2), bit 2 z (0-4)
__device__ __forceinline__ unsigned dmc_axes(unsigned c)
{
    return ((c ^ (c >> 1)) & 1u) | (((c ^ (c >> 2)) & 1u) << 1) | (((c ^ (c >> 4)) & 1u) << 2);
}

__device__ __forceinline__ int dmc_slot_offset(int a, int s, int k)
{
    return -((k == (a + 2) % 3 ? (s & 1) : 0) + (k == (a + 1) % 3 ? (s >> 1) & 1 : 0));
}

template <class S>
__device__ __forceinline__ unsigned dmc_key(const DmcGrid<S>& g, unsigned cx, unsigned cy, unsigned cz, unsigned slot)
{
    const unsigned n = (unsigned)g.size;
    return ((cz * n + cy) * n + cx) * 12u + slot;
}

// The first quad (in the reference's cell / axis / slot order) that uses the dual vertex
// (cell w, piece p of case c), as cell index * 12 + axis * 4 + slot: that quad's
// DmcGetVertIndex call is the one that creates the vertex in the reference's map.  Away
// from the chunk's faces every quad around w lies in the chunk and the table knows the
// first; next to them the quads that fall outside are skipped.
template <class S>
__device__ __forceinline__ unsigned dmc_first_use(const DmcGrid<S>& g, int wx, int wy, int wz, unsigned c, unsigned p)
{
    const unsigned n = (unsigned)g.size;
    if ((unsigned)wx < n - 1u && (unsigned)wy < n - 1u && (unsigned)wz < n - 1u) {
        const int e = __ldg(&kDmc.first[c][p]);
        const unsigned off = (unsigned)(kDmcUseOffs >> (3 * e)) & 7u;
        return dmc_key(g, (unsigned)wx + (off & 1u), (unsigned)wy + ((off >> 1) & 1u), (unsigned)wz + (off >> 2),
                       (unsigned)(kDmcUseSlots >> (4 * e)) & 0xFu);
    }
    unsigned best = 0xFFFFFFFFu;
    for (unsigned m = __ldg(&kDmc.code[c][p]); m; m &= m - 1u) {
        const int e = __ffs(m) - 1;
        const unsigned off = (unsigned)(kDmcUseOffs >> (3 * e)) & 7u;
        const unsigned cx = (unsigned)(wx + (int)(off & 1u)), cy = (unsigned)(wy + (int)((off >> 1) & 1u)),
                       cz = (unsigned)(wz + (int)(off >> 2));
        if (cx >= n || cy >= n || cz >= n) continue;                // also catches -1
        const unsigned key = dmc_key(g, cx, cy, cz, (unsigned)(kDmcUseSlots >> (4 * e)) & 0xFu);
        best = key < best ? key : best;
    }
    return best;
}

// One quad reference: vertex cell w of slot (a, s) of cell (x, y, z), its case and piece.
struct DmcRef {
    int wx, wy, wz;
    unsigned c, p;
};

template <class S>
__device__ __forceinline__ DmcRef dmc_ref(const DmcGrid<S>& g, int x, int y, int z, int a, int s)
{
    DmcRef r;
    r.wx = x + dmc_slot_offset(a, s, 0);
    r.wy = y + dmc_slot_offset(a, s, 1);
    r.wz = z + dmc_slot_offset(a, s, 2);
    r.c = dmc_case_at(g, r.wx, r.wy, r.wz);
    const int e = (int)((kDmcSlotEdges >> (4 * (a * 4 + s))) & 0xFu);
    r.p = (unsigned)(__ldg(&kDmc.edge_piece[r.c]) >> (4 * e)) & 0xFu;    // the piece holding e (:792-800)
    return r;
}

// mean of the piece's edge crossings, relative to the cell's base corner (:810-890)
template <class S>
__device__ __forceinline__ float3 dmc_point(const DmcGrid<S>& g, int i, unsigned code, float iso)
{
    const int X = g.sx, Y = g.sy, Z = g.sz;
    auto t = [&](int a, int b) {
        const float da = g.src.value(a);
        return (iso - da) / (g.src.value(b) - da);
    };
    float x = 0.0f, y = 0.0f, z = 0.0f;
    if (code & 1u) x += t(i, i + X);
    if (code & 2u) { x += 1.0f; z += t(i + X, i + X + Z); }
    if (code & 4u) { x += t(i + Z, i + X + Z); z += 1.0f; }
    if (code & 8u) z += t(i, i + Z);
    if (code & 16u) { x += t(i + Y, i + X + Y); y += 1.0f; }
    if (code & 32u) { x += 1.0f; y += 1.0f; z += t(i + X + Y, i + X + Y + Z); }
    if (code & 64u) { x += t(i + Y + Z, i + X + Y + Z); y += 1.0f; z += 1.0f; }
    if (code & 128u) { y += 1.0f; z += t(i + Y, i + Y + Z); }
    if (code & 256u) y += t(i, i + Y);
    if (code & 512u) { x += 1.0f; y += t(i + X, i + X + Y); }
    if (code & 1024u) { x += 1.0f; y += t(i + X + Z, i + X + Y + Z); z += 1.0f; }
    if (code & 2048u) { y += t(i + Z, i + Y + Z); z += 1.0f; }
    const float n = (float)__popc(code);
    return make_float3(x / n, y / n, z / n);
}

// NormaliseConstExpr(-LIGHT_DIR) (:21-30): Newton square root until it repeats
__device__ __forceinline__ float3 dmc_light_dir()
{
    const float x = -kLightX, y = -kLightY, z = -kLightZ;
    const float len2 = x * x + y * y + z * z;
    float curr = len2, prev = 0.0f;
    for (int k = 0; k < 64 && curr != prev; ++k) {
        const float next = 0.5f * (curr + len2 / curr);
        prev = curr;
        curr = next;
    }
    return make_float3(x / curr, y / curr, z / curr);
}

// One coordinate of the vertex offset DmcGetVertIndex receives: the float of the
// quad's cell coordinate, minus 1 when the vertex cell lies one step back.
__device__ __forceinline__ float dmc_offset(int pos, int cell, int vcell)
{
    const float f = (float)(pos + cell);
    return vcell != cell ? f - 1.0f : f;
}

__device__ __forceinline__ float lerp_(float a, float b, float t) { return a + (b - a) * t; }   // ImLerp

// the vertex light: trilinear central-difference gradient at the point (:902-948)
template <class S>
__device__ __forceinline__ float dmc_light(const DmcGrid<S>& g, int i, float3 v, float3 nl)
{
    auto d = [&](int k) { return g.src.value(k); };
    const int X = g.sx, Y = g.sy, Z = g.sz;
    // STEP & (int)lroundf(-v): v lies in [0, 1], so lroundf gives -1 (offset one step) or 0
    const int ox = lroundf(-v.x) == -1 ? X : 0, oy = lroundf(-v.y) == -1 ? Y : 0, oz = lroundf(-v.z) == -1 ? Z : 0;
    float3 dd = make_float3(v.x + 0.5f, v.y + 0.5f, v.z + 0.5f);
    dd = make_float3(dd.x - floorf(dd.x), dd.y - floorf(dd.y), dd.z - floorf(dd.z));
    float3 der = make_float3(0.0f, 0.0f, 0.0f);
    int cur = i;
#pragma unroll
    for (int z = -1; z < 1; ++z) {
        const float cz = fabsf((float)z + v.z);
#pragma unroll
        for (int y = -1; y < 1; ++y) {
            const float cy = fabsf((float)y + v.y);
#pragma unroll
            for (int x = -1; x < 1; ++x) {
                const float cx = fabsf((float)x + v.x);
                if (x) {
                    const int k = cur + ox;
                    der.x += cy * cz * lerp_(d(k - X) - d(k), d(k) - d(k + X), dd.x);
                }
                if (y) {
                    const int k = cur + oy;
                    der.y += cx * cz * lerp_(d(k - Y) - d(k), d(k) - d(k + Y), dd.y);
                }
                if (z) {
                    const int k = cur + oz;
                    der.z += cx * cy * lerp_(d(k - Z) - d(k), d(k) - d(k + Z), dd.z);
                }
                cur += X;
            }
            cur += Y - X * 2;
        }
        cur += Z - Y * 2;
    }
    float light = dot3(nl, normalized3(der)) * (0.5f - kAmbient * 0.5f) + (0.5f + kAmbient * 0.5f);
    light *= light;
    return light < 1.0f ? light : 1.0f;                        // std::min(1.0f, light): NaN -> 1
}

// Cell counts are scanned in tiles of 2048 cells; the tile sums are accumulated with
// atomics by the passes that produce the counts, so the scan reads each count once.
constexpr int kDmcTile = 2048;

// Work lists, appended warp by warp.
struct DmcLists {
    unsigned* vert_items;   // cell << 4 | slot bit, one per vertex
    unsigned* quad_items;   // cell << 2 | axis, one per quad
    unsigned* counters;     // [0] vertex items, [1] quad items
    uint2* tile_sums;       // per 2048 cells: vertices, quads; then scanned in place
};

// Add v to sums[tile] with one atomic per distinct tile among the warp's lanes.
__device__ __forceinline__ void warp_tile_add(unsigned* sums, unsigned tile, unsigned v)
{
    const unsigned group = __match_any_sync(0xffffffffu, tile);
    const unsigned sum = __reduce_add_sync(group, v);
    if ((threadIdx.x & 31u) == (unsigned)(__ffs(group) - 1) && sum) atomicAdd(&sums[2 * tile], sum);
}

__device__ __forceinline__ unsigned warp_append(unsigned* counter, unsigned n)
{
    const int lane = threadIdx.x & 31;
    unsigned x = n;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    const unsigned total = __shfl_sync(0xffffffffu, x, 31);
    unsigned base = 0;
    if (lane == 31 && total) base = atomicAdd(counter, total);
    return __shfl_sync(0xffffffffu, base, 31) + x - n;
}

// Case pass: the marching-cubes case of every vertex cell (-1 .. size-1 per axis); for the
// chunk's own cells also their quads (one per cut axis): tile sums and work items.
template <class S>
__global__ void dmc_cases(DmcGrid<S> g, float iso, const float* minmax, unsigned* masks, DmcLists lists)
{
    if (early_out(minmax, iso)) return;
    const unsigned s1 = (unsigned)g.size + 1u, n = s1 * s1 * s1, lane = threadIdx.x & 31u;
    unsigned* quad_sums = &lists.tile_sums[0].y;
    for (unsigned t0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); t0 < n; t0 += gridDim.x * blockDim.x) {
        const unsigned t = t0 + lane;
        unsigned axes = 0, cell = 0;
        if (t < n) {
            const int x = (int)(t % s1) - 1, y = (int)((t / s1) % s1) - 1, z = (int)(t / (s1 * s1)) - 1;
            const unsigned c = dmc_case(g, dmc_index(g, x, y, z), iso);
            g.cases[t] = (unsigned char)c;
            if (x >= 0 && y >= 0 && z >= 0) {
                cell = ((unsigned)z * g.size + (unsigned)y) * g.size + (unsigned)x;
                axes = dmc_axes(c);
                if (axes) masks[cell] = 0u;
            }
        }
        warp_tile_add(quad_sums, cell / kDmcTile, __popc(axes));
        unsigned q = warp_append(&lists.counters[1], __popc(axes));
        for (unsigned m = axes; m; m &= m - 1u) lists.quad_items[q++] = cell << 2 | (unsigned)(__ffs(m) - 1);
    }
}

// Count pass: one thread per quad; each of its 4 references that is the vertex's first
// use creates the vertex (bit axis * 4 + slot of the cell's mask) and becomes a vertex item.
template <class S>
__global__ void dmc_count(DmcGrid<S> g, unsigned* masks, DmcLists lists)
{
    const unsigned items = lists.counters[1];
    unsigned* vert_sums = &lists.tile_sums[0].x;
    for (unsigned j0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); j0 < items; j0 += gridDim.x * blockDim.x) {
        const unsigned j = j0 + (threadIdx.x & 31u);
        unsigned bits = 0, t = 0;
        if (j < items) {
            const unsigned it = lists.quad_items[j];
            t = it >> 2;
            const int a = (int)(it & 3u);
            const int x = t % g.size, y = (t / g.size) % g.size, z = t / ((unsigned)g.size * g.size);
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                const DmcRef r = dmc_ref(g, x, y, z, a, s);
                if (dmc_first_use(g, r.wx, r.wy, r.wz, r.c, r.p) == t * 12u + (unsigned)(a * 4 + s)) bits |= 1u << (a * 4 + s);
            }
            if (bits) atomicOr(&masks[t], bits);
        }
        warp_tile_add(vert_sums, t / kDmcTile, __popc(bits));
        unsigned v = warp_append(&lists.counters[0], __popc(bits));
        for (unsigned m = bits; m; m &= m - 1u) lists.vert_items[v++] = t << 4 | (unsigned)(__ffs(m) - 1);
    }
}

// Tile offsets: exclusive scan of the tile sums (one block); the grand total lands in `total`.
__global__ void __launch_bounds__(kScanBlock) dmc_scan_tiles(uint2* tile_sums, unsigned tiles, uint2* total)
{
    __shared__ uint2 ws[32];
    uint2 carry = make_uint2(0u, 0u);
    for (unsigned base = 0; base < tiles; base += kScanBlock) {
        const unsigned i = base + threadIdx.x;
        const uint2 v = i < tiles ? tile_sums[i] : make_uint2(0u, 0u);
        uint2 sum;
        const uint2 ex = block_exclusive_scan(v, ws, sum);
        if (i < tiles) tile_sums[i] = plus(carry, ex);
        carry = plus(carry, sum);
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

// Cell offsets within each tile that holds quads (256 threads x 8 cells, staged through
// shared memory so that global loads and stores stay coalesced).  A cell's counts come from
// its case (one quad per cut axis) and its mask (the vertices it creates).
template <class S>
__global__ void __launch_bounds__(256) dmc_scan_cells(DmcGrid<S> g, const unsigned* masks, uint2* offsets, const uint2* tile_offsets,
                                                      const uint2* total)
{
    __shared__ uint2 tile[kDmcTile];
    __shared__ uint2 ws[32];
    const unsigned n = (unsigned)g.size * g.size * g.size;
    const unsigned base = blockIdx.x * kDmcTile;
    const unsigned next = blockIdx.x + 1u < gridDim.x ? tile_offsets[blockIdx.x + 1].y : total->y;
    if (next == tile_offsets[blockIdx.x].y) return;             // no quads: nobody reads these offsets
    for (int k = threadIdx.x; k < kDmcTile; k += 256) {
        const unsigned t = base + k;
        uint2 c = make_uint2(0u, 0u);
        if (t < n) {
            const int x = t % g.size, y = (t / g.size) % g.size, z = t / ((unsigned)g.size * g.size);
            const unsigned axes = dmc_axes(dmc_case_at(g, x, y, z));
            if (axes) c = make_uint2(__popc(masks[t]), __popc(axes));
        }
        tile[k] = c;
    }
    __syncthreads();
    uint2 local[8];
    uint2 run = make_uint2(0u, 0u);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        local[k] = run;
        run = plus(run, tile[threadIdx.x * 8 + k]);
    }
    uint2 sum;
    const uint2 before = plus(tile_offsets[blockIdx.x], block_exclusive_scan(run, ws, sum));
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 8; ++k) tile[threadIdx.x * 8 + k] = plus(before, local[k]);
    __syncthreads();
    for (int k = threadIdx.x; k < kDmcTile; k += 256)
        if (base + k < n) offsets[base + k] = tile[k];
}

// Vertex pass: one thread per created vertex, written at its cell's scanned offset.
template <class S>
__global__ void dmc_vertices(DmcGrid<S> g, int3 pos, float iso, const unsigned* masks, const uint2* offsets, const uint2* total,
                             DmcLists lists, MeshVertex* verts, unsigned vcap)
{
    __shared__ float3 s_nl;
    if (threadIdx.x == 0) s_nl = dmc_light_dir();
    __syncthreads();
    if (total->x > vcap) return;
    const float3 nl = s_nl;
    const unsigned items = lists.counters[0];
    for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < items; j += gridDim.x * blockDim.x) {
        const unsigned it = lists.vert_items[j];
        const unsigned t = it >> 4, bit = it & 15u;
        const int a = (int)(bit >> 2), s = (int)(bit & 3u);
        const int x = t % g.size, y = (t / g.size) % g.size, z = t / ((unsigned)g.size * g.size);
        const DmcRef r = dmc_ref(g, x, y, z, a, s);
        const int wi = dmc_index(g, r.wx, r.wy, r.wz);
        const float3 p = dmc_point(g, wi, __ldg(&kDmc.code[r.c][r.p]), iso);
        const float light = dmc_light(g, wi, p, nl);
        const unsigned out = offsets[t].x + __popc(masks[t] & ((1u << bit) - 1u));
        verts[out] = MeshVertex{p.x + dmc_offset(pos.x, x, r.wx), p.y + dmc_offset(pos.y, y, r.wy),
                                p.z + dmc_offset(pos.z, z, r.wz), light};
    }
}

// Quad pass: one thread per cut edge, 6 indices (:662-674) with the vertex indices found
// through each vertex's first use; the y-edge quads also give the min air / max solid
// heights (:706-724).
template <class S>
__global__ void dmc_quads(DmcGrid<S> g, int3 pos, float iso, const unsigned* masks, const uint2* offsets, const uint2* total,
                          DmcLists lists, const MeshVertex* verts, unsigned vcap, unsigned* idx, unsigned icap, unsigned* airsolid)
{
    const uint2 tot = *total;
    const bool fits = tot.x <= vcap && (unsigned long long)tot.y * 6ull <= icap;
    const unsigned items = lists.counters[1];
    unsigned air = 0xFFFFFFFFu, solid = 0u;
    for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < items; j += gridDim.x * blockDim.x) {
        const unsigned it = lists.quad_items[j];
        const unsigned t = it >> 2;
        const int a = (int)(it & 3u);
        const int x = t % g.size, y = (t / g.size) % g.size, z = t / ((unsigned)g.size * g.size);
        const unsigned own = dmc_case_at(g, x, y, z);
        const bool inside = !(own & 1u);                      // density <= iso; cut, so also density < neighbour
        const unsigned quad = offsets[t].y + __popc(dmc_axes(own) & ((1u << a) - 1u));
        unsigned q[4];
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const DmcRef r = dmc_ref(g, x, y, z, a, s);
            const unsigned first = dmc_first_use(g, r.wx, r.wy, r.wz, r.c, r.p);
            const unsigned c = first / 12u, bit = first - c * 12u;
            q[s] = offsets[c].x + __popc(masks[c] & ((1u << bit) - 1u));
            if (a == 1) {                       // the stored vertex's y: offset of the quad that created it
                // the vertex pass wrote exactly this value when the buffers fit
                const int cy = (int)((c / (unsigned)g.size) % (unsigned)g.size);
                const float vy = fits ? verts[q[s]].y
                                      : dmc_point(g, dmc_index(g, r.wx, r.wy, r.wz), __ldg(&kDmc.code[r.c][r.p]), iso).y +
                                            dmc_offset(pos.y, cy, r.wy);
                if (inside) solid = max(solid, enc(vy));
                else air = min(air, enc(vy));
            }
        }
        if (fits) {
            const unsigned rot = fabsf(verts[q[0]].light - verts[q[3]].light) > fabsf(verts[q[1]].light - verts[q[2]].light) ? 2u : 0u;
            const unsigned flip = inside ? 2u : 0u;
            unsigned* o = idx + (size_t)quad * 6u;
            o[0] = q[flip];
            o[1] = q[3u - rot];
            o[2] = q[2u - flip];
            o[3] = q[3u - flip];
            o[4] = q[rot];
            o[5] = q[1u + flip];
        }
    }
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

// ---- the sparse density form: which densities a pass reads, and where their values land

// Set bits [start, start + len) of `need`, clipped to the chunk's n densities.
__device__ __forceinline__ void mark_run(unsigned* need, int start, int len, unsigned n)
{
    int a = start < 0 ? 0 : start;
    const int b = start + len < (int)n ? start + len : (int)n;
    while (a < b) {
        const int lo = a & 31, cnt = min(b - a, 32 - lo);
        const unsigned mask = (cnt == 32 ? 0xFFFFFFFFu : ((1u << cnt) - 1u)) << lo;
        atomicOr(&need[a >> 5], mask);
        a += cnt;
    }
}

// The density index of every created vertex's cell (its base corner) -- marked in `cells`;
// need_dilate then adds the densities the vertex and quad passes read around them.
template <class S>
__global__ void dmc_mark_cells(DmcGrid<S> g, DmcLists lists, unsigned* cells)
{
    const unsigned items = lists.counters[0];
    for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < items; j += gridDim.x * blockDim.x) {
        const unsigned it = lists.vert_items[j];
        const unsigned t = it >> 4, bit = it & 15u;
        const int x = t % g.size, y = (t / g.size) % g.size, z = t / ((unsigned)g.size * g.size);
        const DmcRef r = dmc_ref(g, x, y, z, (int)(bit >> 2), (int)(bit & 3u));
        const int wi = dmc_index(g, r.wx, r.wy, r.wz);
        atomicOr(&cells[wi >> 5], 1u << (wi & 31));
    }
}

// 64 bits of a bit array starting at bit b (bits outside [0, 32 nwords) read as 0).
__device__ __forceinline__ unsigned long long bits64(const unsigned* a, long long b, unsigned nwords)
{
    const long long w = b >> 5;                       // floor
    const unsigned sh = (unsigned)(b & 31);
    unsigned v[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) v[k] = (w + k >= 0 && w + k < (long long)nwords) ? __ldg(&a[w + k]) : 0u;
    const unsigned long long lo = (unsigned long long)v[0] | ((unsigned long long)v[1] << 32);
    return sh ? (lo >> sh) | ((unsigned long long)v[2] << (64 - sh)) : lo;
}

// The densities dmc_point and dmc_light read around a vertex cell with base corner i: the
// corners, and the central differences at them, which the vertex position may shift one step
// up each axis -- i + [-1, 3] along the differentiated axis and i + [0, 2] along the other
// two (offsets in the passes' own index arithmetic).  need = cells dilated by that stencil,
// 32 densities per thread: for each stencil row (dy, dz) and its x range [lo, hi],
// need bit j |= cells bit (32w + j - dx - dy sy - dz sz) for dx in [lo, hi].  Also the set bits
// per word, for the scan.
__global__ void need_dilate(const unsigned* cells, unsigned* need, unsigned* counts, unsigned n_dens, int sy, int sz)
{
    const unsigned nwords = (n_dens + 31u) / 32u;
    for (unsigned w = blockIdx.x * blockDim.x + threadIdx.x; w < nwords; w += gridDim.x * blockDim.x) {
        unsigned out = 0;
        for (int dz = -1; dz <= 3; ++dz)
            for (int dy = -1; dy <= 3; ++dy) {
                const bool iny = dy >= 0 && dy <= 2, inz = dz >= 0 && dz <= 2;
                if (!iny && !inz) continue;
                const int lo = iny && inz ? -1 : 0, hi = iny && inz ? 3 : 2;
                const long long b = 32ll * w - (long long)dy * sy - (long long)dz * sz - hi;
                const unsigned long long win = bits64(cells, b, nwords);
                for (int m = 0; m <= hi - lo; ++m) out |= (unsigned)(win >> m);
            }
        if (w == nwords - 1u && (n_dens & 31u)) out &= (1u << (n_dens & 31u)) - 1u;   // past the last density
        need[w] = out;
        counts[w] = __popc(out);
    }
}

__global__ void need_counts(const unsigned* need, unsigned* counts, unsigned nwords)
{
    for (unsigned w = blockIdx.x * blockDim.x + threadIdx.x; w < nwords; w += gridDim.x * blockDim.x) counts[w] = __popc(need[w]);
}

// The marked density indices in ascending order (word w's go to idx[rank[w] ..]), and each
// word's rank packed with its bits for the passes' value lookups.
__global__ void need_compact(const unsigned* need, const unsigned* rank, unsigned nwords, unsigned* idx, uint2* stored)
{
    for (unsigned w = blockIdx.x * blockDim.x + threadIdx.x; w < nwords; w += gridDim.x * blockDim.x) {
        const unsigned bits = need[w];
        unsigned o = rank[w];
        stored[w] = make_uint2(o, bits);
        for (unsigned m = bits; m; m &= m - 1u) idx[o++] = w * 32u + (unsigned)(__ffs(m) - 1);
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
    Vox<DenseSrc> v{DenseSrc{dens}, 1, up_axis_z ? sg * sg : sg, up_axis_z ? sg : sg * sg};
    const unsigned n = (unsigned)size * size * size;
    cudaError_t e = cudaMemsetAsync(s.airsolid, 0, 2 * sizeof(unsigned), stream);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(s.airsolid, 0xFF, sizeof(unsigned), stream);           // min air starts at "none"
    if (e != cudaSuccess) return e;
    const float3 pos = make_float3(px, py, pz);
    bloxel_count<<<grid_for(n, 256), 256, 0, stream>>>(v, size, pos, iso, dminmax, s.counts, s.airsolid, nullptr);
    exclusive_scan<unsigned>(s.counts, s.offsets, s.block_totals, s.total, n, stream);
    bloxel_emit<<<grid_for(n, 256), 256, 0, stream>>>(v, size, pos, iso, dminmax, s.offsets, verts, idx, vcap, icap);
    return cudaGetLastError();
}

namespace {

SparseSrc sparse_src(const SparseScratch& sp)
{
    return SparseSrc{sp.above, sp.solid, sp.stored, sp.vals};
}

// The marked densities' ranks and their index list (total in sp.total); `counted` = the
// counts per word are already in sp.counts.
void need_list(SparseScratch& sp, unsigned n_dens, bool counted, cudaStream_t stream)
{
    const unsigned nwords = (n_dens + 31u) / 32u;
    if (!counted) need_counts<<<grid_for(nwords, 256), 256, 0, stream>>>(sp.need, sp.counts, nwords);
    exclusive_scan<unsigned>(sp.counts, sp.rank, sp.block_totals, sp.total, nwords, stream);
    need_compact<<<grid_for(nwords, 256), 256, 0, stream>>>(sp.need, sp.rank, nwords, sp.idx, sp.stored);
}

}  // namespace

cudaError_t launch_bloxel_sparse_prepare(SparseScratch& sp, int size, bool up_axis_z, float px, float py, float pz, float iso,
                                         const float* dminmax, MeshScratch& s, cudaStream_t stream)
{
    const int sg = size + 2;
    const unsigned n_dens = (unsigned)sg * sg * sg;
    Vox<SparseSrc> v{sparse_src(sp), 1, up_axis_z ? sg * sg : sg, up_axis_z ? sg : sg * sg};
    const unsigned n = (unsigned)size * size * size;
    cudaError_t e = cudaMemsetAsync(s.airsolid, 0, 2 * sizeof(unsigned), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s.airsolid, 0xFF, sizeof(unsigned), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(sp.need, 0, ((n_dens + 31u) / 32u) * sizeof(unsigned), stream);
    if (e != cudaSuccess) return e;
    bloxel_count<<<grid_for(n, 256), 256, 0, stream>>>(v, size, make_float3(px, py, pz), iso, dminmax, s.counts, s.airsolid, sp.need);
    exclusive_scan<unsigned>(s.counts, s.offsets, s.block_totals, s.total, n, stream);
    need_list(sp, n_dens, false, stream);
    return cudaGetLastError();
}

cudaError_t launch_bloxel_sparse_emit(const SparseScratch& sp, int size, bool up_axis_z, float px, float py, float pz, float iso,
                                      const float* dminmax, MeshScratch& s, MeshVertex* verts, unsigned vcap, unsigned* idx,
                                      unsigned icap, cudaStream_t stream)
{
    const int sg = size + 2;
    Vox<SparseSrc> v{sparse_src(sp), 1, up_axis_z ? sg * sg : sg, up_axis_z ? sg : sg * sg};
    const unsigned n = (unsigned)size * size * size;
    bloxel_emit<<<grid_for(n, 256), 256, 0, stream>>>(v, size, make_float3(px, py, pz), iso, dminmax, s.offsets, verts, idx, vcap,
                                                      icap);
    return cudaGetLastError();
}

cudaError_t launch_heightmap(const float* dens, int size, float px, float pz, float mul, MeshVertex* verts, unsigned vcap,
                             unsigned* idx, unsigned icap, cudaStream_t stream)
{
    const unsigned n = (unsigned)size * size;
    heightmap_emit<<<grid_for(n, 256), 256, 0, stream>>>(dens, size, make_float2(px, pz), mul, verts, idx, vcap, icap);
    return cudaGetLastError();
}

cudaError_t launch_dmc(const float* dens, int size, bool up_axis_z, int px, int py, int pz, float iso, const float* dminmax,
                       DmcScratch& s, MeshVertex* verts, unsigned vcap, unsigned* idx, unsigned icap, cudaStream_t stream)
{
    const int sg = size + 4;
    const DmcGrid<DenseSrc> g{DenseSrc{dens}, 1, up_axis_z ? sg * sg : sg, up_axis_z ? sg : sg * sg, size, s.cases};
    const DmcLists lists{s.vert_items, s.quad_items, s.counters, s.tile_sums};
    const unsigned n = (unsigned)size * size * size, s1 = (unsigned)size + 1u;
    const unsigned tiles = (n + kDmcTile - 1) / kDmcTile;
    // air = "none" (all ones), solid = 0; list counters and tile sums = 0 (one contiguous block)
    cudaError_t e = cudaMemsetAsync(s.airsolid, 0, 2 * sizeof(unsigned), stream);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(s.airsolid, 0xFF, sizeof(unsigned), stream);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(s.counters, 0, 2 * sizeof(unsigned), stream);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(s.tile_sums, 0, tiles * sizeof(uint2), stream);
    if (e != cudaSuccess) return e;
    const int3 pos = make_int3(px, py, pz);
    dmc_cases<<<grid_for(s1 * s1 * s1, 256), 256, 0, stream>>>(g, iso, dminmax, s.masks, lists);
    // one thread per quad / vertex: the lists hold a few items per surface cell
    dmc_count<<<grid_for(n / 8, 256), 256, 0, stream>>>(g, s.masks, lists);
    dmc_scan_tiles<<<1, kScanBlock, 0, stream>>>(s.tile_sums, tiles, s.total);
    dmc_scan_cells<<<tiles, 256, 0, stream>>>(g, s.masks, s.offsets, s.tile_sums, s.total);
    dmc_vertices<<<grid_for(n / 8, 256), 256, 0, stream>>>(g, pos, iso, s.masks, s.offsets, s.total, lists, verts, vcap);
    dmc_quads<<<grid_for(n / 8, 256), 256, 0, stream>>>(g, pos, iso, s.masks, s.offsets, s.total, lists, verts, vcap, idx, icap,
                                                        s.airsolid);
    return cudaGetLastError();
}

cudaError_t launch_dmc_sparse_prepare(SparseScratch& sp, int size, bool up_axis_z, float iso, const float* dminmax, DmcScratch& s,
                                      cudaStream_t stream)
{
    const int sg = size + 4;
    const unsigned n_dens = (unsigned)sg * sg * sg;
    const DmcGrid<SparseSrc> g{sparse_src(sp), 1, up_axis_z ? sg * sg : sg, up_axis_z ? sg : sg * sg, size, s.cases};
    const DmcLists lists{s.vert_items, s.quad_items, s.counters, s.tile_sums};
    const unsigned n = (unsigned)size * size * size, s1 = (unsigned)size + 1u;
    const unsigned tiles = (n + kDmcTile - 1) / kDmcTile;
    const unsigned nwords = (n_dens + 31u) / 32u;
    cudaError_t e = cudaMemsetAsync(s.airsolid, 0, 2 * sizeof(unsigned), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s.airsolid, 0xFF, sizeof(unsigned), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s.counters, 0, 2 * sizeof(unsigned), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s.tile_sums, 0, tiles * sizeof(uint2), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(sp.cells, 0, nwords * sizeof(unsigned), stream);
    if (e != cudaSuccess) return e;
    dmc_cases<<<grid_for(s1 * s1 * s1, 256), 256, 0, stream>>>(g, iso, dminmax, s.masks, lists);
    dmc_count<<<grid_for(n / 8, 256), 256, 0, stream>>>(g, s.masks, lists);
    dmc_scan_tiles<<<1, kScanBlock, 0, stream>>>(s.tile_sums, tiles, s.total);
    dmc_scan_cells<<<tiles, 256, 0, stream>>>(g, s.masks, s.offsets, s.tile_sums, s.total);
    dmc_mark_cells<<<grid_for(n / 8, 256), 256, 0, stream>>>(g, lists, sp.cells);
    need_dilate<<<grid_for(nwords, 256), 256, 0, stream>>>(sp.cells, sp.need, sp.counts, n_dens, g.sy, g.sz);
    need_list(sp, n_dens, true, stream);
    return cudaGetLastError();
}

cudaError_t launch_dmc_sparse_finish(const SparseScratch& sp, int size, bool up_axis_z, int px, int py, int pz, float iso,
                                     DmcScratch& s, MeshVertex* verts, unsigned vcap, unsigned* idx, unsigned icap,
                                     cudaStream_t stream)
{
    const int sg = size + 4;
    const DmcGrid<SparseSrc> g{sparse_src(sp), 1, up_axis_z ? sg * sg : sg, up_axis_z ? sg : sg * sg, size, s.cases};
    const DmcLists lists{s.vert_items, s.quad_items, s.counters, s.tile_sums};
    const unsigned n = (unsigned)size * size * size;
    const int3 pos = make_int3(px, py, pz);
    dmc_vertices<<<grid_for(n / 8, 256), 256, 0, stream>>>(g, pos, iso, s.masks, s.offsets, s.total, lists, verts, vcap);
    dmc_quads<<<grid_for(n / 8, 256), 256, 0, stream>>>(g, pos, iso, s.masks, s.offsets, s.total, lists, verts, vcap, idx, icap,
                                                        s.airsolid);
    return cudaGetLastError();
}

}  // namespace fn
