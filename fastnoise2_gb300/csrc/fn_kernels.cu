// fn_kernels.cu -- the program interpreter for sm_103a.
//
// One thread evaluates one point: it builds the root position (grid index,
// tileable torus or position array, as Generator.inl:79-433 do), runs the
// tree's program over a per-point register file, stores the result and folds
// it into a running min/max.  Blocks reduce min/max with warp shuffles and
// shared memory; the last block to finish reduces the per-block partials, so a
// launch needs no separate initialisation or finishing kernel.
//
// The program blob is staged into shared memory once per block; every thread
// of a warp executes the same instruction stream (warp-uniform dispatch).
#include <cuda_runtime.h>

#include <atomic>

#include "fn_eval.cuh"
#include "fn_kernels.cuh"

namespace fn {

using namespace fnd;

namespace {

constexpr int kThreads = 256;
constexpr float kInf = __builtin_huge_valf();

__device__ __forceinline__ int sadd(int a, int b) { return (int)((unsigned)a + (unsigned)b); }

template <int D>
__device__ __forceinline__ float noise_at(int kind, int seed, const float* R, int a, float f)
{
    float p[4];
#pragma unroll
    for (int k = 0; k < D; ++k) p[k] = R[a + k] * f;          // ScalableGenerator::ScalePositions
    if (D == 2) {
        switch (kind) {
        case FN_NOISE_SIMPLEX: return simplex2(seed, p[0], p[1]);
        case FN_NOISE_SUPERSIMPLEX: return supersimplex2(seed, p[0], p[1]);
        case FN_NOISE_PERLIN: return perlin2(seed, p[0], p[1]);
        default: return value2(seed, p[0], p[1]);
        }
    } else if (D == 3) {
        switch (kind) {
        case FN_NOISE_SIMPLEX: return simplex3(seed, p[0], p[1], p[2]);
        case FN_NOISE_SUPERSIMPLEX: return supersimplex3(seed, p[0], p[1], p[2]);
        case FN_NOISE_PERLIN: return perlin3(seed, p[0], p[1], p[2]);
        default: return value3(seed, p[0], p[1], p[2]);
        }
    } else {
        switch (kind) {
        case FN_NOISE_SIMPLEX: return simplex4(seed, p[0], p[1], p[2], p[3]);
        case FN_NOISE_SUPERSIMPLEX: return supersimplex4(seed, p[0], p[1], p[2], p[3]);
        case FN_NOISE_PERLIN: return perlin4(seed, p[0], p[1], p[2], p[3]);
        default: return value4(seed, p[0], p[1], p[2], p[3]);
        }
    }
}

template <int D>
__device__ __forceinline__ CellParams cell_params(const FnInstr& I, const float* P, const float* R)
{
    CellParams cp;
    cp.freq = P[I.prm];
    cp.jitter = CellConst<D>::jitter * R[I.b];
    cp.sizeActive = I.c != FN_REG_NONE;
    cp.sizeJitter = cp.sizeActive ? R[I.c] * CellConst<D>::size : 0.0f;
    cp.distFunc = I.aux & 15;
    cp.minkowski = P[I.prm + 3 - (I.op == FN_OP_CELL_LOOKUP ? 1 : 0)];
    return cp;
}

template <int D>
__device__ __forceinline__ void exec_dim(const FnInstr& I, const float* P, float* R, int seed)
{
    const int sd = sadd(seed, I.seed);
    switch (I.op) {
    case FN_OP_NOISE: {
        float v = noise_at<D>(I.aux, sd, R, I.a, P[I.prm]);
        R[I.dst] = scale_out(v, P[I.prm + 1], P[I.prm + 2], P[I.prm + 3]);
        break;
    }
    case FN_OP_WHITE: {
        float p[4];
#pragma unroll
        for (int k = 0; k < D; ++k) p[k] = R[I.a + k];
        R[I.dst] = scale_out(white<D>(sd, p), -kValueBounds, P[I.prm], P[I.prm + 1]);
        break;
    }
    case FN_OP_CHECKER: {
        float p[4];
#pragma unroll
        for (int k = 0; k < D; ++k) p[k] = R[I.a + k];
        R[I.dst] = scale_out(checkerboard<D>(p, P[I.prm]), 0.0f, P[I.prm + 1], P[I.prm + 2]);
        break;
    }
    case FN_OP_SINE: {
        float p[4];
#pragma unroll
        for (int k = 0; k < D; ++k) p[k] = R[I.a + k];
        R[I.dst] = scale_out(sine_wave<D>(p, P[I.prm]), -1.0f, P[I.prm + 1], P[I.prm + 2]);
        break;
    }
    case FN_OP_CELL_VALUE: {
        float p[4];
#pragma unroll
        for (int k = 0; k < D; ++k) p[k] = R[I.a + k];
        CellParams cp = cell_params<D>(I, P, R);
        float v = cellular_value<D>(sd, p, cp, (I.aux >> 4) & 3);
        R[I.dst] = scale_out(v, -kValueBounds, P[I.prm + 1], P[I.prm + 2]);
        break;
    }
    case FN_OP_CELL_DIST: {
        float p[4];
#pragma unroll
        for (int k = 0; k < D; ++k) p[k] = R[I.a + k];
        CellParams cp = cell_params<D>(I, P, R);
        float dist[4];
        cellular_distances<D>(sd, p, cp, dist);
        float nmax;
        float v = cellular_return<D>(dist, cp.distFunc, (I.aux >> 4) & 3, (I.aux >> 8) & 3, (I.aux >> 12) & 7, nmax);
        R[I.dst] = scale_out(v, 0.0f, P[I.prm + 1], P[I.prm + 2]);
        break;
    }
    case FN_OP_CELL_LOOKUP: {
        float p[4], o[4];
#pragma unroll
        for (int k = 0; k < D; ++k) p[k] = R[I.a + k];
        CellParams cp = cell_params<D>(I, P, R);
        cellular_lookup_pos<D>(sd, p, cp, P[I.prm + 1], o);
#pragma unroll
        for (int k = 0; k < D; ++k) R[I.dst + k] = o[k];
        break;
    }
    case FN_OP_WARP_GRAD: {
        float sp[4], io[4], axis[4];
        const float f = P[I.prm];
#pragma unroll
        for (int k = 0; k < D; ++k) { sp[k] = R[I.a + k] * f; io[k] = R[I.dst + k]; axis[k] = P[I.prm + 1 + k]; }
        float strength = warp_gradient<D>(sd, R[I.b], sp, axis, io);
#pragma unroll
        for (int k = 0; k < D; ++k) R[I.dst + k] = io[k];
        if (I.c != FN_REG_NONE) R[I.c] = strength;
        break;
    }
    case FN_OP_WARP_SIMPLEX: {
        float sp[4], io[4], axis[4];
        const float f = P[I.prm];
#pragma unroll
        for (int k = 0; k < D; ++k) { sp[k] = R[I.a + k] * f; io[k] = R[I.dst + k]; axis[k] = P[I.prm + 1 + k]; }
        float strength = warp_simplex<D>(sd, R[I.b], sp, axis, io, I.aux & 1, (I.aux >> 1) & 1);
#pragma unroll
        for (int k = 0; k < D; ++k) R[I.dst + k] = io[k];
        if (I.c != FN_REG_NONE) R[I.c] = strength;
        break;
    }
    case FN_OP_SCALE_POS: {
        const float f = P[I.prm];
#pragma unroll
        for (int k = 0; k < D; ++k) R[I.dst + k] = R[I.a + k] * f;
        break;
    }
    case FN_OP_SCALE_POS_V:
#pragma unroll
        for (int k = 0; k < D; ++k) R[I.dst + k] = R[I.a + k] * P[I.prm + k];
        break;
    case FN_OP_OFFSET_POS: case FN_OP_SUB_POS: {
        const uint8_t off[4] = {I.b, I.c, I.d, I.e};
        float o[4];
#pragma unroll
        for (int k = 0; k < D; ++k) o[k] = I.op == FN_OP_OFFSET_POS ? R[I.a + k] + R[off[k]] : R[I.a + k] - R[off[k]];
#pragma unroll
        for (int k = 0; k < D; ++k) R[I.dst + k] = o[k];
        break;
    }
    case FN_OP_GRADIENT: {
        const uint8_t off[4] = {I.b, I.c, I.d, I.e};
        float r = 0.0f;
#pragma unroll
        for (int k = 0; k < D; ++k) r = fmaf(R[I.a + k] + R[off[k]], P[I.prm + k], r);
        R[I.dst] = r;
        break;
    }
    case FN_OP_DISTANCE: {
        float p[4];
#pragma unroll
        for (int k = 0; k < D; ++k) p[k] = R[I.a + k];
        R[I.dst] = distance<D>(I.aux & 15, (I.aux >> 4) & 1, p, I.b != FN_REG_NONE ? R[I.b] : 0.0f);
        break;
    }
    case FN_OP_ROTATE3: {
        const float x = R[I.a], y = R[I.a + 1], z = D >= 3 ? R[I.a + 2] : 0.0f;
        const float* m = P + I.prm;
        const float nx = fmaf(x, m[0], fmaf(y, m[1], z * m[2]));
        const float ny = fmaf(x, m[3], fmaf(y, m[4], z * m[5]));
        const float nz = fmaf(x, m[6], fmaf(y, m[7], z * m[8]));
        R[I.dst] = nx; R[I.dst + 1] = ny; R[I.dst + 2] = nz;
        break;
    }
    case FN_OP_ROTPLANE: {
        float x = R[I.a], y = R[I.a + 1], z = D >= 3 ? R[I.a + 2] : 0.0f;
        const float w = D == 4 ? R[I.a + 3] : 0.0f;
        rotate_plane(I.aux, x, y, z);
        R[I.dst] = x; R[I.dst + 1] = y; R[I.dst + 2] = z;
        if (D == 4) R[I.dst + 3] = w;
        break;
    }
    default:
        break;
    }
}

__device__ __noinline__ void exec_program(const FnInstr* ins, int n, const float* P, float* R, int seed)
{
    for (int pc = 0; pc < n; ++pc) {
        const FnInstr I = ins[pc];
        switch (I.op) {
        case FN_OP_CONST: R[I.dst] = P[I.prm]; break;
        case FN_OP_MOV: R[I.dst] = R[I.a]; break;
        case FN_OP_ROTATE2: {
            const float x = R[I.a], y = R[I.a + 1], c = P[I.prm], s = P[I.prm + 1];
            const float nx = fmaf(-y, s, x * c);
            const float ny = fmaf(x, s, y * c);
            R[I.dst] = nx; R[I.dst + 1] = ny;
            break;
        }
        case FN_OP_FRACT_INIT: {
            float noise = R[I.a];
            float sum;
            if (I.aux) { noise = fabs_(noise); R[I.a] = noise; sum = (noise * -2.0f + 1.0f) * 1.0f; }
            else sum = noise * 1.0f;
            R[I.dst] = sum;
            R[I.b] = 1.0f;
            break;
        }
        case FN_OP_FRACT_AMP: {
            const float noise = R[I.a];
            const float t = I.aux ? 1.0f - noise : (noise + 1.0f) * 0.5f;
            float amp = R[I.b] * lerp(1.0f, t, R[I.c]);
            R[I.b] = amp * R[I.d];
            break;
        }
        case FN_OP_FRACT_ACC: {
            float noise = R[I.a];
            if (I.aux) { noise = fabs_(noise); R[I.a] = noise; R[I.dst] = R[I.dst] + (noise * -2.0f + 1.0f) * R[I.b]; }
            else R[I.dst] = R[I.dst] + noise * R[I.b];
            break;
        }
        case FN_OP_DWF_AMP: {
            const float strength = sqrtf(R[I.a]);
            R[I.a] = strength;
            float amp = R[I.b] * lerp(1.0f, 1.0f - strength, R[I.c]);
            R[I.b] = amp * R[I.d];
            break;
        }
        case FN_OP_ADD: R[I.dst] = R[I.a] + R[I.b]; break;
        case FN_OP_SUB: R[I.dst] = R[I.a] - R[I.b]; break;
        case FN_OP_MUL: R[I.dst] = R[I.a] * R[I.b]; break;
        case FN_OP_DIV: R[I.dst] = R[I.a] / R[I.b]; break;
        case FN_OP_MOD: R[I.dst] = mod_(R[I.a], R[I.b]); break;
        case FN_OP_MIN: R[I.dst] = fmin_(R[I.a], R[I.b]); break;
        case FN_OP_MAX: R[I.dst] = fmax_(R[I.a], R[I.b]); break;
        case FN_OP_ABS: R[I.dst] = fabs_(R[I.a]); break;
        case FN_OP_SSQRT: R[I.dst] = signed_sqrt(R[I.a]); break;
        case FN_OP_POWF: R[I.dst] = pow_(fmax_(fabs_(R[I.a]), 1.17549435e-38f), R[I.b]); break;
        case FN_OP_POWI: {
            const float v = R[I.a];
            float p = v * v;
            for (int i = 2; i < I.aux; ++i) p *= v;
            R[I.dst] = p;
            break;
        }
        case FN_OP_MINSMOOTH: R[I.dst] = min_smooth(R[I.a], R[I.b], R[I.c]); break;
        case FN_OP_MAXSMOOTH: R[I.dst] = -min_smooth(-R[I.a], -R[I.b], R[I.c]); break;
        case FN_OP_FADE: R[I.dst] = lerp(R[I.a], R[I.b], fade_t(R[I.c], R[I.d], R[I.e], I.aux)); break;
        case FN_OP_REMAP: R[I.dst] = remap(R[I.a], R[I.b], R[I.c], R[I.d], R[I.e], I.aux != 0); break;
        case FN_OP_TERRACE: {
            const float src = R[I.a] * P[I.prm];
            float rounded = rintf(src);
            if (I.b != FN_REG_NONE) {
                const float sm = R[I.b];
                if (sm != 0.0f) rounded = terrace_smooth(rounded, src, 1.0f + 1.0f / sm);
            } else if (I.aux) {
                rounded = terrace_smooth(rounded, src, P[I.prm + 2]);
            }
            R[I.dst] = rounded * P[I.prm + 1];
            break;
        }
        case FN_OP_PINGPONG: R[I.dst] = ping_pong(R[I.a] * R[I.b]); break;
        case FN_OP_RGBA8: R[I.dst] = to_rgba8(R[I.a], P[I.prm], P[I.prm + 1]); break;
        default:
            if (I.dim == 2) exec_dim<2>(I, P, R, seed);
            else if (I.dim == 3) exec_dim<3>(I, P, R, seed);
            else exec_dim<4>(I, P, R, seed);
            break;
        }
    }
}

__global__ void __launch_bounds__(kThreads, 4) interp_kernel(const FnProgramHeader* gprog, uint32_t bytes, PointArgs args,
                                                          float* __restrict__ out, MinMaxWork* work, float* dminmax)
{
    extern __shared__ uint4 sprog[];
    __shared__ float smn[kThreads / 32], smx[kThreads / 32];
    const uint4* src = reinterpret_cast<const uint4*>(gprog);
    for (uint32_t w = threadIdx.x; w < bytes / 16; w += blockDim.x) sprog[w] = src[w];
    __syncthreads();
    const FnProgramHeader* h = reinterpret_cast<const FnProgramHeader*>(sprog);
    const FnInstr* ins = fn_program_instrs(h);
    const float* P = fn_program_params(h);
    const int n = h->n_instr;
    const int outr = h->out_reg;

    float mn = kInf, mx = -kInf;
    float R[FN_MAX_REGS];
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < args.total; i += stride) {
        fne::root_position(args, i, R);
        exec_program(ins, n, P, R, args.seed);
        const float v = R[outr];
        out[i] = v;
        fne::fold(v, mn, mx);
    }
    fne::grid_minmax(mn, mx, work, dminmax, smn, smx);
}

// SM count per device ordinal, looked up on first use with that device current.
constexpr int kSmCacheDevices = 64;
std::atomic<int> g_num_sms[kSmCacheDevices];

// Let a kernel stage up to 96 KB of program in dynamic shared memory, once per
// device (the attribute is per device; `done` holds one bit per device ordinal).
cudaError_t allow_program_smem(const void* kernel, std::atomic<unsigned long long>& done)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load(std::memory_order_acquire) & bit) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
    if (e == cudaSuccess) done.fetch_or(bit, std::memory_order_release);
    return e;
}

constexpr int kBatchThreads = 256;

__global__ void __launch_bounds__(kBatchThreads, 2) batch_kernel(BatchHeader* hdr, const BatchRequest* __restrict__ reqs,
                                                              BatchState* states, const uint2* __restrict__ items)
{
    extern __shared__ uint4 sprog[];
    __shared__ unsigned int s_item;
    __shared__ float smn[kBatchThreads / 32], smx[kBatchThreads / 32];
    const FnProgramHeader* loaded = nullptr;
    const unsigned int n_items = hdr->n_items;
    const unsigned int tile_points = hdr->tile_points;

    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(&hdr->head, 1u);
        __syncthreads();
        const unsigned int it = s_item;
        if (it >= n_items) break;
        const uint2 item = items[it];
        const BatchRequest& rq = reqs[item.x];
        const FnProgramHeader* gprog = static_cast<const FnProgramHeader*>(rq.prog);
        if (gprog != loaded) {                               // stage this request's program
            const uint4* src = reinterpret_cast<const uint4*>(gprog);
            for (uint32_t w = threadIdx.x; w < rq.prog_bytes / 16; w += blockDim.x) sprog[w] = src[w];
            loaded = gprog;
        }
        __syncthreads();
        const FnProgramHeader* h = reinterpret_cast<const FnProgramHeader*>(sprog);
        const FnInstr* ins = fn_program_instrs(h);
        const float* P = fn_program_params(h);
        const PointArgs args = rq.args;
        const long long begin = (long long)item.y * tile_points;
        long long end = begin + tile_points;
        if (end > args.total) end = args.total;

        float mn = kInf, mx = -kInf;
        float R[FN_MAX_REGS];
        for (long long i = begin + threadIdx.x; i < end; i += blockDim.x) {
            fne::root_position(args, i, R);
            exec_program(ins, h->n_instr, P, R, args.seed);
            const float v = R[h->out_reg];
            rq.out[i] = v;
            fne::fold(v, mn, mx);
        }
        fne::block_minmax(mn, mx, smn, smx);
        if (threadIdx.x == 0) fne::finish_tile(rq, states + item.x, hdr, mn, mx);
        // the next iteration's __syncthreads orders shared-memory reuse
    }
}

}  // namespace

cudaError_t launch_batch(BatchHeader* hdr, const BatchRequest* reqs, BatchState* states, const uint2* items,
                         uint32_t max_prog_bytes, int grid, int block, cudaStream_t stream)
{
    static std::atomic<unsigned long long> attr_set{0};      // one bit per device
    cudaError_t e = allow_program_smem((const void*)batch_kernel, attr_set);
    if (e != cudaSuccess) return e;
    if (block != kBatchThreads || max_prog_bytes > 96 * 1024) return cudaErrorInvalidValue;
    batch_kernel<<<grid, block, max_prog_bytes, stream>>>(hdr, reqs, states, items);
    return cudaGetLastError();
}

int batch_occupancy(int block, uint32_t smem)
{
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel, block, smem) != cudaSuccess || n < 1) n = 1;
    return n;
}



int num_sms()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    const bool cached = dev >= 0 && dev < kSmCacheDevices;
    int n = cached ? g_num_sms[dev].load(std::memory_order_relaxed) : 0;
    if (n > 0) return n;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
    // threads racing here look up and store the same value
    if (cached) g_num_sms[dev].store(n, std::memory_order_relaxed);
    return n;
}

cudaError_t launch_interpreter(const FnProgramHeader* prog, uint32_t prog_bytes, const PointArgs& args, float* out,
                               MinMaxWork* work, float* dminmax, cudaStream_t stream)
{
    static std::atomic<unsigned long long> attr_set{0};      // one bit per device
    cudaError_t e = allow_program_smem((const void*)interp_kernel, attr_set);
    if (e != cudaSuccess) return e;
    if (prog_bytes > 96 * 1024 || (prog_bytes & 15)) return cudaErrorInvalidValue;
    long long blocks = (args.total + kThreads - 1) / kThreads;
    long long cap = (long long)num_sms() * 8;
    if (blocks > cap) blocks = cap;
    if (blocks > kMaxReduceBlocks) blocks = kMaxReduceBlocks;
    if (blocks < 1) blocks = 1;
    interp_kernel<<<(unsigned)blocks, kThreads, prog_bytes, stream>>>(prog, prog_bytes, args, out, work, dminmax);
    return cudaGetLastError();
}

}  // namespace fn
