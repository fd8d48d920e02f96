// fn_capi.cpp -- the FastNoise_C entry points (include/FastNoise/FastNoise_C.h).
//
// Part 1 mirrors reference src/FastNoise/FastNoise_C.cpp:41-476 (same names,
// argument meaning, sentinel return values).  Generation runs on the GPU
// through the program interpreter; host output arrays are filled by a
// device->host copy on this thread's stream.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include <sys/mman.h>
#include <unistd.h>

#include <cuda.h>   // CUpointer_attribute: the range query below goes through the runtime's driver entry point

#include "../../include/FastNoise/FastNoise_C.h"
#include "fn_capi_internal.h"
#include "fn_batch.h"
#include "fn_jit.h"
#include "fn_runtime.h"
#include "fn_server.h"
#include "fn_static_scratch.h"

using namespace fn;

namespace fn {
namespace capi {


Node* N(void* p) { return static_cast<Node*>(p); }
const Node* N(const void* p) { return static_cast<const Node*>(p); }

float f_of(int32_t bits) { float f; std::memcpy(&f, &bits, 4); return f; }
int32_t bits_of(float f) { int32_t i; std::memcpy(&i, &f, 4); return i; }

void store_minmax(float* mm, float mn, float mx)   // FastNoise_C.cpp:32-39
{
    if (mm) { mm[0] = mn; mm[1] = mx; }
}

void fill_nan(float* out, long long n, float* mm)
{
    const float q = std::numeric_limits<float>::quiet_NaN();
    if (out) for (long long i = 0; i < n; ++i) out[i] = q;
    store_minmax(mm, q, q);
}

// Page-locked host memory (cudaHostAlloc, cudaMallocHost, cudaHostRegister): the end of the
// allocation holding `p`, in host addresses; 0 for pageable memory or where the driver does not
// report the allocation's extent.  A device-to-host copy that starts in such an allocation must
// end inside it (the runtime rejects the copy otherwise), so copies are cut there.
using PointerAttrFn = CUresult (*)(void*, CUpointer_attribute, CUdeviceptr);

PointerAttrFn pointer_attr_fn()
{
    static const PointerAttrFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return PointerAttrFn(nullptr);
        }
        return reinterpret_cast<PointerAttrFn>(f);
    }();
    return fn;
}

uintptr_t pinned_end(const void* p)
{
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) { cudaGetLastError(); return 0; }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer) return 0;
    const PointerAttrFn attr = pointer_attr_fn();
    if (!attr) return 0;
    const CUdeviceptr dp = (CUdeviceptr)(uintptr_t)at.devicePointer;
    CUdeviceptr start = 0;
    size_t size = 0;
    if (attr(&start, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, dp) != CUDA_SUCCESS ||
        attr(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, dp) != CUDA_SUCCESS || dp < start || dp - start >= size)
        return 0;
    return (uintptr_t)p + (size_t)(start + size - dp);
}

// The device address of host memory [p, p + bytes) when the whole range lies in one
// page-locked allocation the device addresses (cudaHostAlloc, cudaMallocHost, cudaHostRegister),
// else nullptr.
float* pinned_device_view(float* p, size_t bytes)
{
    cudaPointerAttributes at{};
    if (!p || cudaPointerGetAttributes(&at, p) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
    const uintptr_t a = (uintptr_t)p, end = pinned_end(p);
    return (end > a && bytes <= end - a) ? static_cast<float*>(at.devicePointer) : nullptr;
}

// Host memory the generation kernels may store into directly: page-locked memory (above), or,
// on devices that access pageable memory coherently through the host's page tables (a Grace
// host over NVLink-C2C reports both attributes), any host memory.  FASTNOISE_HOST_DIRECT=0
// turns direct stores off (every host output is then staged in device memory and copied).
bool pageable_direct_supported()
{
    static std::atomic<int> cached[64];                 // per device: 0 unknown, 1 no, 2 yes
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) { cudaGetLastError(); return false; }
    int v = cached[dev].load(std::memory_order_relaxed);
    if (v == 0) {
        int pageable = 0, host_tables = 0;
        const bool ok = cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess &&
                        cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) == cudaSuccess;
        if (!ok) cudaGetLastError();
        v = ok && pageable == 1 && host_tables == 1 ? 2 : 1;
        cached[dev].store(v, std::memory_order_relaxed);
    }
    return v == 2;
}

// True when every page of [p, p + bytes) is mapped and resident (mincore, in windows of 64 Ki
// pages; it fails on unmapped addresses).  A kernel storing into pages nobody has touched yet
// would populate them one device fault at a time (a fresh 64 MB buffer took 20 ms that way), so
// such outputs are staged instead and the host touches them.
bool pages_resident(const void* p, size_t bytes)
{
    static const uintptr_t page = (uintptr_t)sysconf(_SC_PAGESIZE);
    constexpr size_t kWindow = size_t(1) << 16;           // pages per mincore call
    const uintptr_t a = (uintptr_t)p, first = a & ~(page - 1), last = (a + bytes - 1) & ~(page - 1);
    const size_t pages = (size_t)((last - first) / page) + 1;
    thread_local std::vector<unsigned char> v;
    v.resize(std::min(pages, kWindow));
    for (size_t done = 0; done < pages;) {
        const size_t n = std::min(pages - done, kWindow);
        if (mincore(reinterpret_cast<void*>(first + done * page), n * page, v.data()) != 0) return false;
        for (size_t i = 0; i < n; ++i)
            if (!(v[i] & 1)) return false;
        done += n;
    }
    return true;
}

bool host_direct_allowed()
{
    static const bool allowed = [] {
        const char* env = std::getenv("FASTNOISE_HOST_DIRECT");
        return !(env && env[0] == '0');
    }();
    return allowed;
}

// Ordinary (pageable) host memory the device stores into coherently, with every page resident.
bool pageable_direct(float* p, size_t bytes)
{
    if (!p || !host_direct_allowed()) return false;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) { cudaGetLastError(); return false; }
    return at.type == cudaMemoryTypeUnregistered && pageable_direct_supported() && pages_resident(p, bytes);
}

float* host_direct_view(float* p, size_t bytes)
{
    if (!p || !host_direct_allowed()) return nullptr;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    if (at.type == cudaMemoryTypeHost) return pinned_device_view(p, bytes);
    return at.type == cudaMemoryTypeUnregistered && pageable_direct_supported() && pages_resident(p, bytes) ? p : nullptr;
}

// Copy of `bytes` between device memory and host memory that may start in one page-locked
// allocation and continue past it (into pageable memory, or another allocation).
bool copy_host(const void* host, const void* dev, size_t bytes, bool to_host, cudaStream_t s, const char* what)
{
    uintptr_t h = (uintptr_t)host, d = (uintptr_t)dev;
    while (bytes) {
        const uintptr_t end = pinned_end(reinterpret_cast<const void*>(h));
        const size_t n = (end > h && end - h < bytes) ? (size_t)(end - h) : bytes;
        const cudaError_t e = to_host ? cudaMemcpyAsync(reinterpret_cast<void*>(h), reinterpret_cast<const void*>(d), n, cudaMemcpyDeviceToHost, s)
                                      : cudaMemcpyAsync(reinterpret_cast<void*>(d), reinterpret_cast<const void*>(h), n, cudaMemcpyHostToDevice, s);
        if (!cuda_ok(e, what)) return false;
        h += n;
        d += n;
        bytes -= n;
    }
    return true;
}

bool copy_to_host(float* dst, const float* src, size_t bytes, cudaStream_t s)
{
    return copy_host(dst, src, bytes, true, s, "copy output");
}

bool ensure(float*& buf, size_t& cap, size_t n)
{
    if (n <= cap) return true;
    if (buf) cudaFree(buf);
    buf = nullptr;
    cap = 0;
    size_t want = n < 4096 ? 4096 : n;
    if (!cuda_ok(cudaMalloc(&buf, want * sizeof(float)), "cudaMalloc(output)")) return false;
    cap = want;
    return true;
}

// Launch one generation call: the tree's specialised kernel when one is loaded,
// the interpreter otherwise.
cudaError_t launch_points(const DeviceProgram& prog, const PointArgs& args, float* out, MinMaxWork* work, float* dminmax,
                          cudaStream_t stream)
{
    cudaError_t e;
    if (jit_launch(prog.hash, args, out, work, dminmax, stream, e)) return e;
    // the first call on a tree that an earlier process specialised: its kernels from the cache
    if (args.total > 0 && jit_try_cached(prog.host) && jit_launch(prog.hash, args, out, work, dminmax, stream, e)) return e;
    // A tree with per-cell sub-programs cannot run on the interpreter; with no
    // points there is nothing to evaluate and the interpreter only writes min/max.
    if (prog.host->needs_specialisation() && args.total > 0) return cudaErrorNotSupported;
    if (args.total > 0) jit_note_interpreted(prog.host);      // may queue a background specialisation
    return launch_interpreter(prog.dptr, prog.bytes, args, out, work, dminmax, stream);
}

// Specialise trees the interpreter cannot run before their first launch.
bool ensure_runnable(const DeviceProgram& prog)
{
    std::string err;
    if (jit_ensure(prog.host, err)) return true;
    set_error(FN_ERR_COMPILE, err);
    return false;
}

// Run one host-memory generation call end to end.
// Large grids into host memory are generated in slabs along the outermost axis: every slab is
// launched at once, and slab s is copied to the host as soon as it is done, while later slabs
// are still being generated.  Positions come from the point's index in the whole grid (the
// slab's `base`), so the output is the same as one launch's; the slabs' min/max are combined
// in slab order with the same comparisons the kernels' own block reduction uses.
constexpr long long kSlabMinPoints = 1ll << 22;
constexpr int kMaxSlabs = 8;

struct SlabCtx {
    cudaStream_t copy = nullptr;
    cudaEvent_t done[kMaxSlabs] = {};
    float* dmm = nullptr;                  // device: min/max per slab
    float* hmm = nullptr;                  // pinned copy
    ~SlabCtx()
    {
        for (cudaEvent_t& e : done) if (e) cudaEventDestroy(e);
        if (dmm) cudaFree(dmm);
        if (hmm) cudaFreeHost(hmm);
        if (copy) cudaStreamDestroy(copy);
    }
};
thread_local SlabCtx* t_slab = nullptr;

SlabCtx* slab_ctx()
{
    if (t_slab) return t_slab;
    SlabCtx* c = new SlabCtx();
    bool ok = cuda_ok(cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking), "stream") &&
              cuda_ok(cudaMalloc(&c->dmm, 2 * kMaxSlabs * sizeof(float)), "cudaMalloc(slab minmax)") &&
              cuda_ok(cudaMallocHost(&c->hmm, 2 * kMaxSlabs * sizeof(float)), "cudaMallocHost(slab minmax)");
    for (int k = 0; ok && k < kMaxSlabs; ++k) ok = cuda_ok(cudaEventCreateWithFlags(&c->done[k], cudaEventDisableTiming), "event");
    if (!ok) { delete c; return nullptr; }
    return t_slab = c;
}

// Generate a grid in slabs into host memory; false on a CUDA error (already reported).
bool gen_host_slabs(const DeviceProgram& prog, const PointArgs& args, ThreadCtx* ctx, MinMaxWork* work, float* out, float* minmax)
{
    SlabCtx* sc = slab_ctx();
    if (!sc) return false;
    const int k = args.dim - 1;
    const int rows = args.count[k];
    const long long row = args.total / rows;                   // points per index of the outermost axis
    int slabs = (int)std::min<long long>(std::min<long long>(kMaxSlabs, args.total / kSlabMinPoints), rows);
    const int per = (rows + slabs - 1) / slabs;
    slabs = (rows + per - 1) / per;
    for (int s = 0; s < slabs; ++s) {
        PointArgs a = args;
        const long long r0 = (long long)s * per, r1 = std::min<long long>(rows, r0 + per);
        a.base = (unsigned)(r0 * row);
        a.total = (r1 - r0) * row;
        if (!cuda_ok(launch_points(prog, a, ctx->dbuf + a.base, work, sc->dmm + 2 * s, ctx->stream), "launch") ||
            !cuda_ok(cudaEventRecord(sc->done[s], ctx->stream), "record"))
            return false;
    }
    for (int s = 0; s < slabs; ++s) {
        const long long r0 = (long long)s * per, r1 = std::min<long long>(rows, r0 + per);
        if (!cuda_ok(cudaStreamWaitEvent(sc->copy, sc->done[s], 0), "wait") ||
            !copy_to_host(out + r0 * row, ctx->dbuf + r0 * row, (size_t)((r1 - r0) * row) * 4, sc->copy))
            return false;
    }
    if (!cuda_ok(cudaMemcpyAsync(sc->hmm, sc->dmm, 2 * slabs * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream), "copy minmax") ||
        !cuda_ok(cudaStreamSynchronize(sc->copy), "synchronize") || !cuda_ok(cudaStreamSynchronize(ctx->stream), "synchronize"))
        return false;
    float mn = std::numeric_limits<float>::infinity(), mx = -mn;
    for (int s = 0; s < slabs; ++s) {
        mn = mn < sc->hmm[2 * s] ? mn : sc->hmm[2 * s];
        mx = mx > sc->hmm[2 * s + 1] ? mx : sc->hmm[2 * s + 1];
    }
    store_minmax(minmax, mn, mx);
    return true;
}

void gen_host(const void* node, PointArgs args, float* out, float* minmax, const float* const* hpos)
{
    clear_error();
    const long long total = args.total;
    if (!node || total < 0 || (total > 0 && !out)) { set_error(FN_ERR_ARG, "invalid arguments"); fill_nan(out, total > 0 ? total : 0, minmax); return; }
    ThreadCtx* ctx = thread_ctx();
    DeviceProgram prog;
    if (!ctx || !get_program(N(node), args.dim, prog) || !ensure_runnable(prog)) { fill_nan(out, total, minmax); return; }
    MinMaxWork* work = work_for_stream(ctx->stream);
    // Host outputs the device can store into (page-locked memory; any host memory on devices
    // with coherent pageable access): the kernel stores into them directly.  One tree's kernel
    // produces output slower than the host link carries it, so the stores overlap the
    // generation; there is no device buffer, no copy and no slab pipeline to fill and drain.
    float* direct = total > 0 ? host_direct_view(out, (size_t)total * 4) : nullptr;
    if (!work || (!direct && !ensure(ctx->dbuf, ctx->dbuf_cap, (size_t)total))) { fill_nan(out, total, minmax); return; }
    // Position arrays the device can read in place (the same rule as for outputs) are not copied.
    bool pos_direct = args.src == kSrcPositions && total > 0;
    for (int k = 0; pos_direct && k < args.dim; ++k) {
        const float* v = hpos[k] ? host_direct_view(const_cast<float*>(hpos[k]), (size_t)total * 4) : nullptr;
        pos_direct = v != nullptr;
        args.pos[k] = v;
    }
    if (args.src == kSrcPositions && total > 0 && !pos_direct) {
        if ((size_t)total > ctx->dpos_cap) {
            for (float*& p : ctx->dpos) { if (p) cudaFree(p); p = nullptr; }
            ctx->dpos_cap = 0;
            for (int k = 0; k < 4; ++k)      // all four axes, so any dimensionality fits
                if (!cuda_ok(cudaMalloc(&ctx->dpos[k], (size_t)total * 4), "cudaMalloc(positions)")) { fill_nan(out, total, minmax); return; }
            ctx->dpos_cap = (size_t)total;
        }
        for (int k = 0; k < args.dim; ++k) {
            if (!hpos[k]) { set_error(FN_ERR_ARG, "null position array"); fill_nan(out, total, minmax); return; }
            if (!copy_host(hpos[k], ctx->dpos[k], (size_t)total * 4, false, ctx->stream, "copy positions")) {
                fill_nan(out, total, minmax);
                return;
            }
            args.pos[k] = ctx->dpos[k];
        }
    }
    if (!direct && args.src == kSrcGrid && total >= 2 * kSlabMinPoints && total < (1ll << 32)) {
        if (!gen_host_slabs(prog, args, ctx, work, out, minmax)) fill_nan(out, total, minmax);
        return;
    }
    // the kernel's last block stores the min/max straight into pinned host memory when it can
    if (!cuda_ok(launch_points(prog, args, direct ? direct : ctx->dbuf, work, ctx->hminmax_dev, ctx->stream), "launch")) {
        fill_nan(out, total, minmax);
        return;
    }
    if (!direct && total > 0 && !copy_to_host(out, ctx->dbuf, (size_t)total * 4, ctx->stream)) { fill_nan(out, total, minmax); return; }
    if ((!ctx->hminmax_dev &&
         !cuda_ok(cudaMemcpyAsync(ctx->hminmax, work->result, 8, cudaMemcpyDeviceToHost, ctx->stream), "copy minmax")) ||
        !cuda_ok(cudaStreamSynchronize(ctx->stream), "synchronize")) {
        fill_nan(out, total, minmax);
        return;
    }
    store_minmax(minmax, ctx->hminmax[0], ctx->hminmax[1]);
}

int gen_device(const void* node, PointArgs args, float* dout, float* dminmax, void* stream)
{
    clear_error();
    if (!node || args.total < 0 || (args.total > 0 && !dout)) { set_error(FN_ERR_ARG, "invalid arguments"); return FN_ERR_ARG; }
    if (!thread_ctx()) return FN_ERR_CUDA;
    DeviceProgram prog;
    if (!get_program(N(node), args.dim, prog)) return last_error();
    if (!ensure_runnable(prog)) return FN_ERR_COMPILE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    MinMaxWork* work = work_for_stream(s);
    if (!work) return FN_ERR_CUDA;
    if (!cuda_ok(launch_points(prog, args, dout, work, dminmax, s), "launch")) return FN_ERR_CUDA;
    return FN_OK;
}

// Magic numbers for dividing 32-bit point indices by count (PointArgs::divm/divs):
// s = ceil(log2 count), m = 2^32 (2^s - count) / count + 1; count 1 gives s = 0.
void set_divisor(PointArgs& a, int k, int count)
{
    const uint64_t d = count > 0 ? (uint64_t)count : 1u;
    if (d == 1) { a.divm[k] = 0; a.divs[k] = 0; return; }
    unsigned s = 0;
    while ((1ull << s) < d) ++s;
    a.divm[k] = (unsigned)(((1ull << 32) * ((1ull << s) - d)) / d + 1);
    a.divs[k] = s;
}

PointArgs grid_args(int dim, const float* off, const int* cnt, const float* step, int seed)
{
    PointArgs a;
    std::memset(&a, 0, sizeof a);
    a.src = kSrcGrid;
    a.dim = dim;
    a.seed = seed;
    long long total = 1;
    for (int k = 0; k < dim; ++k) {
        a.count[k] = cnt[k];
        a.offset[k] = off[k];
        a.step[k] = step[k];
        total *= cnt[k] > 0 ? cnt[k] : 0;
        if (k < 3) set_divisor(a, k, cnt[k]);
    }
    a.total = total;
    return a;
}

PointArgs tile_args(int xSize, int ySize, float xStep, float yStep, int seed)
{
    PointArgs a;
    std::memset(&a, 0, sizeof a);
    a.src = kSrcTileable;
    a.dim = 4;
    a.seed = seed;
    a.count[0] = xSize;
    a.count[1] = ySize;
    const float pi2Recip = 0.15915493667f;                    // Generator.inl:386-392
    const float xSizePi = (float)xSize * pi2Recip;
    const float ySizePi = (float)ySize * pi2Recip;
    a.tfreq[0] = xSizePi * xStep;
    a.tfreq[1] = ySizePi * yStep;
    a.tmul[0] = 1 / xSizePi;
    a.tmul[1] = 1 / ySizePi;
    a.total = (long long)(xSize > 0 ? xSize : 0) * (ySize > 0 ? ySize : 0);
    set_divisor(a, 0, xSize);
    return a;
}

PointArgs pos_args(int dim, int count, const float* off, int seed)
{
    PointArgs a;
    std::memset(&a, 0, sizeof a);
    a.src = kSrcPositions;
    a.dim = dim;
    a.seed = seed;
    a.total = count > 0 ? count : 0;
    for (int k = 0; k < dim; ++k) a.offset[k] = off[k];
    return a;
}

float gen_single(const void* node, int dim, const float* p, int seed)
{
    const int cnt[4] = {1, 1, 1, 1};
    const float step[4] = {0, 0, 0, 0};
    float out = 0.0f;
    gen_host(node, grid_args(dim, p, cnt, step, seed), &out, nullptr, nullptr);   // fma(0, 0, p) == p
    return out;
}

const NodeMeta* M(int id) { return meta_by_id(id); }

// ------------------------------------------------------------------ batches

bool request_args(const fnGenRequest& r, PointArgs& a)
{
    switch (r.kind) {
    case FN_KIND_GRID2D: case FN_KIND_GRID3D: case FN_KIND_GRID4D:
        a = grid_args(2 + (r.kind - FN_KIND_GRID2D), r.offset, r.count, r.step, r.seed);
        return true;
    case FN_KIND_TILEABLE2D:
        a = tile_args(r.count[0], r.count[1], r.step[0], r.step[1], r.seed);
        return true;
    case FN_KIND_POSITIONS2D: case FN_KIND_POSITIONS3D: case FN_KIND_POSITIONS4D: {
        const int dim = 2 + (r.kind - FN_KIND_POSITIONS2D);
        a = pos_args(dim, r.count[0], r.offset, r.seed);
        for (int k = 0; k < dim; ++k) {
            if (a.total > 0 && !r.positions[k]) return false;
            a.pos[k] = r.positions[k];
        }
        return true;
    }
    default:
        return false;
    }
}

struct BatchCtx {
    BatchRunner runner;
    float* dminmax = nullptr;
    float* hminmax = nullptr;
    size_t cap = 0;
    ~BatchCtx()
    {
        if (dminmax) cudaFree(dminmax);
        if (hminmax) cudaFreeHost(hminmax);
    }
};
thread_local BatchCtx* t_batch = nullptr;

// Size `b`'s min/max buffers for n requests.
bool reserve_batch(BatchCtx* b, size_t n)
{
    if (n > b->cap) {
        if (b->dminmax) cudaFree(b->dminmax);
        if (b->hminmax) cudaFreeHost(b->hminmax);
        b->dminmax = nullptr; b->hminmax = nullptr; b->cap = 0;
        size_t want = n < 256 ? 256 : n;
        if (!cuda_ok(cudaMalloc(&b->dminmax, want * 2 * sizeof(float)), "cudaMalloc(batch minmax)") ||
            !cuda_ok(cudaMallocHost(&b->hminmax, want * 2 * sizeof(float)), "cudaMallocHost(batch minmax)"))
            return false;
        b->cap = want;
    }
    return true;
}

BatchCtx* batch_ctx(size_t n)
{
    if (!t_batch) t_batch = new BatchCtx();
    return reserve_batch(t_batch, n) ? t_batch : nullptr;
}

int build_items(const fnGenRequest* reqs, int n, BatchCtx* b, std::vector<BatchItem>& items)
{
    items.resize((size_t)n);
    for (int i = 0; i < n; ++i) {
        BatchItem& it = items[(size_t)i];
        it.node = N(reqs[i].node);
        if (!it.node || !request_args(reqs[i], it.args)) {
            set_error(FN_ERR_ARG, "batch request " + std::to_string(i) + ": invalid node, kind or positions");
            return FN_ERR_ARG;
        }
        it.dout = reqs[i].out;
        it.dminmax = b->dminmax + 2 * i;
    }
    return FN_OK;
}

// One batch launch on `stream` with the runner and buffers of `b` (b == nullptr: this
// thread's context).
int run_batch(const fnGenRequest* reqs, int n, void* stream, int flags, const BatchTuning* tuning, BatchCtx* b = nullptr)
{
    if (n < 0 || (n > 0 && !reqs)) { set_error(FN_ERR_ARG, "invalid request list"); return FN_ERR_ARG; }
    if (n == 0) return FN_OK;
    if (!thread_ctx()) return FN_ERR_CUDA;
    if (b ? !reserve_batch(b, (size_t)n) : !(b = batch_ctx((size_t)n))) return FN_ERR_CUDA;
    std::vector<BatchItem> items;
    int rc = build_items(reqs, n, b, items);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    rc = b->runner.launch(items, s, tuning, !(flags & FN_BATCH_NO_GRAPH));
    if (rc) return rc;
    if (flags & FN_BATCH_SYNC) {
        if (!cuda_ok(cudaMemcpyAsync(b->hminmax, b->dminmax, (size_t)n * 2 * sizeof(float), cudaMemcpyDeviceToHost, s), "copy minmax") ||
            !cuda_ok(cudaStreamSynchronize(s), "synchronize"))
            return FN_ERR_CUDA;
        for (int i = 0; i < n; ++i)
            if (reqs[i].minMax) { reqs[i].minMax[0] = b->hminmax[2 * i]; reqs[i].minMax[1] = b->hminmax[2 * i + 1]; }
    }
    return FN_OK;
}

// Host-output batches: two device staging buffers, the requests cut into slices that fit one;
// slice k is generated on gen[k % 2] into buffer k % 2 while slice k - 1 is copied to the host
// on `copy`, so the copy engine and the SMs work at the same time.  The two generation streams
// have their own batch runners, so consecutive slices also overlap each other's kernel tails.
// Slices start small (the first copy starts early) and shrink again at the end (little is left
// to copy after the last generation).  Slices are launched without graphs: each has its own
// shape.
constexpr size_t kHostSlicePoints = size_t(1) << 25;       // 128 MB of output per staging buffer
constexpr size_t kHostSliceMin = size_t(1) << 23;

size_t host_slice_cap(int k, size_t remaining)
{
    size_t cap = std::min(kHostSlicePoints, kHostSliceMin << std::min(k, 8));
    if (remaining <= 2 * kHostSlicePoints) cap = std::min(cap, std::max(kHostSliceMin, remaining / 2));
    return cap;
}

struct HostBatchCtx {
    cudaStream_t gen[2] = {}, copy = nullptr;   // slice k is generated on gen[k % 2]
    BatchCtx lane[2];                            // with its own batch runner and buffers
    cudaEvent_t gen_done[2] = {}, copy_done[2] = {};
    float* stage[2] = {};
    size_t stage_cap = 0;                  // floats per staging buffer
    float* hmm = nullptr;                  // pinned: min/max of every request
    size_t hmm_cap = 0;
    fnBatchInfo info{};                    // summed over the slices of the last call
    bool info_valid = false;
    ~HostBatchCtx()
    {
        for (int k = 0; k < 2; ++k) {
            if (stage[k]) cudaFree(stage[k]);
            if (gen_done[k]) cudaEventDestroy(gen_done[k]);
            if (copy_done[k]) cudaEventDestroy(copy_done[k]);
        }
        if (hmm) cudaFreeHost(hmm);
        for (int k = 0; k < 2; ++k)
            if (gen[k]) cudaStreamDestroy(gen[k]);
        if (copy) cudaStreamDestroy(copy);
    }
};
thread_local HostBatchCtx* t_hbatch = nullptr;

// Add one launch of `r` (over `requests` requests) to the summary of a host batch call.
void add_launch(fnBatchInfo& info, const BatchRunner& r, int requests)
{
    info.requests += requests;
    info.specialised = r.last_specialised() ? 1 : 0;
    info.tilePoints = (int)r.last_tile_points();
    info.ctas = r.last_grid();
    info.workItems += r.last_items();
    info.points += r.last_points();
    info.uploadBytes += r.last_upload_bytes();
    info.kernels += r.last_kernels();
}

HostBatchCtx* host_batch_ctx(size_t stage_floats, size_t requests)
{
    if (!t_hbatch) {
        HostBatchCtx* h = new HostBatchCtx();
        bool ok = cuda_ok(cudaStreamCreateWithFlags(&h->gen[0], cudaStreamNonBlocking), "stream") &&
                  cuda_ok(cudaStreamCreateWithFlags(&h->gen[1], cudaStreamNonBlocking), "stream") &&
                  cuda_ok(cudaStreamCreateWithFlags(&h->copy, cudaStreamNonBlocking), "stream");
        for (int k = 0; ok && k < 2; ++k)
            ok = cuda_ok(cudaEventCreateWithFlags(&h->gen_done[k], cudaEventDisableTiming), "event") &&
                 cuda_ok(cudaEventCreateWithFlags(&h->copy_done[k], cudaEventDisableTiming), "event");
        if (!ok) { delete h; return nullptr; }
        t_hbatch = h;
    }
    HostBatchCtx* h = t_hbatch;
    if (stage_floats > h->stage_cap) {
        for (int k = 0; k < 2; ++k) {
            if (h->stage[k]) cudaFree(h->stage[k]);
            h->stage[k] = nullptr;
        }
        h->stage_cap = 0;
        for (int k = 0; k < 2; ++k)
            if (!cuda_ok(cudaMalloc(&h->stage[k], stage_floats * sizeof(float)), "cudaMalloc(host batch staging)")) return nullptr;
        h->stage_cap = stage_floats;
    }
    if (2 * requests > h->hmm_cap) {
        if (h->hmm) cudaFreeHost(h->hmm);
        h->hmm = nullptr;
        h->hmm_cap = 0;
        if (!cuda_ok(cudaMallocHost(&h->hmm, 2 * requests * sizeof(float)), "cudaMallocHost(host batch minmax)")) return nullptr;
        h->hmm_cap = 2 * requests;
    }
    return h;
}

}  // namespace capi
}  // namespace fn

using namespace fn::capi;

extern "C" {

// ------------------------------------------------------------------ lifetime

void* fnNewFromEncodedNodeTree(const char* encodedString, unsigned)
{
    return decode_tree(encodedString);
}

void fnDeleteNodeRef(void* node)
{
    if (node) node_unref(N(node));
}

unsigned fnGetActiveFeatureSet(const void*) { return FN_GB300_FEATURE_SET; }

int fnGetMetadataID(const void* node) { return node ? N(node)->meta->id : -1; }

// ------------------------------------------------------------------ generation (host memory)

void fnGenUniformGrid2D(const void* node, float* noiseOut, float xOffset, float yOffset, int xCount, int yCount,
                        float xStepSize, float yStepSize, int seed, float* outputMinMax)
{
    const float off[2] = {xOffset, yOffset};
    const int cnt[2] = {xCount, yCount};
    const float st[2] = {xStepSize, yStepSize};
    gen_host(node, grid_args(2, off, cnt, st, seed), noiseOut, outputMinMax, nullptr);
}

void fnGenUniformGrid3D(const void* node, float* noiseOut, float xOffset, float yOffset, float zOffset, int xCount,
                        int yCount, int zCount, float xStepSize, float yStepSize, float zStepSize, int seed,
                        float* outputMinMax)
{
    const float off[3] = {xOffset, yOffset, zOffset};
    const int cnt[3] = {xCount, yCount, zCount};
    const float st[3] = {xStepSize, yStepSize, zStepSize};
    gen_host(node, grid_args(3, off, cnt, st, seed), noiseOut, outputMinMax, nullptr);
}

void fnGenUniformGrid4D(const void* node, float* noiseOut, float xOffset, float yOffset, float zOffset, float wOffset,
                        int xCount, int yCount, int zCount, int wCount, float xStepSize, float yStepSize,
                        float zStepSize, float wStepSize, int seed, float* outputMinMax)
{
    const float off[4] = {xOffset, yOffset, zOffset, wOffset};
    const int cnt[4] = {xCount, yCount, zCount, wCount};
    const float st[4] = {xStepSize, yStepSize, zStepSize, wStepSize};
    gen_host(node, grid_args(4, off, cnt, st, seed), noiseOut, outputMinMax, nullptr);
}

void fnGenPositionArray2D(const void* node, float* noiseOut, int count, const float* xPosArray, const float* yPosArray,
                          float xOffset, float yOffset, int seed, float* outputMinMax)
{
    const float off[2] = {xOffset, yOffset};
    const float* p[4] = {xPosArray, yPosArray, nullptr, nullptr};
    gen_host(node, pos_args(2, count, off, seed), noiseOut, outputMinMax, p);
}

void fnGenPositionArray3D(const void* node, float* noiseOut, int count, const float* xPosArray, const float* yPosArray,
                          const float* zPosArray, float xOffset, float yOffset, float zOffset, int seed,
                          float* outputMinMax)
{
    const float off[3] = {xOffset, yOffset, zOffset};
    const float* p[4] = {xPosArray, yPosArray, zPosArray, nullptr};
    gen_host(node, pos_args(3, count, off, seed), noiseOut, outputMinMax, p);
}

void fnGenPositionArray4D(const void* node, float* noiseOut, int count, const float* xPosArray, const float* yPosArray,
                          const float* zPosArray, const float* wPosArray, float xOffset, float yOffset, float zOffset,
                          float wOffset, int seed, float* outputMinMax)
{
    const float off[4] = {xOffset, yOffset, zOffset, wOffset};
    const float* p[4] = {xPosArray, yPosArray, zPosArray, wPosArray};
    gen_host(node, pos_args(4, count, off, seed), noiseOut, outputMinMax, p);
}

void fnGenTileable2D(const void* node, float* noiseOut, int xSize, int ySize, float xStepSize, float yStepSize, int seed,
                     float* outputMinMax)
{
    gen_host(node, tile_args(xSize, ySize, xStepSize, yStepSize, seed), noiseOut, outputMinMax, nullptr);
}

float fnGenSingle2D(const void* node, float x, float y, int seed)
{
    const float p[2] = {x, y};
    return gen_single(node, 2, p, seed);
}

float fnGenSingle3D(const void* node, float x, float y, float z, int seed)
{
    const float p[3] = {x, y, z};
    return gen_single(node, 3, p, seed);
}

float fnGenSingle4D(const void* node, float x, float y, float z, float w, int seed)
{
    const float p[4] = {x, y, z, w};
    return gen_single(node, 4, p, seed);
}

// ------------------------------------------------------------------ metadata (FastNoise_C.cpp:117-476)

int fnGetMetadataCount(void) { return (int)all_meta().size(); }

const char* fnGetMetadataName(int id)
{
    const NodeMeta* m = M(id);
    return m ? m->name : "INVALID NODE ID";
}

void* fnNewFromMetadata(int id, unsigned)
{
    return node_new(id);
}

int fnGetMetadataVariableCount(int id)
{
    const NodeMeta* m = M(id);
    return m ? (int)m->vars.size() : -1;
}

const char* fnGetMetadataVariableName(int id, int i)
{
    const NodeMeta* m = M(id);
    if (!m) return "INVALID NODE ID";
    return (size_t)i < m->vars.size() ? m->vars[i].name : "INVALID VARIABLE INDEX";
}

int fnGetMetadataVariableType(int id, int i)
{
    const NodeMeta* m = M(id);
    return (m && (size_t)i < m->vars.size()) ? (int)m->vars[i].type : -1;
}

int fnGetMetadataVariableDimensionIdx(int id, int i)
{
    const NodeMeta* m = M(id);
    return (m && (size_t)i < m->vars.size()) ? m->vars[i].dim : -1;
}

int fnGetMetadataEnumCount(int id, int i)
{
    const NodeMeta* m = M(id);
    return (m && (size_t)i < m->vars.size()) ? (int)m->vars[i].enums.size() : -1;
}

const char* fnGetMetadataEnumName(int id, int i, int e)
{
    const NodeMeta* m = M(id);
    if (!m) return "INVALID NODE ID";
    if ((size_t)i >= m->vars.size()) return "INVALID VARIABLE INDEX";
    return (size_t)e < m->vars[i].enums.size() ? m->vars[i].enums[e] : "INVALID ENUM INDEX";
}

bool fnSetVariableFloat(void* node, int i, float value)
{
    return node && N(node)->set_var(i, bits_of(value));      // ValueUnion(float)
}

bool fnSetVariableIntEnum(void* node, int i, int value)
{
    return node && N(node)->set_var(i, value);               // ValueUnion(int)
}

int fnGetMetadataNodeLookupCount(int id)
{
    const NodeMeta* m = M(id);
    return m ? (int)m->lookups.size() : -1;
}

const char* fnGetMetadataNodeLookupName(int id, int i)
{
    const NodeMeta* m = M(id);
    if (!m) return "INVALID NODE ID";
    return (size_t)i < m->lookups.size() ? m->lookups[i].name : "INVALID NODE LOOKUP INDEX";
}

int fnGetMetadataNodeLookupDimensionIdx(int id, int i)
{
    const NodeMeta* m = M(id);
    return (m && (size_t)i < m->lookups.size()) ? m->lookups[i].dim : -1;
}

bool fnSetNodeLookup(void* node, int i, const void* lookup)
{
    return node && N(node)->set_lookup(i, const_cast<Node*>(N(lookup)));
}

int fnGetMetadataHybridCount(int id)
{
    const NodeMeta* m = M(id);
    return m ? (int)m->hybrids.size() : -1;
}

const char* fnGetMetadataHybridName(int id, int i)
{
    const NodeMeta* m = M(id);
    if (!m) return "INVALID NODE ID";
    return (size_t)i < m->hybrids.size() ? m->hybrids[i].name : "INVALID HYBRID INDEX";
}

int fnGetMetadataHybridDimensionIdx(int id, int i)
{
    const NodeMeta* m = M(id);
    return (m && (size_t)i < m->hybrids.size()) ? m->hybrids[i].dim : -1;
}

bool fnSetHybridNodeLookup(void* node, int i, const void* lookup)
{
    return node && N(node)->set_hybrid_node(i, const_cast<Node*>(N(lookup)));
}

bool fnSetHybridFloat(void* node, int i, float value)
{
    return node && N(node)->set_hybrid_float(i, value);
}

const char* fnGetMetadataDescription(int id)
{
    const NodeMeta* m = M(id);
    return m ? m->description : "INVALID NODE ID";
}

int fnGetMetadataGroupCount(int id)
{
    const NodeMeta* m = M(id);
    return m ? (int)m->groups.size() : -1;
}

const char* fnGetMetadataGroupName(int id, int g)
{
    const NodeMeta* m = M(id);
    if (!m) return "INVALID NODE ID";
    return (size_t)g < m->groups.size() ? m->groups[g] : "INVALID GROUP INDEX";
}

const char* fnGetMetadataVariableDescription(int id, int i)
{
    const NodeMeta* m = M(id);
    if (!m) return "INVALID NODE ID";
    return (size_t)i < m->vars.size() ? m->vars[i].description : "INVALID VARIABLE INDEX";
}

float fnGetMetadataVariableDefaultFloat(int id, int i)
{
    const NodeMeta* m = M(id);
    return (m && (size_t)i < m->vars.size()) ? f_of(m->vars[i].def) : 0.0f;
}

int fnGetMetadataVariableDefaultIntEnum(int id, int i)
{
    const NodeMeta* m = M(id);
    return (m && (size_t)i < m->vars.size()) ? m->vars[i].def : 0;
}

float fnGetMetadataVariableMinFloat(int id, int i)
{
    const NodeMeta* m = M(id);
    return (m && (size_t)i < m->vars.size()) ? f_of(m->vars[i].vmin) : 0.0f;
}

float fnGetMetadataVariableMaxFloat(int id, int i)
{
    const NodeMeta* m = M(id);
    return (m && (size_t)i < m->vars.size()) ? f_of(m->vars[i].vmax) : 0.0f;
}

const char* fnGetMetadataNodeLookupDescription(int id, int i)
{
    const NodeMeta* m = M(id);
    if (!m) return "INVALID NODE ID";
    return (size_t)i < m->lookups.size() ? m->lookups[i].description : "INVALID NODE LOOKUP INDEX";
}

const char* fnGetMetadataHybridDescription(int id, int i)
{
    const NodeMeta* m = M(id);
    if (!m) return "INVALID NODE ID";
    return (size_t)i < m->hybrids.size() ? m->hybrids[i].description : "INVALID HYBRID INDEX";
}

float fnGetMetadataHybridDefault(int id, int i)
{
    const NodeMeta* m = M(id);
    return (m && (size_t)i < m->hybrids.size()) ? m->hybrids[i].def : 0.0f;
}

// ------------------------------------------------------------------ additions

int fnGetLastError(void) { return last_error(); }
const char* fnGetLastErrorString(void) { return last_error_string(); }

int fnSerialiseNodeTree(const void* node, char* buffer, int bufferSize)
{
    clear_error();
    if (!node) { set_error(FN_ERR_ARG, "null node"); return FN_ERR_ARG; }
    std::string s = encode_tree(N(node));
    if (s.empty()) { set_error(FN_ERR_ARG, "tree has an unset source"); return FN_ERR_ARG; }
    if (buffer && bufferSize > (int)s.size()) std::memcpy(buffer, s.c_str(), s.size() + 1);
    return (int)s.size();
}

int fnGetVariableBits(const void* node, int variableIndex, int* bits)
{
    clear_error();
    if (!node || !bits) { set_error(FN_ERR_ARG, "null node or output"); return FN_ERR_ARG; }
    const Node* n = N(node);
    if (variableIndex < 0 || variableIndex >= (int)n->vars.size()) { set_error(FN_ERR_ARG, "variable index out of range"); return FN_ERR_ARG; }
    *bits = n->vars[variableIndex];
    return FN_OK;
}

void* fnGetNodeLookupRef(const void* node, int nodeLookupIndex)
{
    if (!node) return nullptr;
    const Node* n = N(node);
    if (nodeLookupIndex < 0 || nodeLookupIndex >= (int)n->lookups.size()) return nullptr;
    Node* c = n->lookups[nodeLookupIndex];
    node_ref(c);
    return c;
}

void* fnGetHybridNodeLookupRef(const void* node, int hybridIndex)
{
    if (!node) return nullptr;
    const Node* n = N(node);
    if (hybridIndex < 0 || hybridIndex >= (int)n->hnodes.size()) return nullptr;
    Node* c = n->hnodes[hybridIndex];
    node_ref(c);
    return c;
}

int fnGetHybridFloat(const void* node, int hybridIndex, float* value)
{
    clear_error();
    if (!node || !value) { set_error(FN_ERR_ARG, "null node or output"); return FN_ERR_ARG; }
    const Node* n = N(node);
    if (hybridIndex < 0 || hybridIndex >= (int)n->hvals.size()) { set_error(FN_ERR_ARG, "hybrid index out of range"); return FN_ERR_ARG; }
    *value = n->hvals[hybridIndex];
    return FN_OK;
}

int fnGenBatchDevice(const fnGenRequest* requests, int count, void* stream, int flags)
{
    clear_error();
    if (t_hbatch) t_hbatch->info_valid = false;
    return run_batch(requests, count, stream, flags, nullptr);
}

int fnGenBatchHost(const fnGenRequest* requests, int count, int flags)
{
    (void)flags;
    clear_error();
    if (count < 0 || (count > 0 && !requests)) { set_error(FN_ERR_ARG, "invalid request list"); return FN_ERR_ARG; }
    if (count == 0) return FN_OK;
    if (!thread_ctx()) return FN_ERR_CUDA;
    std::vector<size_t> points((size_t)count);
    size_t largest = 0;
    for (int i = 0; i < count; ++i) {
        PointArgs a;
        if (!requests[i].node || !request_args(requests[i], a) || a.total < 0 || (a.total > 0 && !requests[i].out)) {
            set_error(FN_ERR_ARG, "invalid request " + std::to_string(i));
            return FN_ERR_ARG;
        }
        points[(size_t)i] = (size_t)a.total;
        largest = std::max(largest, points[(size_t)i]);
    }
    // Outputs in ordinary (pageable, resident) memory on a device that stores into it coherently:
    // the batch kernels store into them directly.  Copies into pageable memory run at about half
    // the speed of copies into page-locked memory (the chunk mix: 18.1 ms staged, 13.5 ms direct;
    // into page-locked memory staging stays faster, 9.5 ms).  Checked per run of requests whose
    // outputs are contiguous, for at most 256 runs.
    bool direct = host_direct_allowed();
    int runs = 0;
    for (int j = 0; direct && j < count;) {
        if (!points[(size_t)j]) { ++j; continue; }
        float* dst = requests[j].out;
        size_t n = points[(size_t)j];
        int e = j + 1;
        while (e < count && (!points[(size_t)e] || requests[e].out == dst + n)) n += points[(size_t)e++];
        direct = ++runs <= 256 && pageable_direct(dst, n * sizeof(float));
        j = e;
    }
    const size_t cap = std::max(kHostSlicePoints, largest);
    HostBatchCtx* h = host_batch_ctx(direct ? 0 : cap, (size_t)count);
    if (!h) return FN_ERR_CUDA;
    h->info = fnBatchInfo{};
    h->info_valid = false;
    if (direct) {
        std::vector<fnGenRequest> dreqs(requests, requests + count);
        for (auto& r : dreqs) r.minMax = nullptr;
        BatchCtx* lane = &h->lane[0];
        const int rc = run_batch(dreqs.data(), count, h->gen[0], 0, nullptr, lane);
        if (rc) return rc;
        add_launch(h->info, lane->runner, count);
        if (!cuda_ok(cudaMemcpyAsync(h->hmm, lane->dminmax, (size_t)count * 2 * sizeof(float), cudaMemcpyDeviceToHost, h->gen[0]),
                     "copy minmax") ||
            !cuda_ok(cudaStreamSynchronize(h->gen[0]), "synchronize"))
            return FN_ERR_CUDA;
        for (int i = 0; i < count; ++i)
            if (requests[i].minMax) { requests[i].minMax[0] = h->hmm[2 * i]; requests[i].minMax[1] = h->hmm[2 * i + 1]; }
        h->info_valid = true;
        return FN_OK;
    }
    std::vector<fnGenRequest> slice;
    size_t remaining = 0;
    for (size_t p : points) remaining += p;
    int k = 0;
    for (int i0 = 0; i0 < count; ++k) {
        const int buf = k & 1;
        const size_t want = host_slice_cap(k, remaining);
        size_t used = 0;
        int i1 = i0;
        while (i1 < count && (i1 == i0 || used + points[(size_t)i1] <= want)) used += points[(size_t)i1++];
        remaining -= used;
        slice.assign(requests + i0, requests + i1);
        size_t off = 0;
        for (size_t j = 0; j < slice.size(); ++j) {
            slice[j].out = h->stage[buf] + off;
            slice[j].minMax = nullptr;
            off += points[(size_t)i0 + j];
        }
        // buffer `buf` is free once the copy of slice k - 2 is done; slices k and k + 1 run on
        // different streams with their own runners, so one slice's kernel tails overlap the next
        cudaStream_t gen = h->gen[buf];
        BatchCtx* lane = &h->lane[buf];
        if (!cuda_ok(cudaStreamWaitEvent(gen, h->copy_done[buf], 0), "wait")) return FN_ERR_CUDA;
        const int rc = run_batch(slice.data(), (int)slice.size(), gen, FN_BATCH_NO_GRAPH, nullptr, lane);
        if (rc) return rc;
        add_launch(h->info, lane->runner, (int)slice.size());
        if (!cuda_ok(cudaMemcpyAsync(h->hmm + 2 * (size_t)i0, lane->dminmax, slice.size() * 2 * sizeof(float),
                                     cudaMemcpyDeviceToHost, gen), "copy minmax") ||
            !cuda_ok(cudaEventRecord(h->gen_done[buf], gen), "record") ||
            !cuda_ok(cudaStreamWaitEvent(h->copy, h->gen_done[buf], 0), "wait"))
            return FN_ERR_CUDA;
        // one copy per run of requests whose host outputs are contiguous
        size_t src = 0;
        for (int j = i0; j < i1;) {
            float* dst = requests[j].out;
            size_t n = points[(size_t)j];
            int e = j + 1;
            while (e < i1 && points[(size_t)e] && requests[e].out == dst + n) n += points[(size_t)e++];
            if (n && !copy_to_host(dst, h->stage[buf] + src, n * sizeof(float), h->copy)) return FN_ERR_CUDA;
            src += n;
            j = e;
        }
        if (!cuda_ok(cudaEventRecord(h->copy_done[buf], h->copy), "record")) return FN_ERR_CUDA;
        i0 = i1;
    }
    if (!cuda_ok(cudaStreamSynchronize(h->copy), "synchronize") || !cuda_ok(cudaStreamSynchronize(h->gen[0]), "synchronize") ||
        !cuda_ok(cudaStreamSynchronize(h->gen[1]), "synchronize"))
        return FN_ERR_CUDA;
    for (int i = 0; i < count; ++i)
        if (requests[i].minMax) { requests[i].minMax[0] = h->hmm[2 * i]; requests[i].minMax[1] = h->hmm[2 * i + 1]; }
    h->info_valid = true;
    return FN_OK;
}

int fnGenEachDevice(const fnGenRequest* requests, int count, void* stream, int flags)
{
    clear_error();
    if (count < 0 || (count > 0 && !requests)) { set_error(FN_ERR_ARG, "invalid request list"); return FN_ERR_ARG; }
    if (count == 0) return FN_OK;
    if (!thread_ctx()) return FN_ERR_CUDA;
    BatchCtx* b = batch_ctx((size_t)count);
    if (!b) return FN_ERR_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    for (int i = 0; i < count; ++i) {
        PointArgs a;
        if (!requests[i].node || !request_args(requests[i], a)) { set_error(FN_ERR_ARG, "invalid request"); return FN_ERR_ARG; }
        int rc = gen_device(requests[i].node, a, requests[i].out, b->dminmax + 2 * i, stream);
        if (rc) return rc;
    }
    if (flags & FN_BATCH_SYNC) {
        if (!cuda_ok(cudaMemcpyAsync(b->hminmax, b->dminmax, (size_t)count * 2 * sizeof(float), cudaMemcpyDeviceToHost, s), "copy minmax") ||
            !cuda_ok(cudaStreamSynchronize(s), "synchronize"))
            return FN_ERR_CUDA;
        for (int i = 0; i < count; ++i)
            if (requests[i].minMax) { requests[i].minMax[0] = b->hminmax[2 * i]; requests[i].minMax[1] = b->hminmax[2 * i + 1]; }
    }
    return FN_OK;
}

int fnGenEachPaced(const fnGenRequest* requests, int count, const double* arrivalMicros, void* stream,
                   double* latencyMicros)
{
    clear_error();
    if (count < 0 || (count > 0 && (!requests || !arrivalMicros))) { set_error(FN_ERR_ARG, "invalid request list"); return FN_ERR_ARG; }
    if (count == 0) return FN_OK;
    std::vector<PointArgs> args((size_t)count);
    for (int i = 0; i < count; ++i)
        if (!requests[i].node || !request_args(requests[i], args[i])) { set_error(FN_ERR_ARG, "invalid request"); return FN_ERR_ARG; }
    if (!thread_ctx()) return FN_ERR_CUDA;
    BatchCtx* b = batch_ctx((size_t)count);
    if (!b) return FN_ERR_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int dev = 0;
    cudaGetDevice(&dev);
    std::vector<cudaEvent_t> ev((size_t)count, nullptr);
    for (auto& e : ev)
        if (!cuda_ok(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event")) {
            for (auto& x : ev) if (x) cudaEventDestroy(x);
            return FN_ERR_CUDA;
        }
    using clock = std::chrono::steady_clock;
    std::vector<clock::time_point> done((size_t)count);
    std::atomic<int> issued{0};
    std::atomic<int> stop{0};
    const clock::time_point start = clock::now();
    // completion side: requests finish in stream order, so wait on them in order
    std::thread waiter([&] {
        cudaSetDevice(dev);
        for (int k = 0; k < count; ++k) {
            while (issued.load(std::memory_order_acquire) <= k) {
                if (stop.load(std::memory_order_acquire)) return;
                std::this_thread::yield();
            }
            if (cudaEventSynchronize(ev[(size_t)k]) != cudaSuccess) { stop = 2; return; }
            done[(size_t)k] = clock::now();
        }
    });
    int rc = FN_OK;
    for (int k = 0; k < count && rc == FN_OK; ++k) {
        const clock::time_point due = start + std::chrono::duration_cast<clock::duration>(
                                                  std::chrono::duration<double, std::micro>(arrivalMicros[k]));
        while (clock::now() < due) {
        }
        rc = gen_device(requests[k].node, args[(size_t)k], requests[k].out, b->dminmax + 2 * k, stream);
        if (rc == FN_OK &&
            (!cuda_ok(cudaMemcpyAsync(b->hminmax + 2 * k, b->dminmax + 2 * k, 2 * sizeof(float), cudaMemcpyDeviceToHost, s),
                      "copy minmax") ||
             !cuda_ok(cudaEventRecord(ev[(size_t)k], s), "event record")))
            rc = FN_ERR_CUDA;
        if (rc == FN_OK) issued.store(k + 1, std::memory_order_release);
    }
    if (rc != FN_OK) stop = 1;
    waiter.join();
    if (rc == FN_OK && stop.load() == 2) { set_error(FN_ERR_CUDA, "request failed on the device"); rc = FN_ERR_CUDA; }
    if (rc == FN_OK) {
        for (int k = 0; k < count; ++k) {
            if (latencyMicros)
                latencyMicros[k] = std::chrono::duration<double, std::micro>(done[(size_t)k] - start).count() - arrivalMicros[k];
            if (requests[k].minMax) {
                requests[k].minMax[0] = b->hminmax[2 * k];
                requests[k].minMax[1] = b->hminmax[2 * k + 1];
            }
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    return rc;
}

int fnAutotuneBatch(const fnGenRequest* requests, int count, void* stream)
{
    clear_error();
    if (count <= 0 || !requests) return FN_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaEvent_t e0, e1;
    if (!cuda_ok(cudaEventCreate(&e0), "event") || !cuda_ok(cudaEventCreate(&e1), "event")) return FN_ERR_CUDA;
    BatchTuning best;
    double best_ms = 1e30;
    uint64_t sig = 0;
    for (const BatchTuning& t : Autotuner::instance().candidates()) {
        int rc = run_batch(requests, count, stream, 0, &t);            // warm (first use compiles/captures)
        if (rc) return rc;
        cudaEventRecord(e0, s);
        for (int rep = 0; rep < 2 && rc == 0; ++rep) rc = run_batch(requests, count, stream, 0, &t);
        cudaEventRecord(e1, s);
        if (rc || !cuda_ok(cudaEventSynchronize(e1), "synchronize")) return rc ? rc : FN_ERR_CUDA;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        sig = t_batch->runner.last_signature();
        if (ms < best_ms) { best_ms = ms; best = t; }
    }
    Autotuner::instance().store(sig, best, best_ms / 2);

    // Per tree: the variant of its specialised batch kernel (register bound, block size, points
    // in flight per thread).  The trees' kernels run concurrently, so a variant is judged by the
    // whole batch: coordinate descent over the trees (most points first), each variant of one
    // tree tried with the others' current choices, kept when the batch gets faster by more than
    // the timing noise (0.5 %).
    int rc = FN_OK;
    if (jit_enabled()) {
        std::map<uint64_t, std::pair<const CompiledProgram*, long long>> trees;   // hash -> program, points
        for (int i = 0; i < count && rc == FN_OK; ++i) {
            PointArgs a;
            DeviceProgram p;
            if (!requests[i].node || !request_args(requests[i], a)) continue;
            if (!get_program(N(requests[i].node), a.dim, p)) { rc = last_error(); break; }
            auto& t = trees[p.hash];
            t.first = p.host;
            t.second += std::max(0ll, a.total);
        }
        std::vector<std::pair<long long, uint64_t>> order;
        std::vector<const CompiledProgram*> progs;
        for (auto& kv : trees)
            if (jit_is_specialised(kv.first)) {
                progs.push_back(kv.second.first);
                order.push_back({kv.second.second, kv.first});
            }
        std::sort(order.rbegin(), order.rend());
        std::string err;
        if (rc == FN_OK && !progs.empty() && !jit_build_batch_variants(progs, err)) { set_error(FN_ERR_COMPILE, err); rc = FN_ERR_COMPILE; }
        // the whole batch with the current choices: one warm launch (a new shape compiles and
        // captures), then the fastest of three
        auto time_batch = [&](double& ms_out) -> int {
            int r = run_batch(requests, count, stream, 0, &best);
            double fastest = 1e30;
            for (int rep = 0; rep < 3 && r == FN_OK; ++rep) {
                cudaEventRecord(e0, s);
                r = run_batch(requests, count, stream, 0, &best);
                cudaEventRecord(e1, s);
                if (r == FN_OK && !cuda_ok(cudaEventSynchronize(e1), "synchronize")) r = FN_ERR_CUDA;
                float ms = 0;
                if (r == FN_OK) cudaEventElapsedTime(&ms, e0, e1);
                fastest = std::min(fastest, (double)ms);
            }
            ms_out = fastest;
            return r;
        };
        double base = 0;
        if (rc == FN_OK && !order.empty()) {
            for (auto& o : order) Autotuner::instance().store_tree(o.second, 0, 0.0);
            rc = time_batch(base);
        }
        for (auto& o : order) {
            if (rc != FN_OK) break;
            int keep = 0;
            for (int v = 1; v < (int)batch_variants().size() && rc == FN_OK; ++v) {
                Autotuner::instance().store_tree(o.second, v, 0.0);
                double ms = 0;
                rc = time_batch(ms);
                if (rc == FN_OK && ms < base * 0.995) { base = ms; keep = v; }
            }
            Autotuner::instance().store_tree(o.second, keep, base);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

void* fnServerCreate(const fnServerConfig* config)
{
    clear_error();
    ServerConfig c;
    if (config) {
        if (config->poolBytes) c.pool_bytes = (size_t)config->poolBytes;
        if (config->streams > 0) c.streams = config->streams;
        if (config->maxBatchRequests > 0) c.max_batch_requests = config->maxBatchRequests;
        if (config->maxBatchPoints > 0) c.max_batch_points = config->maxBatchPoints;
        if (config->idleWaitMicros > 0) c.idle_wait_us = config->idleWaitMicros;
    }
    Server* s = new Server(c);
    if (!s->ok()) {
        delete s;
        if (!last_error()) set_error(FN_ERR_CUDA, "server could not start");
        return nullptr;
    }
    return s;
}

void fnServerDestroy(void* server) { delete static_cast<Server*>(server); }

int fnServerSubmit(void* server, const fnGenRequest* request, unsigned long long* ticket)
{
    clear_error();
    if (!server || !request || !ticket) { set_error(FN_ERR_ARG, "invalid arguments"); return FN_ERR_ARG; }
    BatchItem it;
    it.node = N(request->node);
    if (!it.node || !request_args(*request, it.args)) { set_error(FN_ERR_ARG, "invalid node, kind or positions"); return FN_ERR_ARG; }
    it.dout = request->out;
    uint64_t t = 0;
    int rc = static_cast<Server*>(server)->submit(it, t);
    *ticket = t;
    return rc;
}

int fnServerSubmitMany(void* server, const fnGenRequest* requests, int count, unsigned long long* tickets)
{
    clear_error();
    if (!server || count < 0 || (count > 0 && (!requests || !tickets))) { set_error(FN_ERR_ARG, "invalid arguments"); return FN_ERR_ARG; }
    std::vector<BatchItem> items((size_t)count);
    for (int i = 0; i < count; ++i) {
        items[i].node = N(requests[i].node);
        if (!items[i].node || !request_args(requests[i], items[i].args)) {
            set_error(FN_ERR_ARG, "request " + std::to_string(i) + ": invalid node, kind or positions");
            return FN_ERR_ARG;
        }
        items[i].dout = requests[i].out;
    }
    std::vector<uint64_t> t((size_t)count);
    int rc = static_cast<Server*>(server)->submit_many(items.data(), items.size(), t.data());
    if (rc == 0) for (int i = 0; i < count; ++i) tickets[i] = t[i];
    return rc;
}

int fnServerSubmitPaced(void* server, const fnGenRequest* requests, int count, const double* arrivalMicros,
                        unsigned long long* tickets)
{
    clear_error();
    if (!server || count < 0 || (count > 0 && (!requests || !tickets || !arrivalMicros))) {
        set_error(FN_ERR_ARG, "invalid arguments");
        return FN_ERR_ARG;
    }
    std::vector<BatchItem> items((size_t)count);
    for (int i = 0; i < count; ++i) {
        items[i].node = N(requests[i].node);
        if (!items[i].node || !request_args(requests[i], items[i].args)) {
            set_error(FN_ERR_ARG, "request " + std::to_string(i) + ": invalid node, kind or positions");
            return FN_ERR_ARG;
        }
        items[i].dout = requests[i].out;
    }
    std::vector<uint64_t> t((size_t)count);
    int rc = static_cast<Server*>(server)->submit_paced(items.data(), items.size(), arrivalMicros, t.data());
    if (rc == 0) for (int i = 0; i < count; ++i) tickets[i] = t[i];
    return rc;
}

int fnServerWaitMany(void* server, const unsigned long long* tickets, int count, int timeoutMs)
{
    clear_error();
    if (!server || count < 0 || (count > 0 && !tickets)) { set_error(FN_ERR_ARG, "invalid arguments"); return FN_ERR_ARG; }
    std::vector<uint64_t> t(tickets, tickets + count);
    return static_cast<Server*>(server)->wait_many(t.data(), t.size(), timeoutMs);
}

int fnServerPoll(void* server, unsigned long long ticket)
{
    return server ? static_cast<Server*>(server)->poll(ticket) : FN_ERR_ARG;
}

int fnServerWait(void* server, unsigned long long ticket, int timeoutMs, float* minMax, float** dOut)
{
    clear_error();
    if (!server) { set_error(FN_ERR_ARG, "null server"); return FN_ERR_ARG; }
    return static_cast<Server*>(server)->wait(ticket, timeoutMs, minMax, dOut);
}

int fnServerCancel(void* server, unsigned long long ticket)
{
    return server ? static_cast<Server*>(server)->cancel(ticket) : FN_ERR_ARG;
}

int fnServerRelease(void* server, unsigned long long ticket)
{
    return server ? static_cast<Server*>(server)->release(ticket) : FN_ERR_ARG;
}

int fnServerGetStats(void* server, fnServerStats* out)
{
    if (!server || !out) return FN_ERR_ARG;
    ServerStats s;
    static_cast<Server*>(server)->stats(s);
    out->submitted = s.submitted;
    out->completed = s.completed;
    out->failed = s.failed;
    out->batches = s.batches;
    out->points = s.points;
    out->p50Micros = s.p50_us;
    out->p99Micros = s.p99_us;
    out->maxMicros = s.max_us;
    out->meanMicros = s.mean_us;
    out->poolUsed = s.pool_used;
    out->poolCapacity = s.pool_capacity;
    out->queueDepth = s.queue_depth;
    out->inflight = s.inflight;
    out->overlappedBatches = s.overlapped_batches;
    out->maxInflightBatches = s.max_inflight_batches;
    out->maxConcurrentBatches = s.max_concurrent_batches;
    return FN_OK;
}

int fnServerResetStats(void* server)
{
    if (!server) return FN_ERR_ARG;
    static_cast<Server*>(server)->reset_stats();
    return FN_OK;
}

int fnAutotuneLoad(const char* path) { return path && Autotuner::instance().load(path) ? FN_OK : FN_ERR_ARG; }
int fnAutotuneSave(const char* path) { return path && Autotuner::instance().save(path) ? FN_OK : FN_ERR_ARG; }

int fnCompileInfo(const void* node, int dimension, int* nInstr, int* nRegs)
{
    clear_error();
    if (!node) { set_error(FN_ERR_ARG, "null node"); return FN_ERR_ARG; }
    CompiledProgram p;
    std::string err;
    if (!compile_program(N(node), dimension, p, err)) { set_error(FN_ERR_COMPILE, err); return FN_ERR_COMPILE; }
    if (nInstr) *nInstr = p.n_instr;
    if (nRegs) *nRegs = p.n_regs;
    return FN_OK;
}

int fnPrepare(const void* node, int dimension)
{
    clear_error();
    DeviceProgram p;
    if (!thread_ctx()) return FN_ERR_CUDA;
    return get_program(N(node), dimension, p) ? FN_OK : last_error();
}

int fnGenUniformGrid2DDevice(const void* node, float* dOut, float xOffset, float yOffset, int xCount, int yCount,
                             float xStepSize, float yStepSize, int seed, float* dMinMax, void* stream)
{
    const float off[2] = {xOffset, yOffset};
    const int cnt[2] = {xCount, yCount};
    const float st[2] = {xStepSize, yStepSize};
    return gen_device(node, grid_args(2, off, cnt, st, seed), dOut, dMinMax, stream);
}

int fnGenUniformGrid3DDevice(const void* node, float* dOut, float xOffset, float yOffset, float zOffset, int xCount,
                             int yCount, int zCount, float xStepSize, float yStepSize, float zStepSize, int seed,
                             float* dMinMax, void* stream)
{
    const float off[3] = {xOffset, yOffset, zOffset};
    const int cnt[3] = {xCount, yCount, zCount};
    const float st[3] = {xStepSize, yStepSize, zStepSize};
    return gen_device(node, grid_args(3, off, cnt, st, seed), dOut, dMinMax, stream);
}

int fnGenUniformGrid4DDevice(const void* node, float* dOut, float xOffset, float yOffset, float zOffset, float wOffset,
                             int xCount, int yCount, int zCount, int wCount, float xStepSize, float yStepSize,
                             float zStepSize, float wStepSize, int seed, float* dMinMax, void* stream)
{
    const float off[4] = {xOffset, yOffset, zOffset, wOffset};
    const int cnt[4] = {xCount, yCount, zCount, wCount};
    const float st[4] = {xStepSize, yStepSize, zStepSize, wStepSize};
    return gen_device(node, grid_args(4, off, cnt, st, seed), dOut, dMinMax, stream);
}

int fnGenPositionArray2DDevice(const void* node, float* dOut, int count, const float* dX, const float* dY, float xOffset,
                               float yOffset, int seed, float* dMinMax, void* stream)
{
    const float off[2] = {xOffset, yOffset};
    PointArgs a = pos_args(2, count, off, seed);
    a.pos[0] = dX; a.pos[1] = dY;
    if (a.total > 0 && (!dX || !dY)) { set_error(FN_ERR_ARG, "null position array"); return FN_ERR_ARG; }
    return gen_device(node, a, dOut, dMinMax, stream);
}

int fnGenPositionArray3DDevice(const void* node, float* dOut, int count, const float* dX, const float* dY,
                               const float* dZ, float xOffset, float yOffset, float zOffset, int seed, float* dMinMax,
                               void* stream)
{
    const float off[3] = {xOffset, yOffset, zOffset};
    PointArgs a = pos_args(3, count, off, seed);
    a.pos[0] = dX; a.pos[1] = dY; a.pos[2] = dZ;
    if (a.total > 0 && (!dX || !dY || !dZ)) { set_error(FN_ERR_ARG, "null position array"); return FN_ERR_ARG; }
    return gen_device(node, a, dOut, dMinMax, stream);
}

int fnGenPositionArray4DDevice(const void* node, float* dOut, int count, const float* dX, const float* dY,
                               const float* dZ, const float* dW, float xOffset, float yOffset, float zOffset,
                               float wOffset, int seed, float* dMinMax, void* stream)
{
    const float off[4] = {xOffset, yOffset, zOffset, wOffset};
    PointArgs a = pos_args(4, count, off, seed);
    a.pos[0] = dX; a.pos[1] = dY; a.pos[2] = dZ; a.pos[3] = dW;
    if (a.total > 0 && (!dX || !dY || !dZ || !dW)) { set_error(FN_ERR_ARG, "null position array"); return FN_ERR_ARG; }
    return gen_device(node, a, dOut, dMinMax, stream);
}

int fnGenTileable2DDevice(const void* node, float* dOut, int xSize, int ySize, float xStepSize, float yStepSize,
                          int seed, float* dMinMax, void* stream)
{
    return gen_device(node, tile_args(xSize, ySize, xStepSize, yStepSize, seed), dOut, dMinMax, stream);
}

int fnGenPreviewTextureDevice(const void* node, int genType, int sizeX, int sizeY, const float* offset, float scale, int seed,
                              unsigned int* dPixels, float* dMinMax, void* stream)
{
    clear_error();
    if (!node || !offset || genType < 0 || genType > 3 || sizeX < 0 || sizeY < 0) {
        set_error(FN_ERR_ARG, "invalid arguments");
        return FN_ERR_ARG;
    }
    // the editor wraps its tree in a default ConvertRGBA8 (range -1..1) (NoiseTexture.cpp:503-504)
    const NodeMeta* meta = meta_by_name("ConvertRGBA8");
    Node* wrap = meta ? node_new(meta->id) : nullptr;
    if (!wrap || !wrap->set_lookup(0, const_cast<Node*>(N(node)))) {
        if (wrap) node_unref(wrap);
        set_error(FN_ERR_ARG, "cannot wrap the tree in ConvertRGBA8");
        return FN_ERR_ARG;
    }
    // image centred on (offset.x, offset.y) (:508-509)
    const float x0 = offset[0] - ((float)sizeX / 2.0f) * scale;
    const float y0 = offset[1] - ((float)sizeY / 2.0f) * scale;
    float* out = reinterpret_cast<float*>(dPixels);      // packed RGBA8 bits, stored as the node returns them
    int rc;
    switch (genType) {
    case 0:
        rc = fnGenUniformGrid2DDevice(wrap, out, x0, y0, sizeX, sizeY, scale, scale, seed, dMinMax, stream);
        break;
    case 1:
        rc = fnGenTileable2DDevice(wrap, out, sizeX, sizeY, scale, scale, seed, dMinMax, stream);
        break;
    case 2:
        rc = fnGenUniformGrid3DDevice(wrap, out, x0, y0, offset[2], sizeX, sizeY, 1, scale, scale, scale, seed, dMinMax, stream);
        break;
    default:
        rc = fnGenUniformGrid4DDevice(wrap, out, x0, y0, offset[2], offset[3], sizeX, sizeY, 1, 1, scale, scale, scale, scale,
                                      seed, dMinMax, stream);
        break;
    }
    node_unref(wrap);
    return rc;
}

// ---------------------------------------------------------------- run-time specialisation
namespace {
int jit_programs(const void* const* nodes, const int* dims, int count, std::vector<CompiledProgram>& store,
                 std::vector<const CompiledProgram*>& progs)
{
    if (!nodes || !dims || count <= 0) { set_error(FN_ERR_ARG, "invalid arguments"); return FN_ERR_ARG; }
    store.resize((size_t)count);
    for (int i = 0; i < count; ++i) {
        std::string err;
        if (!nodes[i] || dims[i] < 2 || dims[i] > 4) { set_error(FN_ERR_ARG, "invalid node or dimension"); return FN_ERR_ARG; }
        if (!compile_program(N(nodes[i]), dims[i], store[(size_t)i], err)) { set_error(FN_ERR_COMPILE, err); return FN_ERR_COMPILE; }
    }
    for (auto& p : store) {
        bool dup = false;
        for (auto* q : progs) dup = dup || q->hash == p.hash;
        if (!dup) progs.push_back(&p);
    }
    return FN_OK;
}
}  // namespace

int fnGetBatchInfo(fnBatchInfo* info)
{
    clear_error();
    if (!info) { set_error(FN_ERR_ARG, "null info"); return FN_ERR_ARG; }
    std::memset(info, 0, sizeof *info);
    if (t_hbatch && t_hbatch->info_valid) {          // the last call was fnGenBatchHost: its slices summed
        *info = t_hbatch->info;
        return FN_OK;
    }
    if (!t_batch) return FN_OK;
    const BatchRunner& r = t_batch->runner;
    info->requests = (int)r.last_device_minmax().size();
    info->specialised = r.last_specialised() ? 1 : 0;
    info->tilePoints = (int)r.last_tile_points();
    info->ctas = r.last_grid();
    info->workItems = r.last_items();
    info->points = r.last_points();
    info->uploadBytes = r.last_upload_bytes();
    info->kernels = r.last_kernels();
    return FN_OK;
}

int fnJitCompile(const void* const* nodes, const int* dims, int count)
{
    clear_error();
    std::vector<CompiledProgram> store;
    std::vector<const CompiledProgram*> progs;
    int rc = jit_programs(nodes, dims, count, store, progs);
    if (rc) return rc;
    if (!thread_ctx()) return FN_ERR_CUDA;
    for (int i = 0; i < count; ++i) {            // device copies for the interpreter paths (batch staging uses them)
        DeviceProgram dp;
        if (!get_program(N(nodes[i]), dims[i], dp)) return last_error();
    }
    std::string err;
    if (!jit_build(progs, err)) { set_error(FN_ERR_COMPILE, err); return FN_ERR_COMPILE; }
    return FN_OK;
}

int fnSetAutoSpecialise(int uses) { return jit_set_auto_threshold(uses); }

int fnAutoSpecialiseWait(int timeoutMs)
{
    clear_error();
    if (jit_auto_wait(timeoutMs)) return FN_OK;
    set_error(FN_ERR_TIMEOUT, "background specialisation still running");
    return FN_ERR_TIMEOUT;
}

int fnJitIsSpecialised(const void* node, int dimension)
{
    clear_error();
    if (!node || dimension < 2 || dimension > 4) { set_error(FN_ERR_ARG, "invalid node or dimension"); return FN_ERR_ARG; }
    CompiledProgram prog;
    std::string err;
    if (!compile_program(N(node), dimension, prog, err)) { set_error(FN_ERR_COMPILE, err); return FN_ERR_COMPILE; }
    return jit_is_specialised(prog.hash) ? 1 : 0;
}

int fnJitSetCacheDir(const char* dir)
{
    clear_error();
    jit_cache_set_dir(dir);
    return FN_OK;
}

int fnJitGetCacheInfo(char* dir, int dirBytes, unsigned long long* hits, unsigned long long* misses)
{
    clear_error();
    const std::string d = jit_cache_dir();
    if (dir && dirBytes > 0) {
        const size_t n = std::min(d.size(), (size_t)dirBytes - 1);
        std::memcpy(dir, d.data(), n);
        dir[n] = '\0';
    }
    jit_cache_stats(hits, misses);
    return (int)std::min<size_t>(d.size(), 0x7FFFFFFF);
}

int fnJitCheck(const void* const* nodes, const int* dims, int count, int* cubinBytes)
{
    clear_error();
    std::vector<CompiledProgram> store;
    std::vector<const CompiledProgram*> progs;
    int rc = jit_programs(nodes, dims, count, store, progs);
    if (rc) return rc;
    std::vector<std::vector<char>> cubins;
    std::string err;
    if (!jit_compile_all(progs, cubins, err)) { set_error(FN_ERR_COMPILE, err); return FN_ERR_COMPILE; }
    size_t bytes = 0;
    for (auto& c : cubins) bytes += c.size();
    if (cubinBytes) *cubinBytes = bytes > 0x7FFFFFFF ? 0x7FFFFFFF : (int)bytes;
    return FN_OK;
}

int fnJitCheckBatchVariants(const void* const* nodes, const int* dims, int count, int* cubinBytes)
{
    clear_error();
    std::vector<CompiledProgram> store;
    std::vector<const CompiledProgram*> progs;
    int rc = jit_programs(nodes, dims, count, store, progs);
    if (rc) return rc;
    const int nv = (int)batch_variants().size();
    std::vector<std::vector<char>> cubins((size_t)nv);
    std::vector<std::string> logs((size_t)nv);
    std::vector<char> ok((size_t)nv, 1);
    std::vector<std::thread> pool;                 // one NVRTC compilation per variant, concurrently
    for (int v = 1; v < nv; ++v)
        pool.emplace_back([&, v] { ok[(size_t)v] = jit_compile_cubin(jit_batch_source(progs, v), cubins[(size_t)v], logs[(size_t)v]) ? 1 : 0; });
    for (auto& t : pool) t.join();
    size_t bytes = 0;
    for (int v = 1; v < nv; ++v) {
        if (!ok[(size_t)v]) { set_error(FN_ERR_COMPILE, "NVRTC: " + logs[(size_t)v].substr(0, 4000)); return FN_ERR_COMPILE; }
        bytes += cubins[(size_t)v].size();
    }
    if (cubinBytes) *cubinBytes = bytes > 0x7FFFFFFF ? 0x7FFFFFFF : (int)bytes;
    return FN_OK;
}

int fnSetJitEnabled(int enabled)
{
    const int was = jit_enabled() ? 1 : 0;
    jit_set_enabled(enabled != 0);
    return was;
}

// Allocation-free 3D grid: the program is compiled on the host (cached per
// thread, host memory only) and copied into the static device scratch of
// fn_static_scratch.cu on the caller's stream.  No device memory, pinned host
// memory or stream is created, so this never touches thread_ctx().
int fnGenUniformGrid3DDeviceNoAlloc(const void* node, float* dOut, float xOffset, float yOffset, float zOffset,
                                    int xCount, int yCount, int zCount, float xStepSize, float yStepSize,
                                    float zStepSize, int seed, float* dMinMax, void* stream)
{
    clear_error();
    const float off[3] = {xOffset, yOffset, zOffset};
    const int cnt[3] = {xCount, yCount, zCount};
    const float st[3] = {xStepSize, yStepSize, zStepSize};
    const PointArgs args = grid_args(3, off, cnt, st, seed);
    if (!node || args.total < 0 || (args.total > 0 && !dOut)) { set_error(FN_ERR_ARG, "invalid arguments"); return FN_ERR_ARG; }
    struct HostProgram { const Node* node = nullptr; uint64_t epoch = 0; CompiledProgram prog; };
    thread_local HostProgram cached;
    const uint64_t epoch = mutation_epoch();
    if (cached.node != N(node) || cached.epoch != epoch) {
        cached.node = nullptr;
        std::string err;
        if (!compile_program(N(node), 3, cached.prog, err)) { set_error(FN_ERR_COMPILE, err); return FN_ERR_COMPILE; }
        cached.node = N(node);
        cached.epoch = epoch;
    }
    if (cached.prog.needs_specialisation()) {
        set_error(FN_ERR_COMPILE, "the tree evaluates a node per cell (node-driven Minkowski P); the allocation-free "
                                  "path runs the interpreter only");
        return FN_ERR_COMPILE;
    }
    const size_t bytes = cached.prog.blob.size();
    if (bytes > kStaticProgramBytes) {
        set_error(FN_ERR_CAPACITY, "tree program is " + std::to_string(bytes) + " bytes; the allocation-free path holds at most " +
                                       std::to_string(kStaticProgramBytes) + " bytes (use fnGenUniformGrid3DDevice)");
        return FN_ERR_CAPACITY;
    }
    if (!cuda_ok(launch_interpreter_static(cached.prog.blob.data(), (uint32_t)bytes, args, dOut, dMinMax,
                                           static_cast<cudaStream_t>(stream)),
                 "allocation-free launch"))
        return FN_ERR_CUDA;
    return FN_OK;
}

}  // extern "C"
