// fn_runtime.cpp -- error state, device program cache, per-thread contexts.
#include "fn_runtime.h"

#include <cstdio>
#include <map>
#include <memory>
#include <mutex>
#include <unordered_map>

namespace fn {

namespace {
thread_local int t_err = 0;
thread_local std::string t_msg;

struct CacheKey {
    const Node* node;
    int dim;
    bool operator==(const CacheKey& o) const { return node == o.node && dim == o.dim; }
};
struct CacheKeyHash {
    size_t operator()(const CacheKey& k) const { return std::hash<const void*>()(k.node) ^ (size_t)k.dim * 0x9E3779B97F4A7C15ull; }
};
struct NodeEntry {
    uint64_t epoch;
    uint64_t hash;
};
struct ProgEntry {
    std::unique_ptr<CompiledProgram> host;
    void* dptr = nullptr;
};

std::mutex g_mu;
std::unordered_map<CacheKey, NodeEntry, CacheKeyHash> g_node_cache;
std::unordered_map<uint64_t, ProgEntry> g_progs;
}  // namespace

void set_error(int code, const std::string& msg)
{
    t_err = code;
    t_msg = msg;
    if (code) std::fprintf(stderr, "[fastnoise_gb300] error %d: %s\n", code, msg.c_str());
}
void clear_error() { t_err = 0; t_msg.clear(); }
int last_error() { return t_err; }
const char* last_error_string() { return t_msg.c_str(); }

bool cuda_ok(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return true;
    set_error(-3, std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}

bool get_program(const Node* node, int dim, DeviceProgram& out)
{
    if (!node) { set_error(-1, "null node"); return false; }
    const uint64_t epoch = mutation_epoch();
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_node_cache.find({node, dim});
    if (it != g_node_cache.end() && it->second.epoch == epoch) {
        auto p = g_progs.find(it->second.hash);
        if (p != g_progs.end()) {
            out.dptr = static_cast<const FnProgramHeader*>(p->second.dptr);
            out.bytes = (uint32_t)p->second.host->blob.size();
            out.hash = it->second.hash;
            out.dim = dim;
            out.host = p->second.host.get();
            return true;
        }
    }
    auto prog = std::make_unique<CompiledProgram>();
    std::string err;
    if (!compile_program(node, dim, *prog, err)) { set_error(-2, err); return false; }
    const uint64_t h = prog->hash;
    auto p = g_progs.find(h);
    if (p == g_progs.end()) {
        void* d = nullptr;
        if (!cuda_ok(cudaMalloc(&d, prog->blob.size()), "cudaMalloc(program)")) return false;
        if (!cuda_ok(cudaMemcpy(d, prog->blob.data(), prog->blob.size(), cudaMemcpyHostToDevice), "upload program")) {
            cudaFree(d);
            return false;
        }
        ProgEntry e;
        e.host = std::move(prog);
        e.dptr = d;
        p = g_progs.emplace(h, std::move(e)).first;
    }
    g_node_cache[{node, dim}] = NodeEntry{epoch, h};
    out.dptr = static_cast<const FnProgramHeader*>(p->second.dptr);
    out.bytes = (uint32_t)p->second.host->blob.size();
    out.hash = h;
    out.dim = dim;
    out.host = p->second.host.get();
    return true;
}

namespace {
struct ThreadCtxHolder {
    ThreadCtx ctx;
    bool init = false;
    bool failed = false;
    std::map<cudaStream_t, MinMaxWork*> works;
    ~ThreadCtxHolder()
    {
        // Process teardown may already have destroyed the CUDA context; frees are best effort.
        if (!init) return;
        for (auto& w : works) cudaFree(w.second);
        if (ctx.dbuf) cudaFree(ctx.dbuf);
        for (float* p : ctx.dpos) if (p) cudaFree(p);
        if (ctx.hminmax) cudaFreeHost(ctx.hminmax);
        if (ctx.stream) cudaStreamDestroy(ctx.stream);
    }
};
thread_local ThreadCtxHolder t_ctx;
}  // namespace

ThreadCtx* thread_ctx()
{
    if (t_ctx.init) return &t_ctx.ctx;
    if (t_ctx.failed) { set_error(-3, "CUDA is not usable in this process"); return nullptr; }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        t_ctx.failed = true;
        set_error(-3, std::string("no CUDA device available: ") + cudaGetErrorString(e));
        return nullptr;
    }
    if (!cuda_ok(cudaStreamCreateWithFlags(&t_ctx.ctx.stream, cudaStreamNonBlocking), "cudaStreamCreate")) { t_ctx.failed = true; return nullptr; }
    if (!cuda_ok(cudaMallocHost(&t_ctx.ctx.hminmax, 2 * sizeof(float)), "cudaMallocHost")) { t_ctx.failed = true; return nullptr; }
    // Pinned memory is mapped into the device's address space (unified addressing); when the
    // device pointer cannot be had, host calls copy the min/max back instead.
    void* mapped = nullptr;
    if (cudaHostGetDevicePointer(&mapped, t_ctx.ctx.hminmax, 0) == cudaSuccess) t_ctx.ctx.hminmax_dev = static_cast<float*>(mapped);
    else cudaGetLastError();
    t_ctx.init = true;
    return &t_ctx.ctx;
}

MinMaxWork* work_for_stream(cudaStream_t s)
{
    auto it = t_ctx.works.find(s);
    if (it != t_ctx.works.end()) return it->second;
    MinMaxWork* w = nullptr;
    if (!cuda_ok(cudaMalloc(&w, sizeof(MinMaxWork)), "cudaMalloc(workspace)")) return nullptr;
    if (!cuda_ok(cudaMemset(w, 0, sizeof(MinMaxWork)), "cudaMemset(workspace)")) { cudaFree(w); return nullptr; }
    t_ctx.works[s] = w;
    return w;
}

}  // namespace fn
