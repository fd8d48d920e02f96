// fn_runtime.h -- shared runtime services: error state, device program cache,
// per-thread CUDA contexts.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "fn_compile.h"
#include "fn_kernels.cuh"
#include "fn_node.h"

namespace fn {

// thread-local status reported by fnGetLastError / fnGetLastErrorString
void set_error(int code, const std::string& msg);
void clear_error();
int last_error();
const char* last_error_string();

struct DeviceProgram {
    const FnProgramHeader* dptr = nullptr;   // device copy of the blob
    uint32_t bytes = 0;
    uint64_t hash = 0;
    int dim = 0;
    const CompiledProgram* host = nullptr;    // host copy (owned by the cache)
};

// Compile-and-upload with caching by (node, dim, mutation epoch) and by
// program hash.  Returns false (with set_error) when the tree cannot run.
bool get_program(const Node* node, int dim, DeviceProgram& out);

// Per host thread: a non-blocking stream and reduction workspaces.
struct ThreadCtx {
    cudaStream_t stream = nullptr;
    float* dbuf = nullptr;
    size_t dbuf_cap = 0;
    float* dpos[4] = {nullptr, nullptr, nullptr, nullptr};
    size_t dpos_cap = 0;
    float* hminmax = nullptr;                 // pinned float[2]
    float* hminmax_dev = nullptr;             // the same memory as the device sees it (kernels store min/max there)
};
ThreadCtx* thread_ctx();                      // nullptr (and error set) if CUDA is unusable
MinMaxWork* work_for_stream(cudaStream_t s);  // per (thread, stream) workspace

bool cuda_ok(cudaError_t e, const char* what);

}  // namespace fn
