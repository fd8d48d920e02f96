// fn_jit.h -- run-time specialised kernels.
//
// The interpreter (fn_kernels.cu) evaluates any tree but pays for dispatch and
// for a register file in local memory.  For trees that will be evaluated many
// times, the same device program is turned into straight-line CUDA source --
// one call per instruction to the hand-written node functions of
// fn_device.cuh, positions and values in registers, parameters as literals --
// and compiled for sm_103a with NVRTC (-fmad=false, so results are identical
// to the interpreter's).  Each tree gets a module with its grid / position-array
// / tileable per-call kernels; one batch module holds a persistent batch kernel
// per tree, so the trees of a batch run as concurrent kernels, each with the
// register allocation its own code needs.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "fn_compile.h"
#include "fn_types.h"

namespace fn {

struct JitKernels {
    cudaKernel_t grid = nullptr;      // GenUniformGrid for the program's dimensionality
    cudaKernel_t positions = nullptr; // GenPositionArray
    cudaKernel_t tileable = nullptr;  // GenTileable2D (4D programs only)
    cudaKernel_t solid = nullptr;     // chunk meshing (3D programs): classification bitmasks of a grid
    cudaKernel_t list = nullptr;      // chunk meshing (3D programs): grid values at listed point indices
    int slot = -1;                    // index in the module's batch kernel
    int resident[3] = {1, 1, 1};      // 256-thread blocks per SM of grid / positions / tileable at once
};

// Variants of a tree's persistent batch kernel, among which the autotuner picks per
// tree: threads per block, the register bound (the blocks per SM the kernel must fit,
// __launch_bounds__) and how many points a thread has in flight per loop iteration.
// Variant 0 is the one fnJitCompile builds; the others are built when a tuning run
// (or a loaded tuning table) asks for them.
struct BatchVariant {
    int threads;
    int min_blocks;
    int points;
};
const std::vector<BatchVariant>& batch_variants();

struct BatchKernel {
    cudaKernel_t kernel = nullptr;
    int threads = 256;
};

// CUDA source of the batch module for `progs` (slot k = progs[k]) in one variant, and of
// one program's per-call module.
std::string jit_batch_source(const std::vector<const CompiledProgram*>& progs, int variant);
std::string jit_percall_source(const CompiledProgram& prog);

// NVRTC-compile the batch module and every per-call module (concurrently);
// cubins[0] = batch, cubins[1 + k] = program k.  Host only, no GPU needed.
bool jit_compile_all(const std::vector<const CompiledProgram*>& progs, std::vector<std::vector<char>>& cubins,
                     std::string& error);

// Compile and load a module covering `progs`; on success every program gets
// per-call kernels and a batch kernel.  Thread safe.
bool jit_build(const std::vector<const CompiledProgram*>& progs, std::string& error);

// On-disk module cache (see fn_jit.cpp): the directory in use ("" = off, the default; the
// environment variable FASTNOISE_JIT_CACHE names one),
// its hit / miss counts in this process, and the tree's kernels loaded straight from the
// cache when an earlier process built them alone (the way automatic specialisation does):
// true when they are loaded now.  Looks once per program and process.
void jit_cache_set_dir(const char* dir);
std::string jit_cache_dir();
void jit_cache_stats(unsigned long long* hits, unsigned long long* misses);
bool jit_try_cached(const CompiledProgram* prog);

// Build variants 1.. of the batch kernels of `progs` (NVRTC, one module per variant,
// compiled concurrently); programs whose variants exist are skipped.  Thread safe.
bool jit_build_batch_variants(const std::vector<const CompiledProgram*>& progs, std::string& error);

// The batch kernel of `hash` in `variant`, or false when it is not built (or JIT is off).
bool jit_batch_kernel(uint64_t hash, int variant, BatchKernel& out);

// Queue a background build of the batch variants of `prog` (a tuning table loaded in this
// process may name variants that have not been built yet).
void jit_request_batch_variants(const CompiledProgram* prog);

// Kernels for a program hash, or false if none have been built.
bool jit_lookup(uint64_t hash, JitKernels& out);

// Launch the specialised per-call kernel for `hash` if one is loaded (and JIT
// is enabled); returns false when the caller should use the interpreter.
// `err` carries the launch status when true is returned.
bool jit_launch(uint64_t hash, const PointArgs& args, float* out, MinMaxWork* work, float* dminmax, cudaStream_t stream,
                cudaError_t& err);

// Chunk meshing with a specialised 3D tree (false when none is loaded): bit i of `above` /
// `solid` = grid point i's value is > iso / <= iso (both 0 for NaN), and OutputMinMax into
// `dminmax`; and the values at the grid point indices idx[0 .. *count) into out (max_count
// bounds the launch).
bool jit_launch_solid(uint64_t hash, const PointArgs& args, unsigned* above, unsigned* solid, MinMaxWork* work, float* dminmax,
                      float iso, cudaStream_t stream, cudaError_t& err);
bool jit_launch_list(uint64_t hash, const PointArgs& args, const unsigned* idx, const unsigned* count, unsigned max_count,
                     float* out, cudaStream_t stream, cudaError_t& err);

// Programs the interpreter cannot run (CompiledProgram::needs_specialisation)
// get their specialised kernels built on first use; true if they exist now.
bool jit_ensure(const CompiledProgram* prog, std::string& error);

void jit_set_enabled(bool on);
bool jit_enabled();

// Automatic specialisation: the interpreter paths report each launch of a program
// here; once a program has run `threshold` times on the interpreter it is queued
// for a background NVRTC build (one worker thread), and later launches find its
// specialised kernels.  threshold 0 = off; the default comes from the environment
// variable FASTNOISE_AUTO_SPECIALISE (a number, 0 = off), else 4.
void jit_note_interpreted(const CompiledProgram* prog);
int jit_set_auto_threshold(int uses);              // returns the previous threshold
bool jit_auto_wait(int timeout_ms);                // true when no build is queued or running
bool jit_is_specialised(uint64_t hash);

// Compile NVRTC source for sm_103a to a cubin (host only; used by tests).
bool jit_compile_cubin(const std::string& src, std::vector<char>& cubin, std::string& log);

}  // namespace fn
