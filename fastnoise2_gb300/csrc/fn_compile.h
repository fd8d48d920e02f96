// fn_compile.h -- flatten a node tree into an FnProgram (fn_program.h).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "fn_node.h"
#include "fn_program.h"

namespace fn {

struct CompiledProgram {
    std::vector<uint8_t> blob;   // FnProgramHeader + instrs + params (16-byte multiple)
    uint64_t hash = 0;           // of the blob and of every sub-program
    int dim = 0;
    int n_instr = 0;
    int n_regs = 0;
    // Sub-programs evaluated per cell by cellular instructions whose Minkowski P is
    // driven by a node (instruction field d = index here; Utils.inl:326-331 samples
    // the P node at each cell's offset vector).  Only the specialised kernels run
    // them, so a program with sub-programs needs fnJitCompile-style kernels.
    std::vector<CompiledProgram> subs;
    bool needs_specialisation() const { return !subs.empty(); }
};

// Compile `root` for a root dimensionality of 2, 3 or 4.  Returns false and
// fills `error` for trees the GPU path cannot evaluate (missing lookups, node
// kinds without a device implementation, program limits exceeded).
bool compile_program(const Node* root, int dim, CompiledProgram& out, std::string& error);

uint64_t fnv1a64(const void* data, size_t n, uint64_t h = 1469598103934665603ull);

}  // namespace fn
