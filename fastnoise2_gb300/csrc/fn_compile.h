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
    uint64_t hash = 0;
    int dim = 0;
    int n_instr = 0;
    int n_regs = 0;
};

// Compile `root` for a root dimensionality of 2, 3 or 4.  Returns false and
// fills `error` for trees the GPU path cannot evaluate (missing lookups, node
// kinds without a device implementation, program limits exceeded).
bool compile_program(const Node* root, int dim, CompiledProgram& out, std::string& error);

uint64_t fnv1a64(const void* data, size_t n, uint64_t h = 1469598103934665603ull);

}  // namespace fn
