// fn_capi_internal.h -- helpers shared by the C-ABI translation units (fn_capi.cpp,
// fn_capi_mesh.cpp); not part of the public interface.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "fn_node.h"
#include "fn_runtime.h"
#include "fn_types.h"

namespace fn {
namespace capi {

Node* N(void* p);
const Node* N(const void* p);
float f_of(int32_t bits);

// A uniform grid request: x fastest, fma(float(i), step, offset) per axis (Generator.inl).
PointArgs grid_args(int dim, const float* off, const int* cnt, const float* step, int seed);

// Launch one generation call: the tree's specialised kernel when one is loaded,
// the interpreter otherwise (which may queue the tree for background specialisation).
cudaError_t launch_points(const DeviceProgram& prog, const PointArgs& args, float* out, MinMaxWork* work, float* dminmax,
                          cudaStream_t stream);

// Specialise trees the interpreter cannot run before their first launch; false (with the
// error set) when that is impossible.
bool ensure_runnable(const DeviceProgram& prog);

}  // namespace capi
}  // namespace fn
