// fn_jit.cpp -- code generation, NVRTC compilation and the module registry of
// the run-time specialised kernels (see fn_jit.h).
#include "fn_jit.h"

#include <nvrtc.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <thread>
#include <unordered_map>
#include <unordered_set>

#include <sys/stat.h>
#include <unistd.h>

#include "fn_kernels.cuh"
#include "fn_runtime.h"

namespace fn {

// The device headers (fn_types.h, fn_device.cuh, fn_eval.cuh) as one source
// string; the file defining it is generated at build time (build.py).
const char* embedded_device_source();

namespace {

std::string lit(float f)
{
    char b[64];
    if (std::isfinite(f)) {
        std::snprintf(b, sizeof b, "%af", (double)f);         // exact hexadecimal literal
    } else {
        uint32_t u;
        std::memcpy(&u, &f, 4);
        std::snprintf(b, sizeof b, "__int_as_float(0x%08xu)", u);
    }
    return b;
}

std::string r(int i) { return "r" + std::to_string(i); }

const char* noise_fn(int kind)
{
    switch (kind) {
    case FN_NOISE_SIMPLEX: return "simplex";
    case FN_NOISE_SUPERSIMPLEX: return "supersimplex";
    case FN_NOISE_PERLIN: return "perlin";
    default: return "value";
    }
}

// One program -> `__device__ float <name>(int seed, float x, float y, float z, float w)`.
// Its per-cell sub-programs (node-driven Minkowski P) come first, each as a
// function `<name>_s<j>` plus a functor `<name>_s<j>_mk` the cellular walk calls
// with the cell's offset vector.
void emit_eval(const CompiledProgram& prog, const std::string& name, std::ostringstream& o)
{
    for (size_t j = 0; j < prog.subs.size(); ++j) {
        const std::string sub = name + "_s" + std::to_string(j);
        emit_eval(prog.subs[j], sub, o);
        const int sd = prog.subs[j].dim;
        o << "struct " << sub << "_mk {\n    int seed;\n    static constexpr bool kNode = true;\n"
          << "    __device__ __forceinline__ float operator()(const float* v) const { return " << sub << "(seed, v[0], v[1], "
          << (sd > 2 ? "v[2]" : "0.0f") << ", " << (sd > 3 ? "v[3]" : "0.0f") << "); }\n};\n\n";
    }
    const FnProgramHeader* h = reinterpret_cast<const FnProgramHeader*>(prog.blob.data());
    const FnInstr* ins = fn_program_instrs(h);
    const float* P = fn_program_params(h);
    const int nregs = h->n_regs;
    auto mk = [&](const FnInstr& I) {   // trailing functor argument of a cellular call
        return I.d == FN_REG_NONE ? std::string() : ", " + name + "_s" + std::to_string(I.d) + "_mk{seed}";
    };
    o << "__device__ __forceinline__ float " << name << "(int seed, float x, float y, float z, float w)\n{\n";
    o << "    (void)x; (void)y; (void)z; (void)w;\n";
    const char* root[4] = {"x", "y", "z", "w"};
    for (int i = 0; i < nregs; ++i) o << "    float " << r(i) << " = " << (i < h->dim ? root[i] : "0.0f") << ";\n";
    for (int pc = 0; pc < h->n_instr; ++pc) {
        const FnInstr& I = ins[pc];
        const int D = I.dim;
        const std::string sd = "fnd::iadd(seed, " + std::to_string(I.seed) + ")";
        auto p = [&](int j) { return lit(P[I.prm + j]); };
        auto pos = [&](int base) {
            std::string s = "{";
            for (int j = 0; j < D; ++j) s += (j ? ", " : "") + r(base + j);
            return s + "}";
        };
        auto cellp = [&](int mk_index) {
            std::ostringstream c;
            c << "fnd::CellParams cp; cp.freq = " << p(0) << "; cp.jitter = fnd::CellConst<" << D << ">::jitter * " << r(I.b)
              << "; cp.sizeActive = " << (I.c != FN_REG_NONE ? "true" : "false") << "; cp.sizeJitter = "
              << (I.c != FN_REG_NONE ? r(I.c) + " * fnd::CellConst<" + std::to_string(D) + ">::size" : std::string("0.0f"))
              << "; cp.distFunc = " << (I.aux & 15) << "; cp.minkowski = " << p(mk_index) << ";";
            return c.str();
        };
        o << "    { // op " << (int)I.op << "\n";
        switch (I.op) {
        case FN_OP_CONST: o << "        " << r(I.dst) << " = " << p(0) << ";\n"; break;
        case FN_OP_MOV: o << "        " << r(I.dst) << " = " << r(I.a) << ";\n"; break;
        case FN_OP_SCALE_POS:
            for (int j = 0; j < D; ++j) o << "        const float t" << j << " = " << r(I.a + j) << " * " << p(0) << ";\n";
            for (int j = 0; j < D; ++j) o << "        " << r(I.dst + j) << " = t" << j << ";\n";
            break;
        case FN_OP_SCALE_POS_V:
            for (int j = 0; j < D; ++j) o << "        const float t" << j << " = " << r(I.a + j) << " * " << p(j) << ";\n";
            for (int j = 0; j < D; ++j) o << "        " << r(I.dst + j) << " = t" << j << ";\n";
            break;
        case FN_OP_OFFSET_POS: case FN_OP_SUB_POS: {
            const int off[4] = {I.b, I.c, I.d, I.e};
            const char* opch = I.op == FN_OP_OFFSET_POS ? " + " : " - ";
            for (int j = 0; j < D; ++j) o << "        const float t" << j << " = " << r(I.a + j) << opch << r(off[j]) << ";\n";
            for (int j = 0; j < D; ++j) o << "        " << r(I.dst + j) << " = t" << j << ";\n";
            break;
        }
        case FN_OP_ROTATE2:
            o << "        const float px = " << r(I.a) << ", py = " << r(I.a + 1) << ";\n";
            o << "        " << r(I.dst) << " = fmaf(-py, " << p(1) << ", px * " << p(0) << ");\n";
            o << "        " << r(I.dst + 1) << " = fmaf(px, " << p(1) << ", py * " << p(0) << ");\n";
            break;
        case FN_OP_ROTATE3:
            o << "        const float px = " << r(I.a) << ", py = " << r(I.a + 1) << ", pz = " << (D >= 3 ? r(I.a + 2) : "0.0f") << ";\n";
            for (int j = 0; j < 3; ++j)
                o << "        const float n" << j << " = fmaf(px, " << p(3 * j) << ", fmaf(py, " << p(3 * j + 1) << ", pz * " << p(3 * j + 2) << "));\n";
            for (int j = 0; j < 3; ++j) o << "        " << r(I.dst + j) << " = n" << j << ";\n";
            break;
        case FN_OP_ROTPLANE:
            o << "        float px = " << r(I.a) << ", py = " << r(I.a + 1) << ", pz = " << (D >= 3 ? r(I.a + 2) : "0.0f") << ";\n";
            if (D == 4) o << "        const float pw = " << r(I.a + 3) << ";\n";
            o << "        fnd::rotate_plane(" << I.aux << ", px, py, pz);\n";
            o << "        " << r(I.dst) << " = px; " << r(I.dst + 1) << " = py; " << r(I.dst + 2) << " = pz;\n";
            if (D == 4) o << "        " << r(I.dst + 3) << " = pw;\n";
            break;
        case FN_OP_NOISE: {
            o << "        const float f = " << p(0) << ";\n";
            o << "        " << r(I.dst) << " = fnd::scale_out(fnd::" << noise_fn(I.aux) << D << "(" << sd;
            for (int j = 0; j < D; ++j) o << ", " << r(I.a + j) << " * f";
            o << "), " << p(1) << ", " << p(2) << ", " << p(3) << ");\n";
            break;
        }
        case FN_OP_WHITE:
            o << "        const float pp[" << D << "] = " << pos(I.a) << ";\n";
            o << "        " << r(I.dst) << " = fnd::scale_out(fnd::white<" << D << ">(" << sd << ", pp), -fnd::kValueBounds, " << p(0) << ", " << p(1) << ");\n";
            break;
        case FN_OP_CHECKER:
            o << "        const float pp[" << D << "] = " << pos(I.a) << ";\n";
            o << "        " << r(I.dst) << " = fnd::scale_out(fnd::checkerboard<" << D << ">(pp, " << p(0) << "), 0.0f, " << p(1) << ", " << p(2) << ");\n";
            break;
        case FN_OP_SINE:
            o << "        const float pp[" << D << "] = " << pos(I.a) << ";\n";
            o << "        " << r(I.dst) << " = fnd::scale_out(fnd::sine_wave<" << D << ">(pp, " << p(0) << "), -1.0f, " << p(1) << ", " << p(2) << ");\n";
            break;
        case FN_OP_CELL_VALUE:
            o << "        const float pp[" << D << "] = " << pos(I.a) << ";\n        " << cellp(3) << "\n";
            o << "        " << r(I.dst) << " = fnd::scale_out(fnd::cellular_value<" << D << ">(" << sd << ", pp, cp, " << ((I.aux >> 4) & 3)
              << mk(I) << "), -fnd::kValueBounds, " << p(1) << ", " << p(2) << ");\n";
            break;
        case FN_OP_CELL_DIST:
            o << "        const float pp[" << D << "] = " << pos(I.a) << ";\n        " << cellp(3) << "\n";
            o << "        float dist[4]; fnd::cellular_distances<" << D << ", "
              << std::max((I.aux >> 4) & 3, (I.aux >> 8) & 3) + 1 << ">(" << sd << ", pp, cp, dist" << mk(I) << ");\n";
            o << "        float nmax; const float v = fnd::cellular_return<" << D << ">(dist, cp.distFunc, " << ((I.aux >> 4) & 3) << ", "
              << ((I.aux >> 8) & 3) << ", " << ((I.aux >> 12) & 7) << ", nmax);\n";
            o << "        " << r(I.dst) << " = fnd::scale_out(v, 0.0f, " << p(1) << ", " << p(2) << ");\n";
            break;
        case FN_OP_CELL_LOOKUP:
            o << "        const float pp[" << D << "] = " << pos(I.a) << ";\n        " << cellp(2) << "\n";
            o << "        float oo[" << D << "]; fnd::cellular_lookup_pos<" << D << ">(" << sd << ", pp, cp, " << p(1) << ", oo" << mk(I) << ");\n";
            for (int j = 0; j < D; ++j) o << "        " << r(I.dst + j) << " = oo[" << j << "];\n";
            break;
        case FN_OP_WARP_GRAD: case FN_OP_WARP_SIMPLEX:
            o << "        const float f = " << p(0) << ";\n";
            o << "        float sp[" << D << "], io[" << D << "];\n";
            for (int j = 0; j < D; ++j) o << "        sp[" << j << "] = " << r(I.a + j) << " * f; io[" << j << "] = " << r(I.dst + j) << ";\n";
            o << "        const float axis[" << D << "] = {";
            for (int j = 0; j < D; ++j) o << (j ? ", " : "") << p(1 + j);
            if (I.op == FN_OP_WARP_GRAD)
                o << "};\n        const float st = fnd::warp_gradient<" << D << ">(" << sd << ", " << r(I.b) << ", sp, axis, io);\n";
            else
                o << "};\n        const float st = fnd::warp_simplex<" << D << ">(" << sd << ", " << r(I.b) << ", sp, axis, io, "
                  << ((I.aux & 1) ? "true" : "false") << ", " << ((I.aux & 2) ? "true" : "false") << ");\n";
            for (int j = 0; j < D; ++j) o << "        " << r(I.dst + j) << " = io[" << j << "];\n";
            if (I.c != FN_REG_NONE) o << "        " << r(I.c) << " = st;\n";
            else o << "        (void)st;\n";
            break;
        case FN_OP_FRACT_INIT:
            if (I.aux) o << "        const float nz = fnd::fabs_(" << r(I.a) << "); " << r(I.a) << " = nz; " << r(I.dst) << " = (nz * -2.0f + 1.0f) * 1.0f;\n";
            else o << "        " << r(I.dst) << " = " << r(I.a) << " * 1.0f;\n";
            o << "        " << r(I.b) << " = 1.0f;\n";
            break;
        case FN_OP_FRACT_AMP:
            o << "        const float t = " << (I.aux ? "1.0f - " + r(I.a) : "(" + r(I.a) + " + 1.0f) * 0.5f") << ";\n";
            o << "        const float amp = " << r(I.b) << " * fnd::lerp(1.0f, t, " << r(I.c) << ");\n";
            o << "        " << r(I.b) << " = amp * " << r(I.d) << ";\n";
            break;
        case FN_OP_FRACT_ACC:
            if (I.aux) o << "        const float nz = fnd::fabs_(" << r(I.a) << "); " << r(I.a) << " = nz; " << r(I.dst) << " = " << r(I.dst) << " + (nz * -2.0f + 1.0f) * " << r(I.b) << ";\n";
            else o << "        " << r(I.dst) << " = " << r(I.dst) << " + " << r(I.a) << " * " << r(I.b) << ";\n";
            break;
        case FN_OP_DWF_AMP:
            o << "        const float s = sqrtf(" << r(I.a) << "); " << r(I.a) << " = s;\n";
            o << "        const float amp = " << r(I.b) << " * fnd::lerp(1.0f, 1.0f - s, " << r(I.c) << ");\n";
            o << "        " << r(I.b) << " = amp * " << r(I.d) << ";\n";
            break;
        case FN_OP_ADD: o << "        " << r(I.dst) << " = " << r(I.a) << " + " << r(I.b) << ";\n"; break;
        case FN_OP_SUB: o << "        " << r(I.dst) << " = " << r(I.a) << " - " << r(I.b) << ";\n"; break;
        case FN_OP_MUL: o << "        " << r(I.dst) << " = " << r(I.a) << " * " << r(I.b) << ";\n"; break;
        case FN_OP_DIV: o << "        " << r(I.dst) << " = " << r(I.a) << " / " << r(I.b) << ";\n"; break;
        case FN_OP_MOD: o << "        " << r(I.dst) << " = fnd::mod_(" << r(I.a) << ", " << r(I.b) << ");\n"; break;
        case FN_OP_MIN: o << "        " << r(I.dst) << " = fnd::fmin_(" << r(I.a) << ", " << r(I.b) << ");\n"; break;
        case FN_OP_MAX: o << "        " << r(I.dst) << " = fnd::fmax_(" << r(I.a) << ", " << r(I.b) << ");\n"; break;
        case FN_OP_ABS: o << "        " << r(I.dst) << " = fnd::fabs_(" << r(I.a) << ");\n"; break;
        case FN_OP_SSQRT: o << "        " << r(I.dst) << " = fnd::signed_sqrt(" << r(I.a) << ");\n"; break;
        case FN_OP_POWF: o << "        " << r(I.dst) << " = fnd::pow_(fnd::fmax_(fnd::fabs_(" << r(I.a) << "), 1.17549435e-38f), " << r(I.b) << ");\n"; break;
        case FN_OP_POWI:
            o << "        const float v = " << r(I.a) << "; float pw = v * v;\n";
            o << "        for (int i = 2; i < " << I.aux << "; ++i) pw *= v;\n        " << r(I.dst) << " = pw;\n";
            break;
        case FN_OP_MINSMOOTH: o << "        " << r(I.dst) << " = fnd::min_smooth(" << r(I.a) << ", " << r(I.b) << ", " << r(I.c) << ");\n"; break;
        case FN_OP_MAXSMOOTH: o << "        " << r(I.dst) << " = -fnd::min_smooth(-" << r(I.a) << ", -" << r(I.b) << ", " << r(I.c) << ");\n"; break;
        case FN_OP_FADE:
            o << "        " << r(I.dst) << " = fnd::lerp(" << r(I.a) << ", " << r(I.b) << ", fnd::fade_t(" << r(I.c) << ", " << r(I.d) << ", " << r(I.e)
              << ", " << I.aux << "));\n";
            break;
        case FN_OP_REMAP:
            o << "        " << r(I.dst) << " = fnd::remap(" << r(I.a) << ", " << r(I.b) << ", " << r(I.c) << ", " << r(I.d) << ", " << r(I.e) << ", "
              << (I.aux ? "true" : "false") << ");\n";
            break;
        case FN_OP_TERRACE:
            o << "        const float src = " << r(I.a) << " * " << p(0) << ";\n        float rounded = rintf(src);\n";
            if (I.b != FN_REG_NONE)
                o << "        const float sm = " << r(I.b) << ";\n        if (sm != 0.0f) rounded = fnd::terrace_smooth(rounded, src, 1.0f + 1.0f / sm);\n";
            else if (I.aux)
                o << "        rounded = fnd::terrace_smooth(rounded, src, " << p(2) << ");\n";
            o << "        " << r(I.dst) << " = rounded * " << p(1) << ";\n";
            break;
        case FN_OP_PINGPONG: o << "        " << r(I.dst) << " = fnd::ping_pong(" << r(I.a) << " * " << r(I.b) << ");\n"; break;
        case FN_OP_RGBA8: o << "        " << r(I.dst) << " = fnd::to_rgba8(" << r(I.a) << ", " << p(0) << ", " << p(1) << ");\n"; break;
        case FN_OP_GRADIENT: {
            const int off[4] = {I.b, I.c, I.d, I.e};
            o << "        float acc = 0.0f;\n";
            for (int j = 0; j < D; ++j) o << "        acc = fmaf(" << r(I.a + j) << " + " << r(off[j]) << ", " << p(j) << ", acc);\n";
            o << "        " << r(I.dst) << " = acc;\n";
            break;
        }
        case FN_OP_DISTANCE:
            o << "        const float pp[" << D << "] = " << pos(I.a) << ";\n";
            o << "        " << r(I.dst) << " = fnd::distance<" << D << ">(" << (I.aux & 15) << ", " << (((I.aux >> 4) & 1) ? "true" : "false")
              << ", pp, " << (I.b != FN_REG_NONE ? r(I.b) : std::string("0.0f")) << ");\n";
            break;
        default:
            o << "        // unsupported op\n";
            break;
        }
        o << "    }\n";
    }
    o << "    return " << r(h->out_reg) << ";\n}\n\n";
}

// Per-call kernels for program k: grid / position array / tileable.
//
// Each warp owns chunks of 32*ppl consecutive points (ppl = points per lane,
// 1..4, chosen by the host).  Lane l evaluates points chunk + 32*t + l
// (t < ppl, one point at a time, so the tree's code is not replicated) and
// parks the values in shared memory; with ppl == 4 the warp then writes the
// chunk as 32 float4 stores (512 contiguous bytes per warp).  Small calls use
// ppl == 1 so that their few points spread over as many SMs as possible.
void emit_percall(const CompiledProgram& prog, int k, std::ostringstream& o)
{
    const int D = prog.dim;
    const char* pv[4] = {"px", "py", "pz", "pw"};
    std::string call = "fnjit_eval_" + std::to_string(k) + "(A.seed";
    for (int j = 0; j < 4; ++j) call += std::string(", ") + (j < D ? pv[j] : "0.0f");
    call += ")";

    auto kernel = [&](const char* name, const std::string& prologue, const std::string& position) {
        o << "extern \"C\" __global__ void __launch_bounds__(256, 4) " << name << "_" << k
          << "(fn::PointArgs A, float* __restrict__ out, fn::MinMaxWork* work, float* dminmax, unsigned ppl)\n{\n"
          << "    __shared__ float4 stage[8][32];\n"
          << "    __shared__ float smn[8], smx[8];\n"
          << "    float mn = fne::inf(), mx = -fne::inf();\n"
          << "    const unsigned total = (unsigned)A.total;\n"
          << "    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;\n"
          << "    const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;\n"
          << "    const bool aligned = (((unsigned long long)out) & 15ull) == 0;\n"
          << "    float* st = reinterpret_cast<float*>(stage[warp]);\n"
          << prologue
          << "    const unsigned chunk = 32u * ppl;\n"
          << "    for (unsigned base = (((blockIdx.x * blockDim.x) >> 5) + warp) * chunk; base < total; base += nwarps * chunk) {\n"
          << "#pragma unroll 1\n"
          << "        for (unsigned t = 0; t < ppl; ++t) {\n"
          << "            const unsigned i = base + t * 32u + lane;\n"
          << "            float v = 0.0f;\n"
          << "            if (i < total) {\n"
          << position
          << "                v = " << call << ";\n"
          << "                fne::fold(v, mn, mx);\n"
          << "            }\n"
          << "            st[t * 32u + lane] = v;\n"
          << "        }\n"
          << "        __syncwarp();\n"
          << "        if (ppl == 4u && aligned && base + 128u <= total) {\n"
          << "            reinterpret_cast<float4*>(out + base)[lane] = stage[warp][lane];\n"
          << "        } else {\n"
          << "            for (unsigned q = 0; q < ppl; ++q) {\n"
          << "                const unsigned j = base + q * 32u + lane;\n"
          << "                if (j < total) out[j] = st[q * 32u + lane];\n"
          << "            }\n"
          << "        }\n"
          << "        __syncwarp();\n"
          << "    }\n"
          << "    fne::grid_minmax(mn, mx, work, dminmax, smn, smx);\n"
          << "}\n\n";
    };

    // grid: Generator.inl:79-254, pos_k = fma(float(i_k), step_k, offset_k), x fastest
    std::string gridpos;
    {
        std::ostringstream pos;
        pos << "                unsigned r = i + A.base;\n";          // index in the whole request
        const char* ax = "xyzw";
        for (int j = 0; j < D; ++j) {
            if (j < D - 1)
                pos << "                const unsigned q" << j << " = fne::fast_div(r, A.divm[" << j << "], A.divs[" << j << "]);\n"
                    << "                const unsigned i" << ax[j] << " = r - q" << j << " * (unsigned)A.count[" << j << "]; r = q" << j << ";\n";
            else pos << "                const unsigned i" << ax[j] << " = r;\n";
            pos << "                const float " << pv[j] << " = fmaf(fnd::cvtf((int)i" << ax[j] << "), A.step[" << j << "], A.offset[" << j << "]);\n";
        }
        gridpos = pos.str();
        kernel("fnjit_grid", "", gridpos);
    }
    // position arrays: Generator.inl:256-350, pos_k = offset_k + array_k[i]
    {
        std::ostringstream pos;
        for (int j = 0; j < D; ++j)
            pos << "                const float " << pv[j] << " = A.offset[" << j << "] + __ldg(A.pos[" << j << "] + i + A.base);\n";
        kernel("fnjit_pos", "", pos.str());
    }
    // tileable (4D programs): Generator.inl:370-433
    if (D == 4) {
        std::ostringstream pos;
        pos << "                const unsigned g = i + A.base;\n"
            << "                const unsigned iy = fne::fast_div(g, A.divm[0], A.divs[0]), ix = g - iy * (unsigned)A.count[0];\n"
            << "                const float xf = fnd::cvtf((int)ix) * A.tmul[0];\n"
            << "                const float yf = fnd::cvtf((int)iy) * A.tmul[1];\n"
            << "                const float px = fnd::cos_(xf) * A.tfreq[0];\n"
            << "                const float py = fnd::cos_(yf) * A.tfreq[1];\n"
            << "                const float pz = fnd::sin_(xf) * A.tfreq[0];\n"
            << "                const float pw = fnd::sin_(yf) * A.tfreq[1];\n";
        kernel("fnjit_tile", "", pos.str());
    }
    // Chunk meshing (3D programs): the meshers need every density only as "above the iso
    // level" / "at or below it", and exact values at a few voxels near the surface.
    //  fnjit_solid: the grid's two classification bitmasks (bit i of word i / 32; the warp's
    //    32 consecutive points form one word) and OutputMinMax -- no density leaves registers;
    //  fnjit_list: the grid's values at listed point indices (count read from the device).
    if (D == 3) {
        o << "extern \"C\" __global__ void __launch_bounds__(256, 4) fnjit_solid_" << k
          << "(fn::PointArgs A, unsigned* __restrict__ above, unsigned* __restrict__ solid, fn::MinMaxWork* work, float* dminmax,\n"
          << "    float iso, unsigned ppl)\n{\n"
          << "    __shared__ float smn[8], smx[8];\n"
          << "    float mn = fne::inf(), mx = -fne::inf();\n"
          << "    const unsigned total = (unsigned)A.total;\n"
          << "    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;\n"
          << "    const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;\n"
          << "    const unsigned chunk = 32u * ppl;\n"
          << "    for (unsigned base = (((blockIdx.x * blockDim.x) >> 5) + warp) * chunk; base < total; base += nwarps * chunk) {\n"
          << "#pragma unroll 1\n"
          << "        for (unsigned t = 0; t < ppl; ++t) {\n"
          << "            const unsigned i = base + t * 32u + lane;\n"
          << "            bool gt = false, le = false;\n"
          << "            if (i < total) {\n"
          << gridpos
          << "                const float v = " << call << ";\n"
          << "                fne::fold(v, mn, mx);\n"
          << "                gt = v > iso;\n"
          << "                le = v <= iso;\n"
          << "            }\n"
          << "            const unsigned wg = __ballot_sync(0xffffffffu, gt), wl = __ballot_sync(0xffffffffu, le);\n"
          << "            if (lane == 0 && base + t * 32u < total) { above[(base + t * 32u) >> 5] = wg; solid[(base + t * 32u) >> 5] = wl; }\n"
          << "        }\n"
          << "    }\n"
          << "    fne::grid_minmax(mn, mx, work, dminmax, smn, smx);\n"
          << "}\n\n";
        o << "extern \"C\" __global__ void __launch_bounds__(256, 4) fnjit_list_" << k
          << "(fn::PointArgs A, const unsigned* __restrict__ idx, const unsigned* __restrict__ count, float* __restrict__ out)\n{\n"
          << "    const unsigned n = *count;\n"
          << "    for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {\n"
          << "        const unsigned i = idx[j];\n"
          << gridpos
          << "        out[j] = " << call << ";\n"
          << "    }\n"
          << "}\n\n";
    }
}

}  // namespace

const std::vector<BatchVariant>& batch_variants()
{
    // {threads, register bound as blocks per SM, points per thread per loop iteration}
    static const std::vector<BatchVariant> v = {
        {256, 4, 1},     // 64 registers: the kernel fnJitCompile builds
        {256, 3, 1},     // 80 registers: fewer spills for long cellular walks
        {256, 2, 1},     // 128 registers
        {128, 8, 1},     // 64 registers in smaller blocks: finer balance of the work queue
        {256, 2, 2},     // 128 registers, two points in flight per thread
    };
    return v;
}

namespace {

std::string batch_kernel_name(size_t k, int variant)
{
    return "fnjit_batch_" + std::to_string(k) + (variant ? "_v" + std::to_string(variant) : std::string());
}

// The batch kernels: persistent CTAs pull (request, tile) items of their tree's
// group and run a tile loop with that tree's code inlined.  A variant fixes the
// block size, the register bound and how many points a thread has in flight.
void emit_batch(const std::vector<const CompiledProgram*>& progs, std::ostringstream& o, int variant)
{
    const BatchVariant bv = batch_variants()[(size_t)variant];
    for (size_t k = 0; k < progs.size(); ++k) {
        const int D = progs[k]->dim;
        const std::string call = "fnjit_eval_" + std::to_string(k) + "(A.seed, p[0], p[1], " + (D > 2 ? "p[2]" : "0.0f") +
                                 ", " + (D > 3 ? "p[3]" : "0.0f") + ")";
        o << "__device__ __forceinline__ void fnjit_tile_" << k << "_v" << variant
          << "(const fn::PointArgs& A, float* __restrict__ out, unsigned i, unsigned end, float& mn, float& mx)\n{\n";
        if (bv.points == 1) {
            o << "    for (; i < end; i += blockDim.x) {\n"
              << "        float p[4];\n"
              << "        fne::root_position32<" << D << ">(A, i, p);\n"
              << "        const float v = " << call << ";\n"
              << "        out[i] = v;\n"
              << "        fne::fold(v, mn, mx);\n"
              << "    }\n}\n\n";
        } else {
            o << "    for (; i < end; i += " << bv.points << "u * blockDim.x) {\n"
              << "        float v[" << bv.points << "];\n"
              << "#pragma unroll\n"
              << "        for (int q = 0; q < " << bv.points << "; ++q) {\n"
              << "            const unsigned j = i + q * blockDim.x;\n"
              << "            float p[4];\n"
              << "            fne::root_position32<" << D << ">(A, j < end ? j : i, p);\n"
              << "            v[q] = " << call << ";\n"
              << "        }\n"
              << "#pragma unroll\n"
              << "        for (int q = 0; q < " << bv.points << "; ++q) {\n"
              << "            const unsigned j = i + q * blockDim.x;\n"
              << "            if (j < end) { out[j] = v[q]; fne::fold(v[q], mn, mx); }\n"
              << "        }\n"
              << "    }\n}\n\n";
        }
    }
    // one persistent kernel per tree: each gets the register allocation its own
    // code needs, and the trees of a batch run as concurrent kernels
    for (size_t k = 0; k < progs.size(); ++k) {
        o << "extern \"C\" __global__ void __launch_bounds__(" << bv.threads << ", " << bv.min_blocks << ") "
          << batch_kernel_name(k, variant)
          << "(fn::BatchHeader* hdr, const fn::BatchRequest* __restrict__ reqs, fn::BatchState* states,\n"
             "    const uint2* __restrict__ items, fn::BatchGroup* grp)\n{\n"
             "    __shared__ unsigned int s_item;\n"
             "    __shared__ float smn[" << bv.threads / 32 << "], smx[" << bv.threads / 32 << "];\n"
             "    const unsigned int first = grp->item_begin, last = grp->item_end;\n"
             "    const unsigned int tile_points = hdr->tile_points;\n"
             "    for (;;) {\n"
             "        if (threadIdx.x == 0) s_item = first + atomicAdd(&grp->head, 1u);\n"
             "        __syncthreads();\n"
             "        const unsigned int it = s_item;\n"
             "        __syncthreads();\n"
             "        if (it >= last) break;\n"
             "        const uint2 item = items[it];\n"
             "        const fn::BatchRequest& rq = reqs[item.x];\n"
             "        const fn::PointArgs args = rq.args;\n"
             "        const unsigned total = (unsigned)args.total;\n"
             "        const unsigned begin = item.y * tile_points;\n"
             "        const unsigned end = total - begin < tile_points ? total : begin + tile_points;\n"
             "        float mn = fne::inf(), mx = -fne::inf();\n"
             "        fnjit_tile_" << k << "_v" << variant << "(args, rq.out, begin + threadIdx.x, end, mn, mx);\n"
             "        fne::block_minmax(mn, mx, smn, smx);\n"
             "        if (threadIdx.x == 0) fne::finish_tile(rq, states + item.x, hdr, mn, mx);\n"
             "    }\n}\n\n";
    }
}

struct Module {
    cudaLibrary_t lib = nullptr;
    std::vector<uint64_t> hashes;
};

std::mutex g_jit_mu;
std::unordered_map<uint64_t, JitKernels> g_kernels;
std::vector<std::unique_ptr<Module>> g_modules;
std::unordered_map<uint64_t, cudaKernel_t> g_batch_kernels;   // per-tree batch kernel (variant 0)
std::unordered_map<uint64_t, std::vector<BatchKernel>> g_batch_variant_kernels;   // per tree: every variant built
std::atomic<bool> g_enabled{true};

}  // namespace

std::string jit_batch_source(const std::vector<const CompiledProgram*>& progs, int variant)
{
    std::ostringstream o;
    o << "// generated by fn_jit.cpp: batch module, variant " << variant << "\n" << embedded_device_source() << "\n";
    for (size_t k = 0; k < progs.size(); ++k) emit_eval(*progs[k], "fnjit_eval_" + std::to_string(k), o);
    emit_batch(progs, o, variant);
    return o.str();
}

std::string jit_percall_source(const CompiledProgram& prog)
{
    std::ostringstream o;
    o << "// generated by fn_jit.cpp: per-call module\n" << embedded_device_source() << "\n";
    emit_eval(prog, "fnjit_eval_0", o);
    emit_percall(prog, 0, o);
    return o.str();
}

// ---------------------------------------------------------------- on-disk module cache
// Compiled modules are kept on disk, keyed by their CUDA source (which embeds the node
// library's device code), the NVRTC options and the NVRTC version, so a module that any
// earlier process built loads in milliseconds instead of being compiled again.  File:
// "FNJC", format version, the 128-bit key, payload size, the cubin, a checksum of the cubin;
// a file that does not check out is ignored (and replaced by the next compile).
namespace {

constexpr uint32_t kCacheFormat = 1;
const char* const kNvrtcOptions[] = {"--gpu-architecture=sm_103a", "-fmad=false", "--std=c++17", "-default-device",
                                     "-lineinfo", "-diag-suppress=177"};

struct CacheKey {
    uint64_t a = 0, b = 0;
};

uint64_t fnv1a(const void* data, size_t n, uint64_t h)
{
    const unsigned char* p = static_cast<const unsigned char*>(data);
    for (size_t i = 0; i < n; ++i) h = (h ^ p[i]) * 0x100000001B3ull;
    return h;
}

CacheKey cache_key(const std::string& src)
{
    int major = 0, minor = 0;
    nvrtcVersion(&major, &minor);
    std::string salt = "nvrtc " + std::to_string(major) + "." + std::to_string(minor) + " format " + std::to_string(kCacheFormat);
    for (const char* o : kNvrtcOptions) salt += std::string(" ") + o;
    CacheKey k;
    k.a = fnv1a(src.data(), src.size(), fnv1a(salt.data(), salt.size(), 0xCBF29CE484222325ull));
    k.b = fnv1a(src.data(), src.size(), fnv1a(salt.data(), salt.size(), 0x84222325CBF29CE4ull ^ 0x9E3779B97F4A7C15ull));
    return k;
}

std::mutex g_cache_mu;
bool g_cache_resolved = false;
std::string g_cache_dir;                  // empty: off
std::atomic<unsigned long long> g_cache_hits{0}, g_cache_misses{0};

void make_dirs(const std::string& dir)
{
    for (size_t i = 1; i <= dir.size(); ++i)
        if (i == dir.size() || dir[i] == '/') mkdir(dir.substr(0, i).c_str(), 0755);   // existing parts fail harmlessly
}

std::string cache_dir()
{
    std::lock_guard<std::mutex> lk(g_cache_mu);
    if (!g_cache_resolved) {
        g_cache_resolved = true;
        // off unless the application names a directory: a library writes no files of its own
        const char* env = std::getenv("FASTNOISE_JIT_CACHE");
        if (env && *env && std::strcmp(env, "off") != 0) g_cache_dir = env;
        if (!g_cache_dir.empty()) make_dirs(g_cache_dir);
    }
    return g_cache_dir;
}

std::string cache_path(const std::string& dir, const CacheKey& k)
{
    char name[64];
    std::snprintf(name, sizeof name, "/%016llx%016llx.cubin", (unsigned long long)k.a, (unsigned long long)k.b);
    return dir + name;
}

bool cache_read(const std::string& path, const CacheKey& k, std::vector<char>& cubin)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    char magic[4];
    uint32_t format = 0;
    uint64_t ka = 0, kb = 0, size = 0, sum = 0;
    if (!f.read(magic, 4) || std::memcmp(magic, "FNJC", 4) != 0 || !f.read(reinterpret_cast<char*>(&format), 4) ||
        format != kCacheFormat || !f.read(reinterpret_cast<char*>(&ka), 8) || !f.read(reinterpret_cast<char*>(&kb), 8) ||
        ka != k.a || kb != k.b || !f.read(reinterpret_cast<char*>(&size), 8) || size == 0 || size > (uint64_t(1) << 30))
        return false;
    std::vector<char> data((size_t)size);
    if (!f.read(data.data(), (std::streamsize)size) || !f.read(reinterpret_cast<char*>(&sum), 8) ||
        sum != fnv1a(data.data(), data.size(), 0xCBF29CE484222325ull))
        return false;
    cubin.swap(data);
    return true;
}

void cache_write(const std::string& path, const CacheKey& k, const std::vector<char>& cubin)
{
    // written under a name of its own, then renamed: readers see a whole file or none
    const std::string tmp = path + ".tmp" + std::to_string((long long)getpid()) + "_" +
                            std::to_string(std::hash<std::thread::id>()(std::this_thread::get_id()));
    {
        std::ofstream f(tmp, std::ios::binary | std::ios::trunc);
        if (!f) return;
        const uint64_t size = cubin.size(), sum = fnv1a(cubin.data(), cubin.size(), 0xCBF29CE484222325ull);
        f.write("FNJC", 4);
        f.write(reinterpret_cast<const char*>(&kCacheFormat), 4);
        f.write(reinterpret_cast<const char*>(&k.a), 8);
        f.write(reinterpret_cast<const char*>(&k.b), 8);
        f.write(reinterpret_cast<const char*>(&size), 8);
        f.write(cubin.data(), (std::streamsize)cubin.size());
        f.write(reinterpret_cast<const char*>(&sum), 8);
        if (!f) { f.close(); std::remove(tmp.c_str()); return; }
    }
    if (std::rename(tmp.c_str(), path.c_str()) != 0) std::remove(tmp.c_str());
}

// A module from the cache only (no compile); false on a miss.
bool cached_cubin(const std::string& src, std::vector<char>& cubin)
{
    const std::string dir = cache_dir();
    if (dir.empty()) return false;
    const CacheKey k = cache_key(src);
    if (!cache_read(cache_path(dir, k), k, cubin)) return false;
    g_cache_hits.fetch_add(1);
    return true;
}

}  // namespace

void jit_cache_set_dir(const char* dir)
{
    std::lock_guard<std::mutex> lk(g_cache_mu);
    g_cache_resolved = true;
    g_cache_dir = (!dir || !*dir || std::strcmp(dir, "off") == 0) ? std::string() : std::string(dir);
    if (!g_cache_dir.empty()) make_dirs(g_cache_dir);
}

std::string jit_cache_dir() { return cache_dir(); }

void jit_cache_stats(unsigned long long* hits, unsigned long long* misses)
{
    if (hits) *hits = g_cache_hits.load();
    if (misses) *misses = g_cache_misses.load();
}

bool jit_compile_all(const std::vector<const CompiledProgram*>& progs, std::vector<std::vector<char>>& cubins, std::string& error)
{
    // source 0 = the batch module, 1 + k = program k's per-call module; NVRTC
    // compiles independent programs concurrently, so the sources go to a pool of threads
    std::vector<std::string> srcs;
    srcs.push_back(jit_batch_source(progs, 0));
    for (auto* p : progs) srcs.push_back(jit_percall_source(*p));
    cubins.assign(srcs.size(), {});
    std::vector<std::string> logs(srcs.size());
    std::vector<char> ok(srcs.size(), 0);
    std::atomic<size_t> next{0};
    auto worker = [&]() {
        for (size_t i; (i = next.fetch_add(1)) < srcs.size();) ok[i] = jit_compile_cubin(srcs[i], cubins[i], logs[i]) ? 1 : 0;
    };
    unsigned nt = std::thread::hardware_concurrency();
    nt = std::max(1u, std::min<unsigned>(nt ? nt : 4, (unsigned)srcs.size()));
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nt; ++t) pool.emplace_back(worker);
    worker();
    for (auto& t : pool) t.join();
    for (size_t i = 0; i < srcs.size(); ++i)
        if (!ok[i]) { error = "NVRTC: " + logs[i].substr(0, 4000); return false; }
    return true;
}

bool jit_compile_cubin(const std::string& src, std::vector<char>& cubin, std::string& log)
{
    // FASTNOISE_JIT_VERBOSE=1 prints ptxas' register / spill report of every
    // specialised kernel to stderr (useful when tuning trees); it always compiles.
    const char* verbose = std::getenv("FASTNOISE_JIT_VERBOSE");
    const bool v = verbose && verbose[0] == '1';
    if (!v && cached_cubin(src, cubin)) return true;
    const std::string dir = cache_dir();
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, src.c_str(), "fastnoise_jit.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) {
        log = "nvrtcCreateProgram failed";
        return false;
    }
    std::vector<const char*> opts(std::begin(kNvrtcOptions), std::end(kNvrtcOptions));
    if (v) opts.push_back("--ptxas-options=-v");
    nvrtcResult rc = nvrtcCompileProgram(prog, (int)opts.size(), opts.data());
    size_t loglen = 0;
    nvrtcGetProgramLogSize(prog, &loglen);
    log.assign(loglen, '\0');
    if (loglen) nvrtcGetProgramLog(prog, &log[0]);
    if (v) std::fprintf(stderr, "%s\n", log.c_str());
    if (rc != NVRTC_SUCCESS) {
        nvrtcDestroyProgram(&prog);
        return false;
    }
    size_t n = 0;
    nvrtcGetCUBINSize(prog, &n);
    cubin.resize(n);
    nvrtcGetCUBIN(prog, cubin.data());
    nvrtcDestroyProgram(&prog);
    g_cache_misses.fetch_add(1);
    if (!dir.empty() && n > 0) {
        const CacheKey k = cache_key(src);
        cache_write(cache_path(dir, k), k, cubin);
    }
    return true;
}

namespace {

// Load the batch module (cubins[0]) and the per-call modules (cubins[1 + k]) of `progs` and
// register their kernels.
bool jit_load(const std::vector<const CompiledProgram*>& progs, const std::vector<std::vector<char>>& cubins, std::string& error)
{
    std::vector<std::unique_ptr<Module>> mods;
    for (auto& c : cubins) {
        auto mod = std::make_unique<Module>();
        cudaError_t e = cudaLibraryLoadData(&mod->lib, c.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
        if (e != cudaSuccess) {
            error = std::string("cudaLibraryLoadData: ") + cudaGetErrorString(e);
            for (auto& m : mods) cudaLibraryUnload(m->lib);
            return false;
        }
        mods.push_back(std::move(mod));
    }
    std::unordered_map<uint64_t, JitKernels> found;
    std::unordered_map<uint64_t, cudaKernel_t> batch;
    bool ok = true;
    for (size_t k = 0; ok && k < progs.size(); ++k) {
        cudaLibrary_t lib = mods[1 + k]->lib;
        JitKernels jk;
        jk.slot = (int)k;
        cudaKernel_t bk = nullptr;
        ok = cudaLibraryGetKernel(&jk.grid, lib, "fnjit_grid_0") == cudaSuccess &&
             cudaLibraryGetKernel(&jk.positions, lib, "fnjit_pos_0") == cudaSuccess &&
             (progs[k]->dim != 4 || cudaLibraryGetKernel(&jk.tileable, lib, "fnjit_tile_0") == cudaSuccess) &&
             (progs[k]->dim != 3 || (cudaLibraryGetKernel(&jk.solid, lib, "fnjit_solid_0") == cudaSuccess &&
                                     cudaLibraryGetKernel(&jk.list, lib, "fnjit_list_0") == cudaSuccess)) &&
             cudaLibraryGetKernel(&bk, mods[0]->lib, ("fnjit_batch_" + std::to_string(k)).c_str()) == cudaSuccess;
        const cudaKernel_t kern[3] = {jk.grid, jk.positions, jk.tileable};
        for (int j = 0; ok && j < 3; ++j) {
            int n = 0;
            if (kern[j] && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, (const void*)kern[j], 256, 0) == cudaSuccess && n > 0)
                jk.resident[j] = n;
            else
                cudaGetLastError();
        }
        found[progs[k]->hash] = jk;
        batch[progs[k]->hash] = bk;
    }
    if (!ok) {
        error = "kernel lookup failed in a specialised module";
        for (auto& m : mods) cudaLibraryUnload(m->lib);
        return false;
    }
    std::lock_guard<std::mutex> lk(g_jit_mu);
    for (auto& kv : found) g_kernels[kv.first] = kv.second;
    for (auto& kv : batch) {
        g_batch_kernels[kv.first] = kv.second;
        auto& vars = g_batch_variant_kernels[kv.first];
        vars.resize(batch_variants().size());
        vars[0] = BatchKernel{kv.second, batch_variants()[0].threads};
    }
    for (auto& m : mods) g_modules.push_back(std::move(m));   // modules stay loaded: kernels may still be queued
    return true;
}

std::mutex g_build_mu;                           // one build per program, even with concurrent first calls

}  // namespace

bool jit_build(const std::vector<const CompiledProgram*>& progs, std::string& error)
{
    if (progs.empty()) return true;
    std::vector<std::vector<char>> cubins;
    if (!jit_compile_all(progs, cubins, error)) return false;
    return jit_load(progs, cubins, error);
}

bool jit_try_cached(const CompiledProgram* prog)
{
    if (!prog || !g_enabled.load(std::memory_order_relaxed) || cache_dir().empty()) return false;
    static std::mutex tried_mu;
    static std::unordered_set<uint64_t> tried;          // one look per program and process
    {
        std::lock_guard<std::mutex> lk(tried_mu);
        if (!tried.insert(prog->hash).second) return false;
    }
    std::lock_guard<std::mutex> lk(g_build_mu);
    {
        std::lock_guard<std::mutex> rk(g_jit_mu);
        if (g_kernels.count(prog->hash) && g_batch_kernels.count(prog->hash)) return true;
    }
    std::vector<std::vector<char>> cubins(2);
    if (!cached_cubin(jit_batch_source({prog}, 0), cubins[0]) || !cached_cubin(jit_percall_source(*prog), cubins[1])) return false;
    std::string err;
    return jit_load({prog}, cubins, err);
}

bool jit_build_batch_variants(const std::vector<const CompiledProgram*>& progs, std::string& error)
{
    const size_t nv = batch_variants().size();
    std::vector<const CompiledProgram*> todo;
    {
        std::lock_guard<std::mutex> lk(g_jit_mu);
        for (auto* p : progs) {
            auto it = g_batch_variant_kernels.find(p->hash);
            bool all = it != g_batch_variant_kernels.end() && it->second.size() == nv;
            for (size_t v = 1; all && v < nv; ++v) all = it->second[v].kernel != nullptr;
            if (!all && std::find(todo.begin(), todo.end(), p) == todo.end()) todo.push_back(p);
        }
    }
    if (todo.empty()) return true;
    // one module per variant, compiled concurrently
    std::vector<std::string> srcs;
    for (size_t v = 1; v < nv; ++v) srcs.push_back(jit_batch_source(todo, (int)v));
    std::vector<std::vector<char>> cubins(srcs.size());
    std::vector<std::string> logs(srcs.size());
    std::vector<char> ok(srcs.size(), 0);
    std::vector<std::thread> pool;
    for (size_t i = 0; i < srcs.size(); ++i)
        pool.emplace_back([&, i] { ok[i] = jit_compile_cubin(srcs[i], cubins[i], logs[i]) ? 1 : 0; });
    for (auto& t : pool) t.join();
    for (size_t i = 0; i < srcs.size(); ++i)
        if (!ok[i]) { error = "NVRTC: " + logs[i].substr(0, 4000); return false; }
    std::vector<std::unique_ptr<Module>> mods;
    std::vector<std::vector<BatchKernel>> got(todo.size(), std::vector<BatchKernel>(nv));
    for (size_t i = 0; i < cubins.size(); ++i) {
        auto mod = std::make_unique<Module>();
        cudaError_t e = cudaLibraryLoadData(&mod->lib, cubins[i].data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
        if (e != cudaSuccess) {
            error = std::string("cudaLibraryLoadData: ") + cudaGetErrorString(e);
            for (auto& m : mods) cudaLibraryUnload(m->lib);
            return false;
        }
        const int v = (int)i + 1;
        for (size_t k = 0; k < todo.size(); ++k) {
            cudaKernel_t kern = nullptr;
            if (cudaLibraryGetKernel(&kern, mod->lib, batch_kernel_name(k, v).c_str()) != cudaSuccess) {
                error = "kernel lookup failed in a batch variant module";
                cudaLibraryUnload(mod->lib);
                for (auto& m : mods) cudaLibraryUnload(m->lib);
                return false;
            }
            got[k][(size_t)v] = BatchKernel{kern, batch_variants()[(size_t)v].threads};
        }
        mods.push_back(std::move(mod));
    }
    std::lock_guard<std::mutex> lk(g_jit_mu);
    for (size_t k = 0; k < todo.size(); ++k) {
        auto& vars = g_batch_variant_kernels[todo[k]->hash];
        vars.resize(nv);
        for (size_t v = 1; v < nv; ++v) vars[v] = got[k][v];
    }
    for (auto& m : mods) g_modules.push_back(std::move(m));
    return true;
}

bool jit_batch_kernel(uint64_t hash, int variant, BatchKernel& out)
{
    if (!g_enabled.load(std::memory_order_relaxed)) return false;
    std::lock_guard<std::mutex> lk(g_jit_mu);
    auto it = g_batch_variant_kernels.find(hash);
    if (it == g_batch_variant_kernels.end() || variant < 0 || (size_t)variant >= it->second.size() ||
        !it->second[(size_t)variant].kernel)
        return false;
    out = it->second[(size_t)variant];
    return true;
}

bool jit_lookup(uint64_t hash, JitKernels& out)
{
    if (!g_enabled.load(std::memory_order_relaxed)) return false;
    std::lock_guard<std::mutex> lk(g_jit_mu);
    auto it = g_kernels.find(hash);
    if (it == g_kernels.end()) return false;
    out = it->second;
    return true;
}

namespace {
bool is_built(uint64_t hash)
{
    std::lock_guard<std::mutex> lk(g_jit_mu);
    return g_kernels.count(hash) && g_batch_kernels.count(hash);
}
}  // namespace

bool jit_ensure(const CompiledProgram* prog, std::string& error)
{
    if (!prog->needs_specialisation()) return true;
    if (!g_enabled.load()) {
        error = "the tree evaluates a node per cell (node-driven Minkowski P), which only specialised kernels "
                "can do, and specialisation is disabled";
        return false;
    }
    std::lock_guard<std::mutex> lk(g_build_mu);
    {
        std::lock_guard<std::mutex> rk(g_jit_mu);
        if (g_kernels.count(prog->hash) && g_batch_kernels.count(prog->hash)) return true;
    }
    return jit_build({prog}, error);
}

void jit_set_enabled(bool on) { g_enabled.store(on); }
bool jit_enabled() { return g_enabled.load(); }

// ---------------------------------------------------------------- automatic specialisation
namespace {

struct AutoJit {
    std::mutex mu;
    std::condition_variable cv, idle_cv;
    std::unordered_map<uint64_t, int> uses;        // interpreter launches per program hash
    std::unordered_set<uint64_t> queued;           // handed to the worker once, whatever the outcome
    struct Job {
        CompiledProgram prog;                      // a copy: the caller's may go away
        int device;
        bool variants;                             // build the batch variants, not the tree's kernels
    };
    std::deque<Job> work;
    std::unordered_set<uint64_t> variants_queued;
    int running = 0;
    int threshold = -1;                            // -1 = not read from the environment yet
    bool stop = false;
    std::thread worker;
    ~AutoJit()
    {
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
            work.clear();
        }
        cv.notify_all();
        if (worker.joinable()) worker.join();
    }
};

AutoJit& auto_jit()
{
    static AutoJit a;
    return a;
}

int threshold_locked(AutoJit& a)
{
    if (a.threshold < 0) {
        const char* env = std::getenv("FASTNOISE_AUTO_SPECIALISE");
        a.threshold = env && *env ? std::max(0, std::atoi(env)) : 4;
    }
    return a.threshold;
}

void auto_worker()
{
    AutoJit& a = auto_jit();
    std::unique_lock<std::mutex> lk(a.mu);
    for (;;) {
        a.cv.wait(lk, [&] { return a.stop || !a.work.empty(); });
        if (a.stop) return;
        AutoJit::Job job = std::move(a.work.front());
        a.work.pop_front();
        ++a.running;
        lk.unlock();
        cudaSetDevice(job.device);
        std::string err;
        if (job.variants) {
            if (is_built(job.prog.hash)) jit_build_batch_variants({&job.prog}, err);   // a failure keeps variant 0
        } else if (!is_built(job.prog.hash)) {
            jit_build({&job.prog}, err);           // a failure leaves the interpreter in use
        }
        lk.lock();
        --a.running;
        if (a.work.empty() && a.running == 0) a.idle_cv.notify_all();
    }
}

}  // namespace

bool jit_is_specialised(uint64_t hash)
{
    std::lock_guard<std::mutex> lk(g_jit_mu);
    return g_kernels.count(hash) && g_batch_kernels.count(hash);
}

void jit_note_interpreted(const CompiledProgram* prog)
{
    if (!prog || !g_enabled.load(std::memory_order_relaxed)) return;
    AutoJit& a = auto_jit();
    std::lock_guard<std::mutex> lk(a.mu);
    const int t = threshold_locked(a);
    if (t == 0 || a.stop || a.queued.count(prog->hash)) return;
    if (++a.uses[prog->hash] < t) return;
    a.queued.insert(prog->hash);
    a.uses.erase(prog->hash);
    int dev = 0;
    cudaGetDevice(&dev);
    a.work.push_back(AutoJit::Job{*prog, dev, false});
    if (!a.worker.joinable()) a.worker = std::thread(auto_worker);
    a.cv.notify_one();
}

void jit_request_batch_variants(const CompiledProgram* prog)
{
    if (!prog || !g_enabled.load(std::memory_order_relaxed)) return;
    AutoJit& a = auto_jit();
    std::lock_guard<std::mutex> lk(a.mu);
    if (a.stop || a.variants_queued.count(prog->hash)) return;
    a.variants_queued.insert(prog->hash);
    int dev = 0;
    cudaGetDevice(&dev);
    a.work.push_back(AutoJit::Job{*prog, dev, true});
    if (!a.worker.joinable()) a.worker = std::thread(auto_worker);
    a.cv.notify_one();
}

int jit_set_auto_threshold(int uses)
{
    AutoJit& a = auto_jit();
    std::lock_guard<std::mutex> lk(a.mu);
    const int was = threshold_locked(a);
    a.threshold = std::max(0, uses);
    return was;
}

bool jit_auto_wait(int timeout_ms)
{
    AutoJit& a = auto_jit();
    std::unique_lock<std::mutex> lk(a.mu);
    auto idle = [&] { return a.work.empty() && a.running == 0; };
    if (timeout_ms < 0) {
        a.idle_cv.wait(lk, idle);
        return true;
    }
    return a.idle_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), idle);
}

bool jit_launch(uint64_t hash, const PointArgs& args, float* out, MinMaxWork* work, float* dminmax, cudaStream_t stream,
                cudaError_t& err)
{
    err = cudaSuccess;
    JitKernels jk;
    if (args.total <= 0 || args.total > (1ll << 31) || !jit_lookup(hash, jk)) return false;
    const int which = args.src == kSrcGrid ? 0 : args.src == kSrcPositions ? 1 : 2;
    cudaKernel_t k = which == 0 ? jk.grid : which == 1 ? jk.positions : jk.tileable;
    if (!k) return false;
    const int sms = num_sms();
    unsigned ppl;
    long long blocks;
    if (args.total >= (long long)sms * 8 * 128 * 4) {
        // large calls: 4 points per lane (float4 stores), a grid of 8 blocks per SM striding over
        // the warp chunks
        ppl = 4u;
        blocks = std::min<long long>((args.total + 1023) / 1024, (long long)sms * 8);
    } else {
        // small calls are latency-bound: run them in one wave of the blocks that fit at once,
        // with as few points per lane as that allows (the fixed cost of a thread -- index set-up,
        // the min/max reduction -- is shared by its points)
        const long long resident = (long long)sms * std::max(1, jk.resident[which]) * 256;
        ppl = (unsigned)std::min<long long>(4, std::max<long long>(1, (args.total + resident - 1) / resident));
        blocks = (args.total + 256ll * ppl - 1) / (256ll * ppl);
    }
    if (blocks > kMaxReduceBlocks) blocks = kMaxReduceBlocks;
    if (blocks < 1) blocks = 1;
    PointArgs a = args;
    void* params[] = {&a, &out, &work, &dminmax, &ppl};
    err = cudaLaunchKernel((const void*)k, dim3((unsigned)blocks), dim3(256), params, 0, stream);
    return true;
}

bool jit_launch_solid(uint64_t hash, const PointArgs& args, unsigned* above, unsigned* solid, MinMaxWork* work, float* dminmax,
                      float iso, cudaStream_t stream, cudaError_t& err)
{
    err = cudaSuccess;
    JitKernels jk;
    if (args.total <= 0 || args.total > (1ll << 31) || !jit_lookup(hash, jk) || !jk.solid) return false;
    const int sms = num_sms();
    unsigned ppl = 4u;                                     // the grid as the large per-call calls run it
    long long blocks = std::min<long long>((args.total + 1023) / 1024, (long long)sms * 8);
    if (args.total < (long long)sms * 8 * 128 * 4) {
        const long long resident = (long long)sms * std::max(1, jk.resident[0]) * 256;
        ppl = (unsigned)std::min<long long>(4, std::max<long long>(1, (args.total + resident - 1) / resident));
        blocks = (args.total + 256ll * ppl - 1) / (256ll * ppl);
    }
    if (blocks > kMaxReduceBlocks) blocks = kMaxReduceBlocks;
    if (blocks < 1) blocks = 1;
    PointArgs a = args;
    void* params[] = {&a, &above, &solid, &work, &dminmax, &iso, &ppl};
    err = cudaLaunchKernel((const void*)jk.solid, dim3((unsigned)blocks), dim3(256), params, 0, stream);
    return true;
}

bool jit_launch_list(uint64_t hash, const PointArgs& args, const unsigned* idx, const unsigned* count, unsigned max_count,
                     float* out, cudaStream_t stream, cudaError_t& err)
{
    err = cudaSuccess;
    JitKernels jk;
    if (args.total <= 0 || args.total > (1ll << 31) || !jit_lookup(hash, jk) || !jk.list) return false;
    long long blocks = std::min<long long>(((long long)max_count + 255) / 256, (long long)num_sms() * 8);
    if (blocks < 1) blocks = 1;
    PointArgs a = args;
    void* params[] = {&a, &idx, &count, &out};
    err = cudaLaunchKernel((const void*)jk.list, dim3((unsigned)blocks), dim3(256), params, 0, stream);
    return true;
}

}  // namespace fn
