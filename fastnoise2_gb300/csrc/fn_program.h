// fn_program.h -- compact device program for one FastNoise2 node tree.
//
// A tree (FastNoise2's recursive Generator::Gen call graph, reference
// include/FastNoise/Generators/Generator.inl:48-67) is flattened by the host
// compiler (fn_compile.cpp) into a straight-line list of node operations over a
// small per-point register file.  Children evaluated at transformed positions
// (fractal octaves, domain warps, cellular lookups ...) are inlined per use, so
// evaluation order and arithmetic are identical to the reference's recursion.
//
// Layout in device memory (one contiguous, 16-byte aligned blob):
//   FnProgramHeader | FnInstr[n_instr] | float params[n_params]
#pragma once
#include <stdint.h>

#define FN_MAX_REGS 64
#define FN_MAX_INSTR 2048
#define FN_MAX_PARAMS 8192
#define FN_REG_NONE 255

enum FnOp : uint8_t {
    FN_OP_NOP = 0,
    FN_OP_CONST,       // R[dst] = P[prm]
    FN_OP_MOV,         // R[dst] = R[a]
    FN_OP_SCALE_POS,   // R[dst+k] = R[a+k] * P[prm]                       (k < dim)
    FN_OP_SCALE_POS_V, // R[dst+k] = R[a+k] * P[prm+k]
    FN_OP_OFFSET_POS,  // R[dst+k] = R[a+k] + R[{b,c,d,e}[k]]
    FN_OP_SUB_POS,     // R[dst+k] = R[a+k] - R[{b,c,d,e}[k]]
    FN_OP_ROTATE2,     // 2D yaw rotation, P[prm]=cos, P[prm+1]=sin          (dim = 2)
    FN_OP_ROTATE3,     // 3x3 matrix P[prm..prm+8]; dim = input dims (2 => z = 0), output 3
    FN_OP_ROTPLANE,    // DomainRotatePlane, aux = type; dim = input dims, output max(3, dim)
    FN_OP_NOISE,       // R[dst] = ScaleOutput(noise_aux(seed, R[a..]*P[prm]));  P[prm+1..3] = nmin, mul, rmin
    FN_OP_WHITE,       // P[prm..] = mul, rmin
    FN_OP_CHECKER,     // P[prm..] = freq, mul, rmin
    FN_OP_SINE,        // P[prm..] = freq, mul, rmin
    FN_OP_CELL_VALUE,  // a=pos b=jitter c=sizeJitter|NONE; P = freq, mul, rmin, minkowski; aux = df | vidx<<4
    FN_OP_CELL_DIST,   // P = freq, mul, rmin, minkowski; aux = df | i0<<4 | i1<<8 | ret<<12
    FN_OP_CELL_LOOKUP, // dst = out position group; P = freq, scale, minkowski; aux = df
    FN_OP_WARP_GRAD,   // dst = io position group, a = position read (times P[prm]), b = amp, c = strength out|NONE; P[prm+1..4] = axis scale
    FN_OP_FRACT_INIT,  // dst = sum, a = noise (abs'd in place if ridged), b = amp; aux = ridged
    FN_OP_FRACT_AMP,   // b = amp (in/out), a = previous noise, c = weighted strength, d = gain; aux = ridged
    FN_OP_FRACT_ACC,   // dst = sum (in/out), a = noise (in/out), b = amp; aux = ridged
    FN_OP_DWF_AMP,     // b = amp (in/out), a = strength (in/out, sqrt), c = weighted strength, d = gain
    FN_OP_ADD, FN_OP_SUB, FN_OP_MUL, FN_OP_DIV, FN_OP_MOD, FN_OP_MIN, FN_OP_MAX,   // R[dst] = R[a] op R[b]
    FN_OP_ABS, FN_OP_SSQRT,                                                          // R[dst] = f(R[a])
    FN_OP_POWF,        // R[dst] = pow(max(|R[a]|, FLT_MIN), R[b])
    FN_OP_POWI,        // R[dst] = R[a]^aux (aux >= 2, repeated multiply)
    FN_OP_MINSMOOTH, FN_OP_MAXSMOOTH,   // a = lhs, b = rhs, c = smoothness
    FN_OP_FADE,        // a = A, b = B, c = fade, d = fade min, e = fade max; aux = interpolation
    FN_OP_REMAP,       // a = src, b..e = from min/max, to min/max; aux = clamp
    FN_OP_TERRACE,     // a = src; b = dynamic smoothness|NONE; P = steps, step recip, smooth recip; aux = const smoothing on
    FN_OP_PINGPONG,    // a = src, b = strength
    FN_OP_RGBA8,       // a = src; P = min, max
    FN_OP_GRADIENT,    // a = pos, b..e = offsets; P[prm..prm+3] = multipliers
    FN_OP_DISTANCE,    // a = offset vector, b = minkowski reg|NONE; aux = df | sqrt<<4
    FN_OP_WARP_SIMPLEX,// as FN_OP_WARP_GRAD; aux = super (bit 0) | gradient outer product scheme (bit 1)
    FN_OP_COUNT
};

enum FnNoiseKind : uint16_t {
    FN_NOISE_SIMPLEX = 0,
    FN_NOISE_SUPERSIMPLEX,
    FN_NOISE_PERLIN,
    FN_NOISE_VALUE,
};

struct FnInstr {          // 16 bytes
    uint8_t op;
    uint8_t dim;
    uint8_t dst;
    uint8_t a;
    uint8_t b, c, d, e;
    uint16_t prm;
    uint16_t aux;
    int32_t seed;         // added to the call seed
};

struct FnProgramHeader {  // 32 bytes
    uint32_t magic;       // 'FNP1'
    uint16_t n_instr;
    uint16_t n_regs;
    uint16_t n_params;
    uint8_t dim;          // root dimensionality the program was compiled for
    uint8_t out_reg;      // register holding the result
    uint32_t bytes;       // total blob size
    uint32_t flags;
    uint64_t hash;        // content hash (cache key)
};

#define FN_PROGRAM_MAGIC 0x31504E46u

#ifdef __CUDACC__
#define FN_HD __host__ __device__ __forceinline__
#else
#define FN_HD inline
#endif

FN_HD const FnInstr* fn_program_instrs(const FnProgramHeader* h)
{
    return reinterpret_cast<const FnInstr*>(reinterpret_cast<const char*>(h) + sizeof(FnProgramHeader));
}
FN_HD const float* fn_program_params(const FnProgramHeader* h)
{
    return reinterpret_cast<const float*>(fn_program_instrs(h) + h->n_instr);
}
