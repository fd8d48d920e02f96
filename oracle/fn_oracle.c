/*
 * fn_oracle.c -- CPU restatement of FastNoise2's node-tree evaluation.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: tests, the smoke
 * check and the CPU-baseline leg of bench.py call it as the *checker*; the
 * product (fastnoise2_gb300) never links, includes or calls it.
 *
 * It restates, scalar and one point at a time, the reference's hot path:
 *   include/FastNoise/Generators/Generator.inl  (batch drivers, min/max)
 *   include/FastNoise/Generators/Utils.inl      (hash, gradients, fades, distances)
 *   include/FastNoise/Generators/{BasicGenerators,Simplex,Perlin,Value,Cellular,
 *     Fractal,DomainWarp,DomainWarpFractal,Modifiers,Blends}.inl
 * following the portable (non-AVX) branches of the table-driven helpers, and the
 * member setters of the node classes in include/FastNoise/Generators/<Node>.h.
 *
 * PARITY UNPINNED: the reference ships no golden values, and every arithmetic
 * primitive it calls (FS::*) lives in FastSIMD @ 16450dae9528727e500e7254f635a671f9c7ee2d,
 * which is not vendored.  The semantics assumed for FS:: ops (the "strict-FP"
 * build, FASTNOISE2_STRICT_FP=ON) are:
 *   FMulAdd/FNMulAdd/FMulSub  fused (single rounding)  [fused mode, default]
 *                             or mul-then-add          [unfused mode]
 *   Convert<int32>(f)         round-to-nearest-even; NaN / out of range -> INT32_MIN
 *   Convert<float>(i)         round-to-nearest-even
 *   Floor, Round              exact floor, round-half-even
 *   Min(a,b) / Max(a,b)       a<b?a:b / a>b?a:b   (x86 minps/maxps operand order)
 *   InvSqrt(x), Reciprocal(x) 1.0f/sqrtf(x), 1.0f/x (correctly rounded steps)
 *   Sqrt                      correctly rounded
 *   Sin, Cos                  fn_sinf/fn_cosf below (Cody-Waite + Taylor, ~1 ulp)
 *   Pow(x,y)                  fn_powf below (exp2(y*log2 x), ~2 ulp for moderate y)
 *   Modulus(a,b)              a - truncf(a/b)*b
 *   int32 * and + wrap; >> arithmetic; BitShiftRightZeroExtend logical.
 *
 * The file is written in the common subset of C and C++ so that it can also be
 * compiled with a counting scalar type (see opcount.h) to measure FS-level
 * operations per point.
 */
#if !defined(__cplusplus) && !defined(_POSIX_C_SOURCE)
#define _POSIX_C_SOURCE 200809L /* clock_gettime under -std=c11 */
#endif
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#include <pthread.h>
#include <time.h>

#ifdef OC_COUNT
#include "opcount.h"
#else
typedef float f32;
typedef int32_t i32;
#define OC_TICK(n) ((void)0)
#endif

#ifdef __cplusplus
#define OC_EXPORT extern "C" __attribute__((visibility("default")))
#else
#define OC_EXPORT __attribute__((visibility("default")))
#endif

/* ------------------------------------------------------------------------- */
/* FS-level primitives                                                        */
/* ------------------------------------------------------------------------- */

static int g_unfused = 0;   /* 0: FMulAdd fused (AVX2/AVX-512/NEON), 1: scalar-style mul+add */

static inline float bits_f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline uint32_t f_bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

static inline f32 fs_fma(f32 a, f32 b, f32 c)
{
    OC_TICK(1);
    if (g_unfused) { float p = (float)a * (float)b; return p + (float)c; }
    return fmaf((float)a, (float)b, (float)c);
}
/* FS::FNMulAdd(a,b,c) = -(a*b) + c */
static inline f32 fs_fnma(f32 a, f32 b, f32 c)
{
    OC_TICK(1);
    if (g_unfused) { float p = (float)a * (float)b; return (float)c - p; }
    return fmaf(-(float)a, (float)b, (float)c);
}
/* FS::FMulSub(a,b,c) = a*b - c */
static inline f32 fs_fms(f32 a, f32 b, f32 c)
{
    OC_TICK(1);
    if (g_unfused) { float p = (float)a * (float)b; return p - (float)c; }
    return fmaf((float)a, (float)b, -(float)c);
}
static inline f32 fs_min(f32 a, f32 b) { OC_TICK(1); return ((float)a < (float)b) ? a : b; }
static inline f32 fs_max(f32 a, f32 b) { OC_TICK(1); return ((float)a > (float)b) ? a : b; }
static inline f32 fs_abs(f32 a) { OC_TICK(1); return bits_f(f_bits((float)a) & 0x7FFFFFFFu); }
static inline f32 fs_floor(f32 a) { OC_TICK(1); return floorf((float)a); }
static inline f32 fs_round(f32 a) { OC_TICK(1); return nearbyintf((float)a); }
static inline f32 fs_sqrt(f32 a) { OC_TICK(1); return sqrtf((float)a); }
static inline f32 fs_invsqrt(f32 a) { OC_TICK(2); return 1.0f / sqrtf((float)a); }
static inline f32 fs_recip(f32 a) { OC_TICK(1); return 1.0f / (float)a; }
static inline i32 fs_cvt_i(f32 a)
{
    OC_TICK(1);
    float f = (float)a;
    if (f >= -2147483648.0f && f < 2147483648.0f) return (int32_t)nearbyintf(f);
    return INT32_MIN;
}
static inline f32 fs_cvt_f(i32 a) { OC_TICK(1); return (float)(int32_t)a; }
/* sign-bit xor: flips the sign of v when bit 31 of s is set (float ^ Cast<float>(int)) */
static inline f32 fs_xor_sign(f32 v, i32 s) { OC_TICK(1); return bits_f(f_bits((float)v) ^ ((uint32_t)(int32_t)s & 0x80000000u)); }

static inline i32 imul(i32 a, i32 b) { OC_TICK(1); return (int32_t)((uint32_t)(int32_t)a * (uint32_t)(int32_t)b); }
static inline i32 iadd(i32 a, i32 b) { OC_TICK(1); return (int32_t)((uint32_t)(int32_t)a + (uint32_t)(int32_t)b); }
static inline i32 isub(i32 a, i32 b) { OC_TICK(1); return (int32_t)((uint32_t)(int32_t)a - (uint32_t)(int32_t)b); }
static inline i32 ishl(i32 a, int s) { OC_TICK(1); return (int32_t)((uint32_t)(int32_t)a << s); }
static inline i32 isra(i32 a, int s) { OC_TICK(1); return (int32_t)a >> s; }
static inline i32 isrl(i32 a, int s) { OC_TICK(1); return (int32_t)((uint32_t)(int32_t)a >> s); }

/* Sin / Cos: Cody-Waite reduction by pi/2 (three-part constant) and Taylor
 * polynomials on [-pi/4, pi/4].  The CUDA kernels evaluate the identical
 * operation sequence, so both sides agree bit for bit. */
static const float kTwoOverPi = 0x1.45f306p-1f;
static const float kPio2Hi = 0x1.921fb6p+0f;
static const float kPio2Mid = -0x1.777a5cp-25f;
static const float kPio2Lo = -0x1.ee59dap-50f;

static inline float sincos_reduce(float x, int* quadrant)
{
    float k = nearbyintf(x * kTwoOverPi);
    float r = fmaf(-k, kPio2Hi, x);
    r = fmaf(-k, kPio2Mid, r);
    r = fmaf(-k, kPio2Lo, r);
    *quadrant = (int)(int64_t)k & 3;
    return r;
}
static inline float sin_poly(float r)
{
    float r2 = r * r;
    float p = fmaf(r2, -0x1.ae6456p-26f, 0x1.71de3ap-19f);
    p = fmaf(r2, p, -0x1.a01a02p-13f);
    p = fmaf(r2, p, 0x1.111112p-7f);
    p = fmaf(r2, p, -0x1.555556p-3f);
    return fmaf(r * r2, p, r);
}
static inline float cos_poly(float r)
{
    float r2 = r * r;
    float p = fmaf(r2, 0x1.1eed8ep-29f, -0x1.27e4fcp-22f);
    p = fmaf(r2, p, 0x1.a01a02p-16f);
    p = fmaf(r2, p, -0x1.6c16c2p-10f);
    p = fmaf(r2, p, 0x1.555556p-5f);
    p = fmaf(r2, p, -0.5f);
    return fmaf(r2, p, 1.0f);
}
OC_EXPORT float fn_sinf(float x)
{
    int q;
    float r = sincos_reduce(x, &q);
    float s = (q & 1) ? cos_poly(r) : sin_poly(r);
    return (q & 2) ? -s : s;
}
OC_EXPORT float fn_cosf(float x)
{
    int q;
    float r = sincos_reduce(x, &q);
    float c = (q & 1) ? sin_poly(r) : cos_poly(r);
    return ((q + 1) & 2) ? -c : c;
}
static inline f32 fs_sin(f32 x) { OC_TICK(20); return fn_sinf((float)x); }
static inline f32 fs_cos(f32 x) { OC_TICK(20); return fn_cosf((float)x); }

/* Pow for x > 0: 2^(y*log2(x)).  log2 via m in [sqrt(1/2), sqrt(2)) and the
 * atanh series; exp2 via round-to-nearest split and a Taylor polynomial. */
static inline float log2_pos(float x)
{
    uint32_t u = f_bits(x);
    int e = (int)((u >> 23) & 0xFF);
    if (e == 0) {                       /* subnormal: rescale */
        x *= 0x1p23f; u = f_bits(x); e = (int)((u >> 23) & 0xFF) - 23;
    }
    int ex = e - 127;
    float m = bits_f((u & 0x007FFFFFu) | 0x3F800000u);
    if (m > 1.41421356f) { m *= 0.5f; ex += 1; }
    float s = (m - 1.0f) / (m + 1.0f);
    float s2 = s * s;
    float p = fmaf(s2, 0x1.745d18p-4f, 0x1.c71c72p-4f);   /* 1/11, 1/9 */
    p = fmaf(s2, p, 0x1.24924ap-3f);                      /* 1/7 */
    p = fmaf(s2, p, 0x1.99999ap-3f);                      /* 1/5 */
    p = fmaf(s2, p, 0x1.555556p-2f);                      /* 1/3 */
    p = fmaf(s2, p, 1.0f);
    float ln = 2.0f * s * p;
    return fmaf(ln, 0x1.715476p+0f, (float)ex);           /* ln * log2(e) + ex */
}
static inline float exp2_any(float t)
{
    if (!(t < 128.0f)) return (t != t) ? t : INFINITY;
    if (t < -150.0f) return 0.0f;
    float n = nearbyintf(t);
    float f = t - n;
    float a = f * 0x1.62e430p-1f;                         /* f * ln2 */
    float p = fmaf(a, 0x1.a01a02p-13f, 0x1.6c16c2p-10f);  /* 1/5040, 1/720 */
    p = fmaf(a, p, 0x1.111112p-7f);                       /* 1/120 */
    p = fmaf(a, p, 0x1.555556p-5f);                       /* 1/24 */
    p = fmaf(a, p, 0x1.555556p-3f);                       /* 1/6 */
    p = fmaf(a, p, 0.5f);
    p = fmaf(a, p, 1.0f);
    p = fmaf(a, p, 1.0f);
    int ni = (int)n;
    /* scale by 2^ni in two steps so that subnormal results stay representable */
    int n1 = ni / 2, n2 = ni - n1;
    return p * bits_f((uint32_t)(n1 + 127) << 23) * bits_f((uint32_t)(n2 + 127) << 23);
}
OC_EXPORT float fn_powf(float x, float y)
{
    if (y == 0.0f) return 1.0f;
    if (x != x || y != y) return x + y;
    if (x == 0.0f) return y > 0.0f ? 0.0f : INFINITY;
    if (x < 0.0f) return NAN;
    if (x == INFINITY) return y > 0.0f ? INFINITY : 0.0f;
    return exp2_any(y * log2_pos(x));
}
static inline f32 fs_pow(f32 x, f32 y) { OC_TICK(30); return fn_powf((float)x, (float)y); }
static inline f32 fs_mod(f32 a, f32 b)
{
    OC_TICK(4);
    float q = (float)a / (float)b;
    float t = truncf(q);
    return (float)a - t * (float)b;
}

/* ------------------------------------------------------------------------- */
/* Utils.inl restatement                                                      */
/* ------------------------------------------------------------------------- */

#define PRIME_X ((int32_t)0xF797C5C7)   /* Utils.inl:8-11 */
#define PRIME_Y ((int32_t)0x6C060C89)
#define PRIME_Z ((int32_t)0x465FD04F)
#define PRIME_W ((int32_t)0xF7A62279)
#define HASH_A ((int32_t)0xB7E0A5F5)    /* Utils.inl:18 */

static const double kRoot2 = 1.4142135623730950488016887242097;
static const double kRoot3 = 1.7320508075688772935274463415059;
static const double kRoot5 = 2.2360679774997896964091736687313;
static const float kValueBounds = 2147483648.f;

/* HashPrimes (Utils.inl:221-230) */
static inline i32 hash2(i32 seed, i32 a, i32 b)
{
    OC_TICK(2);
    i32 h = (int32_t)seed ^ (int32_t)a ^ (int32_t)b;
    h = imul(h, HASH_A);
    OC_TICK(1);
    return isra(h, 15) ^ (int32_t)h;
}
static inline i32 hash3(i32 seed, i32 a, i32 b, i32 c)
{
    OC_TICK(3);
    i32 h = (int32_t)seed ^ (int32_t)a ^ (int32_t)b ^ (int32_t)c;
    h = imul(h, HASH_A);
    OC_TICK(1);
    return isra(h, 15) ^ (int32_t)h;
}
static inline i32 hash4(i32 seed, i32 a, i32 b, i32 c, i32 d)
{
    OC_TICK(4);
    i32 h = (int32_t)seed ^ (int32_t)a ^ (int32_t)b ^ (int32_t)c ^ (int32_t)d;
    h = imul(h, HASH_A);
    OC_TICK(1);
    return isra(h, 15) ^ (int32_t)h;
}
/* HashPrimesHB (Utils.inl:232-240) */
static inline i32 hashhb2(i32 seed, i32 a, i32 b) { OC_TICK(2); return imul((int32_t)seed ^ (int32_t)a ^ (int32_t)b, HASH_A); }
static inline i32 hashhb3(i32 seed, i32 a, i32 b, i32 c) { OC_TICK(3); return imul((int32_t)seed ^ (int32_t)a ^ (int32_t)b ^ (int32_t)c, HASH_A); }
static inline i32 hashhb4(i32 seed, i32 a, i32 b, i32 c, i32 d) { OC_TICK(4); return imul((int32_t)seed ^ (int32_t)a ^ (int32_t)b ^ (int32_t)c ^ (int32_t)d, HASH_A); }
/* GetValueCoord (Utils.inl:242-250): hash *= hash * A; float(hash) */
static inline f32 valcoord_h(i32 h) { return fs_cvt_f(imul(h, imul(h, HASH_A))); }
static inline f32 valcoord2(i32 seed, i32 a, i32 b) { OC_TICK(2); return valcoord_h((int32_t)seed ^ (int32_t)a ^ (int32_t)b); }
static inline f32 valcoord3(i32 seed, i32 a, i32 b, i32 c) { OC_TICK(3); return valcoord_h((int32_t)seed ^ (int32_t)a ^ (int32_t)b ^ (int32_t)c); }
static inline f32 valcoord4(i32 seed, i32 a, i32 b, i32 c, i32 d) { OC_TICK(4); return valcoord_h((int32_t)seed ^ (int32_t)a ^ (int32_t)b ^ (int32_t)c ^ (int32_t)d); }

/* GetGradientDotCommon, portable branch (Utils.inl:132-158) */
static inline f32 grad_common(i32 hash, f32 fX, f32 fY, f32 fZ)
{
    OC_TICK(1);
    int32_t h13 = (int32_t)hash & 13;
    OC_TICK(4);
    f32 u = (h13 > 7) ? fY : fX;
    f32 v = (h13 == 12) ? fX : fZ;
    v = (h13 < 2) ? fY : v;
    f32 h1u = fs_xor_sign(u, ishl(hash, 31));
    f32 h2v = fs_xor_sign(v, ishl(isra(hash, 1), 31));
    return h1u + h2v;
}
/* GetGradientDotPerlin 2D, portable branch (Utils.inl:181-190) */
static inline f32 grad_perlin2(i32 hash, f32 fX, f32 fY)
{
    fX = fs_xor_sign(fX, ishl(hash, 31));
    fY = fs_xor_sign(fY, ishl(isra(hash, 1), 31));
    i32 sel = ishl(hash, 29);
    OC_TICK(2);
    f32 u = ((int32_t)sel < 0) ? fY : fX;
    f32 v = ((int32_t)sel < 0) ? fX : fY;
    return fs_fma(1.0f + (float)kRoot2, u, v);
}
/* GetGradientDotPerlin 4D, portable branch (Utils.inl:205-218) */
static inline f32 grad_perlin4(i32 hash, f32 fX, f32 fY, f32 fZ, f32 fW)
{
    OC_TICK(1);
    int32_t p = (int32_t)hash & (3 << 3);
    OC_TICK(3);
    f32 a = (p > 0) ? fX : fY;
    f32 b = ((int32_t)ishl(hash, 27) < 0) ? fY : fZ;
    f32 c = (p > (2 << 3)) ? fZ : fW;
    f32 as = fs_xor_sign(a, ishl(hash, 31));
    f32 bs = fs_xor_sign(b, ishl(isra(hash, 1), 31));
    f32 cs = fs_xor_sign(c, ishl(isra(hash, 2), 31));
    return (as + bs) + cs;
}

static inline f32 lerp(f32 a, f32 b, f32 t) { return fs_fma(t, b - a, a); }               /* Utils.inl:252 */
static inline f32 interp_hermite(f32 t) { return t * t * fs_fnma(t, 2.0f, 3.0f); }          /* Utils.inl:257 */
static inline f32 interp_quintic(f32 t) { return t * t * t * fs_fma(t, fs_fma(t, 6.0f, -15.0f), 10.0f); } /* :262 */

/* ------------------------------------------------------------------------- */
/* Node model                                                                 */
/* ------------------------------------------------------------------------- */

enum {
    N_CONSTANT = 0, N_WHITE, N_CHECKERBOARD, N_SINEWAVE, N_GRADIENT, N_DISTANCETOPOINT,
    N_SIMPLEX, N_SUPERSIMPLEX, N_PERLIN, N_VALUE,
    N_CELLULARVALUE, N_CELLULARDISTANCE, N_CELLULARLOOKUP,
    N_FRACTALFBM, N_PINGPONG, N_FRACTALRIDGED,
    N_DOMAINWARPSIMPLEX, N_DOMAINWARPSUPERSIMPLEX, N_DOMAINWARPGRADIENT,
    N_DWFRACTALPROGRESSIVE, N_DWFRACTALINDEPENDENT,
    N_ADD, N_SUBTRACT, N_MULTIPLY, N_DIVIDE,
    N_ABS, N_MIN, N_MAX, N_MINSMOOTH, N_MAXSMOOTH, N_SIGNEDSQRT, N_POWFLOAT, N_POWINT,
    N_DOMAINSCALE, N_DOMAINOFFSET, N_DOMAINROTATE, N_DOMAINAXISSCALE,
    N_SEEDOFFSET, N_CONVERTRGBA8, N_GENERATORCACHE,
    N_FADE, N_REMAP, N_TERRACE, N_ADDDIMENSION, N_REMOVEDIMENSION,
    N_MODULUS, N_DOMAINROTATEPLANE,
    N_COUNT
};

typedef struct on_node {
    int id;
    struct on_node* lookup[2];
    struct on_node* hnode[8];
    float hval[8];
    /* reference member state (as the setters leave it) */
    float scale, frequency;            /* ScalableGenerator */
    int seed_offset;                   /* Seeded / SeedOffset::mOffset */
    float range_min, range_scale;      /* VariableRange */
    float value;                       /* Constant */
    float multiplier[4];               /* Gradient */
    float axis[4];                     /* DomainWarp::mAxisScale, DomainAxisScale::mScale */
    int dist_func, value_index, dist_idx0, dist_idx1, return_type;
    int octaves; float lacunarity;
    int vec_scheme;
    int pow_int;
    float dscale;                      /* DomainScale */
    float yaw_cos, yaw_sin, pitch_cos, pitch_sin, roll_cos, roll_sin;
    float rot[9];                      /* Xa Xb Xc Ya Yb Yc Za Zb Zc */
    float rgba_min, rgba_max;
    int interp, clamp_output;
    float step_count, step_recip, smooth_recip;
    int remove_dim, rot_type;
} on_node;

/* member-variable setter kinds, per node, in metadata order */
enum {
    V_SCALE = 1, V_SEED, V_OMIN, V_OMAX, V_VALUE, V_MULT0, V_DISTF = V_MULT0 + 4, V_VALIDX, V_DIDX0, V_DIDX1,
    V_RET, V_OCT, V_LAC, V_AXIS0, V_VEC = V_AXIS0 + 4, V_POWI, V_DSCALE, V_YAW, V_PITCH, V_ROLL,
    V_SOFF, V_RGBMIN, V_RGBMAX, V_INTERP, V_CLAMP, V_STEPS, V_REMDIM, V_ROTTYPE
};

static const int kVarKinds[N_COUNT][8] = {
    /* Constant */ {V_VALUE},
    /* White */ {V_SEED, V_OMIN, V_OMAX},
    /* Checkerboard */ {V_SCALE, V_OMIN, V_OMAX},
    /* SineWave */ {V_SCALE, V_OMIN, V_OMAX},
    /* Gradient */ {V_MULT0, V_MULT0 + 1, V_MULT0 + 2, V_MULT0 + 3},
    /* DistanceToPoint */ {V_DISTF},
    /* Simplex */ {V_SCALE, V_SEED, V_OMIN, V_OMAX},
    /* SuperSimplex */ {V_SCALE, V_SEED, V_OMIN, V_OMAX},
    /* Perlin */ {V_SCALE, V_SEED, V_OMIN, V_OMAX},
    /* Value */ {V_SCALE, V_SEED, V_OMIN, V_OMAX},
    /* CellularValue */ {V_SCALE, V_SEED, V_OMIN, V_OMAX, V_DISTF, V_VALIDX},
    /* CellularDistance */ {V_SCALE, V_SEED, V_OMIN, V_OMAX, V_DISTF, V_DIDX0, V_DIDX1, V_RET},
    /* CellularLookup */ {V_SCALE, V_SEED, V_DISTF},
    /* FractalFBm */ {V_OCT, V_LAC},
    /* PingPong */ {0},
    /* FractalRidged */ {V_OCT, V_LAC},
    /* DomainWarpSimplex */ {V_SCALE, V_SEED, V_AXIS0, V_AXIS0 + 1, V_AXIS0 + 2, V_AXIS0 + 3, V_VEC},
    /* DomainWarpSuperSimplex */ {V_SCALE, V_SEED, V_AXIS0, V_AXIS0 + 1, V_AXIS0 + 2, V_AXIS0 + 3, V_VEC},
    /* DomainWarpGradient */ {V_SCALE, V_SEED, V_AXIS0, V_AXIS0 + 1, V_AXIS0 + 2, V_AXIS0 + 3},
    /* DWFractalProgressive */ {V_OCT, V_LAC},
    /* DWFractalIndependent */ {V_OCT, V_LAC},
    /* Add */ {0}, /* Subtract */ {0}, /* Multiply */ {0}, /* Divide */ {0},
    /* Abs */ {0}, /* Min */ {0}, /* Max */ {0}, /* MinSmooth */ {0}, /* MaxSmooth */ {0},
    /* SignedSquareRoot */ {0}, /* PowFloat */ {0},
    /* PowInt */ {V_POWI},
    /* DomainScale */ {V_DSCALE},
    /* DomainOffset */ {0},
    /* DomainRotate */ {V_YAW, V_PITCH, V_ROLL},
    /* DomainAxisScale */ {V_AXIS0, V_AXIS0 + 1, V_AXIS0 + 2, V_AXIS0 + 3},
    /* SeedOffset */ {V_SOFF},
    /* ConvertRGBA8 */ {V_RGBMIN, V_RGBMAX},
    /* GeneratorCache */ {0},
    /* Fade */ {V_INTERP},
    /* Remap */ {V_CLAMP},
    /* Terrace */ {V_STEPS},
    /* AddDimension */ {0},
    /* RemoveDimension */ {V_REMDIM},
    /* Modulus */ {0},
    /* DomainRotatePlane */ {V_ROTTYPE},
};

/* hybrid defaults per node (metadata order, include/FastNoise/Generators/<Node>.h) */
static void hybrid_defaults(int id, float* h)
{
    for (int k = 0; k < 8; ++k) h[k] = 0.0f;
    switch (id) {
    case N_DISTANCETOPOINT: h[4] = 1.5f; break;
    case N_CELLULARVALUE: case N_CELLULARDISTANCE: case N_CELLULARLOOKUP: h[0] = 1.5f; h[1] = 1.0f; break;
    case N_FRACTALFBM: case N_FRACTALRIDGED: case N_DWFRACTALPROGRESSIVE: case N_DWFRACTALINDEPENDENT: h[0] = 0.5f; break;
    case N_PINGPONG: h[0] = 2.0f; break;
    case N_DOMAINWARPSIMPLEX: case N_DOMAINWARPSUPERSIMPLEX: case N_DOMAINWARPGRADIENT: h[0] = 50.0f; break;
    case N_MINSMOOTH: case N_MAXSMOOTH: h[1] = 0.1f; break;
    case N_POWFLOAT: h[0] = 2.0f; h[1] = 2.0f; break;
    case N_FADE: h[1] = -1.0f; h[2] = 1.0f; break;
    case N_REMAP: h[0] = -1.0f; h[1] = 1.0f; h[3] = 1.0f; break;
    default: break;
    }
}

static void rotate_calc(on_node* n)   /* DomainRotate::CalculateRotation (Modifiers.h:104-117) */
{
    n->rot[0] = n->yaw_cos * n->pitch_cos;
    n->rot[1] = n->yaw_cos * n->pitch_sin * n->roll_sin - n->yaw_sin * n->roll_cos;
    n->rot[2] = n->yaw_cos * n->pitch_sin * n->roll_cos + n->yaw_sin * n->roll_sin;
    n->rot[3] = n->yaw_sin * n->pitch_cos;
    n->rot[4] = n->yaw_sin * n->pitch_sin * n->roll_sin + n->yaw_cos * n->roll_cos;
    n->rot[5] = n->yaw_sin * n->pitch_sin * n->roll_cos - n->yaw_cos * n->roll_sin;
    n->rot[6] = -n->pitch_sin;
    n->rot[7] = n->pitch_cos * n->roll_sin;
    n->rot[8] = n->pitch_cos * n->roll_cos;
}

static int clamp03(int v) { return v < 0 ? 0 : (v > 3 ? 3 : v); }

OC_EXPORT on_node* on_new(int id)
{
    if (id < 0 || id >= N_COUNT) return NULL;
    on_node* n = (on_node*)calloc(1, sizeof(on_node));
    n->id = id;
    n->scale = 100.0f; n->frequency = 1.0f / 100;          /* BasicGenerators.h:27-28 */
    n->range_min = -1.0f; n->range_scale = 2.0f;            /* BasicGenerators.h:111-112 */
    n->value = 1.0f;
    n->dist_func = 1;                                       /* EuclideanSquared */
    n->dist_idx1 = 1;
    n->octaves = 3; n->lacunarity = 2.0f;
    for (int k = 0; k < 4; ++k) n->axis[k] = 1.0f;
    n->pow_int = 2;
    n->dscale = 1.0f;
    n->yaw_cos = n->pitch_cos = n->roll_cos = 1.0f;
    n->rot[0] = n->rot[4] = n->rot[8] = 1.0f;
    n->rgba_min = -1.0f; n->rgba_max = 1.0f;
    n->step_count = 1.0f; n->step_recip = 1.0f;
    n->remove_dim = 1;
    if (id == N_SEEDOFFSET) n->seed_offset = 1;             /* Modifiers.h:149 */
    hybrid_defaults(id, n->hval);
    return n;
}

OC_EXPORT void on_free(on_node* n) { free(n); }

/* Apply a member-variable setter with raw ValueUnion bits (Metadata.h:75-104). */
OC_EXPORT int on_set_var(on_node* n, int idx, int32_t bits)
{
    if (idx < 0 || idx >= 8) return 0;
    int kind = kVarKinds[n->id][idx];
    if (!kind) return 0;
    float f = bits_f((uint32_t)bits);
    int i = bits;
    switch (kind) {
    case V_SCALE: n->scale = f; n->frequency = 1.0f / f; break;      /* BasicGenerators.h:20-24 */
    case V_SEED: n->seed_offset = i; break;
    case V_OMIN: n->range_scale += n->range_min - f; n->range_min = f; break;   /* :96-100 */
    case V_OMAX: n->range_scale = (f - n->range_min); break;                    /* :105-108 */
    case V_VALUE: n->value = f; break;
    case V_MULT0: case V_MULT0 + 1: case V_MULT0 + 2: case V_MULT0 + 3: n->multiplier[kind - V_MULT0] = f; break;
    case V_DISTF: n->dist_func = i; break;
    case V_VALIDX: n->value_index = clamp03(i); break;                  /* Cellular.h:65 */
    case V_DIDX0: n->dist_idx0 = clamp03(i); break;                     /* Cellular.h:104 */
    case V_DIDX1: n->dist_idx1 = clamp03(i); break;
    case V_RET: n->return_type = i; break;
    case V_OCT: n->octaves = i; break;
    case V_LAC: n->lacunarity = f; break;
    case V_AXIS0: case V_AXIS0 + 1: case V_AXIS0 + 2: case V_AXIS0 + 3: n->axis[kind - V_AXIS0] = f; break;
    case V_VEC: n->vec_scheme = i; break;
    case V_POWI: n->pow_int = i; break;
    case V_DSCALE: n->dscale = f; break;
    case V_YAW: n->yaw_cos = cosf(f); n->yaw_sin = sinf(f); rotate_calc(n); break;     /* Modifiers.h:81-83 */
    case V_PITCH: n->pitch_cos = cosf(f); n->pitch_sin = sinf(f); rotate_calc(n); break;
    case V_ROLL: n->roll_cos = cosf(f); n->roll_sin = sinf(f); rotate_calc(n); break;
    case V_SOFF: n->seed_offset = i; break;
    case V_RGBMIN: n->rgba_min = f; break;
    case V_RGBMAX: n->rgba_max = f; break;
    case V_INTERP: n->interp = i; break;
    case V_CLAMP: n->clamp_output = i; break;
    case V_STEPS: n->step_count = f; n->step_recip = 1 / f; break;    /* Modifiers.h:276 */
    case V_REMDIM: n->remove_dim = i; break;
    case V_ROTTYPE: n->rot_type = i; break;
    default: return 0;
    }
    return 1;
}

OC_EXPORT int on_set_lookup(on_node* n, int idx, on_node* child)
{
    if (idx < 0 || idx >= 2) return 0;
    n->lookup[idx] = child;
    return 1;
}

OC_EXPORT int on_set_hybrid_node(on_node* n, int idx, on_node* child)
{
    if (idx < 0 || idx >= 8) return 0;
    n->hnode[idx] = child;
    return 1;
}

OC_EXPORT int on_set_hybrid_float(on_node* n, int idx, float v)
{
    if (idx < 0 || idx >= 8) return 0;
    n->hnode[idx] = NULL;
    n->hval[idx] = v;
    if (n->id == N_TERRACE && v != 0.0f) n->smooth_recip = 1 + 1 / v;   /* Modifiers.h:278 */
    return 1;
}

/* ------------------------------------------------------------------------- */
/* Evaluation                                                                 */
/* ------------------------------------------------------------------------- */

static f32 gen2(const on_node* n, i32 seed, f32 x, f32 y);
static f32 gen3(const on_node* n, i32 seed, f32 x, f32 y, f32 z);
static f32 gen4(const on_node* n, i32 seed, f32 x, f32 y, f32 z, f32 w);

#define HYB2(n, k, s, x, y) ((n)->hnode[k] ? gen2((n)->hnode[k], s, x, y) : (f32)(n)->hval[k])
#define HYB3(n, k, s, x, y, z) ((n)->hnode[k] ? gen3((n)->hnode[k], s, x, y, z) : (f32)(n)->hval[k])
#define HYB4(n, k, s, x, y, z, w) ((n)->hnode[k] ? gen4((n)->hnode[k], s, x, y, z, w) : (f32)(n)->hval[k])

/* VariableRange::ScaleOutput (BasicGenerators.inl:27-30) */
static inline f32 scale_output(const on_node* n, f32 value, float nmin, float nmax)
{
    float mul = (1.0f / (nmax - nmin)) * n->range_scale;
    return fs_fma(mul, value - nmin, n->range_min);
}

/* ---- Simplex (Simplex.inl:7-286) ---------------------------------------- */

static f32 simplex2(const on_node* n, i32 seed, f32 x, f32 y)
{
    seed = iadd(seed, n->seed_offset);
    x = x * n->frequency; y = y * n->frequency;
    const double kSkew2 = 1.0 / (kRoot3 + 1.0);
    const double kUnskew2 = -1.0 / (kRoot3 + 3.0);
    const double kFalloffRadiusSquared = 0.5;

    f32 skewDelta = (float)kSkew2 * (x + y);
    f32 xSkewed = x + skewDelta, ySkewed = y + skewDelta;
    f32 xSkewedBase = fs_floor(xSkewed), ySkewedBase = fs_floor(ySkewed);
    f32 dxSkewed = xSkewed - xSkewedBase, dySkewed = ySkewed - ySkewedBase;
    i32 xPrimedBase = imul(fs_cvt_i(xSkewedBase), PRIME_X);
    i32 yPrimedBase = imul(fs_cvt_i(ySkewedBase), PRIME_Y);
    int xGreaterEqualY = dxSkewed >= dySkewed;

    f32 unskewDelta = (float)kUnskew2 * (dxSkewed + dySkewed);
    f32 dx0 = dxSkewed + unskewDelta, dy0 = dySkewed + unskewDelta;
    f32 dx1 = (!xGreaterEqualY ? dx0 + 1.0f : dx0) - (float)(kUnskew2 + 1);
    f32 dy1 = (xGreaterEqualY ? dy0 + 1.0f : dy0) - (float)(kUnskew2 + 1);
    f32 dx2 = dx0 - (float)(kUnskew2 * 2 + 1);
    f32 dy2 = dy0 - (float)(kUnskew2 * 2 + 1);

    f32 falloff0 = fs_fnma(dx0, dx0, fs_fnma(dy0, dy0, (float)kFalloffRadiusSquared));
    f32 falloff1 = fs_fnma(dx1, dx1, fs_fnma(dy1, dy1, (float)kFalloffRadiusSquared));
    f32 falloff2 = falloff0 + fs_fma(unskewDelta, (float)(-4.0 * (kRoot3 + 2.0) / (kRoot3 + 3.0)), (float)(-2.0 / 3.0));
    falloff0 = fs_max(falloff0, 0.0f); falloff1 = fs_max(falloff1, 0.0f); falloff2 = fs_max(falloff2, 0.0f);
    falloff0 = falloff0 * falloff0; falloff0 = falloff0 * falloff0;
    falloff1 = falloff1 * falloff1; falloff1 = falloff1 * falloff1;
    falloff2 = falloff2 * falloff2; falloff2 = falloff2 * falloff2;

    f32 g0 = grad_perlin2(hash2(seed, xPrimedBase, yPrimedBase), dx0, dy0);
    f32 g1 = grad_perlin2(hash2(seed, xGreaterEqualY ? iadd(xPrimedBase, PRIME_X) : xPrimedBase,
                                      xGreaterEqualY ? yPrimedBase : iadd(yPrimedBase, PRIME_Y)), dx1, dy1);
    f32 g2 = grad_perlin2(hash2(seed, iadd(xPrimedBase, PRIME_X), iadd(yPrimedBase, PRIME_Y)), dx2, dy2);
    f32 value = fs_fma(g0, falloff0, fs_fma(g1, falloff1, g2 * falloff2));
    const float kBounding = 0.0261208079755306243896484375f;
    return scale_output(n, value, -kBounding, kBounding);
}

static f32 simplex3(const on_node* n, i32 seed, f32 x, f32 y, f32 z)
{
    seed = iadd(seed, n->seed_offset);
    x = x * n->frequency; y = y * n->frequency; z = z * n->frequency;
    const double kSkew3 = 1.0 / 3.0;
    const double kReflectUnskew3 = -1.0 / 2.0;
    const double kFalloffRadiusSquared = 0.6;

    f32 skewDelta = (float)kSkew3 * (x + y + z);
    f32 xSkewed = x + skewDelta, ySkewed = y + skewDelta, zSkewed = z + skewDelta;
    f32 xSkewedBase = fs_floor(xSkewed), ySkewedBase = fs_floor(ySkewed), zSkewedBase = fs_floor(zSkewed);
    f32 dxSkewed = xSkewed - xSkewedBase, dySkewed = ySkewed - ySkewedBase, dzSkewed = zSkewed - zSkewedBase;
    i32 xPrimedBase = imul(fs_cvt_i(xSkewedBase), PRIME_X);
    i32 yPrimedBase = imul(fs_cvt_i(ySkewedBase), PRIME_Y);
    i32 zPrimedBase = imul(fs_cvt_i(zSkewedBase), PRIME_Z);

    int xGEY = dxSkewed >= dySkewed, yGEZ = dySkewed >= dzSkewed, xGEZ = dxSkewed >= dzSkewed;
    f32 unskewDelta = (float)kReflectUnskew3 * (dxSkewed + dySkewed + dzSkewed);
    f32 dx0 = dxSkewed + unskewDelta, dy0 = dySkewed + unskewDelta, dz0 = dzSkewed + unskewDelta;

    int maskX1 = xGEY & xGEZ;
    int maskY1 = yGEZ & !xGEY;           /* BitwiseAndNot(a, b) = a & ~b */
    int maskZ1 = xGEZ | yGEZ;            /* inverse-masked */
    int nMaskX2 = xGEY | xGEZ;           /* inverse-masked */
    int nMaskY2 = xGEY & !yGEZ;
    int nMaskZ2 = xGEZ & yGEZ;

    f32 dx3 = dx0 - (float)(kReflectUnskew3 * 3 + 1);
    f32 dy3 = dy0 - (float)(kReflectUnskew3 * 3 + 1);
    f32 dz3 = dz0 - (float)(kReflectUnskew3 * 3 + 1);
    f32 dx1 = maskX1 ? dx3 - 1.0f : dx3;
    f32 dy1 = maskY1 ? dy3 - 1.0f : dy3;
    f32 dz1 = maskZ1 ? dz3 : dz3 - 1.0f;
    f32 dx2 = !nMaskX2 ? dx0 + 1.0f : dx0;
    f32 dy2 = nMaskY2 ? dy0 + 1.0f : dy0;
    f32 dz2 = nMaskZ2 ? dz0 + 1.0f : dz0;

    f32 falloff0 = fs_fnma(dz0, dz0, fs_fnma(dy0, dy0, fs_fnma(dx0, dx0, (float)kFalloffRadiusSquared)));
    f32 falloff1 = fs_fnma(dz1, dz1, fs_fnma(dy1, dy1, fs_fnma(dx1, dx1, (float)kFalloffRadiusSquared)));
    f32 falloff2 = fs_fnma(dz2, dz2, fs_fnma(dy2, dy2, fs_fnma(dx2, dx2, (float)kFalloffRadiusSquared)));
    f32 falloff3 = falloff0 - (unskewDelta + (float)(3.0 / 4.0));
    falloff0 = fs_max(falloff0, 0.0f); falloff1 = fs_max(falloff1, 0.0f);
    falloff2 = fs_max(falloff2, 0.0f); falloff3 = fs_max(falloff3, 0.0f);
    falloff0 = falloff0 * falloff0; falloff0 = falloff0 * falloff0;
    falloff1 = falloff1 * falloff1; falloff1 = falloff1 * falloff1;
    falloff2 = falloff2 * falloff2; falloff2 = falloff2 * falloff2;
    falloff3 = falloff3 * falloff3; falloff3 = falloff3 * falloff3;

    f32 g0 = grad_common(hash3(seed, xPrimedBase, yPrimedBase, zPrimedBase), dx0, dy0, dz0);
    f32 g1 = grad_common(hash3(seed, maskX1 ? iadd(xPrimedBase, PRIME_X) : xPrimedBase,
                                     maskY1 ? iadd(yPrimedBase, PRIME_Y) : yPrimedBase,
                                     maskZ1 ? zPrimedBase : iadd(zPrimedBase, PRIME_Z)), dx1, dy1, dz1);
    f32 g2 = grad_common(hash3(seed, nMaskX2 ? iadd(xPrimedBase, PRIME_X) : xPrimedBase,
                                     nMaskY2 ? yPrimedBase : iadd(yPrimedBase, PRIME_Y),
                                     nMaskZ2 ? zPrimedBase : iadd(zPrimedBase, PRIME_Z)), dx2, dy2, dz2);
    f32 g3 = grad_common(hash3(seed, iadd(xPrimedBase, PRIME_X), iadd(yPrimedBase, PRIME_Y), iadd(zPrimedBase, PRIME_Z)), dx3, dy3, dz3);
    f32 value = fs_fma(g3, falloff3, fs_fma(g2, falloff2, fs_fma(g1, falloff1, g0 * falloff0)));
    const float kBounding = 0.030586399137973785400390625f;
    return scale_output(n, value, -kBounding, kBounding);
}

static f32 simplex4(const on_node* n, i32 seed, f32 x, f32 y, f32 z, f32 w)
{
    seed = iadd(seed, n->seed_offset);
    x = x * n->frequency; y = y * n->frequency; z = z * n->frequency; w = w * n->frequency;
    const double kSkew4 = 1.0 / (kRoot5 + 1.0);
    const double kUnskew4 = -1.0 / (kRoot5 + 5.0);
    const double kFalloffRadiusSquared = 0.6;

    f32 skewDelta = (float)kSkew4 * (x + y + z + w);
    f32 xSkewed = x + skewDelta, ySkewed = y + skewDelta, zSkewed = z + skewDelta, wSkewed = w + skewDelta;
    f32 xSB = fs_floor(xSkewed), ySB = fs_floor(ySkewed), zSB = fs_floor(zSkewed), wSB = fs_floor(wSkewed);
    f32 dxS = xSkewed - xSB, dyS = ySkewed - ySB, dzS = zSkewed - zSB, dwS = wSkewed - wSB;
    i32 xP = imul(fs_cvt_i(xSB), PRIME_X), yP = imul(fs_cvt_i(ySB), PRIME_Y);
    i32 zP = imul(fs_cvt_i(zSB), PRIME_Z), wP = imul(fs_cvt_i(wSB), PRIME_W);

    f32 unskewDelta = (float)kUnskew4 * (dxS + dyS + dzS + dwS);
    f32 dx0 = dxS + unskewDelta, dy0 = dyS + unskewDelta, dz0 = dzS + unskewDelta, dw0 = dwS + unskewDelta;

    int rankX = 0, rankY = 0, rankZ = 0, rankW = 0;
    if (dx0 >= dy0) rankX++; else rankY++;
    if (dx0 >= dz0) rankX++; else rankZ++;
    if (dx0 >= dw0) rankX++; else rankW++;
    if (dy0 >= dz0) rankY++; else rankZ++;
    if (dy0 >= dw0) rankY++; else rankW++;
    if (dz0 >= dw0) rankZ++; else rankW++;

    const float u1 = (float)kUnskew4, u2 = (float)(kUnskew4 * 2), u3 = (float)(kUnskew4 * 3), u4 = (float)(kUnskew4 * 4 + 1);
    f32 dx1 = (rankX > 2 ? dx0 - 1.0f : dx0) - u1, dy1 = (rankY > 2 ? dy0 - 1.0f : dy0) - u1;
    f32 dz1 = (rankZ > 2 ? dz0 - 1.0f : dz0) - u1, dw1 = (rankW > 2 ? dw0 - 1.0f : dw0) - u1;
    f32 dx2 = (rankX > 1 ? dx0 - 1.0f : dx0) - u2, dy2 = (rankY > 1 ? dy0 - 1.0f : dy0) - u2;
    f32 dz2 = (rankZ > 1 ? dz0 - 1.0f : dz0) - u2, dw2 = (rankW > 1 ? dw0 - 1.0f : dw0) - u2;
    f32 dx3 = (rankX > 0 ? dx0 - 1.0f : dx0) - u3, dy3 = (rankY > 0 ? dy0 - 1.0f : dy0) - u3;
    f32 dz3 = (rankZ > 0 ? dz0 - 1.0f : dz0) - u3, dw3 = (rankW > 0 ? dw0 - 1.0f : dw0) - u3;
    f32 dx4 = dx0 - u4, dy4 = dy0 - u4, dz4 = dz0 - u4, dw4 = dw0 - u4;

    const float R = (float)kFalloffRadiusSquared;
    f32 falloff0 = fs_fnma(dw0, dw0, fs_fnma(dz0, dz0, fs_fnma(dy0, dy0, fs_fnma(dx0, dx0, R))));
    f32 falloff1 = fs_fnma(dw1, dw1, fs_fnma(dz1, dz1, fs_fnma(dy1, dy1, fs_fnma(dx1, dx1, R))));
    f32 falloff2 = fs_fnma(dw2, dw2, fs_fnma(dz2, dz2, fs_fnma(dy2, dy2, fs_fnma(dx2, dx2, R))));
    f32 falloff3 = fs_fnma(dw3, dw3, fs_fnma(dz3, dz3, fs_fnma(dy3, dy3, fs_fnma(dx3, dx3, R))));
    f32 falloff4 = falloff0 + fs_fma(unskewDelta, (float)(-4.0 * (kRoot5 + 3.0) / (kRoot5 + 5.0)), (float)(-4.0 / 5.0));
    falloff0 = fs_max(falloff0, 0.0f); falloff1 = fs_max(falloff1, 0.0f); falloff2 = fs_max(falloff2, 0.0f);
    falloff3 = fs_max(falloff3, 0.0f); falloff4 = fs_max(falloff4, 0.0f);
    falloff0 = falloff0 * falloff0; falloff0 = falloff0 * falloff0;
    falloff1 = falloff1 * falloff1; falloff1 = falloff1 * falloff1;
    falloff2 = falloff2 * falloff2; falloff2 = falloff2 * falloff2;
    falloff3 = falloff3 * falloff3; falloff3 = falloff3 * falloff3;
    falloff4 = falloff4 * falloff4; falloff4 = falloff4 * falloff4;

    f32 g0 = grad_perlin4(hash4(seed, xP, yP, zP, wP), dx0, dy0, dz0, dw0);
    f32 g1 = grad_perlin4(hash4(seed, rankX > 2 ? iadd(xP, PRIME_X) : xP, rankY > 2 ? iadd(yP, PRIME_Y) : yP,
                                      rankZ > 2 ? iadd(zP, PRIME_Z) : zP, rankW > 2 ? iadd(wP, PRIME_W) : wP), dx1, dy1, dz1, dw1);
    f32 g2 = grad_perlin4(hash4(seed, rankX > 1 ? iadd(xP, PRIME_X) : xP, rankY > 1 ? iadd(yP, PRIME_Y) : yP,
                                      rankZ > 1 ? iadd(zP, PRIME_Z) : zP, rankW > 1 ? iadd(wP, PRIME_W) : wP), dx2, dy2, dz2, dw2);
    f32 g3 = grad_perlin4(hash4(seed, rankX > 0 ? iadd(xP, PRIME_X) : xP, rankY > 0 ? iadd(yP, PRIME_Y) : yP,
                                      rankZ > 0 ? iadd(zP, PRIME_Z) : zP, rankW > 0 ? iadd(wP, PRIME_W) : wP), dx3, dy3, dz3, dw3);
    f32 g4 = grad_perlin4(hash4(seed, iadd(xP, PRIME_X), iadd(yP, PRIME_Y), iadd(zP, PRIME_Z), iadd(wP, PRIME_W)), dx4, dy4, dz4, dw4);
    f32 value = fs_fma(g0, falloff0, fs_fma(g1, falloff1, fs_fma(g2, falloff2, fs_fma(g3, falloff3, g4 * falloff4))));
    const float kBounding = 0.036730043590068817138671875f;
    return scale_output(n, value, -kBounding, kBounding);
}

/* ---- SuperSimplex (Simplex.inl:293-936) --------------------------------- */

static f32 supersimplex2(const on_node* n, i32 seed, f32 x, f32 y)
{
    seed = iadd(seed, n->seed_offset);
    x = x * n->frequency; y = y * n->frequency;
    const double kSkew2 = 1.0 / (kRoot3 + 1.0);
    const double kUnskew2 = -1.0 / (kRoot3 + 3.0);
    const double kFalloffRadiusSquared = 2.0 / 3.0;

    f32 skewDelta = (float)kSkew2 * (x + y);
    f32 xSkewed = x + skewDelta, ySkewed = y + skewDelta;
    f32 xSkewedBase = fs_floor(xSkewed), ySkewedBase = fs_floor(ySkewed);
    f32 dxSkewed = xSkewed - xSkewedBase, dySkewed = ySkewed - ySkewedBase;
    i32 xPrimedBase = imul(fs_cvt_i(xSkewedBase), PRIME_X);
    i32 yPrimedBase = imul(fs_cvt_i(ySkewedBase), PRIME_Y);

    int forwardXY = (dxSkewed + dySkewed) > 1.0f;
    f32 boundaryXY = forwardXY ? -1.0f : 0.0f;
    int forwardX = fs_fma(dxSkewed, -2.0f, dySkewed) < boundaryXY;
    int forwardY = fs_fma(dySkewed, -2.0f, dxSkewed) < boundaryXY;

    f32 unskewDelta = (float)kUnskew2 * (dxSkewed + dySkewed);
    f32 dxBase = dxSkewed + unskewDelta, dyBase = dySkewed + unskewDelta;
    f32 falloffBase0, value;
    {
        i32 h = hash2(seed, xPrimedBase, yPrimedBase);
        f32 g = grad_perlin2(h, dxBase, dyBase);
        falloffBase0 = fs_fnma(dxBase, dxBase, fs_fnma(dyBase, dyBase, (float)kFalloffRadiusSquared));
        f32 falloff = falloffBase0; falloff = falloff * falloff; falloff = falloff * falloff;
        value = falloff * g;
    }
    {
        i32 h = hash2(seed, iadd(xPrimedBase, PRIME_X), iadd(yPrimedBase, PRIME_Y));
        f32 g = grad_perlin2(h, dxBase - (float)(2 * kUnskew2 + 1), dyBase - (float)(2 * kUnskew2 + 1));
        f32 falloff = fs_fma(unskewDelta, (float)(-4.0 * (kRoot3 + 2.0) / (kRoot3 + 3.0)), falloffBase0 - (float)kFalloffRadiusSquared);
        falloff = falloff * falloff; falloff = falloff * falloff;
        value = fs_fma(falloff, g, value);
    }
    f32 xyDelta = forwardXY ? (float)(kUnskew2 + 1) : (float)(-kUnskew2);
    dxBase = dxBase - xyDelta;
    dyBase = dyBase - xyDelta;
    {
        i32 xa = forwardX ? iadd(xPrimedBase, (int32_t)((uint32_t)PRIME_X * 2u)) : xPrimedBase;
        i32 h = hash2(seed, forwardXY ? xa : isub(xa, PRIME_X), forwardXY ? iadd(yPrimedBase, PRIME_Y) : yPrimedBase);
        f32 dx = dxBase - (forwardX ? (float)(1 + 2 * kUnskew2) : -1.0f);
        f32 dy = forwardX ? dyBase - (float)(2 * kUnskew2) : dyBase;
        f32 g = grad_perlin2(h, dx, dy);
        f32 falloff = fs_max(fs_fnma(dx, dx, fs_fnma(dy, dy, (float)kFalloffRadiusSquared)), 0.0f);
        falloff = falloff * falloff; falloff = falloff * falloff;
        value = fs_fma(falloff, g, value);
    }
    {
        i32 ya = forwardY ? iadd(yPrimedBase, (int32_t)(uint32_t)((uint64_t)(int64_t)PRIME_Y * 2u)) : yPrimedBase;
        i32 h = hash2(seed, forwardXY ? iadd(xPrimedBase, PRIME_X) : xPrimedBase, forwardXY ? ya : isub(ya, PRIME_Y));
        f32 dx = forwardY ? dxBase - (float)(2 * kUnskew2) : dxBase;
        f32 dy = dyBase - (forwardY ? (float)(1 + 2 * kUnskew2) : -1.0f);
        f32 g = grad_perlin2(h, dx, dy);
        f32 falloff = fs_max(fs_fnma(dx, dx, fs_fnma(dy, dy, (float)kFalloffRadiusSquared)), 0.0f);
        falloff = falloff * falloff; falloff = falloff * falloff;
        value = fs_fma(falloff, g, value);
    }
    const float kBounding = 0.14084912836551666259765625f;
    return scale_output(n, value, -kBounding, kBounding);
}

/* sign-mask helpers used by SuperSimplex 3D/4D: FS::Masked(mask, -0.0f bits) */
static inline f32 sgn_xor(f32 v, int mask) { return mask ? fs_xor_sign(v, (int32_t)0x80000000) : v; }

static f32 supersimplex3(const on_node* n, i32 seed, f32 x, f32 y, f32 z)
{
    seed = iadd(seed, n->seed_offset);
    x = x * n->frequency; y = y * n->frequency; z = z * n->frequency;
    const double kSkew3 = 1.0 / 3.0;
    const double kReflectUnskew3 = -1.0 / 2.0;
    const double kTwiceUnskew3 = -1.0 / 4.0;
    const double kDistanceSquaredA = 3.0 / 4.0;
    const double kDistanceSquaredB = 1.0;
    const double kFalloffRadiusSquared = kDistanceSquaredA;

    f32 skewDelta = (float)kSkew3 * (x + y + z);
    f32 xSkewed = x + skewDelta, ySkewed = y + skewDelta, zSkewed = z + skewDelta;
    f32 xSB = fs_floor(xSkewed), ySB = fs_floor(ySkewed), zSB = fs_floor(zSkewed);
    f32 dxS = xSkewed - xSB, dyS = ySkewed - ySB, dzS = zSkewed - zSB;
    {
        f32 twiceUnskewDelta = (float)kTwiceUnskew3 * (dxS + dyS + dzS);
        f32 xN = dxS + twiceUnskewDelta, yN = dyS + twiceUnskewDelta, zN = dzS + twiceUnskewDelta;
        f32 xyzN = -twiceUnskewDelta;
        f32 maxScore = 0.375f;
        int32_t bits = (xyzN > maxScore) ? -1 : 0;
        maxScore = fs_max(maxScore, xyzN);
#define CONSIDER(score, b) do { f32 s_ = (score); if (s_ > maxScore) bits = (b); maxScore = fs_max(maxScore, s_); } while (0)
        CONSIDER(xN, 1); CONSIDER(yN, 2); CONSIDER(zN, 4);
        maxScore = maxScore + (0.125f - xyzN);
        CONSIDER(-zN, 3); CONSIDER(-yN, 5); CONSIDER(-xN, 6);
        int moveX = (bits & 1) != 0, moveY = (bits & 2) != 0, moveZ = (bits & 4) != 0;
        if (moveX) { xSB = xSB + 1.0f; dxS = dxS - 1.0f; }
        if (moveY) { ySB = ySB + 1.0f; dyS = dyS - 1.0f; }
        if (moveZ) { zSB = zSB + 1.0f; dzS = dzS - 1.0f; }
    }
    i32 xP = imul(fs_cvt_i(xSB), PRIME_X), yP = imul(fs_cvt_i(ySB), PRIME_Y), zP = imul(fs_cvt_i(zSB), PRIME_Z);

    f32 sum = dxS + dyS + dzS;
    f32 twiceUnskewDelta = (float)kTwiceUnskew3 * sum;
    f32 xN = dxS + twiceUnskewDelta, yN = dyS + twiceUnskewDelta, zN = dzS + twiceUnskewDelta;
    f32 xyzN = -twiceUnskewDelta;
    f32 unskewDelta = (float)kReflectUnskew3 * sum;
    f32 dxB = dxS + unskewDelta, dyB = dyS + unskewDelta, dzB = dzS + unskewDelta;
    f32 coordinateSum = (float)(1 + 3 * kReflectUnskew3) * sum;

    f32 value, stemA, stemB;
    {
        f32 g = grad_common(hash3(seed, xP, yP, zP), dxB, dyB, dzB);
        f32 fb = fs_fnma(dzB, dzB, fs_fnma(dyB, dyB, fs_fnma(dxB, dxB, (float)kFalloffRadiusSquared))) * 0.5f;
        stemA = fb - (float)(kDistanceSquaredA * 0.5);
        stemB = fb - (float)(kDistanceSquaredB * 0.5);
        value = (fb * fb) * (fb * fb) * g;
    }
    {   /* <1,1,1> or <-1,-1,-1> */
        int m = xyzN < 0.0f;
        i32 xq = iadd(xP, m ? -PRIME_X : PRIME_X), yq = iadd(yP, m ? -PRIME_Y : PRIME_Y), zq = iadd(zP, m ? -PRIME_Z : PRIME_Z);
        f32 off = sgn_xor((float)(3 * kReflectUnskew3 + 1), m);
        f32 g = grad_common(hash3(seed, xq, yq, zq), dxB - off, dyB - off, dzB - off);
        f32 fb = fs_max(fs_fma(off, coordinateSum, stemA), 0.0f);
        value = fs_fma((fb * fb) * (fb * fb), g, value);
    }
    {   /* <1,1,0> */
        int m = xyzN < zN;
        i32 xq = iadd(xP, m ? -PRIME_X : PRIME_X), yq = iadd(yP, m ? -PRIME_Y : PRIME_Y);
        f32 off0 = sgn_xor((float)(2 * kReflectUnskew3), m);
        f32 g = grad_common(hash3(seed, xq, yq, zP), dxB, dyB, dzB - off0);
        f32 fb = fs_min(sgn_xor(dzB, m) - stemB, 0.0f);
        value = fs_fma((fb * fb) * (fb * fb), g, value);
    }
    {   /* <1,0,1> */
        int m = xyzN < yN;
        i32 xq = iadd(xP, m ? -PRIME_X : PRIME_X), zq = iadd(zP, m ? -PRIME_Z : PRIME_Z);
        f32 off0 = sgn_xor((float)(2 * kReflectUnskew3), m);
        f32 g = grad_common(hash3(seed, xq, yP, zq), dxB, dyB - off0, dzB);
        f32 fb = fs_min(sgn_xor(dyB, m) - stemB, 0.0f);
        value = fs_fma((fb * fb) * (fb * fb), g, value);
    }
    {   /* <0,1,1> */
        int m = xyzN < xN;
        i32 yq = iadd(yP, m ? -PRIME_Y : PRIME_Y), zq = iadd(zP, m ? -PRIME_Z : PRIME_Z);
        f32 off0 = sgn_xor((float)(2 * kReflectUnskew3), m);
        f32 g = grad_common(hash3(seed, xP, yq, zq), dxB - off0, dyB, dzB);
        f32 fb = fs_min(sgn_xor(dxB, m) - stemB, 0.0f);
        value = fs_fma((fb * fb) * (fb * fb), g, value);
    }
    {   /* <1,0,0> */
        int m = xN < 0.0f;
        i32 xq = iadd(xP, m ? -PRIME_X : PRIME_X);
        f32 off0 = sgn_xor((float)kReflectUnskew3, m);
        f32 g = grad_common(hash3(seed, xq, yP, zP), dxB + off0, dyB - off0, dzB - off0);
        f32 fb = fs_max(fs_fma(off0, coordinateSum, stemA) + sgn_xor(dxB, m), 0.0f);
        value = fs_fma((fb * fb) * (fb * fb), g, value);
    }
    {   /* <0,1,0> */
        int m = yN < 0.0f;
        i32 yq = iadd(yP, m ? -PRIME_Y : PRIME_Y);
        f32 off0 = sgn_xor((float)kReflectUnskew3, m);
        f32 g = grad_common(hash3(seed, xP, yq, zP), dxB - off0, dyB + off0, dzB - off0);
        f32 fb = fs_max(fs_fma(off0, coordinateSum, stemA) + sgn_xor(dyB, m), 0.0f);
        value = fs_fma((fb * fb) * (fb * fb), g, value);
    }
    {   /* <0,0,1> */
        int m = zN < 0.0f;
        i32 zq = iadd(zP, m ? -PRIME_Z : PRIME_Z);
        f32 off0 = sgn_xor((float)kReflectUnskew3, m);
        f32 g = grad_common(hash3(seed, xP, yP, zq), dxB - off0, dyB - off0, dzB + off0);
        f32 fb = fs_max(fs_fma(off0, coordinateSum, stemA) + sgn_xor(dzB, m), 0.0f);
        value = fs_fma((fb * fb) * (fb * fb), g, value);
    }
    const float kBounding = 0.0069091119803488254547119140625f;
    return scale_output(n, value, -kBounding, kBounding);
}

static f32 supersimplex4(const on_node* n, i32 seed, f32 x, f32 y, f32 z, f32 w)
{
    seed = iadd(seed, n->seed_offset);
    x = x * n->frequency; y = y * n->frequency; z = z * n->frequency; w = w * n->frequency;
    const double kSkew4 = 1.0 / (kRoot5 + 1.0);
    const double kUnskew4 = -1.0 / (kRoot5 + 5.0);
    const double kTwiceUnskew4 = -1.0 / 5.0;
    const double kDistanceSquaredA = 4.0 / 5.0;
    const double kDistanceSquaredB = 6.0 / 5.0;
    const double kFalloffRadiusSquared = kDistanceSquaredA;

    f32 skewDelta = (float)kSkew4 * (x + y + z + w);
    f32 xSk = x + skewDelta, ySk = y + skewDelta, zSk = z + skewDelta, wSk = w + skewDelta;
    f32 xSB = fs_floor(xSk), ySB = fs_floor(ySk), zSB = fs_floor(zSk), wSB = fs_floor(wSk);
    f32 dxS = xSk - xSB, dyS = ySk - ySB, dzS = zSk - zSB, dwS = wSk - wSB;
    {
        f32 tud = (float)kTwiceUnskew4 * (dxS + dyS + dzS + dwS);
        f32 xN = dxS + tud, yN = dyS + tud, zN = dzS + tud, wN = dwS + tud;
        f32 xyzwN = -tud;
        f32 maxScore = 0.6f - xyzwN;
        int32_t bits = (0.2f > maxScore) ? -1 : 0;
        maxScore = fs_max(maxScore, 0.2f);
        CONSIDER(-wN, 7); CONSIDER(-zN, 11); CONSIDER(-yN, 13); CONSIDER(-xN, 14);
        maxScore = maxScore + (xyzwN - 0.2f);
        CONSIDER(xN, 1); CONSIDER(yN, 2); CONSIDER(zN, 4); CONSIDER(wN, 8);
        maxScore = maxScore + (0.2f - xN);
        CONSIDER(yN, 3); CONSIDER(zN, 5); CONSIDER(wN, 9);
        maxScore = maxScore + xN;
        CONSIDER(yN + zN, 6);
        maxScore = maxScore - wN;
        CONSIDER(yN, 10); CONSIDER(zN, 12);
        if (bits & 1) { xSB = xSB + 1.0f; dxS = dxS - 1.0f; }
        if (bits & 2) { ySB = ySB + 1.0f; dyS = dyS - 1.0f; }
        if (bits & 4) { zSB = zSB + 1.0f; dzS = dzS - 1.0f; }
        if (bits & 8) { wSB = wSB + 1.0f; dwS = dwS - 1.0f; }
    }
#undef CONSIDER
    i32 xP = imul(fs_cvt_i(xSB), PRIME_X), yP = imul(fs_cvt_i(ySB), PRIME_Y);
    i32 zP = imul(fs_cvt_i(zSB), PRIME_Z), wP = imul(fs_cvt_i(wSB), PRIME_W);

    f32 sum = dxS + dyS + dzS + dwS;
    f32 tud = (float)kTwiceUnskew4 * sum;
    f32 xN = dxS + tud, yN = dyS + tud, zN = dzS + tud, wN = dwS + tud;
    f32 xyzwN = -tud;
    f32 ud = (float)kUnskew4 * sum;
    f32 dxB = dxS + ud, dyB = dyS + ud, dzB = dzS + ud, dwB = dwS + ud;
    f32 cs = (float)(1 + 4 * kUnskew4) * sum;

    f32 value, stemA, stemB;
    {
        f32 g = grad_perlin4(hash4(seed, xP, yP, zP, wP), dxB, dyB, dzB, dwB);
        f32 fb = fs_fnma(dwB, dwB, fs_fnma(dzB, dzB, fs_fnma(dyB, dyB, fs_fnma(dxB, dxB, (float)kFalloffRadiusSquared)))) * 0.5f;
        stemA = fb - (float)(kDistanceSquaredA * 0.5);
        stemB = fb - (float)(kDistanceSquaredB * 0.5);
        value = (fb * fb) * (fb * fb) * g;
    }
#define SEL_P(m, base, P) iadd(base, (m) ? -(P) : (P))
#define ACC(fbexpr, gexpr) do { f32 g_ = (gexpr); f32 fb_ = fs_max((fbexpr), 0.0f); value = fs_fma((fb_ * fb_) * (fb_ * fb_), g_, value); } while (0)
    {   /* <1,1,1,1> */
        int m = xyzwN < 0.0f;
        f32 off = sgn_xor((float)(4 * kUnskew4 + 1), m);
        ACC(fs_fma(off, cs, stemA),
            grad_perlin4(hash4(seed, SEL_P(m, xP, PRIME_X), SEL_P(m, yP, PRIME_Y), SEL_P(m, zP, PRIME_Z), SEL_P(m, wP, PRIME_W)),
                         dxB - off, dyB - off, dzB - off, dwB - off));
    }
    {   /* <1,1,1,0> */
        int m = xyzwN < wN;
        f32 o1 = sgn_xor((float)(3 * kUnskew4 + 1), m), o0 = sgn_xor((float)(3 * kUnskew4), m);
        ACC(fs_fma(o1, cs, stemB) - sgn_xor(dwB, m),
            grad_perlin4(hash4(seed, SEL_P(m, xP, PRIME_X), SEL_P(m, yP, PRIME_Y), SEL_P(m, zP, PRIME_Z), wP),
                         dxB - o1, dyB - o1, dzB - o1, dwB - o0));
    }
    {   /* <1,1,0,1> */
        int m = xyzwN < zN;
        f32 o1 = sgn_xor((float)(3 * kUnskew4 + 1), m), o0 = sgn_xor((float)(3 * kUnskew4), m);
        ACC(fs_fma(o1, cs, stemB) - sgn_xor(dzB, m),
            grad_perlin4(hash4(seed, SEL_P(m, xP, PRIME_X), SEL_P(m, yP, PRIME_Y), zP, SEL_P(m, wP, PRIME_W)),
                         dxB - o1, dyB - o1, dzB - o0, dwB - o1));
    }
    {   /* <1,0,1,1> */
        int m = xyzwN < yN;
        f32 o1 = sgn_xor((float)(3 * kUnskew4 + 1), m), o0 = sgn_xor((float)(3 * kUnskew4), m);
        ACC(fs_fma(o1, cs, stemB) - sgn_xor(dyB, m),
            grad_perlin4(hash4(seed, SEL_P(m, xP, PRIME_X), yP, SEL_P(m, zP, PRIME_Z), SEL_P(m, wP, PRIME_W)),
                         dxB - o1, dyB - o0, dzB - o1, dwB - o1));
    }
    {   /* <0,1,1,1> */
        int m = xyzwN < xN;
        f32 o1 = sgn_xor((float)(3 * kUnskew4 + 1), m), o0 = sgn_xor((float)(3 * kUnskew4), m);
        ACC(fs_fma(o1, cs, stemB) - sgn_xor(dxB, m),
            grad_perlin4(hash4(seed, xP, SEL_P(m, yP, PRIME_Y), SEL_P(m, zP, PRIME_Z), SEL_P(m, wP, PRIME_W)),
                         dxB - o0, dyB - o1, dzB - o1, dwB - o1));
    }
    {   /* <1,0,0,0> */
        int m = xN < 0.0f;
        f32 o1 = sgn_xor((float)(kUnskew4 + 1), m), o0 = sgn_xor((float)kUnskew4, m);
        ACC(fs_fma(o0, cs, stemA) + sgn_xor(dxB, m),
            grad_perlin4(hash4(seed, SEL_P(m, xP, PRIME_X), yP, zP, wP), dxB - o1, dyB - o0, dzB - o0, dwB - o0));
    }
    {   /* <1,1,0,0> */
        int m = xN < -yN;
        f32 o1 = sgn_xor((float)(2 * kUnskew4 + 1), m), o0 = sgn_xor((float)(2 * kUnskew4), m);
        ACC(fs_fma(o0, cs, stemB) + sgn_xor(dxB + dyB, m),
            grad_perlin4(hash4(seed, SEL_P(m, xP, PRIME_X), SEL_P(m, yP, PRIME_Y), zP, wP), dxB - o1, dyB - o1, dzB - o0, dwB - o0));
    }
    {   /* <1,0,1,0> */
        int m = xN < -zN;
        f32 o1 = sgn_xor((float)(2 * kUnskew4 + 1), m), o0 = sgn_xor((float)(2 * kUnskew4), m);
        ACC(fs_fma(o0, cs, stemB) + sgn_xor(dxB + dzB, m),
            grad_perlin4(hash4(seed, SEL_P(m, xP, PRIME_X), yP, SEL_P(m, zP, PRIME_Z), wP), dxB - o1, dyB - o0, dzB - o1, dwB - o0));
    }
    {   /* <1,0,0,1> */
        int m = xN < -wN;
        f32 o1 = sgn_xor((float)(2 * kUnskew4 + 1), m), o0 = sgn_xor((float)(2 * kUnskew4), m);
        ACC(fs_fma(o0, cs, stemB) + sgn_xor(dxB + dwB, m),
            grad_perlin4(hash4(seed, SEL_P(m, xP, PRIME_X), yP, zP, SEL_P(m, wP, PRIME_W)), dxB - o1, dyB - o0, dzB - o0, dwB - o1));
    }
    {   /* <0,1,0,0> */
        int m = yN < 0.0f;
        f32 o1 = sgn_xor((float)(kUnskew4 + 1), m), o0 = sgn_xor((float)kUnskew4, m);
        ACC(fs_fma(o0, cs, stemA) + sgn_xor(dyB, m),
            grad_perlin4(hash4(seed, xP, SEL_P(m, yP, PRIME_Y), zP, wP), dxB - o0, dyB - o1, dzB - o0, dwB - o0));
    }
    {   /* <0,1,1,0> */
        int m = yN < -zN;
        f32 o1 = sgn_xor((float)(2 * kUnskew4 + 1), m), o0 = sgn_xor((float)(2 * kUnskew4), m);
        ACC(fs_fma(o0, cs, stemB) + sgn_xor(dyB + dzB, m),
            grad_perlin4(hash4(seed, xP, SEL_P(m, yP, PRIME_Y), SEL_P(m, zP, PRIME_Z), wP), dxB - o0, dyB - o1, dzB - o1, dwB - o0));
    }
    {   /* <0,1,0,1> */
        int m = yN < -wN;
        f32 o1 = sgn_xor((float)(2 * kUnskew4 + 1), m), o0 = sgn_xor((float)(2 * kUnskew4), m);
        ACC(fs_fma(o0, cs, stemB) + sgn_xor(dyB + dwB, m),
            grad_perlin4(hash4(seed, xP, SEL_P(m, yP, PRIME_Y), zP, SEL_P(m, wP, PRIME_W)), dxB - o0, dyB - o1, dzB - o0, dwB - o1));
    }
    {   /* <0,0,1,0> */
        int m = zN < 0.0f;
        f32 o1 = sgn_xor((float)(kUnskew4 + 1), m), o0 = sgn_xor((float)kUnskew4, m);
        ACC(fs_fma(o0, cs, stemA) + sgn_xor(dzB, m),
            grad_perlin4(hash4(seed, xP, yP, SEL_P(m, zP, PRIME_Z), wP), dxB - o0, dyB - o0, dzB - o1, dwB - o0));
    }
    {   /* <0,0,1,1> */
        int m = zN < -wN;
        f32 o1 = sgn_xor((float)(2 * kUnskew4 + 1), m), o0 = sgn_xor((float)(2 * kUnskew4), m);
        ACC(fs_fma(o0, cs, stemB) + sgn_xor(dzB + dwB, m),
            grad_perlin4(hash4(seed, xP, yP, SEL_P(m, zP, PRIME_Z), SEL_P(m, wP, PRIME_W)), dxB - o0, dyB - o0, dzB - o1, dwB - o1));
    }
    {   /* <0,0,0,1> */
        int m = wN < 0.0f;
        f32 o1 = sgn_xor((float)(kUnskew4 + 1), m), o0 = sgn_xor((float)kUnskew4, m);
        ACC(fs_fma(o0, cs, stemA) + sgn_xor(dwB, m),
            grad_perlin4(hash4(seed, xP, yP, zP, SEL_P(m, wP, PRIME_W)), dxB - o0, dyB - o0, dzB - o0, dwB - o1));
    }
#undef ACC
#undef SEL_P
    const float kBounding = 0.011310013942420482635498046875f;
    return scale_output(n, value, -kBounding, kBounding);
}

/* ---- Perlin (Perlin.inl) ------------------------------------------------ */

static f32 perlin2(const on_node* n, i32 seed, f32 x, f32 y)
{
    seed = iadd(seed, n->seed_offset);
    x = x * n->frequency; y = y * n->frequency;
    f32 xs = fs_floor(x), ys = fs_floor(y);
    i32 x0 = imul(fs_cvt_i(xs), PRIME_X), y0 = imul(fs_cvt_i(ys), PRIME_Y);
    i32 x1 = iadd(x0, PRIME_X), y1 = iadd(y0, PRIME_Y);
    f32 xf0 = x - xs, yf0 = y - ys;
    f32 xf1 = xf0 - 1.0f, yf1 = yf0 - 1.0f;
    xs = interp_quintic(xf0); ys = interp_quintic(yf0);
    f32 value = lerp(lerp(grad_perlin2(hash2(seed, x0, y0), xf0, yf0), grad_perlin2(hash2(seed, x1, y0), xf1, yf0), xs),
                     lerp(grad_perlin2(hash2(seed, x0, y1), xf0, yf1), grad_perlin2(hash2(seed, x1, y1), xf1, yf1), xs), ys);
    const float kBounding = 1.726796627044677734375f;
    return scale_output(n, value, -kBounding, kBounding);
}

static f32 perlin3(const on_node* n, i32 seed, f32 x, f32 y, f32 z)
{
    seed = iadd(seed, n->seed_offset);
    x = x * n->frequency; y = y * n->frequency; z = z * n->frequency;
    f32 xs = fs_floor(x), ys = fs_floor(y), zs = fs_floor(z);
    i32 x0 = imul(fs_cvt_i(xs), PRIME_X), y0 = imul(fs_cvt_i(ys), PRIME_Y), z0 = imul(fs_cvt_i(zs), PRIME_Z);
    i32 x1 = iadd(x0, PRIME_X), y1 = iadd(y0, PRIME_Y), z1 = iadd(z0, PRIME_Z);
    f32 xf0 = x - xs, yf0 = y - ys, zf0 = z - zs;
    f32 xf1 = xf0 - 1.0f, yf1 = yf0 - 1.0f, zf1 = zf0 - 1.0f;
    xs = interp_quintic(xf0); ys = interp_quintic(yf0); zs = interp_quintic(zf0);
    f32 value = lerp(
        lerp(lerp(grad_common(hash3(seed, x0, y0, z0), xf0, yf0, zf0), grad_common(hash3(seed, x1, y0, z0), xf1, yf0, zf0), xs),
             lerp(grad_common(hash3(seed, x0, y1, z0), xf0, yf1, zf0), grad_common(hash3(seed, x1, y1, z0), xf1, yf1, zf0), xs), ys),
        lerp(lerp(grad_common(hash3(seed, x0, y0, z1), xf0, yf0, zf1), grad_common(hash3(seed, x1, y0, z1), xf1, yf0, zf1), xs),
             lerp(grad_common(hash3(seed, x0, y1, z1), xf0, yf1, zf1), grad_common(hash3(seed, x1, y1, z1), xf1, yf1, zf1), xs), ys), zs);
    const double kBounding = 1.0363423824310302734375;
    return scale_output(n, value, (float)-kBounding, (float)kBounding);
}

static f32 perlin4(const on_node* n, i32 seed, f32 x, f32 y, f32 z, f32 w)
{
    seed = iadd(seed, n->seed_offset);
    x = x * n->frequency; y = y * n->frequency; z = z * n->frequency; w = w * n->frequency;
    f32 xs = fs_floor(x), ys = fs_floor(y), zs = fs_floor(z), ws = fs_floor(w);
    i32 x0 = imul(fs_cvt_i(xs), PRIME_X), y0 = imul(fs_cvt_i(ys), PRIME_Y);
    i32 z0 = imul(fs_cvt_i(zs), PRIME_Z), w0 = imul(fs_cvt_i(ws), PRIME_W);
    i32 x1 = iadd(x0, PRIME_X), y1 = iadd(y0, PRIME_Y), z1 = iadd(z0, PRIME_Z), w1 = iadd(w0, PRIME_W);
    f32 xf0 = x - xs, yf0 = y - ys, zf0 = z - zs, wf0 = w - ws;
    f32 xf1 = xf0 - 1.0f, yf1 = yf0 - 1.0f, zf1 = zf0 - 1.0f, wf1 = wf0 - 1.0f;
    xs = interp_quintic(xf0); ys = interp_quintic(yf0); zs = interp_quintic(zf0); ws = interp_quintic(wf0);
#define G4(a, b, c, d, fa, fb, fc, fd) grad_perlin4(hash4(seed, a, b, c, d), fa, fb, fc, fd)
    f32 value = lerp(
        lerp(lerp(lerp(G4(x0, y0, z0, w0, xf0, yf0, zf0, wf0), G4(x1, y0, z0, w0, xf1, yf0, zf0, wf0), xs),
                  lerp(G4(x0, y1, z0, w0, xf0, yf1, zf0, wf0), G4(x1, y1, z0, w0, xf1, yf1, zf0, wf0), xs), ys),
             lerp(lerp(G4(x0, y0, z1, w0, xf0, yf0, zf1, wf0), G4(x1, y0, z1, w0, xf1, yf0, zf1, wf0), xs),
                  lerp(G4(x0, y1, z1, w0, xf0, yf1, zf1, wf0), G4(x1, y1, z1, w0, xf1, yf1, zf1, wf0), xs), ys), zs),
        lerp(lerp(lerp(G4(x0, y0, z0, w1, xf0, yf0, zf0, wf1), G4(x1, y0, z0, w1, xf1, yf0, zf0, wf1), xs),
                  lerp(G4(x0, y1, z0, w1, xf0, yf1, zf0, wf1), G4(x1, y1, z0, w1, xf1, yf1, zf0, wf1), xs), ys),
             lerp(lerp(G4(x0, y0, z1, w1, xf0, yf0, zf1, wf1), G4(x1, y0, z1, w1, xf1, yf0, zf1, wf1), xs),
                  lerp(G4(x0, y1, z1, w1, xf0, yf1, zf1, wf1), G4(x1, y1, z1, w1, xf1, yf1, zf1, wf1), xs), ys), zs), ws);
#undef G4
    const float kBounding = 1.33858621120452880859375f;
    return scale_output(n, value, -kBounding, kBounding);
}

/* ---- Value (Value.inl) -------------------------------------------------- */

static f32 value2(const on_node* n, i32 seed, f32 x, f32 y)
{
    seed = iadd(seed, n->seed_offset);
    x = x * n->frequency; y = y * n->frequency;
    f32 xs = fs_floor(x), ys = fs_floor(y);
    i32 x0 = imul(fs_cvt_i(xs), PRIME_X), y0 = imul(fs_cvt_i(ys), PRIME_Y);
    i32 x1 = iadd(x0, PRIME_X), y1 = iadd(y0, PRIME_Y);
    xs = interp_hermite(x - xs); ys = interp_hermite(y - ys);
    return scale_output(n, lerp(lerp(valcoord2(seed, x0, y0), valcoord2(seed, x1, y0), xs),
                                lerp(valcoord2(seed, x0, y1), valcoord2(seed, x1, y1), xs), ys), -kValueBounds, kValueBounds);
}

static f32 value3(const on_node* n, i32 seed, f32 x, f32 y, f32 z)
{
    seed = iadd(seed, n->seed_offset);
    x = x * n->frequency; y = y * n->frequency; z = z * n->frequency;
    f32 xs = fs_floor(x), ys = fs_floor(y), zs = fs_floor(z);
    i32 x0 = imul(fs_cvt_i(xs), PRIME_X), y0 = imul(fs_cvt_i(ys), PRIME_Y), z0 = imul(fs_cvt_i(zs), PRIME_Z);
    i32 x1 = iadd(x0, PRIME_X), y1 = iadd(y0, PRIME_Y), z1 = iadd(z0, PRIME_Z);
    xs = interp_hermite(x - xs); ys = interp_hermite(y - ys); zs = interp_hermite(z - zs);
    return scale_output(n, lerp(
        lerp(lerp(valcoord3(seed, x0, y0, z0), valcoord3(seed, x1, y0, z0), xs),
             lerp(valcoord3(seed, x0, y1, z0), valcoord3(seed, x1, y1, z0), xs), ys),
        lerp(lerp(valcoord3(seed, x0, y0, z1), valcoord3(seed, x1, y0, z1), xs),
             lerp(valcoord3(seed, x0, y1, z1), valcoord3(seed, x1, y1, z1), xs), ys), zs), -kValueBounds, kValueBounds);
}

static f32 value4(const on_node* n, i32 seed, f32 x, f32 y, f32 z, f32 w)
{
    seed = iadd(seed, n->seed_offset);
    x = x * n->frequency; y = y * n->frequency; z = z * n->frequency; w = w * n->frequency;
    f32 xs = fs_floor(x), ys = fs_floor(y), zs = fs_floor(z), ws = fs_floor(w);
    i32 x0 = imul(fs_cvt_i(xs), PRIME_X), y0 = imul(fs_cvt_i(ys), PRIME_Y);
    i32 z0 = imul(fs_cvt_i(zs), PRIME_Z), w0 = imul(fs_cvt_i(ws), PRIME_W);
    i32 x1 = iadd(x0, PRIME_X), y1 = iadd(y0, PRIME_Y), z1 = iadd(z0, PRIME_Z), w1 = iadd(w0, PRIME_W);
    xs = interp_hermite(x - xs); ys = interp_hermite(y - ys); zs = interp_hermite(z - zs); ws = interp_hermite(w - ws);
#define V4(a, b, c, d) valcoord4(seed, a, b, c, d)
    return scale_output(n, lerp(
        lerp(lerp(lerp(V4(x0, y0, z0, w0), V4(x1, y0, z0, w0), xs), lerp(V4(x0, y1, z0, w0), V4(x1, y1, z0, w0), xs), ys),
             lerp(lerp(V4(x0, y0, z1, w0), V4(x1, y0, z1, w0), xs), lerp(V4(x0, y1, z1, w0), V4(x1, y1, z1, w0), xs), ys), zs),
        lerp(lerp(lerp(V4(x0, y0, z0, w1), V4(x1, y0, z0, w1), xs), lerp(V4(x0, y1, z0, w1), V4(x1, y1, z0, w1), xs), ys),
             lerp(lerp(V4(x0, y0, z1, w1), V4(x1, y0, z1, w1), xs), lerp(V4(x0, y1, z1, w1), V4(x1, y1, z1, w1), xs), ys), zs), ws),
        -kValueBounds, kValueBounds);
#undef V4
}

/* ---- CalcDistance (Utils.inl:281-335) ----------------------------------- */

enum { DF_EUCLIDEAN, DF_EUCLIDEAN_SQ, DF_MANHATTAN, DF_HYBRID, DF_MAXAXIS, DF_MINKOWSKI };

static f32 calc_distance(const on_node* n, int hybrid_minkowski, int do_sqrt, i32 seed, int dim, const f32* p)
{
    int df = n->dist_func;
    if (df < 0 || df > DF_MINKOWSKI) df = DF_EUCLIDEAN;   /* default: case Euclidean */
    switch (df) {
    case DF_EUCLIDEAN:
    case DF_EUCLIDEAN_SQ: {
        f32 d = p[0] * p[0];
        for (int k = 1; k < dim; ++k) d = fs_fma(p[k], p[k], d);
        return (df == DF_EUCLIDEAN && do_sqrt) ? fs_sqrt(d) : d;
    }
    case DF_MANHATTAN: {
        f32 tail = fs_abs(p[dim - 1]);                  /* right fold: |y| + (|z| + |w|) */
        for (int k = dim - 2; k >= 1; --k) tail = fs_abs(p[k]) + tail;
        return fs_abs(p[0]) + tail;
    }
    case DF_HYBRID: {
        f32 both = fs_fma(p[0], p[0], fs_abs(p[0]));
        for (int k = 1; k < dim; ++k) both = both + fs_fma(p[k], p[k], fs_abs(p[k]));
        return both;
    }
    case DF_MAXAXIS: {
        f32 mx = fs_abs(p[0]);
        for (int k = 1; k < dim; ++k) mx = fs_max(fs_abs(p[k]), mx);
        return mx;
    }
    default: {  /* Minkowski: hybrid evaluated at the offset vector */
        f32 m;
        if (dim == 2) m = HYB2(n, hybrid_minkowski, seed, p[0], p[1]);
        else if (dim == 3) m = HYB3(n, hybrid_minkowski, seed, p[0], p[1], p[2]);
        else m = HYB4(n, hybrid_minkowski, seed, p[0], p[1], p[2], p[3]);
        f32 tail = fs_pow(fs_abs(p[dim - 1]), m);
        for (int k = dim - 2; k >= 1; --k) tail = fs_pow(fs_abs(p[k]), m) + tail;
        return fs_pow(fs_pow(fs_abs(p[0]), m) + tail, fs_recip(m));
    }
    }
}

/* ---- Cellular (Cellular.inl) ------------------------------------------- */

static const float kJitter2D = 0.437016f, kJitter3D = 0.396144f, kJitter4D = 0.366025f;

typedef struct {
    i32 seed, source_seed;
    f32 jitter, size_jitter;
    int size_active;
} cell_ctx;

static cell_ctx cell_setup(const on_node* n, i32 seed, int dim, const f32* pos)
{
    /* Cellular.inl:22-30: hybrids evaluated at the unscaled position with the
     * un-offset seed; Grid Jitter = hybrid 1, Size Jitter = hybrid 2 */
    static const float kj[5] = {0, 0, 0.437016f, 0.396144f, 0.366025f};
    static const float ks[5] = {0, 0, -1.f / 0x3ff, -1.f / 0xffff, -1.f / 0xfffff};
    cell_ctx c;
    c.source_seed = seed;
    c.seed = iadd(seed, n->seed_offset);
    f32 gj, sj = 0.0f;
    if (dim == 2) gj = HYB2(n, 1, seed, pos[0], pos[1]);
    else if (dim == 3) gj = HYB3(n, 1, seed, pos[0], pos[1], pos[2]);
    else gj = HYB4(n, 1, seed, pos[0], pos[1], pos[2], pos[3]);
    c.jitter = kj[dim] * gj;
    c.size_active = n->hnode[2] != NULL || n->hval[2] != 0.0f;
    if (c.size_active) {
        if (dim == 2) sj = HYB2(n, 2, seed, pos[0], pos[1]);
        else if (dim == 3) sj = HYB3(n, 2, seed, pos[0], pos[1], pos[2]);
        else sj = HYB4(n, 2, seed, pos[0], pos[1], pos[2], pos[3]);
        sj = sj * ks[dim];
    }
    c.size_jitter = sj;
    return c;
}

/* Per-cell jittered offset: hash bit-fields -> direction, scaled by jitter/|dir|. */
static inline void cell_dir(int dim, i32 hash, f32 jitter, f32* d)
{
    if (dim == 2) {
        d[0] = fs_cvt_f((int32_t)hash & 0x7ff) - (0x7ff / 2.0f);
        d[1] = fs_cvt_f(isrl(hash, 21)) - (0x7ff / 2.0f);
        d[2] = jitter * fs_invsqrt(fs_fma(d[0], d[0], d[1] * d[1]));
    } else if (dim == 3) {
        d[0] = fs_cvt_f((int32_t)hash & 0x3ff) - (0x3ff / 2.0f);
        d[1] = fs_cvt_f((int32_t)isra(hash, 11) & 0x3ff) - (0x3ff / 2.0f);
        d[2] = fs_cvt_f(isrl(hash, 22)) - (0x3ff / 2.0f);
        d[3] = jitter * fs_invsqrt(fs_fma(d[0], d[0], fs_fma(d[1], d[1], d[2] * d[2])));
    } else {
        d[0] = fs_cvt_f((int32_t)hash & 0xff) - (0xff / 2.0f);
        d[1] = fs_cvt_f((int32_t)isra(hash, 8) & 0xff) - (0xff / 2.0f);
        d[2] = fs_cvt_f((int32_t)isra(hash, 16) & 0xff) - (0xff / 2.0f);
        d[3] = fs_cvt_f(isrl(hash, 24)) - (0xff / 2.0f);
        d[4] = jitter * fs_invsqrt(fs_fma(d[0], d[0], fs_fma(d[1], d[1], fs_fma(d[2], d[2], d[3] * d[3]))));
    }
}

static inline f32 size_jitter_factor(int dim, i32 hash, f32 sj)
{
    f32 dj;
    if (dim == 2) dj = fs_cvt_f((int32_t)isra(hash, 11) & 0x3ff);
    else if (dim == 3) dj = fs_cvt_f((int32_t)hash & 0xffff);
    else dj = fs_cvt_f((int32_t)hash & 0xfffff);
    return fs_fnma(sj, dj, 1.0f);
}

static const int32_t kPrimes[4] = {PRIME_X, PRIME_Y, PRIME_Z, PRIME_W};

static inline i32 hashhb_n(int dim, i32 seed, const i32* c)
{
    if (dim == 2) return hashhb2(seed, c[0], c[1]);
    if (dim == 3) return hashhb3(seed, c[0], c[1], c[2]);
    return hashhb4(seed, c[0], c[1], c[2], c[3]);
}

/* CellularValue (Cellular.inl:18-292) */
static f32 cellular_value(const on_node* n, i32 seed, int dim, const f32* pin)
{
    cell_ctx cc = cell_setup(n, seed, dim, pin);
    f32 p[4];
    for (int k = 0; k < dim; ++k) p[k] = pin[k] * n->frequency;
    f32 distance[4] = {INFINITY, INFINITY, INFINITY, INFINITY};
    i32 valueHash[4] = {0, 0, 0, 0};
    i32 cbase[4];
    f32 cfbase[4];
    for (int k = 0; k < dim; ++k) {
        cbase[k] = iadd(fs_cvt_i(p[k]), -1);
        cfbase[k] = fs_cvt_f(cbase[k]) - p[k];
        cbase[k] = imul(cbase[k], kPrimes[k]);
    }
    int total = dim == 2 ? 9 : (dim == 3 ? 27 : 81);
    i32 c[4]; f32 cf[4];
    for (int k = 0; k < dim; ++k) { c[k] = cbase[k]; cf[k] = cfbase[k]; }
    int idx[4] = {0, 0, 0, 0};
    for (int it = 0; it < total; ++it) {
        i32 hash = hashhb_n(dim, cc.seed, c);
        f32 d[5];
        cell_dir(dim, hash, cc.jitter, d);
        f32 invMag = d[dim];
        f32 off[4];
        for (int k = 0; k < dim; ++k) off[k] = fs_fma(d[k], invMag, cf[k]);
        i32 newHash = hash;
        /* 2D uses CalcDistance<true>, 3D/4D CalcDistance<false> (Cellular.inl:63,151,251) */
        f32 newDistance = calc_distance(n, 0, dim == 2, cc.source_seed, dim, off);
        if (cc.size_active) newDistance = newDistance * size_jitter_factor(dim, hash, cc.size_jitter);
        for (int i = 0;; i++) {
            int closer = newDistance < distance[i];
            f32 localDistance = distance[i];
            i32 localHash = valueHash[i];
            distance[i] = closer ? newDistance : distance[i];
            valueHash[i] = closer ? newHash : valueHash[i];
            if (i >= n->value_index) break;
            newDistance = closer ? localDistance : newDistance;
            newHash = closer ? localHash : newHash;
        }
        /* advance innermost axis first (x outermost loop ... last axis innermost) */
        for (int k = dim - 1; k >= 0; --k) {
            if (++idx[k] < 3) { cf[k] = cf[k] + 1.0f; c[k] = iadd(c[k], kPrimes[k]); break; }
            idx[k] = 0; cf[k] = cfbase[k]; c[k] = cbase[k];
        }
    }
    return scale_output(n, fs_cvt_f(valueHash[n->value_index]), -kValueBounds, kValueBounds);
}

/* CellularDistance (Cellular.inl:295-566).  The per-axis offsets (cell - pos)
 * are recomputed from the running integer-valued float cell coordinate at each
 * loop level, exactly as the reference nests them. */
static f32 cellular_distance(const on_node* n, i32 seed, int dim, const f32* pin)
{
    cell_ctx cc = cell_setup(n, seed, dim, pin);
    f32 p[4];
    for (int k = 0; k < dim; ++k) p[k] = pin[k] * n->frequency;
    f32 distance[4] = {INFINITY, INFINITY, INFINITY, INFINITY};
    i32 cbase[4]; f32 cfbase[4];
    for (int k = 0; k < dim; ++k) {
        cbase[k] = iadd(fs_cvt_i(p[k]), -1);
        cfbase[k] = fs_cvt_f(cbase[k]);
        cbase[k] = imul(cbase[k], kPrimes[k]);
    }
    int total = dim == 2 ? 9 : (dim == 3 ? 27 : 81);
    i32 c[4]; f32 cf[4];
    for (int k = 0; k < dim; ++k) { c[k] = cbase[k]; cf[k] = cfbase[k]; }
    int idx[4] = {0, 0, 0, 0};
    for (int it = 0; it < total; ++it) {
        i32 hash = hashhb_n(dim, cc.seed, c);
        f32 d[5];
        cell_dir(dim, hash, cc.jitter, d);
        f32 invMag = d[dim];
        f32 off[4];
        for (int k = 0; k < dim; ++k) off[k] = fs_fma(d[k], invMag, cf[k] - p[k]);
        f32 newDistance = calc_distance(n, 0, 0, cc.source_seed, dim, off);
        if (cc.size_active) newDistance = newDistance * size_jitter_factor(dim, hash, cc.size_jitter);
        for (int i = 3; i > 0; i--) distance[i] = fs_max(fs_min(distance[i], newDistance), distance[i - 1]);
        distance[0] = fs_min(distance[0], newDistance);
        for (int k = dim - 1; k >= 0; --k) {
            if (++idx[k] < 3) { cf[k] = cf[k] + 1.0f; c[k] = iadd(c[k], kPrimes[k]); break; }
            idx[k] = 0; cf[k] = cfbase[k]; c[k] = cbase[k];
        }
    }
    /* GetReturn (Cellular.inl:531-565) */
    float maxDist = 1 + (dim == 2 ? kJitter2D : (dim == 3 ? kJitter3D : kJitter4D));
    int i0 = n->dist_idx0, i1 = n->dist_idx1;
    if (n->dist_func == DF_EUCLIDEAN) {
        distance[i0] = distance[i0] * fs_invsqrt(distance[i0]);
        distance[i1] = distance[i1] * fs_invsqrt(distance[i1]);
    }
    maxDist = maxDist * maxDist;
    switch (n->return_type) {
    default:
    case 0: return scale_output(n, distance[i0], 0, maxDist);
    case 1: return scale_output(n, distance[i0] + distance[i1], 0, maxDist * 2);
    case 2: return scale_output(n, fs_abs(distance[i0] - distance[i1]), 0, maxDist);
    case 3: return scale_output(n, distance[i0] * distance[i1], 0, maxDist * maxDist);
    case 4: return scale_output(n, distance[i0] * fs_recip(distance[i1]), 0, maxDist);
    }
}

static f32 gen_n(const on_node* n, i32 seed, int dim, const f32* p)
{
    if (dim == 2) return gen2(n, seed, p[0], p[1]);
    if (dim == 3) return gen3(n, seed, p[0], p[1], p[2]);
    return gen4(n, seed, p[0], p[1], p[2], p[3]);
}

/* CellularLookup (Cellular.inl:569-807) */
static f32 cellular_lookup(const on_node* n, i32 seed, int dim, const f32* pin)
{
    cell_ctx cc = cell_setup(n, seed, dim, pin);
    f32 p[4];
    for (int k = 0; k < dim; ++k) p[k] = pin[k] * n->frequency;
    f32 distance = FLT_MAX;
    f32 cell[4] = {0, 0, 0, 0};
    i32 cbase[4]; f32 cfbase[4];
    for (int k = 0; k < dim; ++k) {
        cbase[k] = iadd(fs_cvt_i(p[k]), -1);
        cfbase[k] = fs_cvt_f(cbase[k]);
        cbase[k] = imul(cbase[k], kPrimes[k]);
    }
    int total = dim == 2 ? 9 : (dim == 3 ? 27 : 81);
    i32 c[4]; f32 cf[4];
    for (int k = 0; k < dim; ++k) { c[k] = cbase[k]; cf[k] = cfbase[k]; }
    int idx[4] = {0, 0, 0, 0};
    for (int it = 0; it < total; ++it) {
        i32 hash = hashhb_n(dim, cc.seed, c);
        f32 d[5];
        cell_dir(dim, hash, cc.jitter, d);
        f32 invMag = d[dim];
        f32 local[4], off[4];
        for (int k = 0; k < dim; ++k) { local[k] = fs_fma(d[k], invMag, cf[k]); off[k] = local[k] - p[k]; }
        f32 newDistance = calc_distance(n, 0, 0, cc.source_seed, dim, off);
        if (cc.size_active) newDistance = newDistance * size_jitter_factor(dim, hash, cc.size_jitter);
        int closer = newDistance < distance;
        distance = fs_min(newDistance, distance);
        for (int k = 0; k < dim; ++k) cell[k] = closer ? local[k] : cell[k];
        for (int k = dim - 1; k >= 0; --k) {
            if (++idx[k] < 3) { cf[k] = cf[k] + 1.0f; c[k] = iadd(c[k], kPrimes[k]); break; }
            idx[k] = 0; cf[k] = cfbase[k]; c[k] = cbase[k];
        }
    }
    f32 q[4];
    for (int k = 0; k < dim; ++k) q[k] = cell[k] * n->scale;
    return gen_n(n->lookup[0], iadd(cc.source_seed, 1), dim, q);
}

/* ---- DomainWarpGradient::Warp (DomainWarp.inl:33-206) ------------------- */

static f32 warp_gradient(const on_node* n, i32 seed, f32 warpAmp, int dim, const f32* pin, f32* out)
{
    seed = iadd(seed, n->seed_offset);
    f32 s[4][2];         /* s[k][0] = 1 - hermite, s[k][1] = hermite */
    i32 c[4][2];
    for (int k = 0; k < dim; ++k) {
        f32 fl = fs_floor(pin[k]);
        c[k][0] = imul(fs_cvt_i(fl), kPrimes[k]);
        c[k][1] = iadd(c[k][0], kPrimes[k]);
        s[k][1] = interp_hermite(pin[k] - fl);
        s[k][0] = 1.0f - s[k][1];
    }
    f32 wv[4];
    float normalise;
    int corners = 1 << dim;
    for (int corner = 0; corner < corners; ++corner) {
        /* corner bit k selects the +1 lattice point on axis k; x toggles fastest */
        int b0 = corner & 1, b1 = (corner >> 1) & 1, b2 = (corner >> 2) & 1, b3 = (corner >> 3) & 1;
        i32 h;
        f32 contrib;
        f32 comp[4];
        if (dim == 2) {
            h = hashhb2(seed, c[0][b0], c[1][b1]);
            contrib = s[0][b0] * s[1][b1];
            comp[0] = fs_cvt_f((int32_t)h & 0xffff);
            comp[1] = fs_cvt_f(isrl(h, 16));
            normalise = 1.0f / (0xffff / 2.0f);
        } else if (dim == 3) {
            h = hashhb3(seed, c[0][b0], c[1][b1], c[2][b2]);
            contrib = s[0][b0] * s[1][b1] * s[2][b2];
            comp[0] = fs_cvt_f((int32_t)h & 0x3ff);
            comp[1] = fs_cvt_f((int32_t)isra(h, 11) & 0x3ff);
            comp[2] = fs_cvt_f(isrl(h, 22));
            normalise = 1.0f / (0x3ff / 2.0f);
        } else {
            h = hashhb4(seed, c[0][b0], c[1][b1], c[2][b2], c[3][b3]);
            contrib = s[0][b0] * s[1][b1] * s[2][b2] * s[3][b3];
            comp[0] = fs_cvt_f((int32_t)h & 0xff);
            comp[1] = fs_cvt_f((int32_t)isra(h, 8) & 0xff);
            comp[2] = fs_cvt_f((int32_t)isra(h, 16) & 0xff);
            comp[3] = fs_cvt_f(isrl(h, 24));
            normalise = 1.0f / (0xff / 2.0f);
        }
        for (int k = 0; k < dim; ++k) wv[k] = corner == 0 ? contrib * comp[k] : fs_fma(contrib, comp[k], wv[k]);
    }
    for (int k = 0; k < dim; ++k) wv[k] = fs_fms(wv[k], normalise, 1.0f);
    for (int k = 0; k < dim; ++k) out[k] = fs_fma(wv[k], warpAmp * n->axis[k], out[k]);
    f32 r = wv[dim - 1] * wv[dim - 1];
    for (int k = dim - 2; k >= 0; --k) r = fs_fma(wv[k], wv[k], r);
    return r;
}

static f32 warp_any(const on_node* w, i32 seed, f32 amp, int dim, const f32* scaled, f32* out);

/* DomainWarp::GenT (DomainWarp.inl:9-17): the node's seed offset is applied
 * here and again inside Warp. */
static f32 domain_warp_gen(const on_node* n, i32 seed, int dim, const f32* pin)
{
    i32 sourceSeed = seed;
    seed = iadd(seed, n->seed_offset);
    f32 amp;
    if (dim == 2) amp = HYB2(n, 0, sourceSeed, pin[0], pin[1]);
    else if (dim == 3) amp = HYB3(n, 0, sourceSeed, pin[0], pin[1], pin[2]);
    else amp = HYB4(n, 0, sourceSeed, pin[0], pin[1], pin[2], pin[3]);
    f32 scaled[4], pos[4];
    for (int k = 0; k < dim; ++k) { scaled[k] = pin[k] * n->frequency; pos[k] = pin[k]; }
    warp_any(n, seed, amp, dim, scaled, pos);
    return gen_n(n->lookup[0], sourceSeed, dim, pos);
}

/* DomainWarpFractalProgressive / Independent (DomainWarpFractal.inl:9-73) */
static f32 domain_warp_fractal(const on_node* n, i32 seed, int dim, const f32* pin, int independent)
{
    const on_node* warp = n->lookup[0];
    f32 noisePos[4], warpPos[4];
    for (int k = 0; k < dim; ++k) { noisePos[k] = pin[k]; warpPos[k] = pin[k]; }
    f32 amp, ws, gain;
    if (dim == 2) {
        amp = HYB2(warp, 0, seed, pin[0], pin[1]); ws = HYB2(n, 1, seed, pin[0], pin[1]); gain = HYB2(n, 0, seed, pin[0], pin[1]);
    } else if (dim == 3) {
        amp = HYB3(warp, 0, seed, pin[0], pin[1], pin[2]); ws = HYB3(n, 1, seed, pin[0], pin[1], pin[2]);
        gain = HYB3(n, 0, seed, pin[0], pin[1], pin[2]);
    } else {
        amp = HYB4(warp, 0, seed, pin[0], pin[1], pin[2], pin[3]); ws = HYB4(n, 1, seed, pin[0], pin[1], pin[2], pin[3]);
        gain = HYB4(n, 0, seed, pin[0], pin[1], pin[2], pin[3]);
    }
    f32 freq = warp->frequency;
    i32 seedInc = seed;
    f32 lac = n->lacunarity;
    f32 scaled[4];
    const f32* src = independent ? noisePos : warpPos;
    for (int k = 0; k < dim; ++k) scaled[k] = src[k] * freq;
    f32 strength = warp_any(warp, seedInc, amp, dim, scaled, warpPos);
    for (int i = 1; i < n->octaves; i++) {
        strength = fs_sqrt(strength);                         /* FastLengthSqrt, strict build */
        seedInc = iadd(seedInc, 1);
        freq = freq * lac;
        amp = amp * lerp(1.0f, 1.0f - strength, ws);
        amp = amp * gain;
        for (int k = 0; k < dim; ++k) scaled[k] = src[k] * freq;
        strength = warp_any(warp, seedInc, amp, dim, scaled, warpPos);
    }
    return gen_n(warp->lookup[0], seed, dim, warpPos);
}

/* ---- DomainWarpSimplex / DomainWarpSuperSimplex (DomainWarpSimplex.inl) --
 * The vector-product helpers follow the portable (non-AVX) branches of
 * DomainWarpSimplex.inl:40-60, 82-116, 148-191, 221-235, 285-316, 560-695;
 * FS::Masked*(m, a, b) are written out as selects, FS::SelectHighBit(m, a, b)
 * as (m < 0 ? a : b). */

static const float kRoot2f = (float)1.4142135623730950488016887242097;
static const float kRoot3f = (float)1.7320508075688772935274463415059;
#define WS_SKEW2F ((float)(1.0 / (1.7320508075688772935274463415059 + 1.0)))
#define WS_SKEW4F ((float)(1.0 / (2.2360679774997896964091736687313 + 1.0)))

static inline f32 ws_selhb(i32 m, f32 a, f32 b) { OC_TICK(1); return (int32_t)m < 0 ? a : b; }
static inline f32 ws_sel(int m, f32 a, f32 b) { OC_TICK(1); return m ? a : b; }

/* ApplyGradientOuterProductVectorProductSimplex 2D (:7-60) */
static void ws_gop2(i32 hash31, f32 fX, f32 fY, f32 mul, f32* vX, f32* vY)
{
    i32 hs = isrl(hash31, 1);
    i32 ig = imul(hs, 12 >> 2);
    i32 io = imul(hs, (int32_t)0xAAAAAAAB) & (int32_t)0xC0000003;
    {
        f32 u = ws_selhb(ishl(ig, 2), fY, fX);
        f32 v = ws_selhb(ishl(ig, 2), fX, fY);
        f32 a = u * ws_selhb(ig, 2.0f, kRoot3f);
        f32 b = fs_xor_sign(v, ishl(isra(ig, 30), 31));
        f32 s = ws_sel((int32_t)ig >= 0, a + b, a);
        mul = mul * fs_xor_sign(s, ishl(isra(ig, 28) ^ (int32_t)io, 31));
    }
    {
        f32 a = mul * ws_selhb(io, 2.0f, kRoot3f);
        f32 b = fs_xor_sign(ws_sel((int32_t)io >= 0, mul, 0.0f), ishl(isra(io, 30), 31));
        *vX = *vX + ws_selhb(ishl(io, 30), b, a);
        *vY = *vY + ws_selhb(ishl(io, 30), a, b);
    }
}

/* ApplyGradientOuterProductVectorProductCommon 3D (:62-116) */
static void ws_gop3(i32 hash31, f32 fX, f32 fY, f32 fZ, f32 mul, f32* vX, f32* vY, f32* vZ)
{
    i32 hs = isrl(hash31, 1);
    i32 ig = isrl(imul(hs, 12 >> 2), 28);
    i32 io = imul(hs, (int32_t)0xAAAAAAAB) & (int32_t)0xC0000003;
    io = (int32_t)io | (int32_t)isra(io, 28);
    {
        f32 u = ws_sel((int32_t)ig >= 8, fY, fX);
        f32 v = ws_sel((int32_t)ig >= 4, fZ, fY);
        mul = mul * (fs_xor_sign(u, ishl(ig, 31)) + fs_xor_sign(v, ishl(isra(ig, 1), 31)));
    }
    {
        io = (int32_t)io & 0xF;
        f32 signed0 = fs_xor_sign(mul, ishl(io, 31));
        f32 signed1 = fs_xor_sign(mul, ishl(isra(io, 1), 31));
        int notYZ = (int32_t)io < 8;
        int notXY = (int32_t)io >= 4;
        *vX = ws_sel(notYZ, *vX + signed0, *vX);
        *vZ = ws_sel(notXY, *vZ + signed1, *vZ);
        *vY = ws_sel(notYZ && notXY, *vY, *vY + ws_sel(notXY, signed0, signed1));
    }
}

/* one gradient of the 4D outer-product table from a [0,20) << 27 index (:150-171) */
static void ws_gop4_vector(i32 index, f32* g)
{
    i32 iA = (int32_t)index & (0x03 << 27);
    i32 iB = (int32_t)isra(index, 2) & (0x07 << 27);
    iB = (int32_t)iB ^ (int32_t)iA;
    int extra = (int32_t)iB >= (0x04 << 27);
    int equal = (int32_t)iA == (int32_t)iB;
    if (equal) iA = -1;
    f32 neutral = ws_sel(equal || extra, ws_sel(extra, WS_SKEW4F * -1.0f, WS_SKEW4F), 0.0f);
    for (int k = 0; k < 4; ++k) {
        f32 t = ws_sel((int32_t)iA == (k << 27), neutral - 1.0f, neutral);
        g[k] = ws_sel((int32_t)iB == (k << 27), t + 1.0f, t);
    }
}

/* ApplyGradientOuterProductVectorProductSimplex 4D (:118-191) */
static void ws_gop4(i32 hash, f32 fX, f32 fY, f32 fZ, f32 fW, f32 mul, f32* v)
{
    i32 hs = isrl(hash, 2);
    i32 ig = imul(hs, 20 >> 2);
    i32 io = imul(hs, (int32_t)0xCCCCCCCD);
    io = imul((int32_t)io & (int32_t)0xE0000003, 3 | (1 << 27));
    f32 g[4];
    ws_gop4_vector(ig, g);
    mul = mul * fs_fma(g[3], fW, fs_fma(g[2], fZ, fs_fma(g[1], fY, g[0] * fX)));
    ws_gop4_vector(io, g);
    for (int k = 0; k < 4; ++k) v[k] = fs_fma(mul, g[k], v[k]);
}

/* ApplyOrthogonalGradientMatrixVectorProductSimplex 2D (:193-235) */
static void ws_ogm2(i32 hash31, f32 fX, f32 fY, f32 mul, f32* vX, f32* vY)
{
    i32 index = imul(isrl(hash31, 1), 12 >> 2);
    i32 ofThree = isrl(index, 30);
    i32 signX = ishl(isra(index, 28), 31);
    i32 signY = ishl(isra(index, 29), 31);
    f32 masked = ws_sel((int32_t)index >= 0, WS_SKEW2F, 0.0f);
    f32 gX = fs_xor_sign(ws_sel((int32_t)ofThree != 0, masked + 1.0f, masked), signX);
    f32 gY = fs_xor_sign(ws_sel((int32_t)ofThree != 1, masked + 1.0f, masked), signY);
    *vX = fs_fma(mul, fs_fma(fY, gY, fX * gX), *vX);
    mul = fs_xor_sign(mul, ishl(hash31, 31));
    *vY = fs_fma(mul, fs_fms(fY, gX, fX * gY), *vY);
}

/* ApplyOrthogonalGradientMatrixVectorProductCommon 3D (:237-316) */
static void ws_ogm3(i32 hash31, f32 fX, f32 fY, f32 fZ, f32 mul, f32* vX, f32* vY, f32* vZ)
{
    const float cA = 2.224744871391589f, cB = -0.224744871391589f, cC = -1.0f, cDE = 1.0f, cF = 2.0f;
    i32 hs = isrl(hash31, 1);
    i32 fb = imul(hs, (int32_t)0xAAAAAAAB);
    i32 p2hb = ishl(fb, 29);
    i32 p3 = isrl(imul(hs, 3), 30);
    i32 finalSign = ishl(hash31, 31);
    i32 sign0 = ishl(fb, 31);
    i32 sign1 = (int32_t)ishl(fb, 30) & (int32_t)0x80000000;
    i32 notYZ = fb;
    i32 notXY = ishl(fb, 1);
    i32 either = (int32_t)notYZ | (int32_t)notXY;

    f32 aX = ws_selhb(notYZ, cC, fs_xor_sign(cA, sign0));
    f32 aY = ws_selhb(either, ws_selhb(notXY, fs_xor_sign(cB, sign1), fs_xor_sign(cA, sign0)), cC);
    f32 aZ = ws_selhb(notXY, cC, fs_xor_sign(cB, sign1));
    f32 valA = fs_fma(aZ, fZ, fs_fma(fY, aY, fX * aX));

    f32 bX = ws_selhb(notYZ, cC, fs_xor_sign(cB, sign0));
    f32 bY = ws_selhb(either, ws_selhb(notXY, fs_xor_sign(cA, sign1), fs_xor_sign(cB, sign0)), cC);
    f32 bZ = ws_selhb(notXY, cC, fs_xor_sign(cA, sign1));
    f32 valB = fs_fma(bZ, fZ, fs_fma(fY, bY, fX * bX));

    f32 cX = ws_selhb(notYZ, cF, fs_xor_sign(cDE, sign0));
    f32 cY = ws_selhb(either, ws_selhb(notXY, fs_xor_sign(cDE, sign1), fs_xor_sign(cDE, sign0)), cF);
    f32 cZ = ws_selhb(notXY, cF, fs_xor_sign(cDE, sign1));
    f32 valC = fs_fma(cZ, fZ, fs_fma(fY, cY, fX * cX));

    f32 valAB = ws_selhb(p2hb, valB, valA);
    f32 valBA = ws_selhb(p2hb, valA, valB);

    mul = fs_xor_sign(mul, finalSign);
    *vX = fs_fma(mul, ws_sel((int32_t)p3 == 0, valC, valAB), *vX);
    *vY = fs_fma(mul, ws_sel((int32_t)p3 == 1, valC, ws_sel((int32_t)p3 == 2, valBA, valAB)), *vY);
    *vZ = fs_fma(mul, ws_sel((int32_t)p3 == 2, valC, valBA), *vZ);
}

/* ApplyOrthogonalGradientMatrixVectorProductSimplex 4D (:318-695) */
static void ws_ogm4(i32 hash31, f32 fX, f32 fY, f32 fZ, f32 fW, f32 mul, f32* v)
{
    const float kNegAB = -0.375999676691291f;        /* kComponentPairwiseIndexedNegativeAB */
    const float kFillAB = 0.222726847849776f;        /* kComponentPairwiseUnindexedFillerAB */
    const float kPosD = -WS_SKEW4F;                  /* kComponentPairwiseIndexedPositiveD */
    const float kUnD = WS_SKEW4F;                    /* kComponentPairwiseUnindexedD */
    const float kToSingleAB = -0.124000323308709f;   /* kDeltaPairwiseToSingleAB */
    const float kToSingleD = 0.190983005625053f;     /* kDeltaPairwiseToSingleD */
    const float kToExtra = WS_SKEW4F;                /* kDeltaSingleToExtra */
    const float kABToC = 0.437016024448821f;         /* kDeltaPairwiseABToC */
    const float kToDiag = -kRoot2f;                  /* kDeltaUnindexedFillerToDiagonal */

    i32 hs = isrl(hash31, 2);
    i32 indexBasis = imul(hs, 20 >> 2);
    i32 p3 = isra(imul(hs, (int32_t)0xD5555556), 29);
    i32 p8 = isra(indexBasis, 24);
    i32 finalSign = ishl(hash31, 31);

    i32 iPos = (int32_t)indexBasis & (0x03 << 27);
    i32 iNeg = (int32_t)isra(indexBasis, 2) & (0x03 << 27);
    iNeg = (int32_t)iNeg ^ (int32_t)iPos;

    /* (0x10 << 27) wraps to INT32_MIN, so with FastSIMD's signed int32 compares
     * this mask is always set in the portable branch (:567) */
    int extraCase = (int32_t)indexBasis >= INT32_MIN;
    int singleCase = (int32_t)iPos == (int32_t)iNeg;
    int singleNonExtra = (int32_t)indexBasis < (0x04 << 27);
    if (singleNonExtra) iPos = -1;

    f32 singleOffsetAB = ws_sel(extraCase, kToSingleAB + kToExtra, kToSingleAB);
    f32 negAB = ws_sel(singleCase, kNegAB + singleOffsetAB, kNegAB);
    f32 fillAB = ws_sel(singleCase, kFillAB + singleOffsetAB, kFillAB);
    f32 negC = ws_sel(singleCase, negAB, negAB + kABToC);
    f32 fillC = ws_sel(singleCase, fillAB, fillAB + kABToC);
    f32 singleOffsetD = ws_sel(extraCase, kToSingleD + kToExtra, kToSingleD);
    f32 posD = ws_sel(singleCase, kPosD + singleOffsetD, kPosD);
    f32 unD = ws_sel(singleCase, kUnD + singleOffsetD, kUnD);

    int counter = -1;
    f32 valA = 0.0f, valB = 0.0f, valC = 0.0f, valD = 0.0f;
    const f32 f[4] = {fX, fY, fZ, fW};
    for (int k = 0; k < 4; ++k) {
        int idxPos = (int32_t)iPos == (k << 27);
        int indexed = idxPos || (int32_t)iNeg == (k << 27);
        f32 icAB = ws_sel(idxPos, negAB + 1.0f, negAB);
        f32 icC = ws_sel(idxPos, negC + 1.0f, negC);
        f32 icD = ws_sel(!idxPos, posD - 1.0f, posD);
        f32 uA, uB, uC;
        if (k == 0) {
            uA = fillAB + kToDiag; uB = fillAB; uC = fillC;
        } else if (k == 1) {
            uA = ws_sel(counter == -2, fillAB + kToDiag, fillAB);
            uB = ws_sel(counter == -1, fillAB + kToDiag, fillAB);
            uC = fillC;
        } else if (k == 2) {
            uA = ws_sel(counter == -3, fillAB + kToDiag, fillAB);
            uB = ws_sel(counter == -2, fillAB + kToDiag, fillAB);
            uC = ws_sel(counter == -1, fillC + kToDiag, fillC);
        } else {
            uA = fillAB;
            uB = ws_sel(counter == -3, fillAB + kToDiag, fillAB);
            uC = ws_sel(counter == -2, fillC + kToDiag, fillC);
        }
        f32 gA = ws_sel(indexed, icAB, uA);
        f32 gB = ws_sel(indexed, icAB, uB);
        f32 gC = ws_sel(indexed, icC, uC);
        f32 gD = ws_sel(indexed, icD, unD);
        if (k < 3 && indexed) counter -= 1;
        if (k == 0) { valA = gA * f[0]; valB = gB * f[0]; valC = gC * f[0]; valD = gD * f[0]; }
        else { valA = fs_fma(gA, f[k], valA); valB = fs_fma(gB, f[k], valB); valC = fs_fma(gC, f[k], valC); valD = fs_fma(gD, f[k], valD); }
    }

    i32 ix = isra(p8, 1);
    i32 iy = iadd(iadd(ix, 1), p3);
    i32 iz = (int32_t)p8 & 1;
    iz = iadd(iadd(ix, 1), (int32_t)iz >= (int32_t)p3 ? iadd(iz, 1) : iz);
    i32 isum = iadd(iadd(ix, iy), iz);

    mul = fs_xor_sign(mul, finalSign);
#define WS_PICK4(I, A_, B_, C_, D_) ws_selhb(ishl(I, 31), ws_selhb(ishl(I, 30), D_, B_), ws_selhb(ishl(I, 30), C_, A_))
    v[0] = fs_fma(mul, WS_PICK4(ix, valA, valB, valC, valD), v[0]);
    v[1] = fs_fma(mul, WS_PICK4(iy, valA, valB, valC, valD), v[1]);
    v[2] = fs_fma(mul, WS_PICK4(iz, valA, valB, valC, valD), v[2]);
    v[3] = fs_fma(mul, ws_selhb(ishl(isum, 31), ws_selhb(ishl(isum, 30), valD, valB), ws_selhb(ishl(isum, 30), valA, valC)), v[3]);
#undef WS_PICK4
}

static void ws_vec2(int gop, i32 h, f32 fX, f32 fY, f32 mul, f32* v)
{
    if (gop) ws_gop2(h, fX, fY, mul, &v[0], &v[1]);
    else ws_ogm2(h, fX, fY, mul, &v[0], &v[1]);
}
static void ws_vec3(int gop, i32 h, f32 fX, f32 fY, f32 fZ, f32 mul, f32* v)
{
    if (gop) ws_gop3(h, fX, fY, fZ, mul, &v[0], &v[1], &v[2]);
    else ws_ogm3(h, fX, fY, fZ, mul, &v[0], &v[1], &v[2]);
}
static void ws_vec4(int gop, i32 h, f32 fX, f32 fY, f32 fZ, f32 fW, f32 mul, f32* v)
{
    if (gop) ws_gop4(h, fX, fY, fZ, fW, mul, v);
    else ws_ogm4(h, fX, fY, fZ, fW, mul, v);
}
static inline f32 ws_pow4(f32 f) { f = f * f; return f * f; }
static inline i32 ws_madd(int m, i32 a, i32 b) { OC_TICK(1); return m ? iadd(a, b) : a; }

/* DomainWarpSimplex Warp_2D (:771-833) */
static void ws_simplex2(int gop, i32 seed, const f32* p, f32* v)
{
    const double kSkew2 = 1.0 / (kRoot3 + 1.0), kUnskew2 = -1.0 / (kRoot3 + 3.0), kR2 = 0.5;
    f32 x = p[0], y = p[1];
    f32 skewDelta = (float)kSkew2 * (x + y);
    f32 xs = x + skewDelta, ys = y + skewDelta;
    f32 xb = fs_floor(xs), yb = fs_floor(ys);
    f32 dxs = xs - xb, dys = ys - yb;
    i32 xp = imul(fs_cvt_i(xb), PRIME_X), yp = imul(fs_cvt_i(yb), PRIME_Y);
    int xGEy = dxs >= dys;
    f32 unskewDelta = (float)kUnskew2 * (dxs + dys);
    f32 dx0 = dxs + unskewDelta, dy0 = dys + unskewDelta;
    f32 dx1 = ws_sel(!xGEy, dx0 + 1.0f, dx0) - (float)(kUnskew2 + 1);
    f32 dy1 = ws_sel(xGEy, dy0 + 1.0f, dy0) - (float)(kUnskew2 + 1);
    f32 dx2 = dx0 - (float)(kUnskew2 * 2 + 1);
    f32 dy2 = dy0 - (float)(kUnskew2 * 2 + 1);
    f32 f0 = fs_fnma(dx0, dx0, fs_fnma(dy0, dy0, (float)kR2));
    f32 f1 = fs_fnma(dx1, dx1, fs_fnma(dy1, dy1, (float)kR2));
    f32 f2 = f0 + fs_fma(unskewDelta, (float)(-4.0 * (kRoot3 + 2.0) / (kRoot3 + 3.0)), (float)(-2.0 / 3.0));
    f0 = ws_pow4(fs_max(f0, 0.0f)); f1 = ws_pow4(fs_max(f1, 0.0f)); f2 = ws_pow4(fs_max(f2, 0.0f));
    v[0] = 0.0f; v[1] = 0.0f;
    ws_vec2(gop, hash2(seed, xp, yp), dx0, dy0, f0, v);
    ws_vec2(gop, hash2(seed, ws_madd(xGEy, xp, PRIME_X), ws_madd(!xGEy, yp, PRIME_Y)), dx1, dy1, f1, v);
    ws_vec2(gop, hash2(seed, iadd(xp, PRIME_X), iadd(yp, PRIME_Y)), dx2, dy2, f2, v);
}

/* DomainWarpSimplex Warp_3D (:835-931) */
static void ws_simplex3(int gop, i32 seed, const f32* p, f32* v)
{
    const double kSkew3 = 1.0 / 3.0, kRU3 = -1.0 / 2.0, kR2 = 0.6;
    f32 x = p[0], y = p[1], z = p[2];
    f32 skewDelta = (float)kSkew3 * (x + y + z);
    f32 xs = x + skewDelta, ys = y + skewDelta, zs = z + skewDelta;
    f32 xb = fs_floor(xs), yb = fs_floor(ys), zb = fs_floor(zs);
    f32 dxs = xs - xb, dys = ys - yb, dzs = zs - zb;
    i32 xp = imul(fs_cvt_i(xb), PRIME_X), yp = imul(fs_cvt_i(yb), PRIME_Y), zp = imul(fs_cvt_i(zb), PRIME_Z);
    int xGEy = dxs >= dys, yGEz = dys >= dzs, xGEz = dxs >= dzs;
    f32 unskewDelta = (float)kRU3 * (dxs + dys + dzs);
    f32 dx0 = dxs + unskewDelta, dy0 = dys + unskewDelta, dz0 = dzs + unskewDelta;
    int maskX1 = xGEy && xGEz;
    int maskY1 = yGEz && !xGEy;
    int maskZ1 = xGEz || yGEz;          /* inverted */
    int nMaskX2 = xGEy || xGEz;         /* inverted */
    int nMaskY2 = xGEy && !yGEz;
    int nMaskZ2 = xGEz && yGEz;
    f32 dx3 = dx0 - (float)(kRU3 * 3 + 1), dy3 = dy0 - (float)(kRU3 * 3 + 1), dz3 = dz0 - (float)(kRU3 * 3 + 1);
    f32 dx1 = ws_sel(maskX1, dx3 - 1.0f, dx3);
    f32 dy1 = ws_sel(maskY1, dy3 - 1.0f, dy3);
    f32 dz1 = ws_sel(maskZ1, dz3, dz3 - 1.0f);
    f32 dx2 = ws_sel(!nMaskX2, dx0 + 1.0f, dx0);
    f32 dy2 = ws_sel(nMaskY2, dy0 + 1.0f, dy0);
    f32 dz2 = ws_sel(nMaskZ2, dz0 + 1.0f, dz0);
    f32 f0 = fs_fnma(dz0, dz0, fs_fnma(dy0, dy0, fs_fnma(dx0, dx0, (float)kR2)));
    f32 f1 = fs_fnma(dz1, dz1, fs_fnma(dy1, dy1, fs_fnma(dx1, dx1, (float)kR2)));
    f32 f2 = fs_fnma(dz2, dz2, fs_fnma(dy2, dy2, fs_fnma(dx2, dx2, (float)kR2)));
    f32 f3 = f0 - (unskewDelta + (float)(3.0 / 4.0));
    f0 = ws_pow4(fs_max(f0, 0.0f)); f1 = ws_pow4(fs_max(f1, 0.0f)); f2 = ws_pow4(fs_max(f2, 0.0f)); f3 = ws_pow4(fs_max(f3, 0.0f));
    v[0] = 0.0f; v[1] = 0.0f; v[2] = 0.0f;
    ws_vec3(gop, hash3(seed, xp, yp, zp), dx0, dy0, dz0, f0, v);
    ws_vec3(gop, hash3(seed, ws_madd(maskX1, xp, PRIME_X), ws_madd(maskY1, yp, PRIME_Y), ws_madd(!maskZ1, zp, PRIME_Z)), dx1, dy1, dz1, f1, v);
    ws_vec3(gop, hash3(seed, ws_madd(nMaskX2, xp, PRIME_X), ws_madd(!nMaskY2, yp, PRIME_Y), ws_madd(!nMaskZ2, zp, PRIME_Z)), dx2, dy2, dz2, f2, v);
    ws_vec3(gop, hash3(seed, iadd(xp, PRIME_X), iadd(yp, PRIME_Y), iadd(zp, PRIME_Z)), dx3, dy3, dz3, f3, v);
    if (gop) {                          /* match gradient orientation (:909-917) */
        f32 d = (float)(-2.0 / 2.0) * (v[0] + v[1] + v[2]);
        v[0] = v[0] + d; v[1] = v[1] + d; v[2] = v[2] + d;
    }
}

/* DomainWarpSimplex Warp_4D (:933-1089) */
static void ws_simplex4(int gop, i32 seed, const f32* p, f32* v)
{
    const double kSkew4 = 1.0 / (kRoot5 + 1.0), kUnskew4 = -1.0 / (kRoot5 + 5.0), kR2 = 0.6;
    static const int32_t primes[4] = {PRIME_X, PRIME_Y, PRIME_Z, PRIME_W};
    f32 skewDelta = (float)kSkew4 * (p[0] + p[1] + p[2] + p[3]);
    f32 ds[4], d0[4];
    i32 pb[4];
    for (int k = 0; k < 4; ++k) {
        f32 sk = p[k] + skewDelta;
        f32 b = fs_floor(sk);
        ds[k] = sk - b;
        pb[k] = imul(fs_cvt_i(b), primes[k]);
    }
    f32 unskewDelta = (float)kUnskew4 * (ds[0] + ds[1] + ds[2] + ds[3]);
    for (int k = 0; k < 4; ++k) d0[k] = ds[k] + unskewDelta;
    int rank[4] = {0, 0, 0, 0};
    for (int a = 0; a < 4; ++a)
        for (int b = a + 1; b < 4; ++b) {
            if (d0[a] >= d0[b]) rank[a]++; else rank[b]++;
        }
    f32 d[5][4];
    f32 fo[5];
    for (int k = 0; k < 4; ++k) {
        d[0][k] = d0[k];
        d[1][k] = ws_sel(rank[k] > 2, d0[k] - 1.0f, d0[k]) - (float)kUnskew4;
        d[2][k] = ws_sel(rank[k] > 1, d0[k] - 1.0f, d0[k]) - (float)(kUnskew4 * 2);
        d[3][k] = ws_sel(rank[k] > 0, d0[k] - 1.0f, d0[k]) - (float)(kUnskew4 * 3);
        d[4][k] = d0[k] - (float)(kUnskew4 * 4 + 1);
    }
    for (int i = 0; i < 4; ++i)
        fo[i] = fs_fnma(d[i][3], d[i][3], fs_fnma(d[i][2], d[i][2], fs_fnma(d[i][1], d[i][1], fs_fnma(d[i][0], d[i][0], (float)kR2))));
    fo[4] = fo[0] + fs_fma(unskewDelta, (float)(-4.0 * (kRoot5 + 3.0) / (kRoot5 + 5.0)), (float)(-4.0 / 5.0));
    for (int i = 0; i < 5; ++i) fo[i] = ws_pow4(fs_max(fo[i], 0.0f));
    v[0] = 0.0f; v[1] = 0.0f; v[2] = 0.0f; v[3] = 0.0f;
    for (int i = 0; i < 5; ++i) {
        i32 c[4];
        for (int k = 0; k < 4; ++k) {
            int m = i == 0 ? 0 : i == 4 ? 1 : rank[k] > 3 - i;
            c[k] = ws_madd(m, pb[k], primes[k]);
        }
        ws_vec4(gop, hash4(seed, c[0], c[1], c[2], c[3]), d[i][0], d[i][1], d[i][2], d[i][3], fo[i], v);
    }
}

/* DomainWarpSuperSimplex Warp_2D (:1131-1218) */
static void ws_super2(int gop, i32 seed, const f32* p, f32* v)
{
    const double kSkew2 = 1.0 / (kRoot3 + 1.0), kUnskew2 = -1.0 / (kRoot3 + 3.0), kR2 = 2.0 / 3.0;
    f32 x = p[0], y = p[1];
    f32 skewDelta = (float)kSkew2 * (x + y);
    f32 xs = x + skewDelta, ys = y + skewDelta;
    f32 xb = fs_floor(xs), yb = fs_floor(ys);
    f32 dxs = xs - xb, dys = ys - yb;
    i32 xp = imul(fs_cvt_i(xb), PRIME_X), yp = imul(fs_cvt_i(yb), PRIME_Y);
    int fXY = dxs + dys > 1.0f;
    f32 boundaryXY = ws_sel(fXY, -1.0f, 0.0f);
    int fX = fs_fma(dxs, -2.0f, dys) < boundaryXY;
    int fY = fs_fma(dys, -2.0f, dxs) < boundaryXY;
    f32 unskewDelta = (float)kUnskew2 * (dxs + dys);
    f32 dxB = dxs + unskewDelta, dyB = dys + unskewDelta;
    v[0] = 0.0f; v[1] = 0.0f;
    f32 fb0;
    {   /* <0, 0> */
        fb0 = fs_fnma(dxB, dxB, fs_fnma(dyB, dyB, (float)kR2));
        ws_vec2(gop, hash2(seed, xp, yp), dxB, dyB, ws_pow4(fb0), v);
    }
    {   /* <1, 1> */
        f32 f = fs_fma(unskewDelta, (float)(-4.0 * (kRoot3 + 2.0) / (kRoot3 + 3.0)), fb0 - (float)kR2);
        ws_vec2(gop, hash2(seed, iadd(xp, PRIME_X), iadd(yp, PRIME_Y)),
                dxB - (float)(2 * kUnskew2 + 1), dyB - (float)(2 * kUnskew2 + 1), ws_pow4(f), v);
    }
    f32 xyDelta = ws_sel(fXY, (float)(kUnskew2 + 1), (float)(-kUnskew2));
    dxB = dxB - xyDelta;
    dyB = dyB - xyDelta;
    {   /* <1, 0> or <-1, 0> or <1, 2> */
        i32 hx = ws_madd(fX, xp, imul(PRIME_X, 2));
        hx = fXY ? hx : isub(hx, PRIME_X);
        i32 h = hash2(seed, hx, ws_madd(fXY, yp, PRIME_Y));
        f32 dx = dxB - ws_sel(fX, (float)(1 + 2 * kUnskew2), -1.0f);
        f32 dy = ws_sel(fX, dyB - (float)(2 * kUnskew2), dyB);
        f32 f = fs_max(fs_fnma(dx, dx, fs_fnma(dy, dy, (float)kR2)), 0.0f);
        ws_vec2(gop, h, dx, dy, ws_pow4(f), v);
    }
    {   /* <0, 1> or <0, -1> or <2, 1> */
        i32 hy = ws_madd(fY, yp, imul(PRIME_Y, 2));
        hy = fXY ? hy : isub(hy, PRIME_Y);
        i32 h = hash2(seed, ws_madd(fXY, xp, PRIME_X), hy);
        f32 dx = ws_sel(fY, dxB - (float)(2 * kUnskew2), dxB);
        f32 dy = dyB - ws_sel(fY, (float)(1 + 2 * kUnskew2), -1.0f);
        f32 f = fs_max(fs_fnma(dx, dx, fs_fnma(dy, dy, (float)kR2)), 0.0f);
        ws_vec2(gop, h, dx, dy, ws_pow4(f), v);
    }
}

static inline f32 ws_fb4(f32 fb) { return (fb * fb) * (fb * fb); }
#define WS_SIGNBIT ((int32_t)0x80000000)

/* DomainWarpSuperSimplex Warp_3D (:1220-1446) */
static void ws_super3(int gop, i32 seed, const f32* p, f32* v)
{
    const double kSkew3 = 1.0 / 3.0, kRU3 = -1.0 / 2.0, kTU3 = -1.0 / 4.0, kDA = 3.0 / 4.0, kDB = 1.0, kR2 = kDA;
    f32 x = p[0], y = p[1], z = p[2];
    f32 skewDelta = (float)kSkew3 * (x + y + z);
    f32 xs = x + skewDelta, ys = y + skewDelta, zs = z + skewDelta;
    f32 xb = fs_floor(xs), yb = fs_floor(ys), zb = fs_floor(zs);
    f32 dxs = xs - xb, dys = ys - yb, dzs = zs - zb;
    {   /* closest vertex of the unit cell */
        f32 tu = (float)kTU3 * (dxs + dys + dzs);
        f32 xN = dxs + tu, yN = dys + tu, zN = dzs + tu;
        f32 xyzN = -tu;
        f32 maxScore = 0.375f;
        int32_t bits = xyzN > maxScore ? -1 : 0;
        maxScore = fs_max(maxScore, xyzN);
#define WS_CONSIDER(score, b) do { f32 s_ = (score); bits = s_ > maxScore ? (b) : bits; maxScore = fs_max(maxScore, s_); } while (0)
        WS_CONSIDER(xN, 1);
        WS_CONSIDER(yN, 2);
        WS_CONSIDER(zN, 4);
        maxScore = maxScore + (0.125f - xyzN);
        WS_CONSIDER(-zN, 3);
        WS_CONSIDER(-yN, 5);
        WS_CONSIDER(-xN, 6);
        int mx = (bits & 1) != 0, my = (bits & 2) != 0, mz = (bits & 4) != 0;
        xb = ws_sel(mx, xb + 1.0f, xb); yb = ws_sel(my, yb + 1.0f, yb); zb = ws_sel(mz, zb + 1.0f, zb);
        dxs = ws_sel(mx, dxs - 1.0f, dxs); dys = ws_sel(my, dys - 1.0f, dys); dzs = ws_sel(mz, dzs - 1.0f, dzs);
    }
    i32 xp = imul(fs_cvt_i(xb), PRIME_X), yp = imul(fs_cvt_i(yb), PRIME_Y), zp = imul(fs_cvt_i(zb), PRIME_Z);
    f32 scs = dxs + dys + dzs;
    f32 tu = (float)kTU3 * scs;
    f32 xN = dxs + tu, yN = dys + tu, zN = dzs + tu;
    f32 xyzN = -tu;
    f32 ud = (float)kRU3 * scs;
    f32 dxB = dxs + ud, dyB = dys + ud, dzB = dzs + ud;
    f32 cs = (float)(1 + 3 * kRU3) * scs;
    v[0] = 0.0f; v[1] = 0.0f; v[2] = 0.0f;
    f32 stemA, stemB;
    {   /* <0,0,0> */
        f32 fb = fs_fnma(dzB, dzB, fs_fnma(dyB, dyB, fs_fnma(dxB, dxB, (float)kR2))) * 0.5f;
        stemA = fb - (float)(kDA * 0.5);
        stemB = fb - (float)(kDB * 0.5);
        ws_vec3(gop, hash3(seed, xp, yp, zp), dxB, dyB, dzB, ws_fb4(fb), v);
    }
    {   /* <1,1,1> or <-1,-1,-1> */
        int sm = xyzN < 0.0f;
        i32 sign = sm ? WS_SIGNBIT : 0;
        f32 off = fs_xor_sign((float)(3 * kRU3 + 1), sign);
        f32 fb = fs_max(fs_fma(off, cs, stemA), 0.0f);
        ws_vec3(gop, hash3(seed, iadd(xp, sm ? -PRIME_X : PRIME_X), iadd(yp, sm ? -PRIME_Y : PRIME_Y), iadd(zp, sm ? -PRIME_Z : PRIME_Z)),
                dxB - off, dyB - off, dzB - off, ws_fb4(fb), v);
    }
    /* <1,1,0>, <1,0,1>, <0,1,1> or their negatives */
    {
        int sm = xyzN < zN;
        i32 sign = sm ? WS_SIGNBIT : 0;
        f32 off0 = fs_xor_sign((float)(2 * kRU3), sign);
        f32 fb = fs_min(fs_xor_sign(dzB, sign) - stemB, 0.0f);
        ws_vec3(gop, hash3(seed, iadd(xp, sm ? -PRIME_X : PRIME_X), iadd(yp, sm ? -PRIME_Y : PRIME_Y), zp),
                dxB, dyB, dzB - off0, ws_fb4(fb), v);
    }
    {
        int sm = xyzN < yN;
        i32 sign = sm ? WS_SIGNBIT : 0;
        f32 off0 = fs_xor_sign((float)(2 * kRU3), sign);
        f32 fb = fs_min(fs_xor_sign(dyB, sign) - stemB, 0.0f);
        ws_vec3(gop, hash3(seed, iadd(xp, sm ? -PRIME_X : PRIME_X), yp, iadd(zp, sm ? -PRIME_Z : PRIME_Z)),
                dxB, dyB - off0, dzB, ws_fb4(fb), v);
    }
    {
        int sm = xyzN < xN;
        i32 sign = sm ? WS_SIGNBIT : 0;
        f32 off0 = fs_xor_sign((float)(2 * kRU3), sign);
        f32 fb = fs_min(fs_xor_sign(dxB, sign) - stemB, 0.0f);
        ws_vec3(gop, hash3(seed, xp, iadd(yp, sm ? -PRIME_Y : PRIME_Y), iadd(zp, sm ? -PRIME_Z : PRIME_Z)),
                dxB - off0, dyB, dzB, ws_fb4(fb), v);
    }
    /* <1,0,0>, <0,1,0>, <0,0,1> or their negatives */
    {
        int sm = xN < 0.0f;
        i32 sign = sm ? WS_SIGNBIT : 0;
        f32 off0 = fs_xor_sign((float)kRU3, sign);
        f32 fb = fs_max(fs_fma(off0, cs, stemA) + fs_xor_sign(dxB, sign), 0.0f);
        ws_vec3(gop, hash3(seed, iadd(xp, sm ? -PRIME_X : PRIME_X), yp, zp), dxB + off0, dyB - off0, dzB - off0, ws_fb4(fb), v);
    }
    {
        int sm = yN < 0.0f;
        i32 sign = sm ? WS_SIGNBIT : 0;
        f32 off0 = fs_xor_sign((float)kRU3, sign);
        f32 fb = fs_max(fs_fma(off0, cs, stemA) + fs_xor_sign(dyB, sign), 0.0f);
        ws_vec3(gop, hash3(seed, xp, iadd(yp, sm ? -PRIME_Y : PRIME_Y), zp), dxB - off0, dyB + off0, dzB - off0, ws_fb4(fb), v);
    }
    {
        int sm = zN < 0.0f;
        i32 sign = sm ? WS_SIGNBIT : 0;
        f32 off0 = fs_xor_sign((float)kRU3, sign);
        f32 fb = fs_max(fs_fma(off0, cs, stemA) + fs_xor_sign(dzB, sign), 0.0f);
        ws_vec3(gop, hash3(seed, xp, yp, iadd(zp, sm ? -PRIME_Z : PRIME_Z)), dxB - off0, dyB - off0, dzB + off0, ws_fb4(fb), v);
    }
    if (gop) {                          /* match gradient orientation (:1424-1432) */
        f32 d = (float)(-2.0 / 3.0) * (v[0] + v[1] + v[2]);
        v[0] = v[0] + d; v[1] = v[1] + d; v[2] = v[2] + d;
    }
}

/* DomainWarpSuperSimplex Warp_4D (:1448-1835).  The sixteen vertices around
 * the closest lattice vertex are visited in the reference's order; a vertex is
 * the set of axes it moves along (bit k = axis k), in the direction given by
 * the sign test of its group. */
static void ws_super4(int gop, i32 seed, const f32* p, f32* v)
{
    const double kSkew4 = 1.0 / (kRoot5 + 1.0), kU4 = -1.0 / (kRoot5 + 5.0), kTU4 = -1.0 / 5.0;
    const double kDA = 4.0 / 5.0, kDB = 6.0 / 5.0, kR2 = kDA;
    static const int32_t primes[4] = {PRIME_X, PRIME_Y, PRIME_Z, PRIME_W};
    static const int order[16] = {0x0, 0xF, 0x7, 0xB, 0xD, 0xE, 0x1, 0x3, 0x5, 0x9, 0x2, 0x6, 0xA, 0x4, 0xC, 0x8};
    f32 skewDelta = (float)kSkew4 * (p[0] + p[1] + p[2] + p[3]);
    f32 b[4], ds[4];
    for (int k = 0; k < 4; ++k) {
        f32 sk = p[k] + skewDelta;
        b[k] = fs_floor(sk);
        ds[k] = sk - b[k];
    }
    {   /* closest vertex of the unit cell */
        f32 tu = (float)kTU4 * (ds[0] + ds[1] + ds[2] + ds[3]);
        f32 n[4];
        for (int k = 0; k < 4; ++k) n[k] = ds[k] + tu;
        f32 xyzwN = -tu;
        f32 maxScore = 0.6f - xyzwN;
        int32_t bits = 0.2f > maxScore ? -1 : 0;
        maxScore = fs_max(maxScore, 0.2f);
        WS_CONSIDER(-n[3], 0x7);
        WS_CONSIDER(-n[2], 0xB);
        WS_CONSIDER(-n[1], 0xD);
        WS_CONSIDER(-n[0], 0xE);
        maxScore = maxScore + (xyzwN - 0.2f);
        WS_CONSIDER(n[0], 0x1);
        WS_CONSIDER(n[1], 0x2);
        WS_CONSIDER(n[2], 0x4);
        WS_CONSIDER(n[3], 0x8);
        maxScore = maxScore + (0.2f - n[0]);
        WS_CONSIDER(n[1], 0x3);
        WS_CONSIDER(n[2], 0x5);
        WS_CONSIDER(n[3], 0x9);
        maxScore = maxScore + n[0];
        WS_CONSIDER(n[1] + n[2], 0x6);
        maxScore = maxScore - n[3];
        WS_CONSIDER(n[1], 0xA);
        WS_CONSIDER(n[2], 0xC);
        for (int k = 0; k < 4; ++k) {
            int m = (bits >> k) & 1;
            b[k] = ws_sel(m, b[k] + 1.0f, b[k]);
            ds[k] = ws_sel(m, ds[k] - 1.0f, ds[k]);
        }
    }
    i32 pb[4];
    for (int k = 0; k < 4; ++k) pb[k] = imul(fs_cvt_i(b[k]), primes[k]);
    f32 scs = ds[0] + ds[1] + ds[2] + ds[3];
    f32 tu = (float)kTU4 * scs;
    f32 n[4], dB[4];
    for (int k = 0; k < 4; ++k) n[k] = ds[k] + tu;
    f32 xyzwN = -tu;
    f32 ud = (float)kU4 * scs;
    for (int k = 0; k < 4; ++k) dB[k] = ds[k] + ud;
    f32 cs = (float)(1 + 4 * kU4) * scs;
    v[0] = 0.0f; v[1] = 0.0f; v[2] = 0.0f; v[3] = 0.0f;
    f32 stemA = 0.0f, stemB = 0.0f;
    for (int vi = 0; vi < 16; ++vi) {
        const int S = order[vi];
        const int cnt = (S & 1) + ((S >> 1) & 1) + ((S >> 2) & 1) + ((S >> 3) & 1);
        if (cnt == 0) {
            f32 fb = fs_fnma(dB[3], dB[3], fs_fnma(dB[2], dB[2], fs_fnma(dB[1], dB[1], fs_fnma(dB[0], dB[0], (float)kR2)))) * 0.5f;
            stemA = fb - (float)(kDA * 0.5);
            stemB = fb - (float)(kDB * 0.5);
            ws_vec4(gop, hash4(seed, pb[0], pb[1], pb[2], pb[3]), dB[0], dB[1], dB[2], dB[3], ws_fb4(fb), v);
            continue;
        }
        int sm;
        f32 off1, off0, fb;
        int a = -1, bb = -1;                      /* the one or two axes of single / pair vertices */
        for (int k = 0; k < 4; ++k) if ((S >> k) & 1) { if (a < 0) a = k; else if (bb < 0) bb = k; }
        int missing = -1;
        for (int k = 0; k < 4; ++k) if (!((S >> k) & 1)) missing = k;
        if (cnt == 4) sm = xyzwN < 0.0f;
        else if (cnt == 3) sm = xyzwN < n[missing];
        else if (cnt == 1) sm = n[a] < 0.0f;
        else sm = n[a] < -n[bb];
        i32 sign = sm ? WS_SIGNBIT : 0;
        if (cnt == 4) {
            off1 = fs_xor_sign((float)(4 * kU4 + 1), sign);
            off0 = off1;
            fb = fs_max(fs_fma(off1, cs, stemA), 0.0f);
        } else if (cnt == 3) {
            off1 = fs_xor_sign((float)(3 * kU4 + 1), sign);
            off0 = fs_xor_sign((float)(3 * kU4), sign);
            fb = fs_max(fs_fma(off1, cs, stemB) - fs_xor_sign(dB[missing], sign), 0.0f);
        } else if (cnt == 1) {
            off1 = fs_xor_sign((float)(kU4 + 1), sign);
            off0 = fs_xor_sign((float)kU4, sign);
            fb = fs_max(fs_fma(off0, cs, stemA) + fs_xor_sign(dB[a], sign), 0.0f);
        } else {
            off1 = fs_xor_sign((float)(2 * kU4 + 1), sign);
            off0 = fs_xor_sign((float)(2 * kU4), sign);
            fb = fs_max(fs_fma(off0, cs, stemB) + fs_xor_sign(dB[a] + dB[bb], sign), 0.0f);
        }
        i32 c[4];
        f32 d[4];
        for (int k = 0; k < 4; ++k) {
            int in = (S >> k) & 1;
            c[k] = in ? iadd(pb[k], sm ? -primes[k] : primes[k]) : pb[k];
            d[k] = dB[k] - (in ? off1 : off0);
        }
        ws_vec4(gop, hash4(seed, c[0], c[1], c[2], c[3]), d[0], d[1], d[2], d[3], ws_fb4(fb), v);
    }
}
#undef WS_CONSIDER

/* DomainWarpSimplex / DomainWarpSuperSimplex ::Warp (:729-769, :1092-1129):
 * seed offset, the vector noise, bounding x axis scale, out += v * amp;
 * returns |v|^2. */
static f32 warp_simplex(const on_node* n, i32 seed, f32 warpAmp, int dim, const f32* pin, f32* out)
{
    const int super = n->id == N_DOMAINWARPSUPERSIMPLEX;
    const int gop = n->vec_scheme == 1;
    seed = iadd(seed, n->seed_offset);
    f32 v[4];
    float bound;
    if (dim == 2) {
        if (super) ws_super2(gop, seed, pin, v); else ws_simplex2(gop, seed, pin, v);
        bound = super ? (gop ? (float)(9.28993664146183 / 2.0) : 12.814453124999995f)
                      : (gop ? (float)(49.918426513671875 / 2.0) : 70.1480577066486f);
    } else if (dim == 3) {
        if (super) ws_super3(gop, seed, pin, v); else ws_simplex3(gop, seed, pin, v);
        bound = super ? (gop ? (float)(144.736422163332608 / 1.4142135623730951) : 37.63698669623629f)
                      : (gop ? (float)(32.69428253173828125 / 1.4142135623730951) : 16.281631889139874f);
    } else {
        if (super) ws_super4(gop, seed, pin, v); else ws_simplex4(gop, seed, pin, v);
        bound = super ? (gop ? (float)(115.21625311930542 / 1.4142135623730951) : 48.80058117543753f)
                      : (gop ? (float)(33.653125584827855 / 1.4142135623730951) : 30.88161777516092f);
    }
    for (int k = 0; k < dim; ++k) v[k] = v[k] * (float)(bound * n->axis[k]);
    for (int k = 0; k < dim; ++k) out[k] = fs_fma(v[k], warpAmp, out[k]);
    f32 r = v[0] * v[0];
    for (int k = 1; k < dim; ++k) r = fs_fma(v[k], v[k], r);
    return r;
}

static f32 warp_any(const on_node* w, i32 seed, f32 amp, int dim, const f32* scaled, f32* out)
{
    if (w->id == N_DOMAINWARPGRADIENT) return warp_gradient(w, seed, amp, dim, scaled, out);
    return warp_simplex(w, seed, amp, dim, scaled, out);
}

/* ---- Fractal (Fractal.inl:10-67) --------------------------------------- */

static f32 fractal(const on_node* n, i32 seed, int dim, const f32* pin, int ridged)
{
    f32 p[4];
    for (int k = 0; k < dim; ++k) p[k] = pin[k];
    f32 gain, ws;
    if (dim == 2) { gain = HYB2(n, 0, seed, p[0], p[1]); ws = HYB2(n, 1, seed, p[0], p[1]); }
    else if (dim == 3) { gain = HYB3(n, 0, seed, p[0], p[1], p[2]); ws = HYB3(n, 1, seed, p[0], p[1], p[2]); }
    else { gain = HYB4(n, 0, seed, p[0], p[1], p[2], p[3]); ws = HYB4(n, 1, seed, p[0], p[1], p[2], p[3]); }
    f32 lac = n->lacunarity;
    f32 amp = 1.0f;
    f32 noise = gen_n(n->lookup[0], seed, dim, p);
    f32 sum;
    if (!ridged) sum = noise * amp;
    else { noise = fs_abs(noise); sum = (noise * -2.0f + 1.0f) * amp; }
    for (int i = 1; i < n->octaves; i++) {
        seed = iadd(seed, 1);
        if (!ridged) amp = amp * lerp(1.0f, (noise + 1.0f) * 0.5f, ws);
        else amp = amp * lerp(1.0f, 1.0f - noise, ws);
        amp = amp * gain;
        for (int k = 0; k < dim; ++k) p[k] = p[k] * lac;
        noise = gen_n(n->lookup[0], seed, dim, p);
        if (!ridged) sum = sum + noise * amp;
        else { noise = fs_abs(noise); sum = sum + (noise * -2.0f + 1.0f) * amp; }
    }
    return sum;
}

/* ---- Basic generators (BasicGenerators.inl:33-125) ----------------------- */

static f32 white(const on_node* n, i32 seed, int dim, const f32* pin)
{
    seed = iadd(seed, n->seed_offset);
    i32 q[4];
    for (int k = 0; k < dim; ++k) {
        i32 b = (int32_t)f_bits((float)pin[k]);
        q[k] = imul((int32_t)b ^ (int32_t)isra(b, 16), kPrimes[k]);
    }
    f32 v;
    if (dim == 2) v = valcoord2(seed, q[0], q[1]);
    else if (dim == 3) v = valcoord3(seed, q[0], q[1], q[2]);
    else v = valcoord4(seed, q[0], q[1], q[2], q[3]);
    return scale_output(n, v, -kValueBounds, kValueBounds);
}

static f32 checkerboard(const on_node* n, int dim, const f32* pin)
{
    int32_t v = 0;
    for (int k = 0; k < dim; ++k) v ^= (int32_t)fs_cvt_i(pin[k] * n->frequency);
    return scale_output(n, bits_f((uint32_t)(v & 1) << 30), 0, 2);
}

static f32 sine_wave(const on_node* n, int dim, const f32* pin)
{
    f32 t = fs_sin(pin[dim - 1] * n->frequency);                 /* right fold of products */
    for (int k = dim - 2; k >= 0; --k) t = fs_sin(pin[k] * n->frequency) * t;
    return scale_output(n, t, -1, 1);
}

static f32 hyb_n(const on_node* n, int k, i32 seed, int dim, const f32* p)
{
    if (dim == 2) return HYB2(n, k, seed, p[0], p[1]);
    if (dim == 3) return HYB3(n, k, seed, p[0], p[1], p[2]);
    return HYB4(n, k, seed, p[0], p[1], p[2], p[3]);
}

static f32 gradient_node(const on_node* n, i32 seed, int dim, const f32* p)
{
    f32 r = 0.0f;
    for (int k = 0; k < dim; ++k) r = fs_fma(p[k] + hyb_n(n, k, seed, dim, p), n->multiplier[k], r);
    return r;
}

static f32 distance_to_point(const on_node* n, i32 seed, int dim, const f32* p)
{
    f32 d[4];
    for (int k = 0; k < dim; ++k) d[k] = p[k] - hyb_n(n, k, seed, dim, p);
    return calc_distance(n, 4, 1, seed, dim, d);
}

/* ---- Modifiers and blends ------------------------------------------------ */

static void rotate_plane(int type, f32* x, f32* y, f32* z)   /* Modifiers.inl:354-388 */
{
    f32 nx = *x, ny = *y, nz = *z;
    if (type == 0) {
        f32 xy = *x + *y;
        f32 s2 = xy * -0.211324865405187f;
        nz = *z * 0.577350269189626f;
        nx = *x + s2 - nz;
        ny = *y + s2 - nz;
        nz = nz + xy * 0.577350269189626f;
    } else if (type == 1) {
        f32 xz = *x + *z;
        f32 s2 = xz * -0.211324865405187f;
        ny = *y * 0.577350269189626f;
        nx = *x + s2 - ny;
        nz = *z + s2 - ny;
        ny = ny + xz * 0.577350269189626f;
    }
    *x = nx; *y = ny; *z = nz;
}

static f32 terrace(const on_node* n, i32 seed, int dim, const f32* p)   /* Modifiers.inl:134-181 */
{
    f32 source = gen_n(n->lookup[0], seed, dim, p);
    source = source * n->step_count;
    f32 rounded = fs_round(source);
    if (n->hnode[0]) {
        f32 smoothness = gen_n(n->hnode[0], seed, dim, p);
        if (smoothness != 0.0f) {
            f32 diff = rounded - source;
            int neg = diff < 0.0f;
            diff = fs_abs(diff);
            diff = 0.5f - diff;
            f32 recip = 1.0f + fs_recip(smoothness);
            diff = diff * recip;
            diff = fs_min(diff, 0.5f);
            diff = neg ? 0.5f - diff : diff - 0.5f;
            rounded = rounded + diff;
        }
    } else if (n->hval[0] != 0.0f) {
        f32 diff = rounded - source;
        int neg = diff < 0.0f;
        diff = fs_abs(diff);
        diff = 0.5f - diff;
        diff = diff * n->smooth_recip;
        diff = fs_min(diff, 0.5f);
        diff = neg ? 0.5f - diff : diff - 0.5f;
        rounded = rounded + diff;
    }
    return rounded * n->step_recip;
}

static f32 eval_node(const on_node* n, i32 seed, int dim, const f32* p)
{
    switch (n->id) {
    case N_CONSTANT: return n->value;
    case N_WHITE: return white(n, seed, dim, p);
    case N_CHECKERBOARD: return checkerboard(n, dim, p);
    case N_SINEWAVE: return sine_wave(n, dim, p);
    case N_GRADIENT: return gradient_node(n, seed, dim, p);
    case N_DISTANCETOPOINT: return distance_to_point(n, seed, dim, p);
    case N_SIMPLEX:
        return dim == 2 ? simplex2(n, seed, p[0], p[1]) : dim == 3 ? simplex3(n, seed, p[0], p[1], p[2]) : simplex4(n, seed, p[0], p[1], p[2], p[3]);
    case N_SUPERSIMPLEX:
        return dim == 2 ? supersimplex2(n, seed, p[0], p[1]) : dim == 3 ? supersimplex3(n, seed, p[0], p[1], p[2]) : supersimplex4(n, seed, p[0], p[1], p[2], p[3]);
    case N_PERLIN:
        return dim == 2 ? perlin2(n, seed, p[0], p[1]) : dim == 3 ? perlin3(n, seed, p[0], p[1], p[2]) : perlin4(n, seed, p[0], p[1], p[2], p[3]);
    case N_VALUE:
        return dim == 2 ? value2(n, seed, p[0], p[1]) : dim == 3 ? value3(n, seed, p[0], p[1], p[2]) : value4(n, seed, p[0], p[1], p[2], p[3]);
    case N_CELLULARVALUE: return cellular_value(n, seed, dim, p);
    case N_CELLULARDISTANCE: return cellular_distance(n, seed, dim, p);
    case N_CELLULARLOOKUP: return cellular_lookup(n, seed, dim, p);
    case N_FRACTALFBM: return fractal(n, seed, dim, p, 0);
    case N_FRACTALRIDGED: return fractal(n, seed, dim, p, 1);
    case N_PINGPONG: {   /* Modifiers.inl:184-201 */
        f32 strength = hyb_n(n, 0, seed, dim, p);
        f32 t = gen_n(n->lookup[0], seed, dim, p) * strength;
        t = t - fs_floor(t * 0.5f) * 2.0f;
        return t < 1.0f ? t : 2.0f - t;
    }
    case N_DOMAINWARPSIMPLEX: case N_DOMAINWARPSUPERSIMPLEX: case N_DOMAINWARPGRADIENT:
        return domain_warp_gen(n, seed, dim, p);
    case N_DWFRACTALPROGRESSIVE: return domain_warp_fractal(n, seed, dim, p, 0);
    case N_DWFRACTALINDEPENDENT: return domain_warp_fractal(n, seed, dim, p, 1);
    case N_ADD: return gen_n(n->lookup[0], seed, dim, p) + hyb_n(n, 0, seed, dim, p);
    case N_SUBTRACT: return hyb_n(n, 0, seed, dim, p) - hyb_n(n, 1, seed, dim, p);
    case N_MULTIPLY: return gen_n(n->lookup[0], seed, dim, p) * hyb_n(n, 0, seed, dim, p);
    case N_DIVIDE: return hyb_n(n, 0, seed, dim, p) / hyb_n(n, 1, seed, dim, p);
    case N_MODULUS: return fs_mod(hyb_n(n, 0, seed, dim, p), hyb_n(n, 1, seed, dim, p));
    case N_ABS: return fs_abs(gen_n(n->lookup[0], seed, dim, p));
    case N_MIN: return fs_min(gen_n(n->lookup[0], seed, dim, p), hyb_n(n, 0, seed, dim, p));
    case N_MAX: return fs_max(gen_n(n->lookup[0], seed, dim, p), hyb_n(n, 0, seed, dim, p));
    case N_MINSMOOTH: case N_MAXSMOOTH: {   /* Blends.inl:124-162 */
        int mx = n->id == N_MAXSMOOTH;
        f32 a = gen_n(n->lookup[0], seed, dim, p);
        f32 b = hyb_n(n, 0, seed, dim, p);
        if (mx) { a = -a; b = -b; }
        f32 sm = fs_max(FLT_MIN, fs_abs(hyb_n(n, 1, seed, dim, p)));
        f32 h = fs_max(sm - fs_abs(a - b), 0.0f);
        h = h * fs_recip(sm);
        f32 r = fs_fnma(1.0f / 6.0f, h * h * h * sm, fs_min(a, b));
        return mx ? -r : r;
    }
    case N_SIGNEDSQRT: {
        f32 v = gen_n(n->lookup[0], seed, dim, p);
        return bits_f(f_bits((float)fs_sqrt(fs_abs(v))) | (f_bits((float)v) & 0x80000000u));
    }
    case N_POWFLOAT: {
        f32 v = fs_max(fs_abs(hyb_n(n, 0, seed, dim, p)), FLT_MIN);
        return fs_pow(v, hyb_n(n, 1, seed, dim, p));
    }
    case N_POWINT: {
        f32 v = gen_n(n->lookup[0], seed, dim, p);
        f32 r = v * v;
        for (int i = 2; i < n->pow_int; i++) r = r * v;
        return r;
    }
    case N_DOMAINSCALE: {
        f32 q[4];
        for (int k = 0; k < dim; ++k) q[k] = p[k] * n->dscale;
        return gen_n(n->lookup[0], seed, dim, q);
    }
    case N_DOMAINOFFSET: {
        f32 q[4];
        for (int k = 0; k < dim; ++k) q[k] = p[k] + hyb_n(n, k, seed, dim, p);
        return gen_n(n->lookup[0], seed, dim, q);
    }
    case N_DOMAINROTATE: {   /* Modifiers.inl:33-61 */
        const float* r = n->rot;
        if (dim == 2) {
            if (n->pitch_sin == 0.0f && n->roll_sin == 0.0f)
                return gen2(n->lookup[0], seed, fs_fnma(p[1], n->yaw_sin, p[0] * n->yaw_cos), fs_fma(p[0], n->yaw_sin, p[1] * n->yaw_cos));
            f32 q[3] = {p[0], p[1], 0.0f};
            return gen3(n->lookup[0], seed, fs_fma(q[0], r[0], fs_fma(q[1], r[1], q[2] * r[2])),
                        fs_fma(q[0], r[3], fs_fma(q[1], r[4], q[2] * r[5])), fs_fma(q[0], r[6], fs_fma(q[1], r[7], q[2] * r[8])));
        }
        if (dim == 3)
            return gen3(n->lookup[0], seed, fs_fma(p[0], r[0], fs_fma(p[1], r[1], p[2] * r[2])),
                        fs_fma(p[0], r[3], fs_fma(p[1], r[4], p[2] * r[5])), fs_fma(p[0], r[6], fs_fma(p[1], r[7], p[2] * r[8])));
        return gen4(n->lookup[0], seed, p[0], p[1], p[2], p[3]);
    }
    case N_DOMAINAXISSCALE: {
        f32 q[4];
        for (int k = 0; k < dim; ++k) q[k] = p[k] * n->axis[k];
        return gen_n(n->lookup[0], seed, dim, q);
    }
    case N_SEEDOFFSET: return gen_n(n->lookup[0], iadd(seed, n->seed_offset), dim, p);
    case N_CONVERTRGBA8: {   /* Modifiers.inl:107-126 */
        f32 s = gen_n(n->lookup[0], seed, dim, p);
        s = fs_min(s, n->rgba_max);
        s = fs_max(s, n->rgba_min);
        s = s - n->rgba_min;
        s = s * (255.0f / (n->rgba_max - n->rgba_min));
        int32_t b = fs_cvt_i(s);
        uint32_t o = 0xFF000000u | (uint32_t)b | ((uint32_t)b << 8) | ((uint32_t)b << 16);
        return bits_f(o);
    }
    case N_GENERATORCACHE: return gen_n(n->lookup[0], seed, dim, p);
    case N_FADE: {   /* Blends.inl:169-198 */
        f32 fade = hyb_n(n, 0, seed, dim, p);
        f32 fmin = hyb_n(n, 1, seed, dim, p);
        f32 fmax = hyb_n(n, 2, seed, dim, p);
        f32 range = fmax - fmin;
        fade = (fade - fmin) / range;
        fade = fs_max(0.0f, fs_min(1.0f, fade));
        if (n->interp == 1) fade = interp_hermite(fade);
        else if (n->interp == 2) fade = interp_quintic(fade);
        fade = (range == 0.0f) ? 0.5f : fade;
        return lerp(gen_n(n->lookup[0], seed, dim, p), gen_n(n->lookup[1], seed, dim, p), fade);
    }
    case N_REMAP: {   /* Modifiers.inl:81-99 */
        f32 s = gen_n(n->lookup[0], seed, dim, p);
        f32 fromMin = hyb_n(n, 0, seed, dim, p), fromMax = hyb_n(n, 1, seed, dim, p);
        f32 toMin = hyb_n(n, 2, seed, dim, p), toMax = hyb_n(n, 3, seed, dim, p);
        f32 r = toMin + ((s - fromMin) / (fromMax - fromMin) * (toMax - toMin));
        if (n->clamp_output == 1) { r = fs_max(r, toMin); r = fs_min(r, toMax); }
        return r;
    }
    case N_TERRACE: return terrace(n, seed, dim, p);
    case N_ADDDIMENSION: {
        if (dim == 4) return gen4(n->lookup[0], seed, p[0], p[1], p[2], p[3]);
        f32 q[4] = {p[0], p[1], p[2], p[3]};
        q[dim] = hyb_n(n, 0, seed, dim, p);
        return gen_n(n->lookup[0], seed, dim + 1, q);
    }
    case N_REMOVEDIMENSION: {   /* Modifiers.inl:240-275 */
        if (dim == 2) return gen2(n->lookup[0], seed, p[0], p[1]);
        int r = n->remove_dim;
        if (r < 0 || r >= dim) return gen_n(n->lookup[0], seed, dim, p);
        f32 q[4]; int m = 0;
        for (int k = 0; k < dim; ++k) if (k != r) q[m++] = p[k];
        return gen_n(n->lookup[0], seed, dim - 1, q);
    }
    case N_DOMAINROTATEPLANE: {
        f32 x = p[0], y = p[1], z = dim >= 3 ? p[2] : 0.0f;
        rotate_plane(dim == 2 ? 0 : n->rot_type, &x, &y, &z);
        if (dim == 4) return gen4(n->lookup[0], seed, x, y, z, p[3]);
        return gen3(n->lookup[0], seed, x, y, z);
    }
    default: return 0.0f;
    }
}

static f32 gen2(const on_node* n, i32 seed, f32 x, f32 y) { f32 p[4] = {x, y, 0, 0}; return eval_node(n, seed, 2, p); }
static f32 gen3(const on_node* n, i32 seed, f32 x, f32 y, f32 z) { f32 p[4] = {x, y, z, 0}; return eval_node(n, seed, 3, p); }
static f32 gen4(const on_node* n, i32 seed, f32 x, f32 y, f32 z, f32 w) { f32 p[4] = {x, y, z, w}; return eval_node(n, seed, 4, p); }

/* ------------------------------------------------------------------------- */
/* Batch drivers (Generator.inl:79-433) with OutputMinMax (Generator.h:85-105) */
/* ------------------------------------------------------------------------- */

enum { K_GRID2, K_GRID3, K_GRID4, K_TILE2, K_POS2, K_POS3, K_POS4 };

typedef struct {
    const on_node* root;
    int kind;
    int seed;
    int count[4];
    float offset[4];
    float step[4];
    const float* posarr[4];
    /* tileable constants */
    float tmul[2], tfreq[2];
    float* out;
    int64_t begin, end;
    float mn, mx;
} job_t;

static void minmax_acc(float v, float* mn, float* mx)
{
    /* OutputMinMax::operator<< uses std::min/std::max: NaN never replaces. */
    if (v < *mn) *mn = v;
    if (*mx < v) *mx = v;
}

static void run_range(job_t* j)
{
    float mn = INFINITY, mx = -INFINITY;
    int dim = (j->kind == K_GRID2 || j->kind == K_POS2) ? 2 : (j->kind == K_GRID3 || j->kind == K_POS3) ? 3 : 4;
    for (int64_t i = j->begin; i < j->end; ++i) {
        f32 p[4] = {0, 0, 0, 0};
        if (j->kind <= K_GRID4) {
            int64_t r = i;
            for (int k = 0; k < dim; ++k) {
                int64_t ik = (k == dim - 1) ? r : r % j->count[k];
                r = (k == dim - 1) ? 0 : r / j->count[k];
                p[k] = fs_fma((float)(int32_t)ik, j->step[k], j->offset[k]);
            }
        } else if (j->kind == K_TILE2) {
            int64_t xi = i % j->count[0], yi = i / j->count[0];
            f32 xF = (float)(int32_t)xi * j->tmul[0];
            f32 yF = (float)(int32_t)yi * j->tmul[1];
            p[0] = fs_cos(xF) * j->tfreq[0];
            p[1] = fs_cos(yF) * j->tfreq[1];
            p[2] = fs_sin(xF) * j->tfreq[0];
            p[3] = fs_sin(yF) * j->tfreq[1];
            dim = 4;
        } else {
            for (int k = 0; k < dim; ++k) p[k] = j->offset[k] + j->posarr[k][i];
        }
        float v = (float)eval_node(j->root, j->seed, dim, p);
        j->out[i] = v;
        minmax_acc(v, &mn, &mx);
    }
    j->mn = mn; j->mx = mx;
}

/* ------------------------------------------------------------------------- */
/* Host worker pool (persistent: threads are created once and reused by every   */
/* call, as an application keeps its job system).  A call hands the pool a list */
/* of tasks; the calling thread works on them too.  Calls are serialised.       */
/* ------------------------------------------------------------------------- */

typedef struct { job_t* job; int64_t begin, end; float mn, mx; } task_t;

#define OC_MAX_THREADS 256

static pthread_mutex_t g_call_mu = PTHREAD_MUTEX_INITIALIZER;   /* one call at a time */
static pthread_mutex_t g_pool_mu = PTHREAD_MUTEX_INITIALIZER;
static pthread_cond_t g_pool_work = PTHREAD_COND_INITIALIZER;
static pthread_cond_t g_pool_done = PTHREAD_COND_INITIALIZER;
static int g_pool_threads = 0;           /* workers started (the caller is extra) */
static uint64_t g_pool_gen = 0;          /* bumped per dispatch */
static task_t* g_tasks = NULL;
static int g_ntasks = 0, g_next_task = 0, g_active = 0, g_busy = 0;

static void run_task(task_t* t)
{
    job_t j = *t->job;
    j.begin = t->begin;
    j.end = t->end;
    run_range(&j);
    t->mn = j.mn;
    t->mx = j.mx;
}

/* Take tasks until none is left (pool mutex held on entry and exit). */
static void drain_tasks_locked(void)
{
    while (g_next_task < g_ntasks) {
        task_t* t = &g_tasks[g_next_task++];
        pthread_mutex_unlock(&g_pool_mu);
        run_task(t);
        pthread_mutex_lock(&g_pool_mu);
    }
}

static void* pool_worker(void* arg)
{
    int index = (int)(intptr_t)arg;
    uint64_t seen = 0;
    pthread_mutex_lock(&g_pool_mu);
    for (;;) {
        while (g_pool_gen == seen) pthread_cond_wait(&g_pool_work, &g_pool_mu);
        seen = g_pool_gen;
        if (index < g_active - 1) {      /* this dispatch asked for fewer threads than the pool has */
            ++g_busy;
            drain_tasks_locked();
            if (--g_busy == 0) pthread_cond_broadcast(&g_pool_done);
        }
    }
    return NULL;
}

/* Run `ntasks` tasks on `threads` threads (the caller included). */
static void pool_run(task_t* tasks, int ntasks, int threads)
{
    if (threads < 1) threads = 1;
    if (threads > OC_MAX_THREADS) threads = OC_MAX_THREADS;
    if (threads > ntasks) threads = ntasks > 0 ? ntasks : 1;
    pthread_mutex_lock(&g_pool_mu);
    while (g_pool_threads < threads - 1) {
        pthread_t tid;
        if (pthread_create(&tid, NULL, pool_worker, (void*)(intptr_t)g_pool_threads) != 0) break;
        pthread_detach(tid);
        ++g_pool_threads;
    }
    if (threads > g_pool_threads + 1) threads = g_pool_threads + 1;
    g_tasks = tasks;
    g_ntasks = ntasks;
    g_next_task = 0;
    g_active = threads;
    g_busy = 1;                          /* the caller */
    ++g_pool_gen;
    if (threads > 1) pthread_cond_broadcast(&g_pool_work);
    drain_tasks_locked();
    --g_busy;
    while (g_busy > 0) pthread_cond_wait(&g_pool_done, &g_pool_mu);
    g_tasks = NULL;
    g_ntasks = 0;
    pthread_mutex_unlock(&g_pool_mu);
}

/* OutputMinMax << OutputMinMax (Generator.h:99-104): min with min, max with max, so a
   range whose values were all NaN (still +inf, -inf) leaves the result unchanged. */
static void merge_minmax(const task_t* tasks, int ntasks, float* minmax)
{
    float mn = INFINITY, mx = -INFINITY;
    for (int t = 0; t < ntasks; ++t) {
        if (tasks[t].begin >= tasks[t].end) continue;
        if (tasks[t].mn < mn) mn = tasks[t].mn;
        if (mx < tasks[t].mx) mx = tasks[t].mx;
    }
    if (minmax) { minmax[0] = mn; minmax[1] = mx; }
}

/* One call: `total` points cut into `threads` contiguous ranges (slabs along the
   outermost axis for grids), one task each. */
static void run_jobs(job_t* proto, int64_t total, int threads, float* minmax)
{
    if (threads < 1) threads = 1;
    if (total < 4096) threads = 1;
    if (threads > OC_MAX_THREADS) threads = OC_MAX_THREADS;
    task_t tasks[OC_MAX_THREADS];
    int64_t chunk = (total + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        int64_t b = (int64_t)t * chunk, e = b + chunk;
        tasks[t].job = proto;
        tasks[t].begin = b < total ? b : total;
        tasks[t].end = e < total ? e : total;
    }
    pthread_mutex_lock(&g_call_mu);
    pool_run(tasks, threads, threads);
    pthread_mutex_unlock(&g_call_mu);
    merge_minmax(tasks, threads, minmax);
}

OC_EXPORT void on_set_unfused(int unfused) { g_unfused = unfused; }

OC_EXPORT void on_gen_grid(const on_node* root, int dim, float* out, const float* offset, const int* count,
                           const float* step, int seed, int threads, float* minmax)
{
    job_t j;
    memset(&j, 0, sizeof j);
    j.root = root; j.kind = dim == 2 ? K_GRID2 : dim == 3 ? K_GRID3 : K_GRID4;
    j.seed = seed; j.out = out;
    int64_t total = 1;
    for (int k = 0; k < dim; ++k) {
        j.count[k] = count[k]; j.offset[k] = offset[k]; j.step[k] = step[k];
        total *= count[k] > 0 ? count[k] : 0;
    }
    run_jobs(&j, total, threads, minmax);
}

OC_EXPORT void on_gen_positions(const on_node* root, int dim, float* out, int64_t count, const float* const* pos,
                                const float* offset, int seed, int threads, float* minmax)
{
    job_t j;
    memset(&j, 0, sizeof j);
    j.root = root; j.kind = dim == 2 ? K_POS2 : dim == 3 ? K_POS3 : K_POS4;
    j.seed = seed; j.out = out;
    for (int k = 0; k < dim; ++k) { j.posarr[k] = pos[k]; j.offset[k] = offset[k]; }
    run_jobs(&j, count > 0 ? count : 0, threads, minmax);
}

OC_EXPORT void on_gen_tileable(const on_node* root, float* out, int xSize, int ySize, float xStep, float yStep,
                               int seed, int threads, float* minmax)
{
    job_t j;
    memset(&j, 0, sizeof j);
    j.root = root; j.kind = K_TILE2; j.seed = seed; j.out = out;
    j.count[0] = xSize; j.count[1] = ySize;
    const float pi2Recip = 0.15915493667f;                 /* Generator.inl:386-392 */
    float xSizePi = (float)xSize * pi2Recip;
    float ySizePi = (float)ySize * pi2Recip;
    j.tfreq[0] = xSizePi * xStep;
    j.tfreq[1] = ySizePi * yStep;
    j.tmul[0] = 1 / xSizePi;
    j.tmul[1] = 1 / ySizePi;
    int64_t total = (int64_t)(xSize > 0 ? xSize : 0) * (ySize > 0 ? ySize : 0);
    run_jobs(&j, total, threads, minmax);
}

/* A batch of requests (the product's fnGenRequest fields; kinds numbered as FN_KIND_*):
 * every request is one task, so whole requests go to threads, largest first; a request
 * of more than `split` points (split > 0) is cut into contiguous ranges of that size. */
typedef struct {
    const on_node* root;
    int kind;
    int seed;
    int count[4];
    float offset[4];
    float step[4];
    const float* positions[4];
    float* out;
    float* minmax;                       /* float[2]: the request's OutputMinMax */
} on_request;

static int64_t setup_request_job(job_t* j, const on_request* r)
{
    memset(j, 0, sizeof *j);
    j->root = r->root;
    j->kind = r->kind;
    j->seed = r->seed;
    j->out = r->out;
    int64_t total = 1;
    if (r->kind <= K_GRID4) {
        int dim = r->kind + 2;
        for (int k = 0; k < dim; ++k) {
            j->count[k] = r->count[k]; j->offset[k] = r->offset[k]; j->step[k] = r->step[k];
            total *= r->count[k] > 0 ? r->count[k] : 0;
        }
    } else if (r->kind == K_TILE2) {
        const float pi2Recip = 0.15915493667f;             /* Generator.inl:386-392 */
        j->count[0] = r->count[0]; j->count[1] = r->count[1];
        float xSizePi = (float)r->count[0] * pi2Recip;
        float ySizePi = (float)r->count[1] * pi2Recip;
        j->tfreq[0] = xSizePi * r->step[0];
        j->tfreq[1] = ySizePi * r->step[1];
        j->tmul[0] = 1 / xSizePi;
        j->tmul[1] = 1 / ySizePi;
        total = (int64_t)(r->count[0] > 0 ? r->count[0] : 0) * (r->count[1] > 0 ? r->count[1] : 0);
    } else {
        int dim = r->kind - K_POS2 + 2;
        for (int k = 0; k < dim; ++k) { j->posarr[k] = r->positions[k]; j->offset[k] = r->offset[k]; }
        total = r->count[0] > 0 ? r->count[0] : 0;
    }
    return total;
}

static int cmp_task_size_desc(const void* a, const void* b)
{
    const task_t* x = (const task_t*)a;
    const task_t* y = (const task_t*)b;
    int64_t sx = x->end - x->begin, sy = y->end - y->begin;
    return sx < sy ? 1 : sx > sy ? -1 : 0;
}

OC_EXPORT int on_gen_requests(const on_request* reqs, int n, int threads, int64_t split)
{
    if (n <= 0) return 0;
    job_t* jobs = (job_t*)malloc(sizeof(job_t) * (size_t)n);
    int64_t* totals = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
    if (!jobs || !totals) { free(jobs); free(totals); return -1; }
    int64_t ntasks = 0;
    for (int i = 0; i < n; ++i) {
        totals[i] = setup_request_job(&jobs[i], &reqs[i]);
        ntasks += (split > 0 && totals[i] > split) ? (totals[i] + split - 1) / split : 1;
    }
    task_t* tasks = (task_t*)malloc(sizeof(task_t) * (size_t)ntasks);
    if (!tasks) { free(jobs); free(totals); return -1; }
    int64_t t = 0;
    for (int i = 0; i < n; ++i) {
        int64_t piece = (split > 0 && totals[i] > split) ? split : (totals[i] > 0 ? totals[i] : 1);
        int64_t b = 0;
        do {
            tasks[t].job = &jobs[i];
            tasks[t].begin = b < totals[i] ? b : totals[i];
            tasks[t].end = b + piece < totals[i] ? b + piece : totals[i];
            tasks[t].mn = INFINITY; tasks[t].mx = -INFINITY;
            ++t;
            b += piece;
        } while (b < totals[i]);
    }
    qsort(tasks, (size_t)t, sizeof(task_t), cmp_task_size_desc);
    pthread_mutex_lock(&g_call_mu);
    pool_run(tasks, (int)t, threads);
    pthread_mutex_unlock(&g_call_mu);
    /* per request: min with min, max with max over its ranges (Generator.h:99-104) */
    for (int i = 0; i < n; ++i) { jobs[i].mn = INFINITY; jobs[i].mx = -INFINITY; }
    for (int64_t k = 0; k < t; ++k) {
        job_t* j = tasks[k].job;
        if (tasks[k].begin >= tasks[k].end) continue;
        if (tasks[k].mn < j->mn) j->mn = tasks[k].mn;
        if (j->mx < tasks[k].mx) j->mx = tasks[k].mx;
    }
    for (int i = 0; i < n; ++i)
        if (reqs[i].minmax) { reqs[i].minmax[0] = jobs[i].mn; reqs[i].minmax[1] = jobs[i].mx; }
    free(tasks); free(jobs); free(totals);
    return 0;
}

/* Open-loop serving on the host cores: request k arrives arrival_us[k] microseconds after the
 * call starts; `threads` workers take the requests in arrival order (a shared FIFO), each
 * waiting for its request's arrival, and latency_us[k] = the request's completion minus its
 * arrival.  Whole requests per worker, as an application's job system would serve them. */
typedef struct {
    const on_request* reqs;
    const double* arrival;
    double* latency;
    int n;
    int next;                            /* guarded by mu */
    pthread_mutex_t mu;
    struct timespec start;
} serve_t;

static double us_since(const struct timespec* t0)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)(t.tv_sec - t0->tv_sec) * 1e6 + (double)(t.tv_nsec - t0->tv_nsec) * 1e-3;
}

static void* serve_worker(void* arg)
{
    serve_t* sv = (serve_t*)arg;
    for (;;) {
        pthread_mutex_lock(&sv->mu);
        const int k = sv->next < sv->n ? sv->next++ : -1;
        pthread_mutex_unlock(&sv->mu);
        if (k < 0) return NULL;
        while (us_since(&sv->start) < sv->arrival[k]) {
            /* spin: arrivals are microseconds apart */
        }
        job_t j;
        const int64_t total = setup_request_job(&j, &sv->reqs[k]);
        j.begin = 0;
        j.end = total;
        run_range(&j);
        if (sv->reqs[k].minmax) {
            sv->reqs[k].minmax[0] = total > 0 ? j.mn : INFINITY;
            sv->reqs[k].minmax[1] = total > 0 ? j.mx : -INFINITY;
        }
        sv->latency[k] = us_since(&sv->start) - sv->arrival[k];
    }
}

OC_EXPORT int on_serve_paced(const on_request* reqs, int n, const double* arrival_us, int threads, double* latency_us)
{
    if (n <= 0) return 0;
    if (threads < 1) threads = 1;
    if (threads > OC_MAX_THREADS) threads = OC_MAX_THREADS;
    serve_t sv;
    sv.reqs = reqs;
    sv.arrival = arrival_us;
    sv.latency = latency_us;
    sv.n = n;
    sv.next = 0;
    pthread_mutex_init(&sv.mu, NULL);
    pthread_t tid[OC_MAX_THREADS];
    clock_gettime(CLOCK_MONOTONIC, &sv.start);
    int started = 0;
    for (int t = 0; t < threads; ++t)
        if (pthread_create(&tid[t], NULL, serve_worker, &sv) == 0) ++started;
    if (started == 0) serve_worker(&sv);
    for (int t = 0; t < started; ++t) pthread_join(tid[t], NULL);
    pthread_mutex_destroy(&sv.mu);
    return 0;
}

OC_EXPORT float on_gen_single(const on_node* root, int dim, const float* pos, int seed)
{
    f32 p[4] = {pos[0], pos[1], dim > 2 ? pos[2] : 0.0f, dim > 3 ? pos[3] : 0.0f};
    return (float)eval_node(root, seed, dim, p);
}

#ifdef OC_COUNT
OC_EXPORT double on_count_ops(const on_node* root, int dim, const float* pos, int seed)
{
    oc_counter = 0;
    f32 p[4] = {pos[0], pos[1], dim > 2 ? pos[2] : 0.0f, dim > 3 ? pos[3] : 0.0f};
    (void)eval_node(root, seed, dim, p);
    return (double)oc_counter;
}
#endif
