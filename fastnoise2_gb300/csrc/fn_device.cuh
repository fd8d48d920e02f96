// fn_device.cuh -- FastNoise2 node math for sm_103a.
//
// Device-side restatement of the node generators in
// include/FastNoise/Generators/*.inl (FastNoise2 v1.1.1).  Every function here
// evaluates ONE point in registers; the interpreter kernel (fn_kernels.cu) and
// the run-time specialised kernels (fn_jit.cpp) both call them.
//
// Arithmetic contract (matches the reference's strict-FP build):
//   * the whole translation unit is compiled with -fmad=false, so a*b+c is a
//     multiply and an add; FS::FMulAdd / FNMulAdd / FMulSub become fmaf();
//   * FS::Convert<int32> rounds to nearest-even and returns INT_MIN for NaN or
//     |x| >= 2^31 (x86 cvtps2dq);
//   * FS::Min(a,b)=a<b?a:b, FS::Max(a,b)=a>b?a:b (minps/maxps operand order);
//   * InvSqrt / Reciprocal / Sqrt / division are the correctly rounded IEEE ops;
//   * Sin / Cos / Pow use the project's own polynomial kernels below, shared
//     bit-for-bit with the CPU restatement used for testing.
#pragma once

#ifndef FN_DEVICE_NO_STDINT
#include <stdint.h>
#endif

#define FND __device__ __forceinline__

namespace fnd {

constexpr int kPrimeX = (int)0xF797C5C7;   // Utils.inl:8-11
constexpr int kPrimeY = (int)0x6C060C89;
constexpr int kPrimeZ = (int)0x465FD04F;
constexpr int kPrimeW = (int)0xF7A62279;
constexpr int kHashA = (int)0xB7E0A5F5;     // Utils.inl:18

constexpr double kRoot2 = 1.4142135623730950488016887242097;
constexpr double kRoot3 = 1.7320508075688772935274463415059;
constexpr double kRoot5 = 2.2360679774997896964091736687313;
constexpr float kValueBounds = 2147483648.f;

// ---------------------------------------------------------------- primitives

FND float fmin_(float a, float b) { return a < b ? a : b; }
FND float fmax_(float a, float b) { return a > b ? a : b; }
// The simplex-family falloffs clamp with fmaxf(v, 0.0f) / fminf(v, 0.0f) (one min/max
// instruction): there the clamped value is only ever raised to an even power, so the one case
// where these differ from FS::Max / FS::Min against 0 (the sign of a zero) cannot show, and a
// NaN becomes 0 in both.
FND float fabs_(float a) { return __int_as_float(__float_as_int(a) & 0x7FFFFFFF); }
FND float flip(float v, int s) { return __int_as_float(__float_as_int(v) ^ (s & (int)0x80000000)); }
FND float flipm(float v, bool m) { return m ? __int_as_float(__float_as_int(v) ^ (int)0x80000000) : v; }
FND int cvti(float x)
{
    // cvt.rni saturates: below -2^31 (and -inf) it already gives INT_MIN, as x86 does; at or
    // above 2^31 and for NaN the comparison fails and INT_MIN is substituted.
    int r = __float2int_rn(x);
    return x < 2147483648.0f ? r : (int)0x80000000;
}
FND float cvtf(int i) { return __int2float_rn(i); }
FND unsigned srl(int a, int s) { return (unsigned)a >> s; }
FND int imul(int a, int b) { return (int)((unsigned)a * (unsigned)b); }
FND int iadd(int a, int b) { return (int)((unsigned)a + (unsigned)b); }
FND float invsqrt(float x) { return 1.0f / sqrtf(x); }

FND int hash_mix(int v) { int h = imul(v, kHashA); return (h >> 15) ^ h; }
FND int hash(int seed, int a, int b) { int h = imul(seed ^ a ^ b, kHashA); return (h >> 15) ^ h; }
FND int hash(int seed, int a, int b, int c) { int h = imul(seed ^ a ^ b ^ c, kHashA); return (h >> 15) ^ h; }
FND int hash(int seed, int a, int b, int c, int d) { int h = imul(seed ^ a ^ b ^ c ^ d, kHashA); return (h >> 15) ^ h; }
FND int hashhb(int seed, int a, int b) { return imul(seed ^ a ^ b, kHashA); }
FND int hashhb(int seed, int a, int b, int c) { return imul(seed ^ a ^ b ^ c, kHashA); }
FND int hashhb(int seed, int a, int b, int c, int d) { return imul(seed ^ a ^ b ^ c ^ d, kHashA); }
FND float valcoord(int h) { return cvtf(imul(h, imul(h, kHashA))); }   // Utils.inl:243-250

FND float lerp(float a, float b, float t) { return fmaf(t, b - a, a); }
FND float hermite(float t) { return t * t * fmaf(-t, 2.0f, 3.0f); }
FND float quintic(float t) { return t * t * t * fmaf(t, fmaf(t, 6.0f, -15.0f), 10.0f); }

// GetGradientDotCommon, portable branch (Utils.inl:132-158)
FND float grad3(int h, float x, float y, float z)
{
    // h & 13 > 7: bit 3;  h & 13 == 12: bits 3, 2 set, bit 0 clear;  h & 13 < 2: bits 3, 2 clear
    const bool b3 = (h & 8) != 0, b2 = (h & 4) != 0, x_case = (h & 9) == 8;
    const float u = b3 ? y : x;
    const float v = b2 ? (x_case ? x : z) : (b3 ? z : y);
    return flip(u, h << 31) + flip(v, h << 30);
}
// GetGradientDotPerlin 2D, portable branch (Utils.inl:181-190)
FND float grad2(int h, float x, float y)
{
    x = flip(x, h << 31);
    y = flip(y, h << 30);
    bool s = (h << 29) < 0;
    return fmaf(1.0f + (float)kRoot2, s ? y : x, s ? x : y);
}
// GetGradientDotPerlin 4D, portable branch (Utils.inl:205-218)
FND float grad4(int h, float x, float y, float z, float w)
{
    // h & 24 > 0: bit 3 or 4;  (h << 27) < 0: bit 4;  h & 24 > 16: bits 3 and 4
    const bool any34 = (h & 24) != 0, b4 = (h & 16) != 0, both34 = (h & 24) == 24;
    const float a = any34 ? x : y;
    const float b = b4 ? y : z;
    const float c = both34 ? z : w;
    return (flip(a, h << 31) + flip(b, h << 30)) + flip(c, h << 29);
}

// Sin / Cos: Cody-Waite reduction by pi/2 (three-part constant), Taylor
// polynomials on [-pi/4, pi/4] evaluated by Horner with fmaf.
FND float sc_reduce(float x, int& q)
{
    float k = rintf(x * 0x1.45f306p-1f);
    float r = fmaf(-k, 0x1.921fb6p+0f, x);
    r = fmaf(-k, -0x1.777a5cp-25f, r);
    r = fmaf(-k, -0x1.ee59dap-50f, r);
    q = (int)(long long)k & 3;
    return r;
}
FND float sin_poly(float r)
{
    float r2 = r * r;
    float p = fmaf(r2, -0x1.ae6456p-26f, 0x1.71de3ap-19f);
    p = fmaf(r2, p, -0x1.a01a02p-13f);
    p = fmaf(r2, p, 0x1.111112p-7f);
    p = fmaf(r2, p, -0x1.555556p-3f);
    return fmaf(r * r2, p, r);
}
FND float cos_poly(float r)
{
    float r2 = r * r;
    float p = fmaf(r2, 0x1.1eed8ep-29f, -0x1.27e4fcp-22f);
    p = fmaf(r2, p, 0x1.a01a02p-16f);
    p = fmaf(r2, p, -0x1.6c16c2p-10f);
    p = fmaf(r2, p, 0x1.555556p-5f);
    p = fmaf(r2, p, -0.5f);
    return fmaf(r2, p, 1.0f);
}
FND float sin_(float x)
{
    int q;
    float r = sc_reduce(x, q);
    float s = (q & 1) ? cos_poly(r) : sin_poly(r);
    return (q & 2) ? -s : s;
}
FND float cos_(float x)
{
    int q;
    float r = sc_reduce(x, q);
    float c = (q & 1) ? sin_poly(r) : cos_poly(r);
    return ((q + 1) & 2) ? -c : c;
}

// Pow for the strict build: 2^(y*log2 x), log2 via the atanh series on
// m in [sqrt(1/2), sqrt(2)), exp2 via a nearest-integer split.
FND float log2_pos(float x)
{
    unsigned u = __float_as_uint(x);
    int e = (int)((u >> 23) & 0xFF);
    if (e == 0) { x *= 0x1p23f; u = __float_as_uint(x); e = (int)((u >> 23) & 0xFF) - 23; }
    int ex = e - 127;
    float m = __uint_as_float((u & 0x007FFFFFu) | 0x3F800000u);
    if (m > 1.41421356f) { m *= 0.5f; ex += 1; }
    float s = (m - 1.0f) / (m + 1.0f);
    float s2 = s * s;
    float p = fmaf(s2, 0x1.745d18p-4f, 0x1.c71c72p-4f);
    p = fmaf(s2, p, 0x1.24924ap-3f);
    p = fmaf(s2, p, 0x1.99999ap-3f);
    p = fmaf(s2, p, 0x1.555556p-2f);
    p = fmaf(s2, p, 1.0f);
    float ln = 2.0f * s * p;
    return fmaf(ln, 0x1.715476p+0f, (float)ex);
}
FND float exp2_any(float t)
{
    if (!(t < 128.0f)) return (t != t) ? t : __int_as_float(0x7F800000);
    if (t < -150.0f) return 0.0f;
    float n = rintf(t);
    float f = t - n;
    float a = f * 0x1.62e430p-1f;
    float p = fmaf(a, 0x1.a01a02p-13f, 0x1.6c16c2p-10f);
    p = fmaf(a, p, 0x1.111112p-7f);
    p = fmaf(a, p, 0x1.555556p-5f);
    p = fmaf(a, p, 0x1.555556p-3f);
    p = fmaf(a, p, 0.5f);
    p = fmaf(a, p, 1.0f);
    p = fmaf(a, p, 1.0f);
    int ni = (int)n;
    int n1 = ni / 2, n2 = ni - n1;
    return p * __uint_as_float((unsigned)(n1 + 127) << 23) * __uint_as_float((unsigned)(n2 + 127) << 23);
}
FND float pow_(float x, float y)
{
    if (y == 0.0f) return 1.0f;
    if (x != x || y != y) return x + y;
    if (x == 0.0f) return y > 0.0f ? 0.0f : __int_as_float(0x7F800000);
    if (x < 0.0f) return __int_as_float(0x7FC00000);
    if (x == __int_as_float(0x7F800000)) return y > 0.0f ? x : 0.0f;
    return exp2_any(y * log2_pos(x));
}
FND float mod_(float a, float b) { return a - truncf(a / b) * b; }

// VariableRange::ScaleOutput (BasicGenerators.inl:27-30); mul = (1/(max-min))*rangeScale
FND float scale_out(float v, float nmin, float mul, float rmin) { return fmaf(mul, v - nmin, rmin); }

// ---------------------------------------------------------------- Simplex

FND float simplex2(int seed, float x, float y)
{
    constexpr double kSkew2 = 1.0 / (kRoot3 + 1.0);
    constexpr double kUnskew2 = -1.0 / (kRoot3 + 3.0);
    float skewDelta = (float)kSkew2 * (x + y);
    float xs = x + skewDelta, ys = y + skewDelta;
    float xb = floorf(xs), yb = floorf(ys);
    float dxs = xs - xb, dys = ys - yb;
    int xp = imul(cvti(xb), kPrimeX), yp = imul(cvti(yb), kPrimeY);
    bool xgey = dxs >= dys;
    float unskew = (float)kUnskew2 * (dxs + dys);
    float dx0 = dxs + unskew, dy0 = dys + unskew;
    float dx1 = (xgey ? dx0 : dx0 + 1.0f) - (float)(kUnskew2 + 1);
    float dy1 = (xgey ? dy0 + 1.0f : dy0) - (float)(kUnskew2 + 1);
    float dx2 = dx0 - (float)(kUnskew2 * 2 + 1);
    float dy2 = dy0 - (float)(kUnskew2 * 2 + 1);
    float f0 = fmaf(-dx0, dx0, fmaf(-dy0, dy0, 0.5f));
    float f1 = fmaf(-dx1, dx1, fmaf(-dy1, dy1, 0.5f));
    float f2 = f0 + fmaf(unskew, (float)(-4.0 * (kRoot3 + 2.0) / (kRoot3 + 3.0)), (float)(-2.0 / 3.0));
    f0 = fmaxf(f0, 0.0f); f1 = fmaxf(f1, 0.0f); f2 = fmaxf(f2, 0.0f);
    f0 *= f0; f0 *= f0; f1 *= f1; f1 *= f1; f2 *= f2; f2 *= f2;
    float g0 = grad2(hash(seed, xp, yp), dx0, dy0);
    float g1 = grad2(hash(seed, xgey ? iadd(xp, kPrimeX) : xp, xgey ? yp : iadd(yp, kPrimeY)), dx1, dy1);
    float g2 = grad2(hash(seed, iadd(xp, kPrimeX), iadd(yp, kPrimeY)), dx2, dy2);
    return fmaf(g0, f0, fmaf(g1, f1, g2 * f2));
}

FND float simplex3(int seed, float x, float y, float z)
{
    constexpr double kReflect = -1.0 / 2.0;
    float skewDelta = (float)(1.0 / 3.0) * (x + y + z);
    float xs = x + skewDelta, ys = y + skewDelta, zs = z + skewDelta;
    float xb = floorf(xs), yb = floorf(ys), zb = floorf(zs);
    float dxs = xs - xb, dys = ys - yb, dzs = zs - zb;
    int xp = imul(cvti(xb), kPrimeX), yp = imul(cvti(yb), kPrimeY), zp = imul(cvti(zb), kPrimeZ);
    bool xgey = dxs >= dys, ygez = dys >= dzs, xgez = dxs >= dzs;
    float unskew = (float)kReflect * (dxs + dys + dzs);
    float dx0 = dxs + unskew, dy0 = dys + unskew, dz0 = dzs + unskew;
    bool mx1 = xgey && xgez, my1 = ygez && !xgey, mz1 = xgez || ygez;
    bool nx2 = xgey || xgez, ny2 = xgey && !ygez, nz2 = xgez && ygez;
    constexpr float c3 = (float)(kReflect * 3 + 1);
    float dx3 = dx0 - c3, dy3 = dy0 - c3, dz3 = dz0 - c3;
    float dx1 = mx1 ? dx3 - 1.0f : dx3;
    float dy1 = my1 ? dy3 - 1.0f : dy3;
    float dz1 = mz1 ? dz3 : dz3 - 1.0f;
    float dx2 = nx2 ? dx0 : dx0 + 1.0f;
    float dy2 = ny2 ? dy0 + 1.0f : dy0;
    float dz2 = nz2 ? dz0 + 1.0f : dz0;
    constexpr float R = (float)0.6;
    float f0 = fmaf(-dz0, dz0, fmaf(-dy0, dy0, fmaf(-dx0, dx0, R)));
    float f1 = fmaf(-dz1, dz1, fmaf(-dy1, dy1, fmaf(-dx1, dx1, R)));
    float f2 = fmaf(-dz2, dz2, fmaf(-dy2, dy2, fmaf(-dx2, dx2, R)));
    float f3 = f0 - (unskew + (float)(3.0 / 4.0));
    f0 = fmaxf(f0, 0.0f); f1 = fmaxf(f1, 0.0f); f2 = fmaxf(f2, 0.0f); f3 = fmaxf(f3, 0.0f);
    f0 *= f0; f0 *= f0; f1 *= f1; f1 *= f1; f2 *= f2; f2 *= f2; f3 *= f3; f3 *= f3;
    float g0 = grad3(hash(seed, xp, yp, zp), dx0, dy0, dz0);
    float g1 = grad3(hash(seed, mx1 ? iadd(xp, kPrimeX) : xp, my1 ? iadd(yp, kPrimeY) : yp, mz1 ? zp : iadd(zp, kPrimeZ)), dx1, dy1, dz1);
    float g2 = grad3(hash(seed, nx2 ? iadd(xp, kPrimeX) : xp, ny2 ? yp : iadd(yp, kPrimeY), nz2 ? zp : iadd(zp, kPrimeZ)), dx2, dy2, dz2);
    float g3 = grad3(hash(seed, iadd(xp, kPrimeX), iadd(yp, kPrimeY), iadd(zp, kPrimeZ)), dx3, dy3, dz3);
    return fmaf(g3, f3, fmaf(g2, f2, fmaf(g1, f1, g0 * f0)));
}

FND float simplex4(int seed, float x, float y, float z, float w)
{
    constexpr double kSkew4 = 1.0 / (kRoot5 + 1.0);
    constexpr double kUnskew4 = -1.0 / (kRoot5 + 5.0);
    float skewDelta = (float)kSkew4 * (x + y + z + w);
    float xs = x + skewDelta, ys = y + skewDelta, zs = z + skewDelta, ws = w + skewDelta;
    float xb = floorf(xs), yb = floorf(ys), zb = floorf(zs), wb = floorf(ws);
    float dxs = xs - xb, dys = ys - yb, dzs = zs - zb, dws = ws - wb;
    int xp = imul(cvti(xb), kPrimeX), yp = imul(cvti(yb), kPrimeY), zp = imul(cvti(zb), kPrimeZ), wp = imul(cvti(wb), kPrimeW);
    float unskew = (float)kUnskew4 * (dxs + dys + dzs + dws);
    float dx0 = dxs + unskew, dy0 = dys + unskew, dz0 = dzs + unskew, dw0 = dws + unskew;
    int rx = 0, ry = 0, rz = 0, rw = 0;
    if (dx0 >= dy0) rx++; else ry++;
    if (dx0 >= dz0) rx++; else rz++;
    if (dx0 >= dw0) rx++; else rw++;
    if (dy0 >= dz0) ry++; else rz++;
    if (dy0 >= dw0) ry++; else rw++;
    if (dz0 >= dw0) rz++; else rw++;
    constexpr float u1 = (float)kUnskew4, u2 = (float)(kUnskew4 * 2), u3 = (float)(kUnskew4 * 3), u4 = (float)(kUnskew4 * 4 + 1);
    float dx1 = (rx > 2 ? dx0 - 1.0f : dx0) - u1, dy1 = (ry > 2 ? dy0 - 1.0f : dy0) - u1;
    float dz1 = (rz > 2 ? dz0 - 1.0f : dz0) - u1, dw1 = (rw > 2 ? dw0 - 1.0f : dw0) - u1;
    float dx2 = (rx > 1 ? dx0 - 1.0f : dx0) - u2, dy2 = (ry > 1 ? dy0 - 1.0f : dy0) - u2;
    float dz2 = (rz > 1 ? dz0 - 1.0f : dz0) - u2, dw2 = (rw > 1 ? dw0 - 1.0f : dw0) - u2;
    float dx3 = (rx > 0 ? dx0 - 1.0f : dx0) - u3, dy3 = (ry > 0 ? dy0 - 1.0f : dy0) - u3;
    float dz3 = (rz > 0 ? dz0 - 1.0f : dz0) - u3, dw3 = (rw > 0 ? dw0 - 1.0f : dw0) - u3;
    float dx4 = dx0 - u4, dy4 = dy0 - u4, dz4 = dz0 - u4, dw4 = dw0 - u4;
    constexpr float R = (float)0.6;
    float f0 = fmaf(-dw0, dw0, fmaf(-dz0, dz0, fmaf(-dy0, dy0, fmaf(-dx0, dx0, R))));
    float f1 = fmaf(-dw1, dw1, fmaf(-dz1, dz1, fmaf(-dy1, dy1, fmaf(-dx1, dx1, R))));
    float f2 = fmaf(-dw2, dw2, fmaf(-dz2, dz2, fmaf(-dy2, dy2, fmaf(-dx2, dx2, R))));
    float f3 = fmaf(-dw3, dw3, fmaf(-dz3, dz3, fmaf(-dy3, dy3, fmaf(-dx3, dx3, R))));
    float f4 = f0 + fmaf(unskew, (float)(-4.0 * (kRoot5 + 3.0) / (kRoot5 + 5.0)), (float)(-4.0 / 5.0));
    f0 = fmaxf(f0, 0.0f); f1 = fmaxf(f1, 0.0f); f2 = fmaxf(f2, 0.0f); f3 = fmaxf(f3, 0.0f); f4 = fmaxf(f4, 0.0f);
    f0 *= f0; f0 *= f0; f1 *= f1; f1 *= f1; f2 *= f2; f2 *= f2; f3 *= f3; f3 *= f3; f4 *= f4; f4 *= f4;
    float g0 = grad4(hash(seed, xp, yp, zp, wp), dx0, dy0, dz0, dw0);
    float g1 = grad4(hash(seed, rx > 2 ? iadd(xp, kPrimeX) : xp, ry > 2 ? iadd(yp, kPrimeY) : yp, rz > 2 ? iadd(zp, kPrimeZ) : zp, rw > 2 ? iadd(wp, kPrimeW) : wp), dx1, dy1, dz1, dw1);
    float g2 = grad4(hash(seed, rx > 1 ? iadd(xp, kPrimeX) : xp, ry > 1 ? iadd(yp, kPrimeY) : yp, rz > 1 ? iadd(zp, kPrimeZ) : zp, rw > 1 ? iadd(wp, kPrimeW) : wp), dx2, dy2, dz2, dw2);
    float g3 = grad4(hash(seed, rx > 0 ? iadd(xp, kPrimeX) : xp, ry > 0 ? iadd(yp, kPrimeY) : yp, rz > 0 ? iadd(zp, kPrimeZ) : zp, rw > 0 ? iadd(wp, kPrimeW) : wp), dx3, dy3, dz3, dw3);
    float g4 = grad4(hash(seed, iadd(xp, kPrimeX), iadd(yp, kPrimeY), iadd(zp, kPrimeZ), iadd(wp, kPrimeW)), dx4, dy4, dz4, dw4);
    return fmaf(g0, f0, fmaf(g1, f1, fmaf(g2, f2, fmaf(g3, f3, g4 * f4))));
}

// ---------------------------------------------------------------- SuperSimplex (OpenSimplex2S)

FND float supersimplex2(int seed, float x, float y)
{
    constexpr double kSkew2 = 1.0 / (kRoot3 + 1.0);
    constexpr double kUnskew2 = -1.0 / (kRoot3 + 3.0);
    constexpr float R = (float)(2.0 / 3.0);
    float skewDelta = (float)kSkew2 * (x + y);
    float xs = x + skewDelta, ys = y + skewDelta;
    float xb = floorf(xs), yb = floorf(ys);
    float dxs = xs - xb, dys = ys - yb;
    int xp = imul(cvti(xb), kPrimeX), yp = imul(cvti(yb), kPrimeY);
    bool fxy = dxs + dys > 1.0f;
    float boundary = fxy ? -1.0f : 0.0f;
    bool fx = fmaf(dxs, -2.0f, dys) < boundary;
    bool fy = fmaf(dys, -2.0f, dxs) < boundary;
    float unskew = (float)kUnskew2 * (dxs + dys);
    float dxb = dxs + unskew, dyb = dys + unskew;
    float fb0 = fmaf(-dxb, dxb, fmaf(-dyb, dyb, R));
    float value;
    {
        float g = grad2(hash(seed, xp, yp), dxb, dyb);
        float f = fb0; f *= f; f *= f;
        value = f * g;
    }
    {
        float g = grad2(hash(seed, iadd(xp, kPrimeX), iadd(yp, kPrimeY)), dxb - (float)(2 * kUnskew2 + 1), dyb - (float)(2 * kUnskew2 + 1));
        float f = fmaf(unskew, (float)(-4.0 * (kRoot3 + 2.0) / (kRoot3 + 3.0)), fb0 - R);
        f *= f; f *= f;
        value = fmaf(f, g, value);
    }
    float xyd = fxy ? (float)(kUnskew2 + 1) : (float)(-kUnskew2);
    dxb = dxb - xyd;
    dyb = dyb - xyd;
    {
        int xa = fx ? iadd(xp, (int)((unsigned)kPrimeX * 2u)) : xp;
        int h = hash(seed, fxy ? xa : iadd(xa, -kPrimeX), fxy ? iadd(yp, kPrimeY) : yp);
        float dx = dxb - (fx ? (float)(1 + 2 * kUnskew2) : -1.0f);
        float dy = fx ? dyb - (float)(2 * kUnskew2) : dyb;
        float g = grad2(h, dx, dy);
        float f = fmaxf(fmaf(-dx, dx, fmaf(-dy, dy, R)), 0.0f);
        f *= f; f *= f;
        value = fmaf(f, g, value);
    }
    {
        int ya = fy ? iadd(yp, (int)((unsigned)kPrimeY * 2u)) : yp;
        int h = hash(seed, fxy ? iadd(xp, kPrimeX) : xp, fxy ? ya : iadd(ya, -kPrimeY));
        float dx = fy ? dxb - (float)(2 * kUnskew2) : dxb;
        float dy = dyb - (fy ? (float)(1 + 2 * kUnskew2) : -1.0f);
        float g = grad2(h, dx, dy);
        float f = fmaxf(fmaf(-dx, dx, fmaf(-dy, dy, R)), 0.0f);
        f *= f; f *= f;
        value = fmaf(f, g, value);
    }
    return value;
}

FND void ss_consider(float& maxScore, int& bits, float score, int b)
{
    bits = score > maxScore ? b : bits;
    maxScore = fmax_(maxScore, score);
}

FND float supersimplex3(int seed, float x, float y, float z)
{
    constexpr double kReflect = -1.0 / 2.0;
    constexpr double kTwice = -1.0 / 4.0;
    constexpr double kDA = 3.0 / 4.0, kDB = 1.0;
    float skewDelta = (float)(1.0 / 3.0) * (x + y + z);
    float xs = x + skewDelta, ys = y + skewDelta, zs = z + skewDelta;
    float xb = floorf(xs), yb = floorf(ys), zb = floorf(zs);
    float dxs = xs - xb, dys = ys - yb, dzs = zs - zb;
    {
        float t = (float)kTwice * (dxs + dys + dzs);
        float xn = dxs + t, yn = dys + t, zn = dzs + t, xyzn = -t;
        float maxScore = 0.375f;
        int bits = xyzn > maxScore ? -1 : 0;
        maxScore = fmax_(maxScore, xyzn);
        ss_consider(maxScore, bits, xn, 1);
        ss_consider(maxScore, bits, yn, 2);
        ss_consider(maxScore, bits, zn, 4);
        maxScore += 0.125f - xyzn;
        ss_consider(maxScore, bits, -zn, 3);
        ss_consider(maxScore, bits, -yn, 5);
        ss_consider(maxScore, bits, -xn, 6);
        if (bits & 1) { xb += 1.0f; dxs -= 1.0f; }
        if (bits & 2) { yb += 1.0f; dys -= 1.0f; }
        if (bits & 4) { zb += 1.0f; dzs -= 1.0f; }
    }
    int xp = imul(cvti(xb), kPrimeX), yp = imul(cvti(yb), kPrimeY), zp = imul(cvti(zb), kPrimeZ);
    float sum = dxs + dys + dzs;
    float t = (float)kTwice * sum;
    float xn = dxs + t, yn = dys + t, zn = dzs + t, xyzn = -t;
    float unskew = (float)kReflect * sum;
    float dx = dxs + unskew, dy = dys + unskew, dz = dzs + unskew;
    float cs = (float)(1 + 3 * kReflect) * sum;
    float value, stemA, stemB;
    {
        float g = grad3(hash(seed, xp, yp, zp), dx, dy, dz);
        float fb = fmaf(-dz, dz, fmaf(-dy, dy, fmaf(-dx, dx, (float)kDA))) * 0.5f;
        stemA = fb - (float)(kDA * 0.5);
        stemB = fb - (float)(kDB * 0.5);
        value = (fb * fb) * (fb * fb) * g;
    }
    {
        bool m = xyzn < 0.0f;
        float off = flipm((float)(3 * kReflect + 1), m);
        float g = grad3(hash(seed, iadd(xp, m ? -kPrimeX : kPrimeX), iadd(yp, m ? -kPrimeY : kPrimeY), iadd(zp, m ? -kPrimeZ : kPrimeZ)), dx - off, dy - off, dz - off);
        float fb = fmaxf(fmaf(off, cs, stemA), 0.0f);
        value = fmaf((fb * fb) * (fb * fb), g, value);
    }
    {
        bool m = xyzn < zn;
        float o0 = flipm((float)(2 * kReflect), m);
        float g = grad3(hash(seed, iadd(xp, m ? -kPrimeX : kPrimeX), iadd(yp, m ? -kPrimeY : kPrimeY), zp), dx, dy, dz - o0);
        float fb = fminf(flipm(dz, m) - stemB, 0.0f);
        value = fmaf((fb * fb) * (fb * fb), g, value);
    }
    {
        bool m = xyzn < yn;
        float o0 = flipm((float)(2 * kReflect), m);
        float g = grad3(hash(seed, iadd(xp, m ? -kPrimeX : kPrimeX), yp, iadd(zp, m ? -kPrimeZ : kPrimeZ)), dx, dy - o0, dz);
        float fb = fminf(flipm(dy, m) - stemB, 0.0f);
        value = fmaf((fb * fb) * (fb * fb), g, value);
    }
    {
        bool m = xyzn < xn;
        float o0 = flipm((float)(2 * kReflect), m);
        float g = grad3(hash(seed, xp, iadd(yp, m ? -kPrimeY : kPrimeY), iadd(zp, m ? -kPrimeZ : kPrimeZ)), dx - o0, dy, dz);
        float fb = fminf(flipm(dx, m) - stemB, 0.0f);
        value = fmaf((fb * fb) * (fb * fb), g, value);
    }
    {
        bool m = xn < 0.0f;
        float o0 = flipm((float)kReflect, m);
        float g = grad3(hash(seed, iadd(xp, m ? -kPrimeX : kPrimeX), yp, zp), dx + o0, dy - o0, dz - o0);
        float fb = fmaxf(fmaf(o0, cs, stemA) + flipm(dx, m), 0.0f);
        value = fmaf((fb * fb) * (fb * fb), g, value);
    }
    {
        bool m = yn < 0.0f;
        float o0 = flipm((float)kReflect, m);
        float g = grad3(hash(seed, xp, iadd(yp, m ? -kPrimeY : kPrimeY), zp), dx - o0, dy + o0, dz - o0);
        float fb = fmaxf(fmaf(o0, cs, stemA) + flipm(dy, m), 0.0f);
        value = fmaf((fb * fb) * (fb * fb), g, value);
    }
    {
        bool m = zn < 0.0f;
        float o0 = flipm((float)kReflect, m);
        float g = grad3(hash(seed, xp, yp, iadd(zp, m ? -kPrimeZ : kPrimeZ)), dx - o0, dy - o0, dz + o0);
        float fb = fmaxf(fmaf(o0, cs, stemA) + flipm(dz, m), 0.0f);
        value = fmaf((fb * fb) * (fb * fb), g, value);
    }
    return value;
}

FND float supersimplex4(int seed, float x, float y, float z, float w)
{
    constexpr double kSkew4 = 1.0 / (kRoot5 + 1.0);
    constexpr double kU = -1.0 / (kRoot5 + 5.0);
    constexpr double kTwice = -1.0 / 5.0;
    constexpr double kDA = 4.0 / 5.0, kDB = 6.0 / 5.0;
    float skewDelta = (float)kSkew4 * (x + y + z + w);
    float xs = x + skewDelta, ys = y + skewDelta, zs = z + skewDelta, ws = w + skewDelta;
    float xb = floorf(xs), yb = floorf(ys), zb = floorf(zs), wb = floorf(ws);
    float dxs = xs - xb, dys = ys - yb, dzs = zs - zb, dws = ws - wb;
    {
        float t = (float)kTwice * (dxs + dys + dzs + dws);
        float xn = dxs + t, yn = dys + t, zn = dzs + t, wn = dws + t, xyzwn = -t;
        float ms = 0.6f - xyzwn;
        int bits = 0.2f > ms ? -1 : 0;
        ms = fmax_(ms, 0.2f);
        ss_consider(ms, bits, -wn, 7);
        ss_consider(ms, bits, -zn, 11);
        ss_consider(ms, bits, -yn, 13);
        ss_consider(ms, bits, -xn, 14);
        ms += xyzwn - 0.2f;
        ss_consider(ms, bits, xn, 1);
        ss_consider(ms, bits, yn, 2);
        ss_consider(ms, bits, zn, 4);
        ss_consider(ms, bits, wn, 8);
        ms += 0.2f - xn;
        ss_consider(ms, bits, yn, 3);
        ss_consider(ms, bits, zn, 5);
        ss_consider(ms, bits, wn, 9);
        ms += xn;
        ss_consider(ms, bits, yn + zn, 6);
        ms -= wn;
        ss_consider(ms, bits, yn, 10);
        ss_consider(ms, bits, zn, 12);
        if (bits & 1) { xb += 1.0f; dxs -= 1.0f; }
        if (bits & 2) { yb += 1.0f; dys -= 1.0f; }
        if (bits & 4) { zb += 1.0f; dzs -= 1.0f; }
        if (bits & 8) { wb += 1.0f; dws -= 1.0f; }
    }
    int xp = imul(cvti(xb), kPrimeX), yp = imul(cvti(yb), kPrimeY), zp = imul(cvti(zb), kPrimeZ), wp = imul(cvti(wb), kPrimeW);
    float sum = dxs + dys + dzs + dws;
    float t = (float)kTwice * sum;
    float xn = dxs + t, yn = dys + t, zn = dzs + t, wn = dws + t, xyzwn = -t;
    float ud = (float)kU * sum;
    float dx = dxs + ud, dy = dys + ud, dz = dzs + ud, dw = dws + ud;
    float cs = (float)(1 + 4 * kU) * sum;
    float value, stemA, stemB;
    {
        float g = grad4(hash(seed, xp, yp, zp, wp), dx, dy, dz, dw);
        float fb = fmaf(-dw, dw, fmaf(-dz, dz, fmaf(-dy, dy, fmaf(-dx, dx, (float)kDA)))) * 0.5f;
        stemA = fb - (float)(kDA * 0.5);
        stemB = fb - (float)(kDB * 0.5);
        value = (fb * fb) * (fb * fb) * g;
    }
#define FND_P(m, base, P) iadd(base, (m) ? -(P) : (P))
#define FND_ACC(fbexpr, gexpr) { float g_ = (gexpr); float fb_ = fmaxf((fbexpr), 0.0f); value = fmaf((fb_ * fb_) * (fb_ * fb_), g_, value); }
    {
        bool m = xyzwn < 0.0f;
        float o = flipm((float)(4 * kU + 1), m);
        FND_ACC(fmaf(o, cs, stemA), grad4(hash(seed, FND_P(m, xp, kPrimeX), FND_P(m, yp, kPrimeY), FND_P(m, zp, kPrimeZ), FND_P(m, wp, kPrimeW)), dx - o, dy - o, dz - o, dw - o));
    }
    {
        bool m = xyzwn < wn;
        float o1 = flipm((float)(3 * kU + 1), m), o0 = flipm((float)(3 * kU), m);
        FND_ACC(fmaf(o1, cs, stemB) - flipm(dw, m), grad4(hash(seed, FND_P(m, xp, kPrimeX), FND_P(m, yp, kPrimeY), FND_P(m, zp, kPrimeZ), wp), dx - o1, dy - o1, dz - o1, dw - o0));
    }
    {
        bool m = xyzwn < zn;
        float o1 = flipm((float)(3 * kU + 1), m), o0 = flipm((float)(3 * kU), m);
        FND_ACC(fmaf(o1, cs, stemB) - flipm(dz, m), grad4(hash(seed, FND_P(m, xp, kPrimeX), FND_P(m, yp, kPrimeY), zp, FND_P(m, wp, kPrimeW)), dx - o1, dy - o1, dz - o0, dw - o1));
    }
    {
        bool m = xyzwn < yn;
        float o1 = flipm((float)(3 * kU + 1), m), o0 = flipm((float)(3 * kU), m);
        FND_ACC(fmaf(o1, cs, stemB) - flipm(dy, m), grad4(hash(seed, FND_P(m, xp, kPrimeX), yp, FND_P(m, zp, kPrimeZ), FND_P(m, wp, kPrimeW)), dx - o1, dy - o0, dz - o1, dw - o1));
    }
    {
        bool m = xyzwn < xn;
        float o1 = flipm((float)(3 * kU + 1), m), o0 = flipm((float)(3 * kU), m);
        FND_ACC(fmaf(o1, cs, stemB) - flipm(dx, m), grad4(hash(seed, xp, FND_P(m, yp, kPrimeY), FND_P(m, zp, kPrimeZ), FND_P(m, wp, kPrimeW)), dx - o0, dy - o1, dz - o1, dw - o1));
    }
    {
        bool m = xn < 0.0f;
        float o1 = flipm((float)(kU + 1), m), o0 = flipm((float)kU, m);
        FND_ACC(fmaf(o0, cs, stemA) + flipm(dx, m), grad4(hash(seed, FND_P(m, xp, kPrimeX), yp, zp, wp), dx - o1, dy - o0, dz - o0, dw - o0));
    }
    {
        bool m = xn < -yn;
        float o1 = flipm((float)(2 * kU + 1), m), o0 = flipm((float)(2 * kU), m);
        FND_ACC(fmaf(o0, cs, stemB) + flipm(dx + dy, m), grad4(hash(seed, FND_P(m, xp, kPrimeX), FND_P(m, yp, kPrimeY), zp, wp), dx - o1, dy - o1, dz - o0, dw - o0));
    }
    {
        bool m = xn < -zn;
        float o1 = flipm((float)(2 * kU + 1), m), o0 = flipm((float)(2 * kU), m);
        FND_ACC(fmaf(o0, cs, stemB) + flipm(dx + dz, m), grad4(hash(seed, FND_P(m, xp, kPrimeX), yp, FND_P(m, zp, kPrimeZ), wp), dx - o1, dy - o0, dz - o1, dw - o0));
    }
    {
        bool m = xn < -wn;
        float o1 = flipm((float)(2 * kU + 1), m), o0 = flipm((float)(2 * kU), m);
        FND_ACC(fmaf(o0, cs, stemB) + flipm(dx + dw, m), grad4(hash(seed, FND_P(m, xp, kPrimeX), yp, zp, FND_P(m, wp, kPrimeW)), dx - o1, dy - o0, dz - o0, dw - o1));
    }
    {
        bool m = yn < 0.0f;
        float o1 = flipm((float)(kU + 1), m), o0 = flipm((float)kU, m);
        FND_ACC(fmaf(o0, cs, stemA) + flipm(dy, m), grad4(hash(seed, xp, FND_P(m, yp, kPrimeY), zp, wp), dx - o0, dy - o1, dz - o0, dw - o0));
    }
    {
        bool m = yn < -zn;
        float o1 = flipm((float)(2 * kU + 1), m), o0 = flipm((float)(2 * kU), m);
        FND_ACC(fmaf(o0, cs, stemB) + flipm(dy + dz, m), grad4(hash(seed, xp, FND_P(m, yp, kPrimeY), FND_P(m, zp, kPrimeZ), wp), dx - o0, dy - o1, dz - o1, dw - o0));
    }
    {
        bool m = yn < -wn;
        float o1 = flipm((float)(2 * kU + 1), m), o0 = flipm((float)(2 * kU), m);
        FND_ACC(fmaf(o0, cs, stemB) + flipm(dy + dw, m), grad4(hash(seed, xp, FND_P(m, yp, kPrimeY), zp, FND_P(m, wp, kPrimeW)), dx - o0, dy - o1, dz - o0, dw - o1));
    }
    {
        bool m = zn < 0.0f;
        float o1 = flipm((float)(kU + 1), m), o0 = flipm((float)kU, m);
        FND_ACC(fmaf(o0, cs, stemA) + flipm(dz, m), grad4(hash(seed, xp, yp, FND_P(m, zp, kPrimeZ), wp), dx - o0, dy - o0, dz - o1, dw - o0));
    }
    {
        bool m = zn < -wn;
        float o1 = flipm((float)(2 * kU + 1), m), o0 = flipm((float)(2 * kU), m);
        FND_ACC(fmaf(o0, cs, stemB) + flipm(dz + dw, m), grad4(hash(seed, xp, yp, FND_P(m, zp, kPrimeZ), FND_P(m, wp, kPrimeW)), dx - o0, dy - o0, dz - o1, dw - o1));
    }
    {
        bool m = wn < 0.0f;
        float o1 = flipm((float)(kU + 1), m), o0 = flipm((float)kU, m);
        FND_ACC(fmaf(o0, cs, stemA) + flipm(dw, m), grad4(hash(seed, xp, yp, zp, FND_P(m, wp, kPrimeW)), dx - o0, dy - o0, dz - o0, dw - o1));
    }
#undef FND_P
#undef FND_ACC
    return value;
}

// ---------------------------------------------------------------- Perlin / Value

FND float perlin2(int seed, float x, float y)
{
    float xs = floorf(x), ys = floorf(y);
    int x0 = imul(cvti(xs), kPrimeX), y0 = imul(cvti(ys), kPrimeY);
    int x1 = iadd(x0, kPrimeX), y1 = iadd(y0, kPrimeY);
    float xf0 = x - xs, yf0 = y - ys, xf1 = xf0 - 1.0f, yf1 = yf0 - 1.0f;
    float u = quintic(xf0), v = quintic(yf0);
    return lerp(lerp(grad2(hash(seed, x0, y0), xf0, yf0), grad2(hash(seed, x1, y0), xf1, yf0), u),
                lerp(grad2(hash(seed, x0, y1), xf0, yf1), grad2(hash(seed, x1, y1), xf1, yf1), u), v);
}

FND float perlin3(int seed, float x, float y, float z)
{
    float xs = floorf(x), ys = floorf(y), zs = floorf(z);
    int x0 = imul(cvti(xs), kPrimeX), y0 = imul(cvti(ys), kPrimeY), z0 = imul(cvti(zs), kPrimeZ);
    int x1 = iadd(x0, kPrimeX), y1 = iadd(y0, kPrimeY), z1 = iadd(z0, kPrimeZ);
    float xf0 = x - xs, yf0 = y - ys, zf0 = z - zs;
    float xf1 = xf0 - 1.0f, yf1 = yf0 - 1.0f, zf1 = zf0 - 1.0f;
    float u = quintic(xf0), v = quintic(yf0), s = quintic(zf0);
    // seed ^ y ^ z shared by each x pair of corners (xor reassociated: the same hashes)
    const int a00 = seed ^ y0 ^ z0, a10 = seed ^ y1 ^ z0, a01 = seed ^ y0 ^ z1, a11 = seed ^ y1 ^ z1;
    return lerp(lerp(lerp(grad3(hash_mix(a00 ^ x0), xf0, yf0, zf0), grad3(hash_mix(a00 ^ x1), xf1, yf0, zf0), u),
                     lerp(grad3(hash_mix(a10 ^ x0), xf0, yf1, zf0), grad3(hash_mix(a10 ^ x1), xf1, yf1, zf0), u), v),
                lerp(lerp(grad3(hash_mix(a01 ^ x0), xf0, yf0, zf1), grad3(hash_mix(a01 ^ x1), xf1, yf0, zf1), u),
                     lerp(grad3(hash_mix(a11 ^ x0), xf0, yf1, zf1), grad3(hash_mix(a11 ^ x1), xf1, yf1, zf1), u), v), s);
}

FND float perlin4(int seed, float x, float y, float z, float w)
{
    float xs = floorf(x), ys = floorf(y), zs = floorf(z), ws = floorf(w);
    int x0 = imul(cvti(xs), kPrimeX), y0 = imul(cvti(ys), kPrimeY), z0 = imul(cvti(zs), kPrimeZ), w0 = imul(cvti(ws), kPrimeW);
    int x1 = iadd(x0, kPrimeX), y1 = iadd(y0, kPrimeY), z1 = iadd(z0, kPrimeZ), w1 = iadd(w0, kPrimeW);
    float xf0 = x - xs, yf0 = y - ys, zf0 = z - zs, wf0 = w - ws;
    float xf1 = xf0 - 1.0f, yf1 = yf0 - 1.0f, zf1 = zf0 - 1.0f, wf1 = wf0 - 1.0f;
    float u = quintic(xf0), v = quintic(yf0), s = quintic(zf0), q = quintic(wf0);
#define G(a, b, c, d, fa, fb, fc, fd) grad4(hash_mix((seed ^ b ^ c ^ d) ^ a), fa, fb, fc, fd)
    return lerp(
        lerp(lerp(lerp(G(x0, y0, z0, w0, xf0, yf0, zf0, wf0), G(x1, y0, z0, w0, xf1, yf0, zf0, wf0), u),
                  lerp(G(x0, y1, z0, w0, xf0, yf1, zf0, wf0), G(x1, y1, z0, w0, xf1, yf1, zf0, wf0), u), v),
             lerp(lerp(G(x0, y0, z1, w0, xf0, yf0, zf1, wf0), G(x1, y0, z1, w0, xf1, yf0, zf1, wf0), u),
                  lerp(G(x0, y1, z1, w0, xf0, yf1, zf1, wf0), G(x1, y1, z1, w0, xf1, yf1, zf1, wf0), u), v), s),
        lerp(lerp(lerp(G(x0, y0, z0, w1, xf0, yf0, zf0, wf1), G(x1, y0, z0, w1, xf1, yf0, zf0, wf1), u),
                  lerp(G(x0, y1, z0, w1, xf0, yf1, zf0, wf1), G(x1, y1, z0, w1, xf1, yf1, zf0, wf1), u), v),
             lerp(lerp(G(x0, y0, z1, w1, xf0, yf0, zf1, wf1), G(x1, y0, z1, w1, xf1, yf0, zf1, wf1), u),
                  lerp(G(x0, y1, z1, w1, xf0, yf1, zf1, wf1), G(x1, y1, z1, w1, xf1, yf1, zf1, wf1), u), v), s), q);
#undef G
}

FND float value2(int seed, float x, float y)
{
    float xs = floorf(x), ys = floorf(y);
    int x0 = imul(cvti(xs), kPrimeX), y0 = imul(cvti(ys), kPrimeY);
    int x1 = iadd(x0, kPrimeX), y1 = iadd(y0, kPrimeY);
    float u = hermite(x - xs), v = hermite(y - ys);
    return lerp(lerp(valcoord(seed ^ x0 ^ y0), valcoord(seed ^ x1 ^ y0), u),
                lerp(valcoord(seed ^ x0 ^ y1), valcoord(seed ^ x1 ^ y1), u), v);
}

FND float value3(int seed, float x, float y, float z)
{
    float xs = floorf(x), ys = floorf(y), zs = floorf(z);
    int x0 = imul(cvti(xs), kPrimeX), y0 = imul(cvti(ys), kPrimeY), z0 = imul(cvti(zs), kPrimeZ);
    int x1 = iadd(x0, kPrimeX), y1 = iadd(y0, kPrimeY), z1 = iadd(z0, kPrimeZ);
    float u = hermite(x - xs), v = hermite(y - ys), s = hermite(z - zs);
    const int a00 = seed ^ y0 ^ z0, a10 = seed ^ y1 ^ z0, a01 = seed ^ y0 ^ z1, a11 = seed ^ y1 ^ z1;   // shared by x pairs
    return lerp(lerp(lerp(valcoord(a00 ^ x0), valcoord(a00 ^ x1), u), lerp(valcoord(a10 ^ x0), valcoord(a10 ^ x1), u), v),
                lerp(lerp(valcoord(a01 ^ x0), valcoord(a01 ^ x1), u), lerp(valcoord(a11 ^ x0), valcoord(a11 ^ x1), u), v), s);
}

FND float value4(int seed, float x, float y, float z, float w)
{
    float xs = floorf(x), ys = floorf(y), zs = floorf(z), ws = floorf(w);
    int x0 = imul(cvti(xs), kPrimeX), y0 = imul(cvti(ys), kPrimeY), z0 = imul(cvti(zs), kPrimeZ), w0 = imul(cvti(ws), kPrimeW);
    int x1 = iadd(x0, kPrimeX), y1 = iadd(y0, kPrimeY), z1 = iadd(z0, kPrimeZ), w1 = iadd(w0, kPrimeW);
    float u = hermite(x - xs), v = hermite(y - ys), s = hermite(z - zs), q = hermite(w - ws);
#define V(a, b, c, d) valcoord((seed ^ b ^ c ^ d) ^ a)
    return lerp(
        lerp(lerp(lerp(V(x0, y0, z0, w0), V(x1, y0, z0, w0), u), lerp(V(x0, y1, z0, w0), V(x1, y1, z0, w0), u), v),
             lerp(lerp(V(x0, y0, z1, w0), V(x1, y0, z1, w0), u), lerp(V(x0, y1, z1, w0), V(x1, y1, z1, w0), u), v), s),
        lerp(lerp(lerp(V(x0, y0, z0, w1), V(x1, y0, z0, w1), u), lerp(V(x0, y1, z0, w1), V(x1, y1, z0, w1), u), v),
             lerp(lerp(V(x0, y0, z1, w1), V(x1, y0, z1, w1), u), lerp(V(x0, y1, z1, w1), V(x1, y1, z1, w1), u), v), s), q);
#undef V
}

// ---------------------------------------------------------------- distances (Utils.inl:281-335)

enum DistFunc { kEuclidean = 0, kEuclideanSq, kManhattan, kHybrid, kMaxAxis, kMinkowski };

// Distance over D components; `sqrt_euclid` mirrors CalcDistance<DO_SQRT>.
// Minkowski takes its exponent `mp` (already evaluated by the caller).
template <int D>
FND float distance(int df, bool sqrt_euclid, const float* p, float mp)
{
    if (df == kManhattan) {
        float tail = fabs_(p[D - 1]);
#pragma unroll
        for (int k = D - 2; k >= 1; --k) tail = fabs_(p[k]) + tail;
        return fabs_(p[0]) + tail;
    }
    if (df == kHybrid) {
        float both = fmaf(p[0], p[0], fabs_(p[0]));
#pragma unroll
        for (int k = 1; k < D; ++k) both = both + fmaf(p[k], p[k], fabs_(p[k]));
        return both;
    }
    if (df == kMaxAxis) {
        float m = fabs_(p[0]);
#pragma unroll
        for (int k = 1; k < D; ++k) m = fmax_(fabs_(p[k]), m);
        return m;
    }
    if (df == kMinkowski) {
        float tail = pow_(fabs_(p[D - 1]), mp);
#pragma unroll
        for (int k = D - 2; k >= 1; --k) tail = pow_(fabs_(p[k]), mp) + tail;
        return pow_(pow_(fabs_(p[0]), mp) + tail, 1.0f / mp);
    }
    float d = p[0] * p[0];
#pragma unroll
    for (int k = 1; k < D; ++k) d = fmaf(p[k], p[k], d);
    return (df != kEuclideanSq && sqrt_euclid) ? sqrtf(d) : d;
}

// ---------------------------------------------------------------- Cellular (Cellular.inl)

constexpr float kJitter2D = 0.437016f, kJitter3D = 0.396144f, kJitter4D = 0.366025f;

template <int D> struct CellConst;
template <> struct CellConst<2> { static constexpr float jitter = kJitter2D; static constexpr float size = -1.f / 0x3ff; static constexpr float sizeMax = 0x3ff; };
template <> struct CellConst<3> { static constexpr float jitter = kJitter3D; static constexpr float size = -1.f / 0xffff; static constexpr float sizeMax = 0xffff; };
template <> struct CellConst<4> { static constexpr float jitter = kJitter4D; static constexpr float size = -1.f / 0xfffff; static constexpr float sizeMax = 0xfffff; };

__device__ constexpr int kPrimes[4] = {kPrimeX, kPrimeY, kPrimeZ, kPrimeW};

template <int D>
FND int cell_hash(int seed, const int* c)
{
    if (D == 2) return hashhb(seed, c[0], c[1]);
    if (D == 3) return hashhb(seed, c[0], c[1], c[2]);
    return hashhb(seed, c[0], c[1], c[2], c[3]);
}

// Jittered cell-point direction scaled by jitter/|dir| (Cellular.inl:55-58, 141-145, 239-244):
// cell_dir_raw gives the D direction components (half-integers, exact), cell_dir_scale the
// factor jitter / |dir| in d[D].
template <int D>
FND void cell_dir_raw(int h, float* d)
{
    if (D == 2) {
        d[0] = cvtf(h & 0x7ff) - (0x7ff / 2.0f);
        d[1] = cvtf((int)srl(h, 21)) - (0x7ff / 2.0f);
    } else if (D == 3) {
        d[0] = cvtf(h & 0x3ff) - (0x3ff / 2.0f);
        d[1] = cvtf((h >> 11) & 0x3ff) - (0x3ff / 2.0f);
        d[2] = cvtf((int)srl(h, 22)) - (0x3ff / 2.0f);
    } else {
        d[0] = cvtf(h & 0xff) - (0xff / 2.0f);
        d[1] = cvtf((h >> 8) & 0xff) - (0xff / 2.0f);
        d[2] = cvtf((h >> 16) & 0xff) - (0xff / 2.0f);
        d[3] = cvtf((int)srl(h, 24)) - (0xff / 2.0f);
    }
}

template <int D>
FND void cell_dir_scale(float jitter, float* d)
{
    if (D == 2) d[2] = jitter * invsqrt(fmaf(d[0], d[0], d[1] * d[1]));
    else if (D == 3) d[3] = jitter * invsqrt(fmaf(d[0], d[0], fmaf(d[1], d[1], d[2] * d[2])));
    else d[4] = jitter * invsqrt(fmaf(d[0], d[0], fmaf(d[1], d[1], fmaf(d[2], d[2], d[3] * d[3]))));
}

template <int D>
FND float size_factor(int h, float sj)
{
    float dj = D == 2 ? cvtf((h >> 11) & 0x3ff) : (D == 3 ? cvtf(h & 0xffff) : cvtf(h & 0xfffff));
    return fmaf(-sj, dj, 1.0f);
}

// The 3^D neighbourhood walk shared by the three cellular nodes.  `mode`:
// 0 = CellularValue (offset base = cell - pos, incremented),
// 1 = CellularDistance (offset = running cell - pos),
// 2 = CellularLookup (cell point, then - pos).
struct CellParams {
    float freq;        // ScalableGenerator::mFrequency
    float jitter;      // kJitterND * grid jitter (already multiplied)
    float sizeJitter;  // size jitter * -1/mask (already multiplied), used if sizeActive
    bool sizeActive;
    int distFunc;
    float minkowski;   // constant Minkowski P
};

// Visit the 3^D cells around the point in the reference's order (last axis
// fastest): visit(c, cf, kRefOrder, nullptr) gets the primed cell coordinates and the
// running float cell offsets (cfb[k] + 0, 1, 2); kRefOrder tells the visitor that cells
// arrive in the reference's order, so its ties need no order index, and the null bound
// array that the cell is not to be skipped.  Nested loops over scalars rather than an
// odometer over arrays, so the per-cell state stays in registers; the innermost
// axis is unrolled so three cells' hashing and distances can overlap.
// Minkowski P of the cellular distance: the node's constant (NoMink), or a
// functor evaluating the P node at each cell's offset vector (specialised kernels;
// Cellular.inl:63 passes the offset to CalcDistance, Utils.inl:326-331).
struct NoMink {
    static constexpr bool kNode = false;
    FND float operator()(const float*) const { return 0.0f; }
};

constexpr int kRefOrder = 0x7fffffff;

template <int D, typename F>
FND void for_each_cell(const int* cb, const float* cfb, F&& visit)
{
    if constexpr (D == 2) {
        int cx = cb[0];
        float fx = cfb[0];
#pragma unroll 1
        for (int xi = 0; xi < 3; ++xi, cx = iadd(cx, kPrimeX), fx += 1.0f) {
            int cy = cb[1];
            float fy = cfb[1];
#pragma unroll
            for (int yi = 0; yi < 3; ++yi, cy = iadd(cy, kPrimeY), fy += 1.0f) {
                const int c[2] = {cx, cy};
                const float cf[2] = {fx, fy};
                visit(c, cf, kRefOrder, nullptr);
            }
        }
    } else if constexpr (D == 3) {
        int cx = cb[0];
        float fx = cfb[0];
#pragma unroll 1
        for (int xi = 0; xi < 3; ++xi, cx = iadd(cx, kPrimeX), fx += 1.0f) {
            int cy = cb[1];
            float fy = cfb[1];
#pragma unroll 1
            for (int yi = 0; yi < 3; ++yi, cy = iadd(cy, kPrimeY), fy += 1.0f) {
                int cz = cb[2];
                float fz = cfb[2];
#pragma unroll
                for (int zi = 0; zi < 3; ++zi, cz = iadd(cz, kPrimeZ), fz += 1.0f) {
                    const int c[3] = {cx, cy, cz};
                    const float cf[3] = {fx, fy, fz};
                    visit(c, cf, kRefOrder, nullptr);
                }
            }
        }
    } else {
        int cx = cb[0];
        float fx = cfb[0];
#pragma unroll 1
        for (int xi = 0; xi < 3; ++xi, cx = iadd(cx, kPrimeX), fx += 1.0f) {
            int cy = cb[1];
            float fy = cfb[1];
#pragma unroll 1
            for (int yi = 0; yi < 3; ++yi, cy = iadd(cy, kPrimeY), fy += 1.0f) {
                int cz = cb[2];
                float fz = cfb[2];
#pragma unroll 1
                for (int zi = 0; zi < 3; ++zi, cz = iadd(cz, kPrimeZ), fz += 1.0f) {
                    int cw = cb[3];
                    float fw = cfb[3];
#pragma unroll
                    for (int wi = 0; wi < 3; ++wi, cw = iadd(cw, kPrimeW), fw += 1.0f) {
                        const int c[4] = {cx, cy, cz, cw};
                        const float cf[4] = {fx, fy, fz, fw};
                        visit(c, cf, kRefOrder, nullptr);
                    }
                }
            }
        }
    }
}

// Skipping cells that cannot change the result.  A cell's point is its lattice point plus
// the jitter vector d * (jitter / |d|): |d|^2 is exact (half-integer components below 2^11),
// so the vector's length is |jitter| within three roundings, below J = |jitter| (1 + 2^-16),
// and so is each of its components.  The cell's fma adds that component to an offset t_k
// (cell - position, as the walk computes it), and since rounding is monotone
// |offset_k| >= lb_k = max(0, RN(|t_k| - J)).  The distance formula evaluated on lb, with
// the axes not yet fixed at 0, uses the same monotone operations as the cell's own distance
// (sums of squares / absolute values, max, square root, the size-jitter factor >= fmin > 0),
// so it bounds that distance from below.  A plane, row or cell whose bound is above the
// current threshold (the last distance slot the walk keeps) cannot enter the kept slots and
// is skipped.
//
// Pruned walks visit each axis middle-first (reference index 1, 0, 2), which finds the near
// cells early (3D: ~12 of 27 cells left per warp for one slot, ~35 of 81 in 4D for two).
// Kept distances do not depend on the visiting order; where the walk keeps one cell's hash or
// point, ties are broken on the reference's visiting index `o`, which makes the result the
// one the reference's strictly-closer rule gives in its own order.  CellularValue with a
// value index above 0 keeps several hashes, and the reference's insertion moves a displaced
// hash past equal distances only when strictly closer, so which of two tied hashes ends in
// which slot depends on the visiting order: that walk prunes in the reference's order.
// Pruning and the order change are used only where no NaN can reach a distance unless every
// cell's is NaN: a finite jitter, a finite size jitter whose factor stays positive, and not
// Minkowski (whose power functions are not shown monotone here); otherwise the unpruned
// reference-order walk runs.
// 2D walks (9 cells, few to skip) also run in the reference's order: the checks cost there
// about what the skipped cells save (CellularLookup 2D measured 1.6 % faster without).
struct CellBound {
    int df;
    bool sq;       // the walk takes the square root of Euclidean distances
    bool size;     // distances are multiplied by a size-jitter factor >= fmin
    float fmin;
    float J;       // bound on each jitter component
    bool on;       // pruned walk (middle-first unless the walk must keep the reference's order)
};

template <int D>
FND CellBound cell_bound_params(const CellParams& cp, bool sq)
{
    CellBound B;
    B.df = cp.distFunc;
    B.sq = sq && cp.distFunc != kEuclideanSq;
    B.size = cp.sizeActive;
    B.J = fabs_(cp.jitter) * 1.00001526f;                      // 1 + 2^-16
    const bool sizeFinite = fabs_(cp.sizeJitter) <= 3.40282347e38f;
    B.fmin = cp.sizeJitter > 0.0f ? fmaf(-cp.sizeJitter, CellConst<D>::sizeMax, 1.0f) : 1.0f;
    B.on = D > 2 && B.J <= 3.40282347e38f && cp.distFunc >= kEuclidean && cp.distFunc <= kMaxAxis &&
           (!cp.sizeActive || (sizeFinite && B.fmin > 0.0f));
    return B;
}

// Lower bound of the distance with axes 0..K at lb and the others at 0 (same operation
// order as distance<D>).
template <int K>
FND float cell_bound(const CellBound& B, const float* lb)
{
    float b;
    if (B.df == kManhattan) {
        float t = lb[K];
#pragma unroll
        for (int k = K - 1; k >= 1; --k) t = lb[k] + t;
        b = K == 0 ? lb[0] : lb[0] + t;
    } else if (B.df == kHybrid) {
        b = fmaf(lb[0], lb[0], lb[0]);
#pragma unroll
        for (int k = 1; k <= K; ++k) b = b + fmaf(lb[k], lb[k], lb[k]);
    } else if (B.df == kMaxAxis) {
        b = lb[0];
#pragma unroll
        for (int k = 1; k <= K; ++k) b = fmax_(lb[k], b);
    } else {
        b = lb[0] * lb[0];
#pragma unroll
        for (int k = 1; k <= K; ++k) b = fmaf(lb[k], lb[k], b);
        if (B.sq) b = sqrtf(b);
    }
    return B.size ? b * B.fmin : b;
}

// Second bound, once the cell's hash gives its jitter direction d (before the normalisation
// and distance): on an axis where the jitter component d_k * jitter has the sign of the
// offset t_k it is added to, the cell point lies beyond t_k, so |offset_k| >= |t_k| (rounding
// is monotone; for CellularLookup, whose cell point is rounded before the position is
// subtracted, the rounded point lies beyond cf as well); elsewhere lb_k stands.  Used by the
// 81-cell 4D walks only: terrain tileable (4D) measured 3.51 -> 3.65 Gpts/s with it, while in
// 3D the per-lane test after the hash cost more than it saved (chunk mix 47.6 -> 46.8; for the
// 3D distance walks alone 48.65 -> 48.0, terrain 128^3 unchanged).
template <int D>
FND float cell_bound_dir(const CellBound& B, const float* lb, const float* t, const float* d, float jitter)
{
    float l2[D];
#pragma unroll
    for (int k = 0; k < D; ++k)
        l2[k] = ((__float_as_uint(d[k]) ^ __float_as_uint(jitter) ^ __float_as_uint(t[k])) >> 31) ? lb[k] : fabs_(t[k]);
    return cell_bound<D - 1>(B, l2);
}

// Pruned walk over axis K and the axes after it, middle-first (Mid) or in the reference's
// order.  axis_lb(k, cf) gives lb_k for the cell offset cf on axis k; thr() the current
// threshold; visit(c, cf, o) as above with the cell's index in the reference's order
// (kRefOrder when the walk keeps the reference's order).
template <bool Mid, int D, int K, typename LbF, typename ThrF, typename F>
FND void walk_mid(const int* cb, const float* cfb, int* c, float* cf, float* lb, int o, const CellBound& B,
                  LbF& axis_lb, ThrF& thr, F& visit)
{
    const int c1 = iadd(cb[K], kPrimes[K]), c2 = iadd(c1, kPrimes[K]);
    const float f1 = cfb[K] + 1.0f, f2 = f1 + 1.0f;
    auto step = [&](int m) {
        const int j = Mid ? (m == 0 ? 1 : (m == 1 ? 0 : 2)) : m;
        c[K] = j == 0 ? cb[K] : (j == 1 ? c1 : c2);
        cf[K] = j == 0 ? cfb[K] : (j == 1 ? f1 : f2);
        lb[K] = axis_lb(K, cf[K]);
        if (cell_bound<K>(B, lb) > thr()) return;
        if constexpr (K + 1 < D) walk_mid<Mid, D, K + 1>(cb, cfb, c, cf, lb, o * 3 + j, B, axis_lb, thr, visit);
        else visit(c, cf, Mid ? o * 3 + j : kRefOrder, static_cast<const float*>(lb));
    };
    if constexpr (K == D - 1) {
#pragma unroll
        for (int m = 0; m < 3; ++m) step(m);
    } else {
#pragma unroll 1
        for (int m = 0; m < 3; ++m) step(m);
    }
}

template <int D, bool Mid = true, typename LbF, typename ThrF, typename F>
FND void for_each_cell_pruned(const int* cb, const float* cfb, const CellBound& B, LbF&& axis_lb, ThrF&& thr, F&& visit)
{
    int c[D];
    float cf[D], lb[D];
    walk_mid<Mid, D, 0>(cb, cfb, c, cf, lb, 0, B, axis_lb, thr, visit);
}

template <int D, typename MinkF = NoMink>
FND float cellular_value(int seed, const float* pin, const CellParams& cp, int valueIndex, const MinkF& mink = MinkF())
{
    float p[D];
#pragma unroll
    for (int k = 0; k < D; ++k) p[k] = pin[k] * cp.freq;
    float dist[4] = {__int_as_float(0x7F800000), __int_as_float(0x7F800000), __int_as_float(0x7F800000), __int_as_float(0x7F800000)};
    int vh[4] = {0, 0, 0, 0};
    int ord[4] = {-1, -1, -1, -1};   // the initial slots precede every cell
    int cb[D];
    float cfb[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        cb[k] = iadd(cvti(p[k]), -1);
        cfb[k] = cvtf(cb[k]) - p[k];
        cb[k] = imul(cb[k], kPrimes[k]);
    }
    const CellBound B = cell_bound_params<D>(cp, D == 2);
    auto thr = [&]() {
        float t = dist[0];
#pragma unroll
        for (int i = 1; i < 4; ++i) t = valueIndex == i ? dist[i] : t;
        return t;
    };
    auto visit = [&](const int* c, const float* cf, int o, const float* lb) {
        int h = cell_hash<D>(seed, c);
        float d[D + 1];
        cell_dir_raw<D>(h, d);
        if (D == 4 && lb && cell_bound_dir<D>(B, lb, cf, d, cp.jitter) > thr()) return;
        cell_dir_scale<D>(cp.jitter, d);
        float off[D];
#pragma unroll
        for (int k = 0; k < D; ++k) off[k] = fmaf(d[k], d[D], cf[k]);
        const float mk = (MinkF::kNode && cp.distFunc == 5) ? mink(off) : cp.minkowski;
        float nd = distance<D>(cp.distFunc, D == 2, off, mk);
        if (cp.sizeActive) nd *= size_factor<D>(h, cp.sizeJitter);
        int nh = h, no = o;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            bool closer = nd < dist[i] || (nd == dist[i] && no < ord[i]);
            float ld = dist[i];
            int lh = vh[i], lo = ord[i];
            dist[i] = closer ? nd : dist[i];
            vh[i] = closer ? nh : vh[i];
            ord[i] = closer ? no : ord[i];
            if (i >= valueIndex) break;
            nd = closer ? ld : nd;
            nh = closer ? lh : nh;
            no = closer ? lo : no;
        }
    };
    auto axis_lb = [&](int, float cf) { return fmaxf(0.0f, fabs_(cf) - B.J); };
    if (B.on && valueIndex == 0) {
        for_each_cell_pruned<D>(cb, cfb, B, axis_lb, thr, visit);
    } else if (B.on) {
        for_each_cell_pruned<D, false>(cb, cfb, B, axis_lb, thr, visit);
    } else {
        for_each_cell<D>(cb, cfb, visit);
    }
    int sel = vh[0];
#pragma unroll
    for (int i = 1; i < 4; ++i) sel = valueIndex == i ? vh[i] : sel;
    return cvtf(sel);
}

// NS = sorted distance slots kept (the reference keeps 4).  Slot i only ever depends on
// slots i and i - 1, so a caller that reads slots below NS alone may keep fewer: the
// specialised kernels pass max(index0, index1) + 1; the other slots stay +inf.
template <int D, int NS = 4, typename MinkF = NoMink>
FND void cellular_distances(int seed, const float* pin, const CellParams& cp, float* dist, const MinkF& mink = MinkF())
{
    float p[D];
#pragma unroll
    for (int k = 0; k < D; ++k) p[k] = pin[k] * cp.freq;
#pragma unroll
    for (int i = 0; i < 4; ++i) dist[i] = __int_as_float(0x7F800000);
    int cb[D];
    float cfb[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        cb[k] = iadd(cvti(p[k]), -1);
        cfb[k] = cvtf(cb[k]);
        cb[k] = imul(cb[k], kPrimes[k]);
    }
    const CellBound B = cell_bound_params<D>(cp, false);
    auto thr = [&]() { return dist[NS - 1]; };
    auto visit = [&](const int* c, const float* cf, int, const float* lb) {
        int h = cell_hash<D>(seed, c);
        float d[D + 1], t[D];
        cell_dir_raw<D>(h, d);
#pragma unroll
        for (int k = 0; k < D; ++k) t[k] = cf[k] - p[k];
        if (D == 4 && lb && cell_bound_dir<D>(B, lb, t, d, cp.jitter) > thr()) return;
        cell_dir_scale<D>(cp.jitter, d);
        float off[D];
#pragma unroll
        for (int k = 0; k < D; ++k) off[k] = fmaf(d[k], d[D], t[k]);
        const float mk = (MinkF::kNode && cp.distFunc == 5) ? mink(off) : cp.minkowski;
        float nd = distance<D>(cp.distFunc, false, off, mk);
        if (cp.sizeActive) nd *= size_factor<D>(h, cp.sizeJitter);
#pragma unroll
        for (int i = NS - 1; i > 0; i--) dist[i] = fmax_(fmin_(dist[i], nd), dist[i - 1]);
        dist[0] = fmin_(dist[0], nd);
    };
    if (B.on) {
        for_each_cell_pruned<D>(cb, cfb, B,
            [&](int k, float cf) { return fmaxf(0.0f, fabs_(cf - p[k]) - B.J); },
            thr, visit);
    } else {
        for_each_cell<D>(cb, cfb, visit);
    }
}

// CellularDistance::GetReturn (Cellular.inl:531-565) without the final ScaleOutput;
// returns the combined distance and writes the native max through `nmax`.
template <int D>
FND float cellular_return(float* dist, int distFunc, int i0, int i1, int ret, float& nmax)
{
    float maxDist = 1 + CellConst<D>::jitter;
    float d0 = dist[0], d1 = dist[0];
#pragma unroll
    for (int i = 1; i < 4; ++i) { d0 = i0 == i ? dist[i] : d0; d1 = i1 == i ? dist[i] : d1; }
    if (distFunc == kEuclidean) {
        d0 = d0 * invsqrt(d0);
        // both indices alias the same slot when i0 == i1: the reference scales it twice
        d1 = (i1 == i0) ? d0 * invsqrt(d0) : d1 * invsqrt(d1);
        if (i1 == i0) d0 = d1;
    }
    maxDist *= maxDist;
    switch (ret) {
    case 1: nmax = maxDist * 2; return d0 + d1;
    case 2: nmax = maxDist; return fabs_(d0 - d1);
    case 3: nmax = maxDist * maxDist; return d0 * d1;
    case 4: nmax = maxDist; return d0 * (1.0f / d1);
    default: nmax = maxDist; return d0;
    }
}

template <int D, typename MinkF = NoMink>
FND void cellular_lookup_pos(int seed, const float* pin, const CellParams& cp, float scale, float* out, const MinkF& mink = MinkF())
{
    float p[D];
#pragma unroll
    for (int k = 0; k < D; ++k) p[k] = pin[k] * cp.freq;
    float best = 3.40282347e+38f;
    int bo = -1;
    float cell[D];
#pragma unroll
    for (int k = 0; k < D; ++k) cell[k] = 0.0f;
    int cb[D];
    float cfb[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        cb[k] = iadd(cvti(p[k]), -1);
        cfb[k] = cvtf(cb[k]);
        cb[k] = imul(cb[k], kPrimes[k]);
    }
    const CellBound B = cell_bound_params<D>(cp, false);
    auto thr = [&]() { return best; };
    auto visit = [&](const int* c, const float* cf, int o, const float* lb) {
        int h = cell_hash<D>(seed, c);
        float d[D + 1];
        cell_dir_raw<D>(h, d);
        if (D == 4 && lb) {
            float t[D];
#pragma unroll
            for (int k = 0; k < D; ++k) t[k] = cf[k] - p[k];
            if (cell_bound_dir<D>(B, lb, t, d, cp.jitter) > thr()) return;
        }
        cell_dir_scale<D>(cp.jitter, d);
        float local[D], off[D];
#pragma unroll
        for (int k = 0; k < D; ++k) { local[k] = fmaf(d[k], d[D], cf[k]); off[k] = local[k] - p[k]; }
        const float mk = (MinkF::kNode && cp.distFunc == 5) ? mink(off) : cp.minkowski;
        float nd = distance<D>(cp.distFunc, false, off, mk);
        if (cp.sizeActive) nd *= size_factor<D>(h, cp.sizeJitter);
        const bool closer = nd < best || (nd == best && o < bo);
        best = fmin_(nd, best);
        bo = closer ? o : bo;
#pragma unroll
        for (int k = 0; k < D; ++k) cell[k] = closer ? local[k] : cell[k];
    };
    if (B.on) {
        // the cell point is rounded before the position is subtracted: widen J by the
        // rounding of the cell point and of cf - p (2^-22 covers both with room)
        for_each_cell_pruned<D>(cb, cfb, B,
            [&](int k, float cf) {
                const float t = fabs_(cf - p[k]);
                return fmaxf(0.0f, t - fmaf(t + fabs_(cf) + B.J, 2.38418579e-7f, B.J));
            },
            thr, visit);
    } else {
        for_each_cell<D>(cb, cfb, visit);
    }
#pragma unroll
    for (int k = 0; k < D; ++k) out[k] = cell[k] * scale;
}

// ---------------------------------------------------------------- DomainWarpGradient::Warp (DomainWarp.inl:33-206)

template <int D>
FND float warp_gradient(int seed, float amp, const float* sp, const float* axis, float* io)
{
    float s[D][2];
    int c[D][2];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        float fl = floorf(sp[k]);
        c[k][0] = imul(cvti(fl), kPrimes[k]);
        c[k][1] = iadd(c[k][0], kPrimes[k]);
        s[k][1] = hermite(sp[k] - fl);
        s[k][0] = 1.0f - s[k][1];
    }
    float wv[D];
    constexpr float normalise = D == 2 ? 1.0f / (0xffff / 2.0f) : (D == 3 ? 1.0f / (0x3ff / 2.0f) : 1.0f / (0xff / 2.0f));
#pragma unroll
    for (int corner = 0; corner < (1 << D); ++corner) {
        const int b0 = corner & 1, b1 = (corner >> 1) & 1, b2 = (corner >> 2) & 1, b3 = (corner >> 3) & 1;
        int h;
        float contrib, comp[D];
        if (D == 2) {
            h = hashhb(seed, c[0][b0], c[1][b1]);
            contrib = s[0][b0] * s[1][b1];
            comp[0] = cvtf(h & 0xffff);
            comp[1] = cvtf((int)srl(h, 16));
        } else if (D == 3) {
            h = hashhb(seed, c[0][b0], c[1][b1], c[2 % D][b2]);
            contrib = s[0][b0] * s[1][b1] * s[2 % D][b2];
            comp[0] = cvtf(h & 0x3ff);
            comp[1] = cvtf((h >> 11) & 0x3ff);
            comp[2 % D] = cvtf((int)srl(h, 22));
        } else {
            h = hashhb(seed, c[0][b0], c[1][b1], c[2 % D][b2], c[3 % D][b3]);
            contrib = s[0][b0] * s[1][b1] * s[2 % D][b2] * s[3 % D][b3];
            comp[0] = cvtf(h & 0xff);
            comp[1] = cvtf((h >> 8) & 0xff);
            comp[2 % D] = cvtf((h >> 16) & 0xff);
            comp[3 % D] = cvtf((int)srl(h, 24));
        }
#pragma unroll
        for (int k = 0; k < D; ++k) wv[k] = corner == 0 ? contrib * comp[k] : fmaf(contrib, comp[k], wv[k]);
    }
#pragma unroll
    for (int k = 0; k < D; ++k) wv[k] = fmaf(wv[k], normalise, -1.0f);
#pragma unroll
    for (int k = 0; k < D; ++k) io[k] = fmaf(wv[k], amp * axis[k], io[k]);
    float r = wv[D - 1] * wv[D - 1];
#pragma unroll
    for (int k = D - 2; k >= 0; --k) r = fmaf(wv[k], wv[k], r);
    return r;
}

// ---------------------------------------------------------------- DomainWarpSimplex / DomainWarpSuperSimplex
//
// Restatement of DomainWarpSimplex.inl.  The vector-product helpers follow the
// portable (non-AVX) branches (:40-60, :82-116, :148-191, :221-235, :285-316,
// :560-695); FS::Masked*(m, a, b) are written as selects and
// FS::SelectHighBit(m, a, b) as (m < 0 ? a : b).  `v` accumulates the vector.

constexpr float kRoot2f = (float)kRoot2, kRoot3f = (float)kRoot3;
constexpr float kSkew2f = (float)(1.0 / (kRoot3 + 1.0)), kSkew4f = (float)(1.0 / (kRoot5 + 1.0));

FND int shl(int a, int s) { return (int)((unsigned)a << s); }
FND float selhb(int m, float a, float b) { return m < 0 ? a : b; }

// ApplyGradientOuterProductVectorProductSimplex 2D (:7-60)
FND void wgop2(int hash31, float fX, float fY, float mul, float* v)
{
    const int hs = (int)srl(hash31, 1);
    const int ig = imul(hs, 12 >> 2);
    const int io = imul(hs, (int)0xAAAAAAAB) & (int)0xC0000003;
    {
        const float u = selhb(shl(ig, 2), fY, fX);
        const float w = selhb(shl(ig, 2), fX, fY);
        const float a = u * selhb(ig, 2.0f, kRoot3f);
        const float b = flip(w, shl(ig >> 30, 31));
        const float s = ig >= 0 ? a + b : a;
        mul = mul * flip(s, shl((ig >> 28) ^ io, 31));
    }
    {
        const float a = mul * selhb(io, 2.0f, kRoot3f);
        const float b = flip(io >= 0 ? mul : 0.0f, shl(io >> 30, 31));
        v[0] = v[0] + selhb(shl(io, 30), b, a);
        v[1] = v[1] + selhb(shl(io, 30), a, b);
    }
}

// ApplyGradientOuterProductVectorProductCommon 3D (:62-116)
FND void wgop3(int hash31, float fX, float fY, float fZ, float mul, float* v)
{
    const int hs = (int)srl(hash31, 1);
    const int ig = (int)srl(imul(hs, 12 >> 2), 28);
    int io = imul(hs, (int)0xAAAAAAAB) & (int)0xC0000003;
    io = io | (io >> 28);
    {
        const float u = ig >= 8 ? fY : fX;
        const float w = ig >= 4 ? fZ : fY;
        mul = mul * (flip(u, shl(ig, 31)) + flip(w, shl(ig >> 1, 31)));
    }
    {
        io &= 0xF;
        const float s0 = flip(mul, shl(io, 31));
        const float s1 = flip(mul, shl(io >> 1, 31));
        const bool notYZ = io < 8, notXY = io >= 4;
        v[0] = notYZ ? v[0] + s0 : v[0];
        v[2] = notXY ? v[2] + s1 : v[2];
        v[1] = (notYZ && notXY) ? v[1] : v[1] + (notXY ? s0 : s1);
    }
}

// one 4D outer-product gradient from a [0,20) << 27 table index (:150-171)
FND void wgop4_vector(int index, float* g)
{
    int iA = index & (0x03 << 27);
    int iB = (index >> 2) & (0x07 << 27);
    iB ^= iA;
    const bool extra = iB >= (0x04 << 27);
    const bool equal = iA == iB;
    if (equal) iA = -1;
    const float neutral = (equal || extra) ? (extra ? kSkew4f * -1.0f : kSkew4f) : 0.0f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float t = iA == (k << 27) ? neutral - 1.0f : neutral;
        g[k] = iB == (k << 27) ? t + 1.0f : t;
    }
}

// ApplyGradientOuterProductVectorProductSimplex 4D (:118-191)
FND void wgop4(int hash, float fX, float fY, float fZ, float fW, float mul, float* v)
{
    const int hs = (int)srl(hash, 2);
    const int ig = imul(hs, 20 >> 2);
    int io = imul(hs, (int)0xCCCCCCCD);
    io = imul(io & (int)0xE0000003, 3 | (1 << 27));
    float g[4];
    wgop4_vector(ig, g);
    mul = mul * fmaf(g[3], fW, fmaf(g[2], fZ, fmaf(g[1], fY, g[0] * fX)));
    wgop4_vector(io, g);
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = fmaf(mul, g[k], v[k]);
}

// ApplyOrthogonalGradientMatrixVectorProductSimplex 2D (:193-235)
FND void wogm2(int hash31, float fX, float fY, float mul, float* v)
{
    const int index = imul((int)srl(hash31, 1), 12 >> 2);
    const int ofThree = (int)srl(index, 30);
    const float masked = index >= 0 ? kSkew2f : 0.0f;
    const float gX = flip(ofThree != 0 ? masked + 1.0f : masked, shl(index >> 28, 31));
    const float gY = flip(ofThree != 1 ? masked + 1.0f : masked, shl(index >> 29, 31));
    v[0] = fmaf(mul, fmaf(fY, gY, fX * gX), v[0]);
    mul = flip(mul, shl(hash31, 31));
    v[1] = fmaf(mul, fmaf(fY, gX, -(fX * gY)), v[1]);
}

// ApplyOrthogonalGradientMatrixVectorProductCommon 3D (:237-316)
FND void wogm3(int hash31, float fX, float fY, float fZ, float mul, float* v)
{
    constexpr float cA = 2.224744871391589f, cB = -0.224744871391589f, cC = -1.0f, cDE = 1.0f, cF = 2.0f;
    const int hs = (int)srl(hash31, 1);
    const int fb = imul(hs, (int)0xAAAAAAAB);
    const int p2hb = shl(fb, 29);
    const int p3 = (int)srl(imul(hs, 3), 30);
    const int sign0 = shl(fb, 31);
    const int sign1 = shl(fb, 30) & (int)0x80000000;
    const int notYZ = fb, notXY = shl(fb, 1), either = notYZ | notXY;

    const float aX = selhb(notYZ, cC, flip(cA, sign0));
    const float aY = selhb(either, selhb(notXY, flip(cB, sign1), flip(cA, sign0)), cC);
    const float aZ = selhb(notXY, cC, flip(cB, sign1));
    const float valA = fmaf(aZ, fZ, fmaf(fY, aY, fX * aX));
    const float bX = selhb(notYZ, cC, flip(cB, sign0));
    const float bY = selhb(either, selhb(notXY, flip(cA, sign1), flip(cB, sign0)), cC);
    const float bZ = selhb(notXY, cC, flip(cA, sign1));
    const float valB = fmaf(bZ, fZ, fmaf(fY, bY, fX * bX));
    const float cX = selhb(notYZ, cF, flip(cDE, sign0));
    const float cY = selhb(either, selhb(notXY, flip(cDE, sign1), flip(cDE, sign0)), cF);
    const float cZ = selhb(notXY, cF, flip(cDE, sign1));
    const float valC = fmaf(cZ, fZ, fmaf(fY, cY, fX * cX));

    const float valAB = selhb(p2hb, valB, valA);
    const float valBA = selhb(p2hb, valA, valB);
    mul = flip(mul, shl(hash31, 31));
    v[0] = fmaf(mul, p3 == 0 ? valC : valAB, v[0]);
    v[1] = fmaf(mul, p3 == 1 ? valC : (p3 == 2 ? valBA : valAB), v[1]);
    v[2] = fmaf(mul, p3 == 2 ? valC : valBA, v[2]);
}

// ApplyOrthogonalGradientMatrixVectorProductSimplex 4D (:318-695)
FND void wogm4(int hash31, float fX, float fY, float fZ, float fW, float mul, float* v)
{
    constexpr float kNegAB = -0.375999676691291f, kFillAB = 0.222726847849776f;
    constexpr float kPosD = -kSkew4f, kUnD = kSkew4f;
    constexpr float kToSingleAB = -0.124000323308709f, kToSingleD = 0.190983005625053f;
    constexpr float kToExtra = kSkew4f, kABToC = 0.437016024448821f, kToDiag = -kRoot2f;

    const int hs = (int)srl(hash31, 2);
    const int basis = imul(hs, 20 >> 2);
    const int p3 = imul(hs, (int)0xD5555556) >> 29;
    const int p8 = basis >> 24;

    int iPos = basis & (0x03 << 27);
    int iNeg = (basis >> 2) & (0x03 << 27);
    iNeg ^= iPos;
    // (0x10 << 27) wraps to INT_MIN: with signed int32 compares the mask is always set (:567)
    const bool extraCase = basis >= (int)0x80000000;
    const bool singleCase = iPos == iNeg;
    const bool singleNonExtra = basis < (0x04 << 27);
    if (singleNonExtra) iPos = -1;

    const float offAB = extraCase ? kToSingleAB + kToExtra : kToSingleAB;
    const float negAB = singleCase ? kNegAB + offAB : kNegAB;
    const float fillAB = singleCase ? kFillAB + offAB : kFillAB;
    const float negC = singleCase ? negAB : negAB + kABToC;
    const float fillC = singleCase ? fillAB : fillAB + kABToC;
    const float offD = extraCase ? kToSingleD + kToExtra : kToSingleD;
    const float posD = singleCase ? kPosD + offD : kPosD;
    const float unD = singleCase ? kUnD + offD : kUnD;

    int counter = -1;
    float vA = 0.0f, vB = 0.0f, vC = 0.0f, vD = 0.0f;
    const float f[4] = {fX, fY, fZ, fW};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const bool idxPos = iPos == (k << 27);
        const bool indexed = idxPos || iNeg == (k << 27);
        const float icAB = idxPos ? negAB + 1.0f : negAB;
        const float icC = idxPos ? negC + 1.0f : negC;
        const float icD = !idxPos ? posD - 1.0f : posD;
        float uA, uB, uC;
        if (k == 0) {
            uA = fillAB + kToDiag; uB = fillAB; uC = fillC;
        } else if (k == 1) {
            uA = counter == -2 ? fillAB + kToDiag : fillAB;
            uB = counter == -1 ? fillAB + kToDiag : fillAB;
            uC = fillC;
        } else if (k == 2) {
            uA = counter == -3 ? fillAB + kToDiag : fillAB;
            uB = counter == -2 ? fillAB + kToDiag : fillAB;
            uC = counter == -1 ? fillC + kToDiag : fillC;
        } else {
            uA = fillAB;
            uB = counter == -3 ? fillAB + kToDiag : fillAB;
            uC = counter == -2 ? fillC + kToDiag : fillC;
        }
        const float gA = indexed ? icAB : uA, gB = indexed ? icAB : uB;
        const float gC = indexed ? icC : uC, gD = indexed ? icD : unD;
        if (k < 3 && indexed) counter -= 1;
        if (k == 0) { vA = gA * f[0]; vB = gB * f[0]; vC = gC * f[0]; vD = gD * f[0]; }
        else { vA = fmaf(gA, f[k], vA); vB = fmaf(gB, f[k], vB); vC = fmaf(gC, f[k], vC); vD = fmaf(gD, f[k], vD); }
    }
    const int ix = p8 >> 1;
    const int iy = iadd(iadd(ix, 1), p3);
    int iz = p8 & 1;
    iz = iadd(iadd(ix, 1), iz >= p3 ? iadd(iz, 1) : iz);
    const int isum = iadd(iadd(ix, iy), iz);
    mul = flip(mul, shl(hash31, 31));
    auto pick = [&](int i) { return selhb(shl(i, 31), selhb(shl(i, 30), vD, vB), selhb(shl(i, 30), vC, vA)); };
    v[0] = fmaf(mul, pick(ix), v[0]);
    v[1] = fmaf(mul, pick(iy), v[1]);
    v[2] = fmaf(mul, pick(iz), v[2]);
    v[3] = fmaf(mul, selhb(shl(isum, 31), selhb(shl(isum, 30), vD, vB), selhb(shl(isum, 30), vA, vC)), v[3]);
}

template <int D>
FND void wvec(bool gop, int h, const float* d, float mul, float* v)
{
    if (D == 2) { if (gop) wgop2(h, d[0], d[1], mul, v); else wogm2(h, d[0], d[1], mul, v); }
    else if (D == 3) { if (gop) wgop3(h, d[0], d[1], d[2 % D], mul, v); else wogm3(h, d[0], d[1], d[2 % D], mul, v); }
    else { if (gop) wgop4(h, d[0], d[1], d[2 % D], d[3 % D], mul, v); else wogm4(h, d[0], d[1], d[2 % D], d[3 % D], mul, v); }
}
FND float pow4(float f) { f = f * f; return f * f; }
FND float fb4(float f) { return (f * f) * (f * f); }

// DomainWarpSimplex::Warp_2D/3D/4D (:771-1089)
FND void ws_simplex2(bool gop, int seed, const float* p, float* v)
{
    constexpr double kSkew2 = 1.0 / (kRoot3 + 1.0), kUnskew2 = -1.0 / (kRoot3 + 3.0), kR2 = 0.5;
    const float x = p[0], y = p[1];
    const float skewDelta = (float)kSkew2 * (x + y);
    const float xs = x + skewDelta, ys = y + skewDelta;
    const float xb = floorf(xs), yb = floorf(ys);
    const float dxs = xs - xb, dys = ys - yb;
    const int xp = imul(cvti(xb), kPrimeX), yp = imul(cvti(yb), kPrimeY);
    const bool xGEy = dxs >= dys;
    const float ud = (float)kUnskew2 * (dxs + dys);
    const float dx0 = dxs + ud, dy0 = dys + ud;
    const float dx1 = (!xGEy ? dx0 + 1.0f : dx0) - (float)(kUnskew2 + 1);
    const float dy1 = (xGEy ? dy0 + 1.0f : dy0) - (float)(kUnskew2 + 1);
    const float dx2 = dx0 - (float)(kUnskew2 * 2 + 1), dy2 = dy0 - (float)(kUnskew2 * 2 + 1);
    float f0 = fmaf(-dx0, dx0, fmaf(-dy0, dy0, (float)kR2));
    float f1 = fmaf(-dx1, dx1, fmaf(-dy1, dy1, (float)kR2));
    float f2 = f0 + fmaf(ud, (float)(-4.0 * (kRoot3 + 2.0) / (kRoot3 + 3.0)), (float)(-2.0 / 3.0));
    f0 = pow4(fmaxf(f0, 0.0f)); f1 = pow4(fmaxf(f1, 0.0f)); f2 = pow4(fmaxf(f2, 0.0f));
    v[0] = 0.0f; v[1] = 0.0f;
    { const float d[2] = {dx0, dy0}; wvec<2>(gop, hash(seed, xp, yp), d, f0, v); }
    { const float d[2] = {dx1, dy1}; wvec<2>(gop, hash(seed, xGEy ? iadd(xp, kPrimeX) : xp, !xGEy ? iadd(yp, kPrimeY) : yp), d, f1, v); }
    { const float d[2] = {dx2, dy2}; wvec<2>(gop, hash(seed, iadd(xp, kPrimeX), iadd(yp, kPrimeY)), d, f2, v); }
}

FND void ws_simplex3(bool gop, int seed, const float* p, float* v)
{
    constexpr double kSkew3 = 1.0 / 3.0, kRU3 = -1.0 / 2.0, kR2 = 0.6;
    const float x = p[0], y = p[1], z = p[2];
    const float skewDelta = (float)kSkew3 * (x + y + z);
    const float xs = x + skewDelta, ys = y + skewDelta, zs = z + skewDelta;
    const float xb = floorf(xs), yb = floorf(ys), zb = floorf(zs);
    const float dxs = xs - xb, dys = ys - yb, dzs = zs - zb;
    const int xp = imul(cvti(xb), kPrimeX), yp = imul(cvti(yb), kPrimeY), zp = imul(cvti(zb), kPrimeZ);
    const bool xGEy = dxs >= dys, yGEz = dys >= dzs, xGEz = dxs >= dzs;
    const float ud = (float)kRU3 * (dxs + dys + dzs);
    const float dx0 = dxs + ud, dy0 = dys + ud, dz0 = dzs + ud;
    const bool mX1 = xGEy && xGEz, mY1 = yGEz && !xGEy, mZ1 = xGEz || yGEz;
    const bool nX2 = xGEy || xGEz, nY2 = xGEy && !yGEz, nZ2 = xGEz && yGEz;
    const float dx3 = dx0 - (float)(kRU3 * 3 + 1), dy3 = dy0 - (float)(kRU3 * 3 + 1), dz3 = dz0 - (float)(kRU3 * 3 + 1);
    const float dx1 = mX1 ? dx3 - 1.0f : dx3, dy1 = mY1 ? dy3 - 1.0f : dy3, dz1 = mZ1 ? dz3 : dz3 - 1.0f;
    const float dx2 = !nX2 ? dx0 + 1.0f : dx0, dy2 = nY2 ? dy0 + 1.0f : dy0, dz2 = nZ2 ? dz0 + 1.0f : dz0;
    float f0 = fmaf(-dz0, dz0, fmaf(-dy0, dy0, fmaf(-dx0, dx0, (float)kR2)));
    float f1 = fmaf(-dz1, dz1, fmaf(-dy1, dy1, fmaf(-dx1, dx1, (float)kR2)));
    float f2 = fmaf(-dz2, dz2, fmaf(-dy2, dy2, fmaf(-dx2, dx2, (float)kR2)));
    float f3 = f0 - (ud + (float)(3.0 / 4.0));
    f0 = pow4(fmaxf(f0, 0.0f)); f1 = pow4(fmaxf(f1, 0.0f)); f2 = pow4(fmaxf(f2, 0.0f)); f3 = pow4(fmaxf(f3, 0.0f));
    v[0] = 0.0f; v[1] = 0.0f; v[2] = 0.0f;
    { const float d[3] = {dx0, dy0, dz0}; wvec<3>(gop, hash(seed, xp, yp, zp), d, f0, v); }
    { const float d[3] = {dx1, dy1, dz1};
      wvec<3>(gop, hash(seed, mX1 ? iadd(xp, kPrimeX) : xp, mY1 ? iadd(yp, kPrimeY) : yp, !mZ1 ? iadd(zp, kPrimeZ) : zp), d, f1, v); }
    { const float d[3] = {dx2, dy2, dz2};
      wvec<3>(gop, hash(seed, nX2 ? iadd(xp, kPrimeX) : xp, !nY2 ? iadd(yp, kPrimeY) : yp, !nZ2 ? iadd(zp, kPrimeZ) : zp), d, f2, v); }
    { const float d[3] = {dx3, dy3, dz3}; wvec<3>(gop, hash(seed, iadd(xp, kPrimeX), iadd(yp, kPrimeY), iadd(zp, kPrimeZ)), d, f3, v); }
    if (gop) {
        const float dl = (float)(-2.0 / 2.0) * (v[0] + v[1] + v[2]);
        v[0] = v[0] + dl; v[1] = v[1] + dl; v[2] = v[2] + dl;
    }
}

FND void ws_simplex4(bool gop, int seed, const float* p, float* v)
{
    constexpr double kSkew4 = 1.0 / (kRoot5 + 1.0), kUnskew4 = -1.0 / (kRoot5 + 5.0), kR2 = 0.6;
    const float skewDelta = (float)kSkew4 * (p[0] + p[1] + p[2] + p[3]);
    float ds[4], d0[4];
    int pb[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float sk = p[k] + skewDelta;
        const float b = floorf(sk);
        ds[k] = sk - b;
        pb[k] = imul(cvti(b), kPrimes[k]);
    }
    const float ud = (float)kUnskew4 * (ds[0] + ds[1] + ds[2] + ds[3]);
#pragma unroll
    for (int k = 0; k < 4; ++k) d0[k] = ds[k] + ud;
    int rank[4] = {0, 0, 0, 0};
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = a + 1; b < 4; ++b) {
            if (d0[a] >= d0[b]) rank[a]++; else rank[b]++;
        }
    v[0] = 0.0f; v[1] = 0.0f; v[2] = 0.0f; v[3] = 0.0f;
    float f0 = 0.0f;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        float d[4];
        int c[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const bool m = i == 0 ? false : i == 4 ? true : rank[k] > 3 - i;
            if (i == 0) d[k] = d0[k];
            else if (i == 4) d[k] = d0[k] - (float)(kUnskew4 * 4 + 1);
            else d[k] = (m ? d0[k] - 1.0f : d0[k]) - (float)(kUnskew4 * i);
            c[k] = m ? iadd(pb[k], kPrimes[k]) : pb[k];
        }
        float f;
        if (i < 4) f = fmaf(-d[3], d[3], fmaf(-d[2], d[2], fmaf(-d[1], d[1], fmaf(-d[0], d[0], (float)kR2))));
        else f = f0 + fmaf(ud, (float)(-4.0 * (kRoot5 + 3.0) / (kRoot5 + 5.0)), (float)(-4.0 / 5.0));
        if (i == 0) f0 = f;
        wvec<4>(gop, hash(seed, c[0], c[1], c[2], c[3]), d, pow4(fmaxf(f, 0.0f)), v);
    }
}

// DomainWarpSuperSimplex::Warp_2D (:1131-1218)
FND void ws_super2(bool gop, int seed, const float* p, float* v)
{
    constexpr double kSkew2 = 1.0 / (kRoot3 + 1.0), kUnskew2 = -1.0 / (kRoot3 + 3.0), kR2 = 2.0 / 3.0;
    const float x = p[0], y = p[1];
    const float skewDelta = (float)kSkew2 * (x + y);
    const float xs = x + skewDelta, ys = y + skewDelta;
    const float xb = floorf(xs), yb = floorf(ys);
    const float dxs = xs - xb, dys = ys - yb;
    const int xp = imul(cvti(xb), kPrimeX), yp = imul(cvti(yb), kPrimeY);
    const bool fXY = dxs + dys > 1.0f;
    const float boundary = fXY ? -1.0f : 0.0f;
    const bool fX = fmaf(dxs, -2.0f, dys) < boundary;
    const bool fY = fmaf(dys, -2.0f, dxs) < boundary;
    const float ud = (float)kUnskew2 * (dxs + dys);
    float dxB = dxs + ud, dyB = dys + ud;
    v[0] = 0.0f; v[1] = 0.0f;
    const float fb0 = fmaf(-dxB, dxB, fmaf(-dyB, dyB, (float)kR2));
    { const float d[2] = {dxB, dyB}; wvec<2>(gop, hash(seed, xp, yp), d, pow4(fb0), v); }
    {
        const float f = fmaf(ud, (float)(-4.0 * (kRoot3 + 2.0) / (kRoot3 + 3.0)), fb0 - (float)kR2);
        const float d[2] = {dxB - (float)(2 * kUnskew2 + 1), dyB - (float)(2 * kUnskew2 + 1)};
        wvec<2>(gop, hash(seed, iadd(xp, kPrimeX), iadd(yp, kPrimeY)), d, pow4(f), v);
    }
    const float xyDelta = fXY ? (float)(kUnskew2 + 1) : (float)(-kUnskew2);
    dxB = dxB - xyDelta;
    dyB = dyB - xyDelta;
    {
        int hx = fX ? iadd(xp, imul(kPrimeX, 2)) : xp;
        hx = fXY ? hx : iadd(hx, -kPrimeX);
        const float dx = dxB - (fX ? (float)(1 + 2 * kUnskew2) : -1.0f);
        const float dy = fX ? dyB - (float)(2 * kUnskew2) : dyB;
        const float f = fmaxf(fmaf(-dx, dx, fmaf(-dy, dy, (float)kR2)), 0.0f);
        const float d[2] = {dx, dy};
        wvec<2>(gop, hash(seed, hx, fXY ? iadd(yp, kPrimeY) : yp), d, pow4(f), v);
    }
    {
        int hy = fY ? iadd(yp, imul(kPrimeY, 2)) : yp;
        hy = fXY ? hy : iadd(hy, -kPrimeY);
        const float dx = fY ? dxB - (float)(2 * kUnskew2) : dxB;
        const float dy = dyB - (fY ? (float)(1 + 2 * kUnskew2) : -1.0f);
        const float f = fmaxf(fmaf(-dx, dx, fmaf(-dy, dy, (float)kR2)), 0.0f);
        const float d[2] = {dx, dy};
        wvec<2>(gop, hash(seed, fXY ? iadd(xp, kPrimeX) : xp, hy), d, pow4(f), v);
    }
}

// closest-vertex search of the super-simplex warps: one candidate
FND void ws_consider(float& maxScore, int& bits, float score, int b)
{
    bits = score > maxScore ? b : bits;
    maxScore = fmax_(maxScore, score);
}

// DomainWarpSuperSimplex::Warp_3D (:1220-1446)
FND void ws_super3(bool gop, int seed, const float* p, float* v)
{
    constexpr double kSkew3 = 1.0 / 3.0, kRU3 = -1.0 / 2.0, kTU3 = -1.0 / 4.0, kDA = 3.0 / 4.0, kDB = 1.0, kR2 = kDA;
    const float x = p[0], y = p[1], z = p[2];
    const float skewDelta = (float)kSkew3 * (x + y + z);
    const float xs = x + skewDelta, ys = y + skewDelta, zs = z + skewDelta;
    float b[3] = {floorf(xs), floorf(ys), floorf(zs)};
    float ds[3] = {xs - b[0], ys - b[1], zs - b[2]};
    {
        const float tu = (float)kTU3 * (ds[0] + ds[1] + ds[2]);
        const float xN = ds[0] + tu, yN = ds[1] + tu, zN = ds[2] + tu, xyzN = -tu;
        float maxScore = 0.375f;
        int bits = xyzN > maxScore ? -1 : 0;
        maxScore = fmax_(maxScore, xyzN);
        ws_consider(maxScore, bits, xN, 1);
        ws_consider(maxScore, bits, yN, 2);
        ws_consider(maxScore, bits, zN, 4);
        maxScore = maxScore + (0.125f - xyzN);
        ws_consider(maxScore, bits, -zN, 3);
        ws_consider(maxScore, bits, -yN, 5);
        ws_consider(maxScore, bits, -xN, 6);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const bool m = (bits >> k) & 1;
            b[k] = m ? b[k] + 1.0f : b[k];
            ds[k] = m ? ds[k] - 1.0f : ds[k];
        }
    }
    int pb[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) pb[k] = imul(cvti(b[k]), kPrimes[k]);
    const float scs = ds[0] + ds[1] + ds[2];
    const float tu = (float)kTU3 * scs;
    const float n[3] = {ds[0] + tu, ds[1] + tu, ds[2] + tu};
    const float xyzN = -tu;
    const float ud = (float)kRU3 * scs;
    const float dB[3] = {ds[0] + ud, ds[1] + ud, ds[2] + ud};
    const float cs = (float)(1 + 3 * kRU3) * scs;
    v[0] = 0.0f; v[1] = 0.0f; v[2] = 0.0f;
    const float fb0 = fmaf(-dB[2], dB[2], fmaf(-dB[1], dB[1], fmaf(-dB[0], dB[0], (float)kR2))) * 0.5f;
    const float stemA = fb0 - (float)(kDA * 0.5), stemB = fb0 - (float)(kDB * 0.5);
    wvec<3>(gop, hash(seed, pb[0], pb[1], pb[2]), dB, fb4(fb0), v);
    {   // <1,1,1> or <-1,-1,-1>
        const bool sm = xyzN < 0.0f;
        const float off = flipm((float)(3 * kRU3 + 1), sm);
        const float fb = fmaxf(fmaf(off, cs, stemA), 0.0f);
        int c[3];
        float d[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) { c[k] = iadd(pb[k], sm ? -kPrimes[k] : kPrimes[k]); d[k] = dB[k] - off; }
        wvec<3>(gop, hash(seed, c[0], c[1], c[2]), d, fb4(fb), v);
    }
    // <1,1,0>, <1,0,1>, <0,1,1> or their negatives: the axis left out is m
#pragma unroll
    for (int m = 2; m >= 0; --m) {
        const bool sm = xyzN < n[m];
        const float off0 = flipm((float)(2 * kRU3), sm);
        const float fb = fminf(flipm(dB[m], sm) - stemB, 0.0f);
        int c[3];
        float d[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            c[k] = k == m ? pb[k] : iadd(pb[k], sm ? -kPrimes[k] : kPrimes[k]);
            d[k] = k == m ? dB[k] - off0 : dB[k];
        }
        wvec<3>(gop, hash(seed, c[0], c[1], c[2]), d, fb4(fb), v);
    }
    // <1,0,0>, <0,1,0>, <0,0,1> or their negatives
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const bool sm = n[a] < 0.0f;
        const float off0 = flipm((float)kRU3, sm);
        const float fb = fmaxf(fmaf(off0, cs, stemA) + flipm(dB[a], sm), 0.0f);
        int c[3];
        float d[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            c[k] = k == a ? iadd(pb[k], sm ? -kPrimes[k] : kPrimes[k]) : pb[k];
            d[k] = k == a ? dB[k] + off0 : dB[k] - off0;
        }
        wvec<3>(gop, hash(seed, c[0], c[1], c[2]), d, fb4(fb), v);
    }
    if (gop) {
        const float dl = (float)(-2.0 / 3.0) * (v[0] + v[1] + v[2]);
        v[0] = v[0] + dl; v[1] = v[1] + dl; v[2] = v[2] + dl;
    }
}

// DomainWarpSuperSimplex::Warp_4D (:1448-1835): the sixteen vertices around the
// closest lattice vertex in the reference's order; a vertex is the set of axes
// it moves along (bit k = axis k), in the direction of its group's sign test.
FND void ws_super4(bool gop, int seed, const float* p, float* v)
{
    constexpr double kSkew4 = 1.0 / (kRoot5 + 1.0), kU4 = -1.0 / (kRoot5 + 5.0), kTU4 = -1.0 / 5.0;
    constexpr double kDA = 4.0 / 5.0, kDB = 6.0 / 5.0, kR2 = kDA;
    const float skewDelta = (float)kSkew4 * (p[0] + p[1] + p[2] + p[3]);
    float b[4], ds[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float sk = p[k] + skewDelta;
        b[k] = floorf(sk);
        ds[k] = sk - b[k];
    }
    {
        const float tu = (float)kTU4 * (ds[0] + ds[1] + ds[2] + ds[3]);
        float n[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) n[k] = ds[k] + tu;
        const float xyzwN = -tu;
        float maxScore = 0.6f - xyzwN;
        int bits = 0.2f > maxScore ? -1 : 0;
        maxScore = fmax_(maxScore, 0.2f);
        ws_consider(maxScore, bits, -n[3], 0x7);
        ws_consider(maxScore, bits, -n[2], 0xB);
        ws_consider(maxScore, bits, -n[1], 0xD);
        ws_consider(maxScore, bits, -n[0], 0xE);
        maxScore = maxScore + (xyzwN - 0.2f);
        ws_consider(maxScore, bits, n[0], 0x1);
        ws_consider(maxScore, bits, n[1], 0x2);
        ws_consider(maxScore, bits, n[2], 0x4);
        ws_consider(maxScore, bits, n[3], 0x8);
        maxScore = maxScore + (0.2f - n[0]);
        ws_consider(maxScore, bits, n[1], 0x3);
        ws_consider(maxScore, bits, n[2], 0x5);
        ws_consider(maxScore, bits, n[3], 0x9);
        maxScore = maxScore + n[0];
        ws_consider(maxScore, bits, n[1] + n[2], 0x6);
        maxScore = maxScore - n[3];
        ws_consider(maxScore, bits, n[1], 0xA);
        ws_consider(maxScore, bits, n[2], 0xC);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const bool m = (bits >> k) & 1;
            b[k] = m ? b[k] + 1.0f : b[k];
            ds[k] = m ? ds[k] - 1.0f : ds[k];
        }
    }
    int pb[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) pb[k] = imul(cvti(b[k]), kPrimes[k]);
    const float scs = ds[0] + ds[1] + ds[2] + ds[3];
    const float tu = (float)kTU4 * scs;
    float n[4], dB[4];
    const float ud = (float)kU4 * scs;
#pragma unroll
    for (int k = 0; k < 4; ++k) { n[k] = ds[k] + tu; dB[k] = ds[k] + ud; }
    const float xyzwN = -tu;
    const float cs = (float)(1 + 4 * kU4) * scs;
    v[0] = 0.0f; v[1] = 0.0f; v[2] = 0.0f; v[3] = 0.0f;
    const float fb0 = fmaf(-dB[3], dB[3], fmaf(-dB[2], dB[2], fmaf(-dB[1], dB[1], fmaf(-dB[0], dB[0], (float)kR2)))) * 0.5f;
    const float stemA = fb0 - (float)(kDA * 0.5), stemB = fb0 - (float)(kDB * 0.5);
    wvec<4>(gop, hash(seed, pb[0], pb[1], pb[2], pb[3]), dB, fb4(fb0), v);
    constexpr int order[15] = {0xF, 0x7, 0xB, 0xD, 0xE, 0x1, 0x3, 0x5, 0x9, 0x2, 0x6, 0xA, 0x4, 0xC, 0x8};
#pragma unroll
    for (int vi = 0; vi < 15; ++vi) {
        const int S = order[vi];
        const int cnt = (S & 1) + ((S >> 1) & 1) + ((S >> 2) & 1) + ((S >> 3) & 1);
        const int a = (S & 1) ? 0 : (S & 2) ? 1 : (S & 4) ? 2 : 3;             // lowest axis in S
        const int bb = (S >> (a + 1)) & 1 ? a + 1 : ((S >> (a + 2)) & 1 ? a + 2 : a + 3);   // second axis (pairs)
        const int missing = !(S & 8) ? 3 : !(S & 4) ? 2 : !(S & 2) ? 1 : 0;    // axis outside S (triples)
        bool sm;
        if (cnt == 4) sm = xyzwN < 0.0f;
        else if (cnt == 3) sm = xyzwN < n[missing];
        else if (cnt == 1) sm = n[a] < 0.0f;
        else sm = n[a] < -n[bb & 3];
        float off1, off0, fb;
        if (cnt == 4) {
            off1 = flipm((float)(4 * kU4 + 1), sm);
            off0 = off1;
            fb = fmaxf(fmaf(off1, cs, stemA), 0.0f);
        } else if (cnt == 3) {
            off1 = flipm((float)(3 * kU4 + 1), sm);
            off0 = flipm((float)(3 * kU4), sm);
            fb = fmaxf(fmaf(off1, cs, stemB) - flipm(dB[missing], sm), 0.0f);
        } else if (cnt == 1) {
            off1 = flipm((float)(kU4 + 1), sm);
            off0 = flipm((float)kU4, sm);
            fb = fmaxf(fmaf(off0, cs, stemA) + flipm(dB[a], sm), 0.0f);
        } else {
            off1 = flipm((float)(2 * kU4 + 1), sm);
            off0 = flipm((float)(2 * kU4), sm);
            fb = fmaxf(fmaf(off0, cs, stemB) + flipm(dB[a] + dB[bb & 3], sm), 0.0f);
        }
        int c[4];
        float d[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const bool in = (S >> k) & 1;
            c[k] = in ? iadd(pb[k], sm ? -kPrimes[k] : kPrimes[k]) : pb[k];
            d[k] = dB[k] - (in ? off1 : off0);
        }
        wvec<4>(gop, hash(seed, c[0], c[1], c[2], c[3]), d, fb4(fb), v);
    }
}

// DomainWarpSimplex / DomainWarpSuperSimplex ::Warp (:729-769, :1092-1129) on
// frequency-scaled positions `sp`: the vector noise, scaled by the bounding
// constant x axis scale, added to io with amplitude `amp`; returns |v|^2.
template <int D>
FND float warp_simplex(int seed, float amp, const float* sp, const float* axis, float* io, bool super, bool gop)
{
    float v[4];
    float bound;
    if (D == 2) {
        if (super) ws_super2(gop, seed, sp, v); else ws_simplex2(gop, seed, sp, v);
        bound = super ? (gop ? (float)(9.28993664146183 / 2.0) : 12.814453124999995f)
                      : (gop ? (float)(49.918426513671875 / 2.0) : 70.1480577066486f);
    } else if (D == 3) {
        if (super) ws_super3(gop, seed, sp, v); else ws_simplex3(gop, seed, sp, v);
        bound = super ? (gop ? (float)(144.736422163332608 / 1.4142135623730951) : 37.63698669623629f)
                      : (gop ? (float)(32.69428253173828125 / 1.4142135623730951) : 16.281631889139874f);
    } else {
        if (super) ws_super4(gop, seed, sp, v); else ws_simplex4(gop, seed, sp, v);
        bound = super ? (gop ? (float)(115.21625311930542 / 1.4142135623730951) : 48.80058117543753f)
                      : (gop ? (float)(33.653125584827855 / 1.4142135623730951) : 30.88161777516092f);
    }
#pragma unroll
    for (int k = 0; k < D; ++k) v[k] = v[k] * (bound * axis[k]);
#pragma unroll
    for (int k = 0; k < D; ++k) io[k] = fmaf(v[k], amp, io[k]);
    float r = v[0] * v[0];
#pragma unroll
    for (int k = 1; k < D; ++k) r = fmaf(v[k], v[k], r);
    return r;
}

// ---------------------------------------------------------------- basic generators

template <int D>
FND float white(int seed, const float* p)
{
    int h = seed;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        int b = __float_as_int(p[k]);
        h ^= imul(b ^ (b >> 16), kPrimes[k]);
    }
    return valcoord(h);
}

template <int D>
FND float checkerboard(const float* p, float freq)
{
    int v = 0;
#pragma unroll
    for (int k = 0; k < D; ++k) v ^= cvti(p[k] * freq);
    return __int_as_float((v & 1) << 30);
}

template <int D>
FND float sine_wave(const float* p, float freq)
{
    float t = sin_(p[D - 1] * freq);
#pragma unroll
    for (int k = D - 2; k >= 0; --k) t = sin_(p[k] * freq) * t;
    return t;
}

// ---------------------------------------------------------------- modifiers

FND void rotate_plane(int type, float& x, float& y, float& z)   // Modifiers.inl:354-388
{
    float nx = x, ny = y, nz = z;
    if (type == 0) {
        float xy = x + y;
        float s2 = xy * -0.211324865405187f;
        nz = z * 0.577350269189626f;
        nx = x + s2 - nz;
        ny = y + s2 - nz;
        nz = nz + xy * 0.577350269189626f;
    } else if (type == 1) {
        float xz = x + z;
        float s2 = xz * -0.211324865405187f;
        ny = y * 0.577350269189626f;
        nx = x + s2 - ny;
        nz = z + s2 - ny;
        ny = ny + xz * 0.577350269189626f;
    }
    x = nx; y = ny; z = nz;
}

// Terrace (Modifiers.inl:134-181).  recip = 1 + 1/smoothness (constant) or computed.
FND float terrace_smooth(float rounded, float source, float recip)
{
    float diff = rounded - source;
    bool neg = diff < 0.0f;
    diff = fabs_(diff);
    diff = 0.5f - diff;
    diff = diff * recip;
    diff = fmin_(diff, 0.5f);
    diff = neg ? 0.5f - diff : diff - 0.5f;
    return rounded + diff;
}

FND float min_smooth(float a, float b, float smooth)   // Blends.inl:130-141
{
    float sm = fmax_(1.17549435e-38f, fabs_(smooth));
    float h = fmax_(sm - fabs_(a - b), 0.0f);
    h = h * (1.0f / sm);
    return fmaf(-(1.0f / 6.0f), h * h * h * sm, fmin_(a, b));
}

FND float fade_t(float fade, float fmn, float fmx, int interp)   // Blends.inl:172-195
{
    float range = fmx - fmn;
    fade = (fade - fmn) / range;
    fade = fmax_(0.0f, fmin_(1.0f, fade));
    if (interp == 1) fade = hermite(fade);
    else if (interp == 2) fade = quintic(fade);
    return range == 0.0f ? 0.5f : fade;
}

FND float remap(float s, float fromMin, float fromMax, float toMin, float toMax, bool clampOut)
{
    float r = toMin + ((s - fromMin) / (fromMax - fromMin) * (toMax - toMin));
    if (clampOut) { r = fmax_(r, toMin); r = fmin_(r, toMax); }
    return r;
}

FND float ping_pong(float t)
{
    t = t - floorf(t * 0.5f) * 2.0f;
    return t < 1.0f ? t : 2.0f - t;
}

FND float to_rgba8(float s, float mn, float mx)   // Modifiers.inl:107-126
{
    s = fmin_(s, mx);
    s = fmax_(s, mn);
    s = s - mn;
    s = s * (255.0f / (mx - mn));
    int b = cvti(s);
    unsigned o = 0xFF000000u | (unsigned)b | ((unsigned)b << 8) | ((unsigned)b << 16);
    return __uint_as_float(o);
}

FND float signed_sqrt(float v)
{
    return __uint_as_float(__float_as_uint(sqrtf(fabs_(v))) | (__float_as_uint(v) & 0x80000000u));
}

}  // namespace fnd
