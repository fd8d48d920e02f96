/*
 * opcount.h -- counting scalar type for the oracle (TEST INFRASTRUCTURE).
 *
 * fn_oracle.c is written in the common subset of C and C++.  Compiled as C++
 * with -DOC_COUNT, its per-point float type `f32` becomes this class, whose
 * arithmetic and comparison operators increment a thread-local counter; the
 * FS-level helpers (fma, floor, convert, min/max, hash steps ...) add their own
 * ticks.  on_count_ops() then reports the FS-level operations one point of a
 * tree costs -- the algorithmic work figure of the compute roofline.
 */
#ifndef FN_OPCOUNT_H
#define FN_OPCOUNT_H
#include <stdint.h>

static thread_local unsigned long long oc_counter = 0;
#define OC_TICK(n) (oc_counter += (unsigned long long)(n))

struct f32 {
    float v;
    f32() = default;
    f32(float x) : v(x) {}
    explicit operator float() const { return v; }
};
static inline f32 operator+(f32 a, f32 b) { OC_TICK(1); return f32(a.v + b.v); }
static inline f32 operator-(f32 a, f32 b) { OC_TICK(1); return f32(a.v - b.v); }
static inline f32 operator*(f32 a, f32 b) { OC_TICK(1); return f32(a.v * b.v); }
static inline f32 operator/(f32 a, f32 b) { OC_TICK(1); return f32(a.v / b.v); }
static inline f32 operator-(f32 a) { OC_TICK(1); return f32(-a.v); }
static inline bool operator<(f32 a, f32 b) { OC_TICK(1); return a.v < b.v; }
static inline bool operator>(f32 a, f32 b) { OC_TICK(1); return a.v > b.v; }
static inline bool operator<=(f32 a, f32 b) { OC_TICK(1); return a.v <= b.v; }
static inline bool operator>=(f32 a, f32 b) { OC_TICK(1); return a.v >= b.v; }
static inline bool operator==(f32 a, f32 b) { OC_TICK(1); return a.v == b.v; }
static inline bool operator!=(f32 a, f32 b) { OC_TICK(1); return a.v != b.v; }

typedef int32_t i32;

#endif
