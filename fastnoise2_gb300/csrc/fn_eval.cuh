// fn_eval.cuh -- per-point driver pieces shared by the compiled interpreter
// kernels (fn_kernels.cu) and the run-time specialised kernels (fn_jit.cpp):
// root positions of the batch drivers, the min/max reductions and the
// order-preserving float encoding used for per-request min/max atomics.
#pragma once

#include "fn_device.cuh"
#include "fn_types.h"

namespace fne {

using fnd::cvtf;
using fnd::fmax_;
using fnd::fmin_;

// +infinity (a bit pattern, so that NVRTC, which lacks the compiler builtins, accepts it)
__device__ __forceinline__ float inf() { return __int_as_float(0x7f800000); }

// Root position of point i (Generator.inl:104-105, 160-162, 225-228, 295-297, 400-406).
__device__ __forceinline__ void root_position(const fn::PointArgs& a, long long i, float* R)
{
    i += a.base;
    if (a.src == fn::kSrcGrid) {
        long long r = i;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (k >= a.dim) break;
            long long ik = (k == a.dim - 1) ? r : r % a.count[k];
            r = (k == a.dim - 1) ? 0 : r / a.count[k];
            R[k] = fmaf(cvtf((int)ik), a.step[k], a.offset[k]);
        }
    } else if (a.src == fn::kSrcTileable) {
        const long long xi = i % a.count[0], yi = i / a.count[0];
        const float xf = cvtf((int)xi) * a.tmul[0];
        const float yf = cvtf((int)yi) * a.tmul[1];
        R[0] = fnd::cos_(xf) * a.tfreq[0];
        R[1] = fnd::cos_(yf) * a.tfreq[1];
        R[2] = fnd::sin_(xf) * a.tfreq[0];
        R[3] = fnd::sin_(yf) * a.tfreq[1];
    } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (k >= a.dim) break;
            R[k] = a.offset[k] + __ldg(a.pos[k] + i);
        }
    }
}

// n / count[k] with the precomputed magic numbers of PointArgs (exact for every
// 32-bit n): a multiply-high and shifts instead of an integer division.
__device__ __forceinline__ unsigned fast_div(unsigned n, unsigned m, unsigned s)
{
    if (s == 0u) return n;                       // divisor 1
    const unsigned t = __umulhi(n, m);
    return (t + ((n - t) >> 1)) >> (s - 1u);
}

// root_position for a known dimensionality and requests below 2^32 points:
// 32-bit index arithmetic, same positions bit for bit.
template <int D>
__device__ __forceinline__ void root_position32(const fn::PointArgs& a, unsigned i, float* R)
{
    i += a.base;
    if (a.src == fn::kSrcGrid) {
        unsigned r = i;
#pragma unroll
        for (int k = 0; k < D - 1; ++k) {
            const unsigned q = fast_div(r, a.divm[k], a.divs[k]);
            const unsigned ik = r - q * (unsigned)a.count[k];
            r = q;
            R[k] = fmaf(cvtf((int)ik), a.step[k], a.offset[k]);
        }
        R[D - 1] = fmaf(cvtf((int)r), a.step[D - 1], a.offset[D - 1]);
    } else if (D == 4 && a.src == fn::kSrcTileable) {
        const unsigned q = fast_div(i, a.divm[0], a.divs[0]);
        const float xf = cvtf((int)(i - q * (unsigned)a.count[0])) * a.tmul[0];
        const float yf = cvtf((int)q) * a.tmul[1];
        R[0] = fnd::cos_(xf) * a.tfreq[0];
        R[1] = fnd::cos_(yf) * a.tfreq[1];
        R[2 % D] = fnd::sin_(xf) * a.tfreq[0];
        R[3 % D] = fnd::sin_(yf) * a.tfreq[1];
    } else {
#pragma unroll
        for (int k = 0; k < D; ++k) R[k] = a.offset[k] + __ldg(a.pos[k] + i);
    }
}

// OutputMinMax::operator<< (Generator.h:91-96): NaN never replaces.
__device__ __forceinline__ void fold(float v, float& mn, float& mx)
{
    mn = v < mn ? v : mn;
    mx = mx < v ? v : mx;
}

__device__ __forceinline__ void warp_minmax(float& mn, float& mx)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn = fmin_(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmax_(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
}

// Block-wide min/max (result valid in thread 0).  `smn`/`smx` hold one slot per warp.
__device__ __forceinline__ void block_minmax(float& mn, float& mx, float* smn, float* smx)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    warp_minmax(mn, mx);
    if (lane == 0) { smn[warp] = mn; smx[warp] = mx; }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) { mn = fmin_(mn, smn[w]); mx = fmax_(mx, smx[w]); }
}

// Order-preserving float <-> uint encoding for atomicMin / atomicMax.
__device__ __forceinline__ unsigned int enc_ordered(float f)
{
    const unsigned int b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float dec_ordered(unsigned int u)
{
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

// Per-launch min/max: each block folds its result into the workspace keys with
// two atomics; the block that counts itself last decodes them (no per-block
// partials to re-read) and clears the workspace for the next launch.  A block
// without a non-NaN output folds nothing, so an all-NaN launch gives (+inf, -inf).
__device__ __forceinline__ void grid_minmax(float mn, float mx, fn::MinMaxWork* work, float* dminmax, float* smn, float* smx)
{
    block_minmax(mn, mx, smn, smx);
    if (threadIdx.x != 0) return;
    if (mn <= mx) {
        atomicMax(&work->mn_key, ~enc_ordered(mn));
        atomicMax(&work->mx_key, enc_ordered(mx));
    }
    __threadfence();
    if (atomicAdd(&work->counter, 1u) != gridDim.x - 1) return;
    __threadfence();
    const unsigned int a = atomicExch(&work->mn_key, 0u), b = atomicExch(&work->mx_key, 0u);
    const float fmn = a == 0u ? inf() : dec_ordered(~a);
    const float fmx = b == 0u ? -inf() : dec_ordered(b);
    work->result[0] = fmn;
    work->result[1] = fmx;
    if (dminmax) { dminmax[0] = fmn; dminmax[1] = fmx; }
    work->counter = 0;
}

// Fold one finished tile's min/max into its request; the tile that completes
// the request publishes the result (device, and mapped host memory).
__device__ __forceinline__ void finish_tile(const fn::BatchRequest& rq, fn::BatchState* st, fn::BatchHeader* hdr, float mn, float mx)
{
    if (mn <= mx) {
        atomicMin(&st->mn_enc, enc_ordered(mn));
        atomicMax(&st->mx_enc, enc_ordered(mx));
    }
    __threadfence();
    const unsigned int done = atomicAdd(&st->tiles_done, 1u);
    if (done + 1 == rq.n_tiles) {
        __threadfence();
        const unsigned int me = atomicAdd(&st->mn_enc, 0u), xe = atomicAdd(&st->mx_enc, 0u);
        const float fmn = me == 0xFFFFFFFFu ? inf() : dec_ordered(me);
        const float fmx = xe == 0u ? -inf() : dec_ordered(xe);
        if (rq.minmax) { rq.minmax[0] = fmn; rq.minmax[1] = fmx; }
        if (rq.host_minmax) {
            volatile float* hm = rq.host_minmax;
            hm[0] = fmn;
            hm[1] = fmx;
        }
        if (rq.host_time) {
            unsigned long long t;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
            *(volatile unsigned long long*)rq.host_time = t;
        }
        __threadfence_system();
        if (rq.host_done) atomicExch_system(rq.host_done, 1u);
        atomicAdd(&hdr->requests_done, 1u);
    }
}

}  // namespace fne
