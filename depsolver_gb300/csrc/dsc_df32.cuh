// dsc_df32.cuh -- double-FP32 arithmetic for the Krylov vectors of the
// mixed sweep.
//
// A value is the unevaluated sum hi + lo of two floats (a float2: x = hi,
// y = lo), a 48-bit significand.  Products are made exact with an FMA
// (Dekker's product via fma: p = a*b, e = fma(a, b, -p)), sums with Knuth's
// TwoSum; the cross terms hi*lo and lo*hi go into the low part and lo*lo is
// dropped.  An accumulator keeps its error terms in .y without
// renormalising; it is renormalised once at the end (df_norm), which keeps
// the error of a length-n sum near n * 2^-48 of its largest partial sum.
//
// These run on the FP32 pipes, which on sm_103a issue 64 times as many
// operations per clock as the FP64 pipe.  The _rn intrinsics stop the
// compiler from contracting the error-free transforms into FMAs.
#pragma once

#include <cuda_runtime.h>

namespace dsc {

__device__ __forceinline__ float2 df_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return make_float2(s, e);
}

// (hi, lo) with |lo| <= ulp(hi) / 2, for |a| >= |b| or a == 0
__device__ __forceinline__ float2 df_fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ float2 df_norm(float2 a)
{
    return df_two_sum(a.x, a.y);
}

// acc += a * b
__device__ __forceinline__ void df_mac(float2 &acc, float2 a, float2 b)
{
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    const float2 s = df_two_sum(acc.x, p);
    acc.x = s.x;
    acc.y = __fadd_rn(acc.y, __fadd_rn(s.y, e));
}

// a * b, renormalised
__device__ __forceinline__ float2 df_mul(float2 a, float2 b)
{
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    return df_fast_two_sum(p, e);
}

__device__ __forceinline__ float2 df_add(float2 a, float2 b)
{
    const float2 s = df_two_sum(a.x, b.x);
    return df_fast_two_sum(s.x, __fadd_rn(s.y, __fadd_rn(a.y, b.y)));
}

__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }

__device__ __forceinline__ float2 df_sub(float2 a, float2 b) { return df_add(a, df_neg(b)); }

// a * a, renormalised
__device__ __forceinline__ float2 df_sqr(float2 a)
{
    const float p = __fmul_rn(a.x, a.x);
    float e = __fmaf_rn(a.x, a.x, -p);
    e = __fmaf_rn(2.0f * a.x, a.y, e);
    return df_fast_two_sum(p, e);
}

// 1 / sqrt(a) for a > 0: an FP32 seed refined by one FP32 Newton step
// (relative error about 2^-23), then one Newton step y <- y + y (1 - a
// y^2) / 2 with a y^2 in double-FP32 (which squares it: about 2^-45).
__device__ __forceinline__ float2 df_rsqrt(float2 a)
{
    float y0 = rsqrtf(a.x);
    y0 = y0 * (1.5f - 0.5f * a.x * y0 * y0);
    float2 y = make_float2(y0, 0.0f);
    const float2 t = df_mul(a, df_sqr(y));
    const float u = __fsub_rn(__fsub_rn(1.0f, t.x), t.y);  // 1 - t.x is exact
    y = df_add(y, df_mul(y, make_float2(0.5f * u, 0.0f)));
    return y;
}

// FP64 <-> double-FP32 (these conversions run on the FP64 pipe: use them
// per block or per system, not per element, in the streaming kernels)
__device__ __forceinline__ float2 df_from(double v)
{
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
}

__device__ __forceinline__ double df_to(float2 a) { return (double)a.x + (double)a.y; }

// a = hi + lo with hi = (float)a (round to nearest; one FP64-pipe
// conversion) and lo = a - hi (exact in FP64, at most 2^-24 |a|) rounded to
// FP32, without further FP64 operations: the difference of the two
// significands, in units of a's last place, fits in 29 bits and equals the
// low word of a minus hi's low three significand bits shifted to a's
// weights (two's complement, also when rounding carried into the next
// binade).  lo is 0 for |a| below 2^-74.
__device__ __forceinline__ void f64_split_rn(double a, float &hi, float &lo)
{
    hi = (float)a;
    const unsigned hw = (unsigned)__double2hiint(a), lw = (unsigned)__double2loint(a);
    const int E = (int)((hw >> 20) & 0x7FFu);                          // biased FP64 exponent
    const int d = (int)(lw - ((__float_as_uint(hi) & 7u) << 29));    // a - hi in units of 2^(E - 1075)
    const float m = (float)(((int)hw < 0) ? -d : d);                   // with a's sign
    lo = E >= 949 ? m * __int_as_float((E - 1075 + 127) << 23) : 0.0f;
}

// Warp-wide sum of accumulators (fixed shuffle order).
__device__ __forceinline__ float2 df_warp_sum(float2 v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        float2 u;
        u.x = __shfl_xor_sync(0xffffffffu, v.x, o);
        u.y = __shfl_xor_sync(0xffffffffu, v.y, o);
        const float2 s = df_two_sum(v.x, u.x);
        v.x = s.x;
        v.y = __fadd_rn(s.y, __fadd_rn(v.y, u.y));
    }
    return v;
}

// Block-wide sum (blockDim.x a multiple of 32, at most 32 warps): warps by
// shuffles, then thread 0 adds the warps in order in FP64.  The result is
// valid in thread 0; sh holds one float2 per warp.  Every thread must call.
__device__ __forceinline__ double df_block_sum(float2 v, float2 *sh)
{
    v = df_warp_sum(v);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += df_to(sh[w]);
    return t;
}

}  // namespace dsc
