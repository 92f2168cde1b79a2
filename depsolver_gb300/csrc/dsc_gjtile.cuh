// dsc_gjtile.cuh -- 128 x 128 FP32 tiles of blocked Gauss-Jordan and block
// LU on the device (not exported): tile loads, scaled fp16 pairs of rows
// for the tensor-core updates, and the inversion of one diagonal tile in
// the registers of one CTA.
#pragma once

#include <cuda_fp16.h>

namespace dsc {

constexpr int kPB = 128;  // Gauss-Jordan / block-LU tile

// A 128 x 128 FP32 tile at base (element (a, b) at base[a * stride + b], b
// contiguous, 16-byte aligned rows) into shared memory through put(a, b,
// value): 16 float4 loads per thread (256 threads) issued before the stores.
template <typename Put>
__device__ __forceinline__ void load_tile128(const float *__restrict__ base, size_t stride, Put put)
{
    float4 v[16];
#pragma unroll
    for (int u = 0; u < 16; u++) {
        const int t = threadIdx.x + 256 * u, a = t >> 5, b = 4 * (t & 31);
        v[u] = *(const float4 *)(base + (size_t)a * stride + b);
    }
#pragma unroll
    for (int u = 0; u < 16; u++) {
        const int t = threadIdx.x + 256 * u, a = t >> 5, b = 4 * (t & 31);
        put(a, b, v[u].x);
        put(a, b + 1, v[u].y);
        put(a, b + 2, v[u].z);
        put(a, b + 3, v[u].w);
    }
}

// Shift of a row whose largest magnitude has FP32 biased exponent e (see
// scale_shift in the tensor-core product: largest entry to [2^14, 2^15)).
__device__ __forceinline__ int pre_shift(int e) { return e == 0 ? 0 : max(-100, min(100, 14 - (e - 127))); }

__device__ __forceinline__ float pre_pow2(int k) { return __int_as_float((127 + k) << 23); }

// One 128-value row v[0..127] (in shared memory, stride 1) to a scaled fp16
// pair at h, l and its factor; a warp per row.
__device__ __forceinline__ void pre_row_pair(const float *v, __half *h, __half *l, float *factor)
{
    const int lane = threadIdx.x & 31;
    int e = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) e = max(e, (__float_as_int(v[lane + 32 * q]) >> 23) & 0xFF);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
    const int sh = pre_shift(e);
    const float f = pre_pow2(sh);
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const float x = v[lane + 32 * q] * f;
        const __half a = __float2half_rn(x);
        h[lane + 32 * q] = a;
        l[lane + 32 * q] = __float2half_rn(x - __half2float(a));
    }
    if (lane == 0) *factor = pre_pow2(-sh);
}

// Threads of the CTA that inverts one tile (gj_invert_tile).
constexpr int kGjThreads = 1024;

// One pivot of gj_invert_tile: pivot j = 4 m + S (S a compile-time slot:
// row S of warp m holds row j, slot S of lane m holds column j).
template <int S>
__device__ __forceinline__ void gj_pivot_step(float (&a)[4][4], int m, float *pr, float tol, int *bad, int row0)
{
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (w == m) {
        // row j: a_jj from lane m, replaced by 1, the row divided by it
        const float pv = __shfl_sync(0xffffffffu, a[S][S], m);
        if (bad && l == 0 && !(fabsf(pv) > tol)) atomicMin(bad, row0 + 4 * m + S);
        const float inv = __frcp_rn(pv);
        float rv[4];
#pragma unroll
        for (int c = 0; c < 4; c++) rv[c] = (c == S && l == m ? 1.0f : a[S][c]) * inv;
        *(float4 *)&pr[4 * l] = make_float4(rv[0], rv[1], rv[2], rv[3]);
    }
    __syncthreads();
    const float4 q = *(const float4 *)&pr[4 * l];
    const float qv[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int r = 0; r < 4; r++) {
        const float f = __shfl_sync(0xffffffffu, a[r][S], m);  // a_ij of this row
        if (r == S && w == m) {
#pragma unroll
            for (int c = 0; c < 4; c++) a[r][c] = qv[c];
        } else {
            if (l == m) a[r][S] = 0.0f;
#pragma unroll
            for (int c = 0; c < 4; c++) a[r][c] = fmaf(-f, qv[c], a[r][c]);
        }
    }
}

// P (row-major, 128 x 128) = inverse of the tile at T (column-major: element
// (r, c) at T[c * ldt + r], 16-byte aligned columns) by Gauss-Jordan without
// pivoting, in one CTA of kGjThreads threads.  Warp w holds rows 4w .. 4w+3,
// lane l columns 4l .. 4l+3 of them: 16 values in registers.  Per pivot j
// the warp holding row j takes a_jj from the lane holding column j, replaces
// it by 1, divides the row by the pivot and publishes it in shared memory;
// after one barrier every other row i takes a_ic -= a_ij r_c with a_ij
// replaced by 0 first (a_ij read by shuffle from the lane that holds column
// j), and row j becomes the published row.  The pivot loop is unrolled by
// four so that the row and column slot of every pivot is a compile-time
// index.  The published rows alternate between two buffers by the parity of
// j, so one barrier a pivot suffices.  With bad not null, a pivot whose
// magnitude is at most tol sets *bad to row0 + j (the lowest such j wins)
// and the inversion goes on.
__device__ __forceinline__ void gj_invert_tile(const float *__restrict__ T, int ldt, float *__restrict__ P,
                                               float tol, int *bad, int row0)
{
    __shared__ __align__(16) float prow[2][kPB];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    float a[4][4];  // a[r][c] = A(4 w + r, 4 l + c)
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const float4 v = *(const float4 *)(T + (size_t)(4 * l + c) * ldt + 4 * w);
        a[0][c] = v.x;
        a[1][c] = v.y;
        a[2][c] = v.z;
        a[3][c] = v.w;
    }
    for (int m = 0; m < kPB / 4; m++) {
        gj_pivot_step<0>(a, m, prow[0], tol, bad, row0);
        gj_pivot_step<1>(a, m, prow[1], tol, bad, row0);
        gj_pivot_step<2>(a, m, prow[0], tol, bad, row0);
        gj_pivot_step<3>(a, m, prow[1], tol, bad, row0);
    }
#pragma unroll
    for (int r = 0; r < 4; r++)
        *(float4 *)(P + (size_t)(4 * w + r) * kPB + 4 * l) = make_float4(a[r][0], a[r][1], a[r][2], a[r][3]);
}

}  // namespace dsc
