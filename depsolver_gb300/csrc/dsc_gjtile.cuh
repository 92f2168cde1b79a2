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

// P (row-major, 128 x 128) = inverse of the tile at T (column-major: element
// (r, c) at T[c * ldt + r], 16-byte aligned columns) by Gauss-Jordan without
// pivoting, in one CTA of 256 threads.  The tile lives in registers: thread
// (tr, tc) = (t / 16, t % 16) owns rows 8 tr .. 8 tr + 7 and columns
// 8 tc .. 8 tc + 7.  Per pivot j: the owners of column j publish it and
// replace it by the unit vector e_j; the owners of row j scale it by
// 1 / a_jj and publish it (a_jj becomes the reciprocal); then every thread
// takes a_rc -= a_rj a_jc (with a_jj's row left alone) on its 64 entries
// without branches.  Shared rows and columns alternate between two buffers
// by the parity of j: two barriers a pivot.  With bad not null, a pivot
// whose magnitude is at most tol sets *bad to row0 + j (the lowest such j
// wins) and the inversion goes on.
__device__ __forceinline__ void gj_invert_tile(const float *__restrict__ T, int ldt, float *__restrict__ P,
                                               float tol, int *bad, int row0)
{
    __shared__ __align__(16) float col[2][kPB], row[2][kPB];
    const int tr = threadIdx.x >> 4, tc = threadIdx.x & 15;
    float a[8][8];
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const float *src = T + (size_t)(8 * tc + c) * ldt + 8 * tr;
        const float4 lo = *(const float4 *)src, hi = *(const float4 *)(src + 4);
        a[0][c] = lo.x; a[1][c] = lo.y; a[2][c] = lo.z; a[3][c] = lo.w;
        a[4][c] = hi.x; a[5][c] = hi.y; a[6][c] = hi.z; a[7][c] = hi.w;
    }
    for (int j = 0; j < kPB; j++) {
        const int p = j & 1, jb = j >> 3, jo = j & 7;
        if (tc == jb) {
#pragma unroll
            for (int c = 0; c < 8; c++) {
                if (c != jo) continue;
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    col[p][8 * tr + i] = a[i][c];
                    a[i][c] = (8 * tr + i == j) ? 1.0f : 0.0f;
                }
            }
        }
        __syncthreads();
        if (tr == jb) {
            const float pv = col[p][j];
            if (bad && tc == 0 && !(fabsf(pv) > tol)) atomicMin(bad, row0 + j);
            const float piv = __frcp_rn(pv);
#pragma unroll
            for (int i = 0; i < 8; i++) {
                if (i != jo) continue;
#pragma unroll
                for (int c = 0; c < 8; c++) {
                    a[i][c] *= piv;
                    row[p][8 * tc + c] = a[i][c];
                }
            }
        }
        __syncthreads();
        const float4 f0 = *(const float4 *)&col[p][8 * tr], f1 = *(const float4 *)&col[p][8 * tr + 4];
        const float4 r0 = *(const float4 *)&row[p][8 * tc], r1 = *(const float4 *)&row[p][8 * tc + 4];
        float f[8] = {f0.x, f0.y, f0.z, f0.w, f1.x, f1.y, f1.z, f1.w};
        const float rv[8] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w};
#pragma unroll
        for (int i = 0; i < 8; i++) {
            if (8 * tr + i == j) f[i] = 0.0f;
#pragma unroll
            for (int c = 0; c < 8; c++) a[i][c] = fmaf(-f[i], rv[c], a[i][c]);
        }
    }
#pragma unroll
    for (int i = 0; i < 8; i++) {
        float *o = P + (size_t)(8 * tr + i) * kPB + 8 * tc;
        *(float4 *)o = make_float4(a[i][0], a[i][1], a[i][2], a[i][3]);
        *(float4 *)(o + 4) = make_float4(a[i][4], a[i][5], a[i][6], a[i][7]);
    }
}

}  // namespace dsc
