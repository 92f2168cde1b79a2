// dsc_gjtile.cuh -- 128 x 128 FP32 tiles of blocked Gauss-Jordan and block
// LU on the device (not exported): tile loads, scaled fp16 pairs of rows
// for the tensor-core updates, and the inversion of one diagonal tile in
// the registers of one CTA.
#pragma once

#include <cuda_fp16.h>

namespace dsc {

constexpr int kPB = 128;  // Gauss-Jordan / block-LU tile
// SMs that the rest of a look-ahead update (a persistent grid on a side
// stream) leaves free for the next step's pivot inverses and row blocks.
constexpr int kGjReserveSms = 16;

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
constexpr int kGjThreads = 512;

// 1 / x to within an ulp (the pivots of the FP32 factors and inverses,
// which iterative refinement or the Krylov solver correct).
__device__ __forceinline__ float gj_rcp(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// One pivot of warp m's elimination among its own eight rows: pivot
// 8 m + S, whose column is slot S & 3 of lane 2 m + (S >> 2).  The pivot
// comes from that lane; every lane scales its entries of row S (the pivot's
// own entry replaced by 1) and takes, for each other row r, a_rc -= a_rS r_c
// with a_rS read from that lane (and replaced by 0 there).
template <int S>
__device__ __forceinline__ void gj_own_pivot8(float (&a)[8][4], int m, float tol, int *bad, int row0)
{
    constexpr int C = S & 3;
    const int l = threadIdx.x & 31, L = 2 * m + (S >> 2);
    const float pv = __shfl_sync(0xffffffffu, a[S][C], L);
    if (bad && l == 0 && !(fabsf(pv) > tol)) atomicMin(bad, row0 + 8 * m + S);
    const float inv = gj_rcp(pv);
#pragma unroll
    for (int c = 0; c < 4; c++) a[S][c] = (c == C && l == L ? 1.0f : a[S][c]) * inv;
#pragma unroll
    for (int r = 0; r < 8; r++) {
        if (r == S) continue;
        const float f = __shfl_sync(0xffffffffu, a[r][C], L);
        if (l == L) a[r][C] = 0.0f;
#pragma unroll
        for (int c = 0; c < 4; c++) a[r][c] = fmaf(-f, a[S][c], a[r][c]);
    }
}

// P (row-major, 128 x 128) and PT (its transpose, row-major), each when not
// null, = inverse of the tile at T (column-major: element (r, c) at
// T[c * ldt + r], 16-byte aligned columns) by Gauss-Jordan without
// pivoting, eight pivots per block barrier, in one CTA of kGjThreads
// threads.  Warp w holds rows 8w .. 8w+7, lane l columns 4l .. 4l+3 of
// them: 32 values in registers.  Step m takes pivots 8m .. 8m+7, whose rows
// are warp m's and whose columns are lanes 2m and 2m+1's: warp m eliminates
// them among its own rows (gj_own_pivot8), which leaves those rows final
// for the step, and publishes them in shared memory; after one barrier
// every other warp takes the rank-8 update a_ic -= sum_q a_iq r_qc, its
// entries a_iq in the pivot columns read from shared memory (staged there
// by lanes 2m and 2m+1 at the end of the step before) and replaced by 0
// first.  The published rows alternate between two buffers by the parity
// of m.  With bad not null, a pivot whose magnitude is at most tol sets
// *bad to row0 + its row (the lowest such row wins) and the inversion goes
// on.
__device__ __forceinline__ void gj_invert_tile(const float *__restrict__ T, int ldt, float *__restrict__ P,
                                               float *__restrict__ PT, float tol, int *bad, int row0)
{
    constexpr int kW = kGjThreads / 32;                  // 16 warps of 8 rows
    __shared__ __align__(16) float prow[2][8][kPB];     // the published rows
    __shared__ __align__(16) float fsl[kW][8][8];       // per warp: its rows' entries in the step's pivot columns
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    float a[8][4];  // a[r][c] = A(8 w + r, 4 l + c)
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const float4 v0 = *(const float4 *)(T + (size_t)(4 * l + c) * ldt + 8 * w);
        const float4 v1 = *(const float4 *)(T + (size_t)(4 * l + c) * ldt + 8 * w + 4);
        a[0][c] = v0.x;
        a[1][c] = v0.y;
        a[2][c] = v0.z;
        a[3][c] = v0.w;
        a[4][c] = v1.x;
        a[5][c] = v1.y;
        a[6][c] = v1.z;
        a[7][c] = v1.w;
    }
    // step 0's pivot columns are lanes 0 and 1's
    if ((l >> 1) == 0) {
#pragma unroll
        for (int r = 0; r < 8; r++)
            *(float4 *)&fsl[w][r][4 * (l & 1)] = make_float4(a[r][0], a[r][1], a[r][2], a[r][3]);
    }
#pragma unroll 1
    for (int m = 0; m < kW; m++) {
        float(*pr)[kPB] = prow[m & 1];
        if (w == m) {
            gj_own_pivot8<0>(a, m, tol, bad, row0);
            gj_own_pivot8<1>(a, m, tol, bad, row0);
            gj_own_pivot8<2>(a, m, tol, bad, row0);
            gj_own_pivot8<3>(a, m, tol, bad, row0);
            gj_own_pivot8<4>(a, m, tol, bad, row0);
            gj_own_pivot8<5>(a, m, tol, bad, row0);
            gj_own_pivot8<6>(a, m, tol, bad, row0);
            gj_own_pivot8<7>(a, m, tol, bad, row0);
#pragma unroll
            for (int r = 0; r < 8; r++)
                *(float4 *)&pr[r][4 * l] = make_float4(a[r][0], a[r][1], a[r][2], a[r][3]);
        }
        __syncthreads();
        if (w != m) {
            if ((l >> 1) == m) {
#pragma unroll
                for (int r = 0; r < 8; r++)
#pragma unroll
                    for (int c = 0; c < 4; c++) a[r][c] = 0.0f;
            }
#pragma unroll
            for (int hq = 0; hq < 2; hq++) {
                float F[8][4];  // F[r][q] = A(8 w + r, 8 m + 4 hq + q) before the step
#pragma unroll
                for (int r = 0; r < 8; r++) {
                    const float4 v = *(const float4 *)&fsl[w][r][4 * hq];
                    F[r][0] = v.x;
                    F[r][1] = v.y;
                    F[r][2] = v.z;
                    F[r][3] = v.w;
                }
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    // packed FP32x2 FMAs (each half rounded as an FMA)
                    const float4 x = *(const float4 *)&pr[4 * hq + q][4 * l];
                    const float2 x01 = make_float2(x.x, x.y), x23 = make_float2(x.z, x.w);
#pragma unroll
                    for (int r = 0; r < 8; r++) {
                        const float2 nf = make_float2(-F[r][q], -F[r][q]);
                        float2 a01 = make_float2(a[r][0], a[r][1]), a23 = make_float2(a[r][2], a[r][3]);
                        a01 = __ffma2_rn(nf, x01, a01);
                        a23 = __ffma2_rn(nf, x23, a23);
                        a[r][0] = a01.x;
                        a[r][1] = a01.y;
                        a[r][2] = a23.x;
                        a[r][3] = a23.y;
                    }
                }
            }
        }
        // the next step's pivot columns, once every lane has read fsl[w]
        if (m + 1 < kW) {
            __syncwarp();
            if ((l >> 1) == m + 1) {
#pragma unroll
                for (int r = 0; r < 8; r++)
                    *(float4 *)&fsl[w][r][4 * (l & 1)] = make_float4(a[r][0], a[r][1], a[r][2], a[r][3]);
            }
        }
    }
    if (P) {
#pragma unroll
        for (int r = 0; r < 8; r++)
            *(float4 *)(P + (size_t)(8 * w + r) * kPB + 4 * l) = make_float4(a[r][0], a[r][1], a[r][2], a[r][3]);
    }
    if (PT) {
#pragma unroll
        for (int c = 0; c < 4; c++) {
            *(float4 *)(PT + (size_t)(4 * l + c) * kPB + 8 * w) = make_float4(a[0][c], a[1][c], a[2][c], a[3][c]);
            *(float4 *)(PT + (size_t)(4 * l + c) * kPB + 8 * w + 4) = make_float4(a[4][c], a[5][c], a[6][c], a[7][c]);
        }
    }
}

// Shared memory of gj_row_product.
constexpr int kGjRowXs = 36;  // row stride of the 32 X columns in shared memory (float4-aligned)
constexpr size_t kGjRowSmem = sizeof(float) * (kPB * kPB + kPB * kGjRowXs);

// R(kk, jj) = sum_q P(kk, q) X(q, j0 + jj) for 32 columns of one 128 x 128
// tile, by 256 threads: PT is P transposed (PT[q * 128 + kk] = P(kk, q)),
// X the tile, column-major with leading dimension ld (X(q, j) at
// X[j * ld + q]).  sm holds kGjRowSmem bytes; the result is left in
// T[jj * 129 + kk] (32 rows of 129 floats, in sm after P's copy) after a
// block barrier.  Thread (ty, tx) forms kk = 4 ty + u, jj = 4 tx + v
// (u, v < 4): per q one float4 of P's column and one of X's row.
__device__ __forceinline__ float *gj_row_product(const float *__restrict__ PT, const float *__restrict__ X,
                                                 size_t ld, int j0, float *sm)
{
    float *Ps = sm;              // Ps[q * 128 + kk] = P(kk, q)
    float *Xs = sm + kPB * kPB;  // Xs[q * kGjRowXs + jj] = X(q, j0 + jj)
#pragma unroll 4
    for (int u = 0; u < kPB * kPB / 4 / 256; u++) {
        const int t = threadIdx.x + 256 * u;
        *(float4 *)&Ps[4 * t] = *(const float4 *)&PT[4 * t];
    }
    {
        // lanes along q (coalesced columns of X), 16 values a thread
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        float v[16];
#pragma unroll
        for (int u = 0; u < 16; u++) {
            const int jj = warp + 8 * (u >> 2), q = lane + 32 * (u & 3);
            v[u] = X[(size_t)(j0 + jj) * ld + q];
        }
#pragma unroll
        for (int u = 0; u < 16; u++) {
            const int jj = warp + 8 * (u >> 2), q = lane + 32 * (u & 3);
            Xs[q * kGjRowXs + jj] = v[u];
        }
    }
    __syncthreads();
    const int ty = threadIdx.x >> 3, tx = threadIdx.x & 7;
    float acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
        for (int v = 0; v < 4; v++) acc[u][v] = 0.0f;
#pragma unroll 8
    for (int q = 0; q < kPB; q++) {
        const float4 p = *(const float4 *)&Ps[q * kPB + 4 * ty];
        const float4 x = *(const float4 *)&Xs[q * kGjRowXs + 4 * tx];
        const float pv[4] = {p.x, p.y, p.z, p.w}, xv[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
            for (int v = 0; v < 4; v++) acc[u][v] = fmaf(pv[u], xv[v], acc[u][v]);
    }
    __syncthreads();  // every read of Xs is done: T takes its place
    float *T = Xs;
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
        for (int v = 0; v < 4; v++) T[(4 * tx + v) * 129 + 4 * ty + u] = acc[u][v];
    __syncthreads();
    return T;
}

// The tile (column-major, leading dimension ld) as T[i * 129 + kk] = X(i,
// kk) (in sm, 128 rows of 129 floats) after a block barrier, by 256
// threads: lanes along i (coalesced columns), conflict-free stores.
__device__ __forceinline__ void gj_load_rows(const float *__restrict__ X, size_t ld, float *T)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll 1
    for (int kb = 0; kb < kPB; kb += 32) {
        float v[16];
#pragma unroll
        for (int u = 0; u < 16; u++) {
            const int kk = kb + warp + 8 * (u >> 2), i = lane + 32 * (u & 3);
            v[u] = X[(size_t)kk * ld + i];
        }
#pragma unroll
        for (int u = 0; u < 16; u++) {
            const int kk = kb + warp + 8 * (u >> 2), i = lane + 32 * (u & 3);
            T[i * 129 + kk] = v[u];
        }
    }
    __syncthreads();
}

}  // namespace dsc
