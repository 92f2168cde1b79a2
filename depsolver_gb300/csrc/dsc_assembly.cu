// dsc_assembly.cu -- dense geometric matrix K of the collocation system.
//
// Restates the element loops of electricFormA_tria3/tria6
// (src/assembly_el.c:63-307) without the frequency: K[c][i] (column-major)
// holds C * int G N_c for conductor rows and int H N_c for interface rows.
//
// Regular pairs (row node not in the element) -- k_asm_regular:
//   CTA = 32 collocation rows x one group of 32 elements (Morton order).
//   Phase A: each warp takes one element at a time, lane = row; the 7-point
//   rule (src/kernelIntegrals.c:109-142, :231-282) gives nen values per
//   (row, element) pair, staged in shared memory as V[slot][row].
//   Phase B: each footprint node of the group sums its slots and writes one
//   coalesced 32-row segment of its K column (or of a partial-sum slot when
//   other groups touch the node too).
// Partial slots are added in group order by k_asm_fixup (deterministic).
// Singular pairs -- k_asm_singular: one warp per row, the row's elements in
// element order, quadrature points split over the lanes (dsc_singular.cuh).
#include "dsc_common.cuh"
#include "dsc_df32.cuh"
#include "dsc_internal.h"
#include "dsc_singular.cuh"
#include "dsc_singular_df.cuh"

namespace dsc {

// Shape-function values at the 7 points of the regular rule.
struct Shape7 {
    double v[kTriPts][6];
};

constexpr Shape7 make_shape(int nen)
{
    Shape7 s{};
    for (int q = 0; q < kTriPts; q++) {
        double l1 = kTri7.v[q][0], l2 = kTri7.v[q][1], l3 = 1.0 - l1 - l2;
        if (nen == 3) {
            s.v[q][0] = l1;
            s.v[q][1] = l2;
            s.v[q][2] = l3;
        } else {
            s.v[q][0] = l1 * (2.0 * l1 - 1.0);
            s.v[q][1] = 4.0 * l1 * l2;
            s.v[q][2] = l2 * (2.0 * l2 - 1.0);
            s.v[q][3] = 4.0 * l2 * l3;
            s.v[q][4] = l3 * (2.0 * l3 - 1.0);
            s.v[q][5] = 4.0 * l1 * l3;
        }
    }
    return s;
}

__constant__ Shape7 c_shape3 = make_shape(3);
__constant__ Shape7 c_shape6 = make_shape(6);

// The same values as double-FP32 pairs (hi = value rounded to FP32, lo = the
// rest).
struct Shape7df {
    float hi[kTriPts][6], lo[kTriPts][6];
};

constexpr Shape7df make_shape_df(int nen)
{
    Shape7df d{};
    const Shape7 s = make_shape(nen);
    for (int q = 0; q < kTriPts; q++)
        for (int k = 0; k < 6; k++) {
            d.hi[q][k] = (float)s.v[q][k];
            d.lo[q][k] = (float)(s.v[q][k] - (double)d.hi[q][k]);
        }
    return d;
}

__constant__ Shape7df c_shape3_df = make_shape_df(3);
__constant__ Shape7df c_shape6_df = make_shape_df(6);

template <int NEN>
__device__ __forceinline__ float2 shape_q_df(int q, int k)
{
    return NEN == 3 ? make_float2(c_shape3_df.hi[q][k], c_shape3_df.lo[q][k])
                    : make_float2(c_shape6_df.hi[q][k], c_shape6_df.lo[q][k]);
}

template <int NEN>
__device__ __forceinline__ double shape_q(int q, int k)
{
    return NEN == 3 ? c_shape3.v[q][k] : c_shape6.v[q][k];
}

// Quadrature points of every element: x, y, z and w_q * J_q.
template <int NEN>
__global__ void k_elem_qp(const double *__restrict__ X, const double *__restrict__ Y,
                          const double *__restrict__ Z, const int *__restrict__ elems, int E,
                          double *__restrict__ qp)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= E * kTriPts) return;
    int e = t / kTriPts, q = t % kTriPts;
    double Xe[NEN][3], N[NEN], XL[3];
#pragma unroll
    for (int k = 0; k < NEN; k++) {
        int v = elems[(size_t)e * NEN + k];
        Xe[k][0] = X[v];
        Xe[k][1] = Y[v];
        Xe[k][2] = Z[v];
    }
    double l1 = c_tri7[q][0], l2 = c_tri7[q][1];
    shape<NEN>(l1, l2, N);
    double J = map_point<NEN>(Xe, l1, l2, N, XL);
    double *o = qp + (size_t)t * 4;
    o[0] = XL[0];
    o[1] = XL[1];
    o[2] = XL[2];
    o[3] = c_tri7[q][2] * J;
}

struct AsmArgs {
    const double *X, *Y, *Z, *normals, *row_fac, *qp;
    const int *row_kind, *elems, *grp_elem, *fp_ptr, *fp_dest, *fp_sl_ptr;
    const uint16_t *fp_sl;
    int N, row_lo, row_hi;
    size_t ld, ldp;
};

// MODE 0: every row of the warp is a conductor row (G = 1/r);
// MODE 1: every row is an interface row (H = n.(x-y)/r^3); MODE 2: mixed.
template <int NEN, int MODE>
__device__ __forceinline__ void pair_regular_f64(const double *__restrict__ q7, double xi, double yi,
                                                 double zi, double nx, double ny, double nz,
                                                 bool isH, double *acc)
{
#pragma unroll
    for (int q = 0; q < kTriPts; q++) {
        const double *Q = q7 + q * 4;
        double dx = xi - Q[0], dy = yi - Q[1], dz = zi - Q[2];
        double r2 = dx * dx + dy * dy + dz * dz;
        double inv = rsqrt(r2);
        double w;
        if (MODE == 0) {
            w = Q[3] * inv;
        } else {
            double h = Q[3] * inv * inv * inv * (dx * nx + dy * ny + dz * nz);
            w = (MODE == 1 || isH) ? h : Q[3] * inv;
        }
#pragma unroll
        for (int k = 0; k < NEN; k++) acc[k] += w * shape_q<NEN>(q, k);
    }
}

template <int NEN>
__global__ void __launch_bounds__(128) k_asm_regular_f64(AsmArgs a, double *__restrict__ K,
                                                         double *__restrict__ P)
{
    constexpr int R = kRowTile, EG = kGroup;
    extern __shared__ double smem[];
    double *s_qp = smem;                                   // EG * 28
    double *s_V = smem + EG * kTriPts * 4;                 // EG * NEN * R
    int *s_nodes = (int *)(s_V + EG * NEN * R);            // EG * NEN
    const int g = blockIdx.y;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;

    for (int t = threadIdx.x; t < EG * kTriPts * 4; t += blockDim.x) {
        int e = a.grp_elem[g * EG + t / (kTriPts * 4)];
        s_qp[t] = e >= 0 ? a.qp[(size_t)e * kTriPts * 4 + t % (kTriPts * 4)] : 0.0;
    }
    for (int t = threadIdx.x; t < EG * NEN; t += blockDim.x) {
        int e = a.grp_elem[g * EG + t / NEN];
        s_nodes[t] = e >= 0 ? a.elems[(size_t)e * NEN + t % NEN] : -1;
    }
    __syncthreads();

    const int i = a.row_lo + blockIdx.x * R + lane;
    const bool valid = i < a.row_hi;
    const int ii = valid ? i : a.row_lo;
    const double xi = a.X[ii], yi = a.Y[ii], zi = a.Z[ii];
    const double nx = a.normals[3 * (size_t)ii], ny = a.normals[3 * (size_t)ii + 1],
                 nz = a.normals[3 * (size_t)ii + 2];
    const int kind = valid ? a.row_kind[ii] : 0;
    const double fac = a.row_fac[ii];
    const bool allG = __all_sync(0xffffffffu, kind == 0);
    const bool allH = __all_sync(0xffffffffu, kind == 1);

    for (int el = w; el < EG; el += 4) {
        double acc[NEN];
#pragma unroll
        for (int k = 0; k < NEN; k++) acc[k] = 0.0;
        const int *en = s_nodes + el * NEN;
        bool drop = en[0] < 0;
#pragma unroll
        for (int k = 0; k < NEN; k++) drop |= en[k] == i;
        if (en[0] >= 0) {
            const double *q7 = s_qp + el * kTriPts * 4;
            if (allG) pair_regular_f64<NEN, 0>(q7, xi, yi, zi, nx, ny, nz, false, acc);
            else if (allH) pair_regular_f64<NEN, 1>(q7, xi, yi, zi, nx, ny, nz, true, acc);
            else pair_regular_f64<NEN, 2>(q7, xi, yi, zi, nx, ny, nz, kind == 1, acc);
        }
#pragma unroll
        for (int k = 0; k < NEN; k++) s_V[(el * NEN + k) * R + lane] = drop ? 0.0 : fac * acc[k];
    }
    __syncthreads();

    const int f0 = a.fp_ptr[g], f1 = a.fp_ptr[g + 1];
    for (int j = f0 + w; j < f1; j += 4) {
        const int s0 = a.fp_sl_ptr[j], s1 = a.fp_sl_ptr[j + 1];
        double sum = 0.0;
        for (int m = s0; m < s1; m++) sum += s_V[a.fp_sl[m] * R + lane];
        const int dest = a.fp_dest[j];
        if (valid) {
            if (dest >= 0) K[(size_t)dest * a.ld + i] = sum;
            else P[(size_t)(-dest - 1) * a.ldp + (i - a.row_lo)] = sum;
        }
    }
}

// ---- the same regular pairs in double-FP32 on the FP32 pipes
// (about 2^-46 per operation instead of FP64's 2^-53; GB300 issues FP64 at
// 1/64 of the FP32 rate, and k_asm_regular_f64 runs at that FP64 roof).

// Quadrature points of every element as double-FP32: x, y, z, w_q J_q.
__global__ void k_qp_to_df(const double *__restrict__ qp, size_t n, float2 *__restrict__ out)
{
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n;
         t += (size_t)gridDim.x * blockDim.x)
        out[t] = df_from(qp[t]);
}

template <int NEN, int MODE>
__device__ __forceinline__ void pair_regular_df(const float2 *__restrict__ q7, float2 xi, float2 yi,
                                                float2 zi, float2 nx, float2 ny, float2 nz, bool isH,
                                                float2 *acc)
{
#pragma unroll
    for (int q = 0; q < kTriPts; q++) {
        const float2 *Q = q7 + q * 4;
        const float2 dx = df_sub(xi, Q[0]), dy = df_sub(yi, Q[1]), dz = df_sub(zi, Q[2]);
        const float2 r2 = df_add(df_add(df_sqr(dx), df_sqr(dy)), df_sqr(dz));
        const float2 inv = df_rsqrt(r2);
        float2 w;
        if (MODE == 0) {
            w = df_mul(Q[3], inv);
        } else {
            const float2 dot = df_add(df_add(df_mul(dx, nx), df_mul(dy, ny)), df_mul(dz, nz));
            const float2 h = df_mul(df_mul(Q[3], df_mul(df_sqr(inv), inv)), dot);
            w = (MODE == 1 || isH) ? h : df_mul(Q[3], inv);
        }
#pragma unroll
        for (int k = 0; k < NEN; k++) df_mac(acc[k], w, shape_q_df<NEN>(q, k));
    }
}

// As k_asm_regular_f64 (same tiles, footprints and partial slots), with the
// pair integrals in double-FP32; K and the partial slots stay FP64.
template <int NEN>
__global__ void __launch_bounds__(128) k_asm_regular_df32(AsmArgs a, const float2 *__restrict__ qpd,
                                                          double *__restrict__ K, double *__restrict__ P)
{
    constexpr int R = kRowTile, EG = kGroup;
    extern __shared__ double smem[];
    float2 *s_qp = (float2 *)smem;                          // EG * 28
    float2 *s_V = s_qp + EG * kTriPts * 4;                  // EG * NEN * R
    int *s_nodes = (int *)(s_V + EG * NEN * R);             // EG * NEN
    const int g = blockIdx.y;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;

    for (int t = threadIdx.x; t < EG * kTriPts * 4; t += blockDim.x) {
        const int e = a.grp_elem[g * EG + t / (kTriPts * 4)];
        s_qp[t] = e >= 0 ? qpd[(size_t)e * kTriPts * 4 + t % (kTriPts * 4)] : make_float2(0.f, 0.f);
    }
    for (int t = threadIdx.x; t < EG * NEN; t += blockDim.x) {
        const int e = a.grp_elem[g * EG + t / NEN];
        s_nodes[t] = e >= 0 ? a.elems[(size_t)e * NEN + t % NEN] : -1;
    }
    __syncthreads();

    const int i = a.row_lo + blockIdx.x * R + lane;
    const bool valid = i < a.row_hi;
    const int ii = valid ? i : a.row_lo;
    const float2 xi = df_from(a.X[ii]), yi = df_from(a.Y[ii]), zi = df_from(a.Z[ii]);
    const float2 nx = df_from(a.normals[3 * (size_t)ii]), ny = df_from(a.normals[3 * (size_t)ii + 1]),
                 nz = df_from(a.normals[3 * (size_t)ii + 2]);
    const int kind = valid ? a.row_kind[ii] : 0;
    const float2 fac = df_from(a.row_fac[ii]);
    const bool allG = __all_sync(0xffffffffu, kind == 0);
    const bool allH = __all_sync(0xffffffffu, kind == 1);

    for (int el = w; el < EG; el += 4) {
        float2 acc[NEN];
#pragma unroll
        for (int k = 0; k < NEN; k++) acc[k] = make_float2(0.f, 0.f);
        const int *en = s_nodes + el * NEN;
        bool drop = en[0] < 0;
#pragma unroll
        for (int k = 0; k < NEN; k++) drop |= en[k] == i;
        if (en[0] >= 0) {
            const float2 *q7 = s_qp + el * kTriPts * 4;
            if (allG) pair_regular_df<NEN, 0>(q7, xi, yi, zi, nx, ny, nz, false, acc);
            else if (allH) pair_regular_df<NEN, 1>(q7, xi, yi, zi, nx, ny, nz, true, acc);
            else pair_regular_df<NEN, 2>(q7, xi, yi, zi, nx, ny, nz, kind == 1, acc);
        }
#pragma unroll
        for (int k = 0; k < NEN; k++)
            s_V[(el * NEN + k) * R + lane] = drop ? make_float2(0.f, 0.f) : df_mul(fac, df_norm(acc[k]));
    }
    __syncthreads();

    const int f0 = a.fp_ptr[g], f1 = a.fp_ptr[g + 1];
    for (int j = f0 + w; j < f1; j += 4) {
        const int s0 = a.fp_sl_ptr[j], s1 = a.fp_sl_ptr[j + 1];
        float2 sum = make_float2(0.f, 0.f);
        for (int m = s0; m < s1; m++) sum = df_add(sum, s_V[a.fp_sl[m] * R + lane]);
        const int dest = a.fp_dest[j];
        if (valid) {
            if (dest >= 0) K[(size_t)dest * a.ld + i] = df_to(sum);
            else P[(size_t)(-dest - 1) * a.ldp + (i - a.row_lo)] = df_to(sum);
        }
    }
}

// ---- the regular pairs in FP32 (the mixed mode's far-field assembly):
// each element's quadrature points as FP32 offsets from its centroid, the
// row point's offset from the centroid from double-FP32 coordinates, so the
// differences x - y carry FP32's relative accuracy whatever the distance
// from the origin; about 1e-7 of each entry.  The centroid-relative form is
// also what makes near pairs safe (no cancellation of large coordinates).

// Per element: centroid (double-FP32 x, y, z) and the points' offsets from
// it, negated, with w_q J_q, in FP32, as four point pairs (q = 2p, 2p + 1)
// of two float4 each: {-x_q, -x_q+1, -y_q, -y_q+1}, {-z_q, -z_q+1, w_q,
// w_q+1}.  The eighth point is a pad of weight 0 far away (1e18: its 1 / r
// and 1 / r^3 stay finite or zero whatever the row point).
constexpr int kQpPairs = (kTriPts + 1) / 2;
constexpr float kQpPad = 1e18f;

__global__ void k_qp_local(const double *__restrict__ qp, int E, float2 *__restrict__ cen,
                           float4 *__restrict__ qloc)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const double *q = qp + (size_t)e * kTriPts * 4;
    double c[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int t = 0; t < kTriPts; t++)
#pragma unroll
        for (int d = 0; d < 3; d++) c[d] += q[4 * t + d];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const float2 cd = df_from(c[d] / kTriPts);
        cen[(size_t)e * 3 + d] = cd;
        c[d] = (double)cd.x + (double)cd.y;  // the centroid as the kernel sees it
    }
    float o[2 * kQpPairs][4];
#pragma unroll
    for (int t = 0; t < 2 * kQpPairs; t++) {
        const bool pt = t < kTriPts;
        o[t][0] = pt ? (float)(c[0] - q[4 * t]) : -kQpPad;
        o[t][1] = pt ? (float)(c[1] - q[4 * t + 1]) : 0.f;
        o[t][2] = pt ? (float)(c[2] - q[4 * t + 2]) : 0.f;
        o[t][3] = pt ? (float)q[4 * t + 3] : 0.f;
    }
#pragma unroll
    for (int p = 0; p < kQpPairs; p++) {
        const float *a = o[2 * p], *b = o[2 * p + 1];
        qloc[((size_t)e * kQpPairs + p) * 2] = make_float4(a[0], b[0], a[1], b[1]);
        qloc[((size_t)e * kQpPairs + p) * 2 + 1] = make_float4(a[2], b[2], a[3], b[3]);
    }
}

// FP32 to FP64 by integer operations (a register move, no FP64-pipe work):
// sign, exponent rebiased by 1023 - 127, significand shifted into place.
// Subnormal FP32 values (below 1.2e-38) become zero.
__device__ __forceinline__ double f32_widen(float v)
{
    const unsigned u = __float_as_uint(v);
    const unsigned e = (u >> 23) & 0xFFu;
    if (e == 0) return __hiloint2double((int)(u & 0x80000000u), 0);
    const unsigned e64 = e == 0xFFu ? 0x7FFu : e + 896u;
    return __hiloint2double((int)((u & 0x80000000u) | (e64 << 20) | ((u >> 3) & 0xFFFFFu)), (int)(u << 29));
}

template <int NEN>
__device__ __forceinline__ float shape_q_f(int q, int k)
{
    return NEN == 3 ? c_shape3_df.hi[q][k] : c_shape6_df.hi[q][k];
}

// The points in pairs on the packed FP32x2 pipe: per pair 15 instructions
// (3 FADD2, 1 FMUL2 + 2 FFMA2 for r^2, 2 MUFU, 1 FMUL2, NEN FFMA2) where
// two single points take 28; each shape function's two partial sums are
// added at the end.  S holds the shape values in point pairs.
template <int NEN, int MODE>
__device__ __forceinline__ void pair_regular_f32(const float4 *__restrict__ q8, float dx0, float dy0, float dz0,
                                                 float nx, float ny, float nz, bool isH,
                                                 const float2 (&S)[kQpPairs][NEN], float *acc)
{
    const float2 d0x = make_float2(dx0, dx0), d0y = make_float2(dy0, dy0), d0z = make_float2(dz0, dz0);
    float2 a2[NEN];
#pragma unroll
    for (int k = 0; k < NEN; k++) a2[k] = make_float2(0.f, 0.f);
#pragma unroll
    for (int p = 0; p < kQpPairs; p++) {
        const float4 A = q8[2 * p], B = q8[2 * p + 1];
        const float2 dx = __fadd2_rn(d0x, make_float2(A.x, A.y));
        const float2 dy = __fadd2_rn(d0y, make_float2(A.z, A.w));
        const float2 dz = __fadd2_rn(d0z, make_float2(B.x, B.y));
        const float2 wq = make_float2(B.z, B.w);
        const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
        const float2 inv = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
        float2 w;
        if (MODE == 0) {
            w = __fmul2_rn(wq, inv);
        } else {
            const float2 t = __ffma2_rn(dz, make_float2(nz, nz),
                                        __ffma2_rn(dy, make_float2(ny, ny), __fmul2_rn(dx, make_float2(nx, nx))));
            const float2 h = __fmul2_rn(__fmul2_rn(wq, __fmul2_rn(__fmul2_rn(inv, inv), inv)), t);
            w = (MODE == 1 || isH) ? h : __fmul2_rn(wq, inv);
        }
#pragma unroll
        for (int k = 0; k < NEN; k++) a2[k] = __ffma2_rn(w, S[p][k], a2[k]);
    }
#pragma unroll
    for (int k = 0; k < NEN; k++) acc[k] = a2[k].x + a2[k].y;
}

// Per-row data of the FP32 assembly, once per assembly (its conversions run
// on the FP64 pipe): x, y, z as double-FP32 pairs, the normal and the row
// factor in FP32.
struct RowF32 {
    float2 x, y, z;
    float nx, ny, nz, fac;
};

__global__ void k_rows_f32(const double *__restrict__ X, const double *__restrict__ Y, const double *__restrict__ Z,
                           const double *__restrict__ normals, const double *__restrict__ row_fac, int N,
                           RowF32 *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    RowF32 r;
    r.x = df_from(X[i]);
    r.y = df_from(Y[i]);
    r.z = df_from(Z[i]);
    r.nx = (float)normals[3 * (size_t)i];
    r.ny = (float)normals[3 * (size_t)i + 1];
    r.nz = (float)normals[3 * (size_t)i + 2];
    r.fac = (float)row_fac[i];
    out[i] = r;
}

// As k_asm_regular_df32 (same tiles, footprints and partial slots), with the
// pair integrals, the row factor and the footprint sums in FP32; K's
// entries widened to FP64, the partial slots kept in FP32 (k_asm_fixup_f32).
template <int NEN>
__global__ void __launch_bounds__(128) k_asm_regular_f32(AsmArgs a, const RowF32 *__restrict__ rows,
                                                         const float2 *__restrict__ cen,
                                                         const float4 *__restrict__ qloc, double *__restrict__ K,
                                                         float *__restrict__ P)
{
    constexpr int R = kRowTile, EG = kGroup;
    __shared__ float4 s_q[EG * 2 * kQpPairs];
    __shared__ float2 s_c[EG * 3];
    __shared__ float s_V[EG * NEN * R];
    __shared__ int s_nodes[EG * NEN];
    // the group's footprint lists (at most EG * NEN nodes and slots)
    __shared__ int s_ptr[EG * NEN + 1], s_dest[EG * NEN];
    __shared__ uint16_t s_sl[EG * NEN];
    const int g = blockIdx.y;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int f0 = a.fp_ptr[g], nfp = a.fp_ptr[g + 1] - f0;
    const int sl0 = a.fp_sl_ptr[f0], nsl = a.fp_sl_ptr[f0 + nfp] - sl0;
    for (int t = threadIdx.x; t <= nfp; t += blockDim.x) s_ptr[t] = a.fp_sl_ptr[f0 + t] - sl0;
    for (int t = threadIdx.x; t < nfp; t += blockDim.x) s_dest[t] = a.fp_dest[f0 + t];
    for (int t = threadIdx.x; t < nsl; t += blockDim.x) s_sl[t] = a.fp_sl[sl0 + t];

    constexpr int Q8 = 2 * kQpPairs;
    for (int t = threadIdx.x; t < EG * Q8; t += blockDim.x) {
        const int e = a.grp_elem[g * EG + t / Q8];
        s_q[t] = e >= 0 ? qloc[(size_t)e * Q8 + t % Q8] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    for (int t = threadIdx.x; t < EG * 3; t += blockDim.x) {
        const int e = a.grp_elem[g * EG + t / 3];
        s_c[t] = e >= 0 ? cen[(size_t)e * 3 + t % 3] : make_float2(0.f, 0.f);
    }
    float2 S[kQpPairs][NEN];
#pragma unroll
    for (int p = 0; p < kQpPairs; p++)
#pragma unroll
        for (int k = 0; k < NEN; k++)
            S[p][k] = make_float2(shape_q_f<NEN>(2 * p, k), 2 * p + 1 < kTriPts ? shape_q_f<NEN>(2 * p + 1, k) : 0.f);
    for (int t = threadIdx.x; t < EG * NEN; t += blockDim.x) {
        const int e = a.grp_elem[g * EG + t / NEN];
        s_nodes[t] = e >= 0 ? a.elems[(size_t)e * NEN + t % NEN] : -1;
    }
    __syncthreads();

    const int i = a.row_lo + blockIdx.x * R + lane;
    const bool valid = i < a.row_hi;
    const int ii = valid ? i : a.row_lo;
    const RowF32 rd = rows[ii];
    const float2 xi = rd.x, yi = rd.y, zi = rd.z;
    const float nx = rd.nx, ny = rd.ny, nz = rd.nz;
    const int kind = valid ? a.row_kind[ii] : 0;
    const float fac = rd.fac;
    const bool allG = __all_sync(0xffffffffu, kind == 0);
    const bool allH = __all_sync(0xffffffffu, kind == 1);

    for (int el = w; el < EG; el += 4) {
        float acc[NEN];
#pragma unroll
        for (int k = 0; k < NEN; k++) acc[k] = 0.f;
        const int *en = s_nodes + el * NEN;
        bool drop = en[0] < 0;
#pragma unroll
        for (int k = 0; k < NEN; k++) drop |= en[k] == i;
        if (en[0] >= 0) {
            // the row point relative to the centroid: both parts of each
            // double-FP32 coordinate, the high parts' difference first
            const float2 *c = s_c + el * 3;
            const float dx = (xi.x - c[0].x) + (xi.y - c[0].y);
            const float dy = (yi.x - c[1].x) + (yi.y - c[1].y);
            const float dz = (zi.x - c[2].x) + (zi.y - c[2].y);
            const float4 *q8 = s_q + el * Q8;
            if (allG) pair_regular_f32<NEN, 0>(q8, dx, dy, dz, nx, ny, nz, false, S, acc);
            else if (allH) pair_regular_f32<NEN, 1>(q8, dx, dy, dz, nx, ny, nz, true, S, acc);
            else pair_regular_f32<NEN, 2>(q8, dx, dy, dz, nx, ny, nz, kind == 1, S, acc);
        }
#pragma unroll
        for (int k = 0; k < NEN; k++) s_V[(el * NEN + k) * R + lane] = drop ? 0.f : fac * acc[k];
    }
    __syncthreads();

    for (int j = w; j < nfp; j += 4) {
        const int s0 = s_ptr[j], s1 = s_ptr[j + 1];
        float sum = 0.f;
        for (int m = s0; m < s1; m++) sum += s_V[s_sl[m] * R + lane];
        const int dest = s_dest[j];
        if (valid) {
            if (dest >= 0) K[(size_t)dest * a.ld + i] = f32_widen(sum);
            else P[(size_t)(-dest - 1) * a.ldp + (i - a.row_lo)] = sum;
        }
    }
}

// k_asm_fixup for FP32 partial slots: the sum in FP32, K in FP64.
__global__ void k_asm_fixup_f32(const int *__restrict__ fix_ptr, const int *__restrict__ fix_slot,
                                const int *__restrict__ fix_col, int n_fix, const float *__restrict__ P,
                                size_t ldp, double *__restrict__ K, size_t ld, int row_lo, int nrows)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    // four columns at a time, their slot loads interleaved (each column's
    // slots still summed in order): four dependent load chains in flight
    constexpr int U = 4;
    const int stride = gridDim.y;
    for (int b0 = blockIdx.y; b0 < n_fix; b0 += U * stride) {
        int lo[U], hi[U];
        int len = 0;
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int b = b0 + u * stride;
            lo[u] = b < n_fix ? fix_ptr[b] : 0;
            hi[u] = b < n_fix ? fix_ptr[b + 1] : 0;
            len = max(len, hi[u] - lo[u]);
        }
        float sum[U];
#pragma unroll
        for (int u = 0; u < U; u++) sum[u] = 0.f;
        for (int j = 0; j < len; j++) {
#pragma unroll
            for (int u = 0; u < U; u++)
                if (lo[u] + j < hi[u]) sum[u] += P[(size_t)fix_slot[lo[u] + j] * ldp + r];
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int b = b0 + u * stride;
            if (b < n_fix) K[(size_t)fix_col[b] * ld + row_lo + r] = f32_widen(sum[u]);
        }
    }
}

// K column of every node shared by several groups = sum of its slots in
// group order; nodes in no element get a zero column.
template <typename T>
__global__ void k_asm_fixup(const int *__restrict__ fix_ptr, const int *__restrict__ fix_slot,
                            const int *__restrict__ fix_col, int n_fix, const T *__restrict__ P,
                            size_t ldp, T *__restrict__ K, size_t ld, int row_lo, int nrows)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    for (int b = blockIdx.y; b < n_fix; b += gridDim.y) {
        T sum = 0;
        for (int t = fix_ptr[b]; t < fix_ptr[b + 1]; t++) sum += P[(size_t)fix_slot[t] * ldp + r];
        K[(size_t)fix_col[b] * ld + row_lo + r] = sum;
    }
}

// Singular pairs: warp per row, adds into K (FP64 sums, stored as T).
// Rows with row_grad[i] set (row_grad may be null) also store the gradient
// integral of each of their singular elements (warp_singular_H's FLAG 1
// sums, 3 NEN per tuple t of ne_ptr's numbering) at Wg + t * 3 NEN: the
// field's singular part at that node, taken from the same points as the
// row's H integral.  Summed as the reference sums them (the FP64 mode; the
// mixed mode takes k_asm_singular_df).
template <int NEN, typename T>
__global__ void __launch_bounds__(128) k_asm_singular(const double *__restrict__ X,
                                                      const double *__restrict__ Y,
                                                      const double *__restrict__ Z,
                                                      const double *__restrict__ normals,
                                                      const int *__restrict__ row_kind,
                                                      const double *__restrict__ row_fac,
                                                      const int *__restrict__ elems,
                                                      const int *__restrict__ ne_ptr,
                                                      const int *__restrict__ ne_elem,
                                                      const int *__restrict__ ne_pos, int row_lo,
                                                      int row_hi, T *__restrict__ K, size_t ld,
                                                      const int *__restrict__ row_grad,
                                                      double *__restrict__ Wg)
{
    const int i = row_lo + (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= row_hi) return;
    const bool grad = row_grad && row_grad[i];
    const double xe[3] = {X[i], Y[i], Z[i]};
    const double n[3] = {normals[3 * (size_t)i], normals[3 * (size_t)i + 1],
                         normals[3 * (size_t)i + 2]};
    const int kind = row_kind[i];
    // warp_singular_H already carries the reference's minus sign
    // (Int[k] -= ...), so interface rows take factor 1 here; conductor rows
    // take C = 1/(4 pi eps0).
    const double fac = kind == 0 ? row_fac[i] : 1.0;
    for (int t = ne_ptr[i]; t < ne_ptr[i + 1]; t++) {
        const int e = ne_elem[t], s = ne_pos[t] + 1;
        double Xe[NEN][3], out[NEN];
#pragma unroll
        for (int k = 0; k < NEN; k++) {
            int v = elems[(size_t)e * NEN + k];
            Xe[k][0] = X[v];
            Xe[k][1] = Y[v];
            Xe[k][2] = Z[v];
        }
        double g[4 * NEN];  // FLAG 2: out's values, then the gradient
        if (kind == 0) {
            warp_singular_G<NEN>(s, Xe, xe, out);
            if (grad) warp_singular_H<NEN, 1>(s, Xe, xe, n, g + NEN);
        } else if (grad) {
            warp_singular_H<NEN, 2>(s, Xe, xe, n, g);
#pragma unroll
            for (int k = 0; k < NEN; k++) out[k] = g[k];
        } else {
            warp_singular_H<NEN, 0>(s, Xe, xe, n, out);
        }
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < NEN; k++) {
                size_t o = (size_t)elems[(size_t)e * NEN + k] * ld + i;
                K[o] = (T)((double)K[o] + fac * out[k]);
            }
            if (grad)
#pragma unroll
                for (int j = 0; j < 3 * NEN; j++) Wg[(size_t)t * 3 * NEN + j] = g[NEN + j];
        }
        __syncwarp();
    }
}

// k_asm_singular<NEN, double, true> in double-FP32 (the mixed mode): node
// coordinates and normals from Xd / Nd (double-FP32, 3 per node), the
// integrals by warp_singular_G_df / warp_singular_H_df; lane k adds output
// k into K (FP64) and stores gradient entry k, so that each pair takes one
// FP64 operation per lane.
template <int NEN>
__global__ void __launch_bounds__(128) k_asm_singular_df(const float2 *__restrict__ Xd,
                                                         const float2 *__restrict__ Nd,
                                                         const int *__restrict__ row_kind,
                                                         const double *__restrict__ row_fac,
                                                         const int *__restrict__ elems,
                                                         const int *__restrict__ ne_ptr,
                                                         const int *__restrict__ ne_elem,
                                                         const int *__restrict__ ne_pos, int row_lo, int row_hi,
                                                         double *__restrict__ K, size_t ld,
                                                         const int *__restrict__ row_grad, double *__restrict__ Wg)
{
    const int i = row_lo + (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= row_hi) return;
    const bool grad = row_grad && row_grad[i];
    const float2 xe[3] = {Xd[3 * (size_t)i], Xd[3 * (size_t)i + 1], Xd[3 * (size_t)i + 2]};
    const float2 nd[3] = {Nd[3 * (size_t)i], Nd[3 * (size_t)i + 1], Nd[3 * (size_t)i + 2]};
    const int kind = row_kind[i];
    const double fac = kind == 0 ? row_fac[i] : 1.0;  // as in k_asm_singular
    for (int t = ne_ptr[i]; t < ne_ptr[i + 1]; t++) {
        const int e = ne_elem[t], s = ne_pos[t] + 1;
        float2 Xe[NEN][3];
        int v[NEN];
#pragma unroll
        for (int k = 0; k < NEN; k++) {
            v[k] = elems[(size_t)e * NEN + k];
#pragma unroll
            for (int d = 0; d < 3; d++) Xe[k][d] = Xd[3 * (size_t)v[k] + d];
        }
        float2 g[4 * NEN];  // out's values, then the gradient
        if (kind == 0) {
            warp_singular_G_df<NEN>(s, Xe, xe, g);
            if (grad) warp_singular_H_df<NEN, 1>(s, Xe, xe, nd, g + NEN);
        } else if (grad) {
            warp_singular_H_df<NEN, 2>(s, Xe, xe, nd, g);
        } else {
            warp_singular_H_df<NEN, 0>(s, Xe, xe, nd, g);
        }
        // every lane holds every sum: lane k takes value k
        float2 mine = g[0];
        int dst = v[0];
#pragma unroll
        for (int k = 1; k < NEN; k++)
            if (lane == k) {
                mine = g[k];
                dst = v[k];
            }
        if (lane < NEN) {
            double *o = K + (size_t)dst * ld + i;
            *o += fac * df_to(mine);
        }
        if (grad) {
            float2 gj = g[NEN];
#pragma unroll
            for (int j = 1; j < 3 * NEN; j++)
                if (lane == j) gj = g[NEN + j];
            if (lane < 3 * NEN) Wg[(size_t)t * 3 * NEN + lane] = df_to(gj);
        }
        __syncwarp();
    }
}

// Xd, Nd = the node coordinates and normals in double-FP32 (3 per node).
__global__ void k_nodes_df(const double *__restrict__ X, const double *__restrict__ Y,
                           const double *__restrict__ Z, const double *__restrict__ normals, int N,
                           float2 *__restrict__ Xd, float2 *__restrict__ Nd)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    Xd[3 * (size_t)i] = df_from(X[i]);
    Xd[3 * (size_t)i + 1] = df_from(Y[i]);
    Xd[3 * (size_t)i + 2] = df_from(Z[i]);
#pragma unroll
    for (int d = 0; d < 3; d++) Nd[3 * (size_t)i + d] = df_from(normals[3 * (size_t)i + d]);
}

static size_t regular_smem(int nen)
{
    return (size_t)kGroup * kTriPts * 4 * sizeof(double) +
           (size_t)kGroup * nen * kRowTile * sizeof(double) + (size_t)kGroup * nen * sizeof(int);
}

template <int NEN>
static int assemble_fp64_impl(const DeviceMesh &m, double *K, size_t ld, cudaStream_t st, Timer *tm,
                              int prec, AsmWorkspace *ws, const int *row_grad, double *Wg,
                              const std::function<int(const int **, double **)> *late)
{
    AsmWorkspace local;
    AsmWorkspace &w = ws ? *ws : local;
    const bool df32 = prec == kAsmDf32, f32 = prec == kAsmF32;
    DSC_LAUNCH(k_elem_qp<NEN><<<(m.E * kTriPts + 255) / 256, 256, 0, st>>>(m.x.p, m.y.p, m.z.p, m.elems.p, m.E,
                                                                  m.qp.p));
    DSC_CUDA(cudaGetLastError());
    DevBuf<float2> &qpd = w.qpd;
    if (df32) {
        DSC_TRY(qpd.alloc((size_t)m.E * kTriPts * 4));
        DSC_LAUNCH(k_qp_to_df<<<4 * 152, 256, 0, st>>>(m.qp.p, (size_t)m.E * kTriPts * 4, qpd.p));
    }
    if (f32) {
        DSC_TRY(w.cen.alloc((size_t)m.E * 3));
        DSC_TRY(w.qloc.alloc((size_t)m.E * 2 * kQpPairs));
        DSC_TRY(w.rows.alloc((size_t)m.N * sizeof(RowF32)));
        DSC_LAUNCH(k_qp_local<<<(m.E + 127) / 128, 128, 0, st>>>(m.qp.p, m.E, w.cen.p, w.qloc.p));
        DSC_LAUNCH(k_rows_f32<<<(m.N + 127) / 128, 128, 0, st>>>(m.x.p, m.y.p, m.z.p, m.normals.p, m.row_fac.p,
                                                                 m.N, (RowF32 *)w.rows.p));
    }
    // Partial-sum buffer: n_slots columns of a row chunk, at most ~1 GiB.
    const size_t budget = (size_t)1 << 30;
    int rc = m.N;
    if (m.n_slots > 0) {
        size_t per_row = (size_t)m.n_slots * sizeof(double);
        size_t fit = budget / per_row;
        if (fit < (size_t)rc) rc = (int)std::max<size_t>(kRowTile, fit / kRowTile * kRowTile);
    }
    DevBuf<double> &P = w.P;
    if (f32) DSC_TRY(w.P32.alloc((size_t)std::max(m.n_slots, 1) * rc));
    else DSC_TRY(P.alloc((size_t)std::max(m.n_slots, 1) * rc));
    const size_t smem = regular_smem(NEN);
    DSC_CUDA(cudaFuncSetAttribute(k_asm_regular_f64<NEN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    DSC_CUDA(cudaFuncSetAttribute(k_asm_regular_df32<NEN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    AsmArgs a{m.x.p, m.y.p, m.z.p, m.normals.p, m.row_fac.p, m.qp.p, m.row_kind.p, m.elems.p,
              m.grp_elem.p, m.fp_ptr.p, m.fp_dest.p, m.fp_sl_ptr.p, m.fp_sl.p, m.N, 0, 0, ld,
              (size_t)rc};
    if (prec != kAsmF64) {
        // the singular pairs' nodes and normals in double-FP32
        DSC_TRY(w.nodes_df.alloc((size_t)m.N * 6));
        DSC_LAUNCH(k_nodes_df<<<(m.N + 255) / 256, 256, 0, st>>>(m.x.p, m.y.p, m.z.p, m.normals.p, m.N,
                                                                w.nodes_df.p, w.nodes_df.p + 3 * (size_t)m.N));
    }
    for (int lo = 0; lo < m.N; lo += rc) {
        int hi = std::min(m.N, lo + rc);
        a.row_lo = lo;
        a.row_hi = hi;
        dim3 grid((hi - lo + kRowTile - 1) / kRowTile, m.G);
        {
            TimerScope ts(tm, kTAsmRegular, st);
            if (f32)
                DSC_LAUNCH(k_asm_regular_f32<NEN><<<grid, 128, 0, st>>>(a, (const RowF32 *)w.rows.p, w.cen.p, w.qloc.p,
                                                                        K, w.P32.p));
            else if (df32) DSC_LAUNCH(k_asm_regular_df32<NEN><<<grid, 128, smem, st>>>(a, qpd.p, K, P.p));
            else DSC_LAUNCH(k_asm_regular_f64<NEN><<<grid, 128, smem, st>>>(a, K, P.p));
            if (tm) tm->add_work(kTAsmRegular, (double)(hi - lo) * m.E);  // (row, element) pairs
        }
        DSC_CUDA(cudaGetLastError());
        if (m.n_fix > 0) {
            // each block walks many shared columns (a block per column would
            // be hundreds of thousands of tiny blocks)
            dim3 fg((hi - lo + 255) / 256, std::min(m.n_fix, 256));
            TimerScope ts(tm, kTAsmFixup, st);
            if (f32)
                DSC_LAUNCH(k_asm_fixup_f32<<<fg, 256, 0, st>>>(m.fix_ptr.p, m.fix_slot.p, m.fix_col.p, m.n_fix,
                                                               w.P32.p, (size_t)rc, K, ld, lo, hi - lo));
            else
                DSC_LAUNCH(k_asm_fixup<double><<<fg, 256, 0, st>>>(m.fix_ptr.p, m.fix_slot.p, m.fix_col.p,
                                                                   m.n_fix, P.p, (size_t)rc, K, ld, lo, hi - lo));
            DSC_CUDA(cudaGetLastError());
        }
        if (late) {
            DSC_TRY((*late)(&row_grad, &Wg));
            late = nullptr;
        }
        int warps = hi - lo;
        TimerScope ts(tm, kTAsmSingular, st);
        if (prec == kAsmF64) {
            DSC_LAUNCH(k_asm_singular<NEN, double><<<(warps * 32 + 127) / 128, 128, 0, st>>>(
                m.x.p, m.y.p, m.z.p, m.normals.p, m.row_kind.p, m.row_fac.p, m.elems.p, m.ne_ptr.p,
                m.ne_elem.p, m.ne_pos.p, lo, hi, K, ld, Wg ? row_grad : nullptr, Wg));
        } else {
            // the mixed mode: double-FP32 on the FP32 pipes
            DSC_LAUNCH(k_asm_singular_df<NEN><<<(warps * 32 + 127) / 128, 128, 0, st>>>(
                w.nodes_df.p, w.nodes_df.p + 3 * (size_t)m.N, m.row_kind.p, m.row_fac.p, m.elems.p, m.ne_ptr.p,
                m.ne_elem.p, m.ne_pos.p, lo, hi, K, ld, Wg ? row_grad : nullptr, Wg));
        }
        DSC_CUDA(cudaGetLastError());
    }
    // a local workspace is released at scope exit: wait for the kernels
    // that read it
    if (!ws) DSC_CUDA(cudaStreamSynchronize(st));
    return kOk;
}

int assemble_K_fp64(const DeviceMesh &m, double *K, size_t ld, cudaStream_t st, Timer *tm, int prec,
                    AsmWorkspace *ws, const int *row_grad, double *Wg,
                    const std::function<int(const int **, double **)> *late)
{
    return m.nen == 6 ? assemble_fp64_impl<6>(m, K, ld, st, tm, prec, ws, row_grad, Wg, late)
                      : assemble_fp64_impl<3>(m, K, ld, st, tm, prec, ws, row_grad, Wg, late);
}

}  // namespace dsc
