// dsc_singular_df.cuh -- the mixed mode's singular element integrals in
// double-FP32 on the FP32 pipes.
//
// The integrals of warp_singular_G / warp_singular_H (dsc_singular.cuh:
// the same points, weights, node rotation and sums) with the element's map
// written as a polynomial about its node at local (0, 0) -- X = k0 + k1 l1 +
// k2 l2 (+ d11 l1^2 / 2 + k12 l1 l2 + d22 l2^2 / 2 for tria6), tangents
// dX/dl1 = k1 + d11 l1 + k12 l2, dX/dl2 = k2 + k12 l1 + d22 l2, and X - k0
// = (l1 (t1 + k1) + l2 (t2 + k2)) / 2, so that a point's offset from the
// collocation point comes from the tangents without cancellation -- and
// |J| / r^k from one reciprocal square root, taken in double-FP32 (a
// 48-bit significand, dsc_df32.cuh): about 1e-13 of the FP64 values, at a
// fraction of the FP64 pipe's time (the FP32 pipes issue 64 times as many
// operations per clock on sm_103a).  The node coordinates and normals come
// in double-FP32 (converted once per assembly), the element's polynomial is
// formed from them in double-FP32, and the sums go back in double-FP32
// (every lane holds them): nothing per point or per pair runs on the FP64
// pipe.  Each pair is evaluated in coordinates scaled by a power of two
// near the element's size, so that r^6 J^2 stays inside FP32's exponent
// range for meshes in any unit; G comes back times that power of two, H
// and the gradient are scale-free.
#pragma once

#include "dsc_common.cuh"
#include "dsc_df32.cuh"
#include "dsc_singular.cuh"

namespace dsc {

// a * b for a float b, renormalised
__device__ __forceinline__ float2 df_mulf(float2 a, float b)
{
    const float p = __fmul_rn(a.x, b);
    float e = __fmaf_rn(a.x, b, -p);
    e = __fmaf_rn(a.y, b, e);
    return df_fast_two_sum(p, e);
}

// a * s for a power of two s (exact)
__device__ __forceinline__ float2 df_pow2(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

// (hi, lo) of a double at compile time
struct DfC {
    float hi, lo;
};
constexpr DfC df_c(double v) { return {(float)v, (float)(v - (double)(float)v)}; }

// The quadrature tables in double-FP32: the 7-point rule's weights, the
// 8-point Gauss-Legendre and Gauss-Jacobi points and weights, and the
// subdivision's level-0 points (SubdivPts).
struct SingDfTables {
    DfC w7[kTriPts];
    DfC gl[kLinePts][2], gj[kLinePts][2];
    DfC l[3][kTriPts][2];
    DfC ab[3][3][kTriPts][4];
};

constexpr SingDfTables make_sing_df_tables()
{
    SingDfTables t{};
    const double gl[kLinePts][2] = {
        {-0.960289856497536, 0.101228536290370}, {-0.796666477413627, 0.222381034453376},
        {-0.525532409916329, 0.313706645877887}, {-0.183434642495650, 0.362683783378362},
        {0.183434642495650, 0.362683783378362},  {0.525532409916329, 0.313706645877887},
        {0.796666477413627, 0.222381034453376},  {0.960289856497536, 0.101228536290370}};
    const double gj[kLinePts][2] = {
        {-0.910732089420060, 0.0131807657689955}, {-0.711267485915709, 0.0713716106239446},
        {-0.426350485711139, 0.181757278018796},  {-0.0903733696068533, 0.316798397969277},
        {0.256135670833455, 0.424189437743720},   {0.571383041208738, 0.450023197883551},
        {0.817352784200412, 0.364476094545495},   {0.964440169705273, 0.178203217446225}};
    for (int q = 0; q < kTriPts; q++) t.w7[q] = df_c(kTri7.v[q][2]);
    for (int i = 0; i < kLinePts; i++)
        for (int c = 0; c < 2; c++) {
            t.gl[i][c] = df_c(gl[i][c]);
            t.gj[i][c] = df_c(gj[i][c]);
        }
    const SubdivPts sp = make_subdiv_pts();
    for (int i = 0; i < 3; i++)
        for (int q = 0; q < kTriPts; q++) {
            for (int c = 0; c < 2; c++) t.l[i][q][c] = df_c(sp.l[i][q][c]);
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 4; c++) t.ab[r][i][q][c] = df_c(sp.ab[r][i][q][c]);
        }
    return t;
}

__device__ const SingDfTables g_sing_df = make_sing_df_tables();

__device__ __forceinline__ float2 df_ld(const DfC &c)
{
    const float2 v = __ldg((const float2 *)&c);
    return v;
}

// The element's polynomial map in double-FP32 from the nodes in
// double-FP32, scaled by sc, a power of two near the element's size (from its first
// tangent: the factor that brings the pair's coordinates to order one).
template <int NEN>
struct ElemMapDf {
    float2 k0[3], k1[3], k2[3], d11[3], k12[3], d22[3];
    float sc;
    __device__ __forceinline__ void init(const float2 (*X)[3])
    {
#pragma unroll
        for (int d = 0; d < 3; d++) {
            if (NEN == 3) {
                k0[d] = X[2][d];
                k1[d] = df_sub(X[0][d], X[2][d]);
                k2[d] = df_sub(X[1][d], X[2][d]);
                d11[d] = k12[d] = d22[d] = make_float2(0.0f, 0.0f);
            } else {
                k0[d] = X[4][d];
                const float2 t3 = df_mulf(X[4][d], 3.0f);
                k1[d] = df_sub(df_sub(df_pow2(X[5][d], 4.0f), X[0][d]), t3);
                k2[d] = df_sub(df_sub(df_pow2(X[3][d], 4.0f), X[2][d]), t3);
                d11[d] = df_pow2(df_sub(df_add(X[0][d], X[4][d]), df_pow2(X[5][d], 2.0f)), 4.0f);
                k12[d] = df_pow2(df_sub(df_add(df_sub(X[1][d], X[3][d]), X[4][d]), X[5][d]), 4.0f);
                d22[d] = df_pow2(df_sub(df_add(X[2][d], X[4][d]), df_pow2(X[3][d], 2.0f)), 4.0f);
            }
        }
        const float h = fabsf(k1[0].x) + fabsf(k1[1].x) + fabsf(k1[2].x);
        int e = 0;
        frexpf(h > 0.0f ? h : 1.0f, &e);
        sc = ldexpf(1.0f, -e);
#pragma unroll
        for (int d = 0; d < 3; d++) {
            k1[d] = df_pow2(k1[d], sc);
            k2[d] = df_pow2(k2[d], sc);
            d11[d] = df_pow2(d11[d], sc);
            k12[d] = df_pow2(k12[d], sc);
            d22[d] = df_pow2(d22[d], sc);
        }
    }
    // e0 = (xe - k0) sc
    __device__ __forceinline__ void offset(const float2 *xe, float2 *e0) const
    {
#pragma unroll
        for (int d = 0; d < 3; d++) e0[d] = df_pow2(df_sub(xe[d], k0[d]), sc);
    }
    // dd = xe - X(l1, l2) given e0 = xe - k0; returns |t1 x t2|^2
    __device__ __forceinline__ float2 at_sq(float2 l1, float2 l2, const float2 *e0, float2 *dd) const
    {
        float2 t1[3], t2[3];
        const float2 h1 = df_pow2(l1, 0.5f), h2 = df_pow2(l2, 0.5f);
#pragma unroll
        for (int d = 0; d < 3; d++) {
            if (NEN == 3) {
                t1[d] = k1[d];
                t2[d] = k2[d];
                dd[d] = df_sub(e0[d], df_add(df_mul(l1, k1[d]), df_mul(l2, k2[d])));
            } else {
                t1[d] = df_add(df_add(df_mul(d11[d], l1), df_mul(k12[d], l2)), k1[d]);
                t2[d] = df_add(df_add(df_mul(k12[d], l1), df_mul(d22[d], l2)), k2[d]);
                dd[d] = df_sub(e0[d], df_add(df_mul(h1, df_add(t1[d], k1[d])), df_mul(h2, df_add(t2[d], k2[d]))));
            }
        }
        const float2 j1 = df_sub(df_mul(t1[1], t2[2]), df_mul(t2[1], t1[2]));
        const float2 j2 = df_sub(df_mul(t2[0], t1[2]), df_mul(t1[0], t2[2]));
        const float2 j3 = df_sub(df_mul(t1[0], t2[1]), df_mul(t2[0], t1[1]));
        return df_add(df_add(df_sqr(j1), df_sqr(j2)), df_sqr(j3));
    }
};

template <int NEN>
__device__ __forceinline__ void shape_df(float2 l1, float2 l2, float2 *N)
{
    const float2 one = make_float2(1.0f, 0.0f);
    const float2 l3 = df_sub(df_sub(one, l1), l2);
    if (NEN == 3) {
        N[0] = l1;
        N[1] = l2;
        N[2] = l3;
    } else {
        N[0] = df_mul(l1, df_sub(df_pow2(l1, 2.0f), one));
        N[1] = df_pow2(df_mul(l1, l2), 4.0f);
        N[2] = df_mul(l2, df_sub(df_pow2(l2, 2.0f), one));
        N[3] = df_pow2(df_mul(l2, l3), 4.0f);
        N[4] = df_mul(l3, df_sub(df_pow2(l3, 2.0f), one));
        N[5] = df_pow2(df_mul(l1, l3), 4.0f);
    }
}

__device__ __forceinline__ float2 df_dot3(const float2 *a, const float2 *b)
{
    return df_add(df_add(df_mul(a[0], b[0]), df_mul(a[1], b[1])), df_mul(a[2], b[2]));
}

// The Duffy maps of duffy() on double-FP32 (u1, u2); returns the
// sub-triangle count.
template <int NEN>
__device__ __forceinline__ int duffy_df(int s, float2 u1, float2 u2, float2 *La, float2 *Lb)
{
    const float2 one = make_float2(1.0f, 0.0f), half = make_float2(0.5f, 0.0f);
    const float2 p1 = df_add(one, u1), m1 = df_sub(one, u1), p2 = df_add(one, u2), m2 = df_sub(one, u2);
    const float2 q = df_pow2(df_mul(u1, p2), 0.25f);  // u1 (1 + u2) / 4
    if (NEN == 3) {
        if (s == 1) { La[0] = df_pow2(m2, 0.5f); La[1] = df_pow2(df_mul(p1, p2), 0.25f); }
        else if (s == 2) { La[0] = df_pow2(df_mul(m1, p2), 0.25f); La[1] = df_pow2(m2, 0.5f); }
        else { La[0] = df_pow2(df_mul(p1, p2), 0.25f); La[1] = df_pow2(df_mul(m1, p2), 0.25f); }
        return 1;
    }
    switch (s) {
    case 1: La[0] = df_pow2(m2, 0.5f); La[1] = df_pow2(df_mul(p1, p2), 0.25f); return 1;
    case 2:
        La[0] = df_pow2(m2, 0.25f); La[1] = df_add(half, q);
        Lb[0] = df_sub(half, q); Lb[1] = df_pow2(m2, 0.25f);
        return 2;
    case 3: La[0] = df_pow2(df_mul(m1, p2), 0.25f); La[1] = df_pow2(m2, 0.5f); return 1;
    case 4:
        La[0] = df_pow2(df_mul(p1, p2), 0.25f); La[1] = df_sub(half, q);
        Lb[0] = df_pow2(df_mul(m1, p2), 0.25f); Lb[1] = df_pow2(m2, 0.25f);
        return 2;
    case 5: La[0] = df_pow2(df_mul(p1, p2), 0.25f); La[1] = df_pow2(df_mul(m1, p2), 0.25f); return 1;
    default:
        La[0] = df_add(half, q); La[1] = df_pow2(df_mul(m1, p2), 0.25f);
        Lb[0] = df_pow2(m2, 0.25f); Lb[1] = df_pow2(df_mul(p1, p2), 0.25f);
        return 2;
    }
}

// warp_singular_G in double-FP32: out[k] (every lane) = sum
// over 8 x 8 (x2) points of w1 w2 J B N_k / r; X and xe in double-FP32.
template <int NEN>
__device__ void warp_singular_G_df(int s, const float2 (*X)[3], const float2 *xe, float2 *out)
{
    const int lane = threadIdx.x & 31;
    ElemMapDf<NEN> ed;
    ed.init(X);
    float2 e0[3];
    ed.offset(xe, e0);
    float2 acc[NEN];
#pragma unroll
    for (int k = 0; k < NEN; k++) acc[k] = make_float2(0.0f, 0.0f);
    float2 La[2], Lb[2], N[6], dd[3];
    const int T = duffy_df<NEN>(s, make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f), La, Lb);
    const float B = T == 1 ? 0.125f : 0.0625f;
    for (int p = lane; p < 64 * T; p += 32) {
        const int ij = p / T, t = p % T;
        const int i = ij / 8, j = ij % 8;
        const float2 u1 = df_ld(g_sing_df.gl[i][0]), w1 = df_ld(g_sing_df.gl[i][1]);
        const float2 u2 = df_ld(g_sing_df.gj[j][0]), w2 = df_ld(g_sing_df.gj[j][1]);
        duffy_df<NEN>(s, u1, u2, La, Lb);
        const float2 *L = t == 0 ? La : Lb;
        shape_df<NEN>(L[0], L[1], N);
        // |J| / r = J^2 / sqrt(J^2 r^2)
        const float2 j2 = ed.at_sq(L[0], L[1], e0, dd);
        const float2 rsq = df_dot3(dd, dd);
        const float2 jr = df_mul(j2, df_rsqrt(df_mul(j2, rsq)));
        const float2 A = df_pow2(df_mul(df_mul(w1, w2), jr), B);
#pragma unroll
        for (int k = 0; k < NEN; k++) df_mac(acc[k], A, N[k]);
    }
    const float back = 1.0f / ed.sc;  // G scales with the length (a power of two: exact)
#pragma unroll
    for (int k = 0; k < NEN; k++) out[k] = df_pow2(df_warp_sum(acc[k]), back);
}

// warp_singular_H<NEN, FLAG> in double-FP32 (the same outputs, in
// double-FP32 in every lane); X0, xe and the normal n in double-FP32.
template <int NEN, int FLAG>
__device__ void warp_singular_H_df(int s, const float2 (*X0)[3], const float2 *xe, const float2 *nd,
                                   float2 *out)
{
    constexpr int NOUT = FLAG == 2 ? 4 * NEN : FLAG ? 3 * NEN : NEN;
    constexpr int G0 = FLAG == 2 ? NEN : 0;
    const int lane = threadIdx.x & 31;
    float2 X[NEN][3];
#pragma unroll
    for (int p = 0; p < NEN; p++)
#pragma unroll
        for (int d = 0; d < 3; d++) X[p][d] = X0[singular_perm<NEN>(s, p)][d];
    ElemMapDf<NEN> ed;
    ed.init(X);
    float2 e0[3];
    ed.offset(xe, e0);
    float2 acc[NOUT];
#pragma unroll
    for (int k = 0; k < NOUT; k++) acc[k] = make_float2(0.0f, 0.0f);
    const bool two = (NEN == 6) && (s % 2 == 0);
    float2 N1[6], N2[6], D1[3], D2[3];
    for (int p = lane; p < kSubdiv * 3 * kTriPts; p += 32) {
        const int m = p / (3 * kTriPts), i = (p / kTriPts) % 3, q = p % kTriPts;
        const float scale = ldexpf(1.0f, -m);                // xs halves each level (exact)
        const float Jm = ldexpf(1.0f, -2 * (m + 1));         // 0.25^(m+1) (exact)
        const float2 W = df_ld(g_sing_df.w7[q]);
        if (!two) {
            const float2 l1 = df_pow2(df_ld(g_sing_df.l[i][q][0]), scale);
            const float2 l2 = df_pow2(df_ld(g_sing_df.l[i][q][1]), scale);
            shape_df<NEN>(l1, l2, N1);
            const float2 j2 = ed.at_sq(l1, l2, e0, D1);
            const float2 rsq = df_dot3(D1, D1);
            // |J| / r^3 = J^2 / sqrt(J^2 r^6)
            const float2 jr3 = df_mul(j2, df_rsqrt(df_mul(j2, df_mul(rsq, df_sqr(rsq)))));
            const float2 A = df_pow2(df_mul(W, jr3), Jm);
            if (FLAG != 1) {
                const float2 An = df_neg(df_mul(A, df_dot3(D1, nd)));
#pragma unroll
                for (int k = 0; k < NEN; k++) df_mac(acc[k], An, N1[k]);
            }
            if (FLAG != 0) {
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const float2 Ad = df_mul(A, D1[c]);
#pragma unroll
                    for (int k = 0; k < NEN; k++) df_mac(acc[G0 + 3 * k + c], Ad, N1[k]);
                }
            }
        } else {
            const DfC *ab = g_sing_df.ab[s / 2 - 1][i][q];
            const float2 a1 = df_pow2(df_ld(ab[0]), scale), a2 = df_pow2(df_ld(ab[1]), scale);
            const float2 b1 = df_pow2(df_ld(ab[2]), scale), b2 = df_pow2(df_ld(ab[3]), scale);
            shape_df<NEN>(a1, a2, N1);
            shape_df<NEN>(b1, b2, N2);
            const float2 j21 = ed.at_sq(a1, a2, e0, D1);
            const float2 j22 = ed.at_sq(b1, b2, e0, D2);
            const float2 r1 = df_dot3(D1, D1), r2 = df_dot3(D2, D2);
            const float2 hJW = df_pow2(W, 0.5f * Jm);
            const float2 A1 = df_mul(hJW, df_mul(j21, df_rsqrt(df_mul(j21, df_mul(r1, df_sqr(r1))))));
            const float2 A2 = df_mul(hJW, df_mul(j22, df_rsqrt(df_mul(j22, df_mul(r2, df_sqr(r2))))));
            if (FLAG != 1) {
                const float2 An1 = df_neg(df_mul(A1, df_dot3(D1, nd)));
                const float2 An2 = df_neg(df_mul(A2, df_dot3(D2, nd)));
#pragma unroll
                for (int k = 0; k < NEN; k++) {
                    df_mac(acc[k], An1, N1[k]);
                    df_mac(acc[k], An2, N2[k]);
                }
            }
            if (FLAG != 0) {
                // the second point's z term with its y distance, as in the
                // reference (src/kernelIntegrals.c:762)
                const float2 Ad1[3] = {df_mul(A1, D1[0]), df_mul(A1, D1[1]), df_mul(A1, D1[2])};
                const float2 Ad2[3] = {df_mul(A2, D2[0]), df_mul(A2, D2[1]), df_mul(A2, D2[1])};
#pragma unroll
                for (int c = 0; c < 3; c++)
#pragma unroll
                    for (int k = 0; k < NEN; k++) {
                        df_mac(acc[G0 + 3 * k + c], Ad1[c], N1[k]);
                        df_mac(acc[G0 + 3 * k + c], Ad2[c], N2[k]);
                    }
            }
        }
    }
    float2 red[NOUT];
#pragma unroll
    for (int k = 0; k < NOUT; k++) red[k] = df_warp_sum(acc[k]);
#pragma unroll
    for (int p = 0; p < NEN; p++) {
        const int o = singular_perm<NEN>(s, p);
        if (FLAG != 1) out[o] = red[p];
        if (FLAG != 0) {
            out[G0 + 3 * o + 0] = red[G0 + 3 * p + 0];
            out[G0 + 3 * o + 1] = red[G0 + 3 * p + 1];
            out[G0 + 3 * o + 2] = red[G0 + 3 * p + 2];
        }
    }
}

}  // namespace dsc
