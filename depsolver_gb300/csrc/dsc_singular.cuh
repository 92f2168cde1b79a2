// dsc_singular.cuh -- FP64 singular element integrals, one warp per
// (collocation point, element) pair with the quadrature points split over
// the lanes.  Restates depSolver's intSingularG_* / intSingularH_*
// (src/kernelIntegrals.c:299-805): the values are the same sums, taken in a
// lane-strided order and combined by a warp reduction.
#pragma once

#include "dsc_common.cuh"

namespace dsc {

// Collapsed-square (Duffy) maps of the weakly singular G integral
// (src/kernelIntegrals.c:322-336 tria3, :391-429 tria6).  Returns the number
// of sub-triangles (1 or 2).
template <int NEN>
__device__ __forceinline__ int duffy(int s, double u1, double u2, double *La, double *Lb)
{
    if (NEN == 3) {
        if (s == 1) { La[0] = 0.5 * (1.0 - u2); La[1] = 0.25 * (1.0 + u1) * (1.0 + u2); }
        else if (s == 2) { La[0] = 0.25 * (1.0 - u1) * (1.0 + u2); La[1] = 0.5 * (1.0 - u2); }
        else { La[0] = 0.25 * (1.0 + u1) * (1.0 + u2); La[1] = 0.25 * (1.0 - u1) * (1.0 + u2); }
        return 1;
    }
    switch (s) {
    case 1: La[0] = 0.5 * (1.0 - u2); La[1] = 0.25 * (1.0 + u1) * (1.0 + u2); return 1;
    case 2:
        La[0] = 0.25 * (1.0 - u2); La[1] = 0.5 + 0.25 * u1 * (1.0 + u2);
        Lb[0] = 0.5 - 0.25 * u1 * (1.0 + u2); Lb[1] = 0.25 * (1.0 - u2);
        return 2;
    case 3: La[0] = 0.25 * (1.0 - u1) * (1.0 + u2); La[1] = 0.5 * (1.0 - u2); return 1;
    case 4:
        La[0] = 0.25 * (1.0 + u1) * (1.0 + u2); La[1] = 0.5 - 0.25 * u1 * (1.0 + u2);
        Lb[0] = 0.25 * (1.0 - u1) * (1.0 + u2); Lb[1] = 0.25 * (1.0 - u2);
        return 2;
    case 5: La[0] = 0.25 * (1.0 + u1) * (1.0 + u2); La[1] = 0.25 * (1.0 - u1) * (1.0 + u2); return 1;
    default:
        La[0] = 0.5 + 0.25 * u1 * (1.0 + u2); La[1] = 0.25 * (1.0 - u1) * (1.0 + u2);
        Lb[0] = 0.25 * (1.0 - u2); Lb[1] = 0.25 * (1.0 + u1) * (1.0 + u2);
        return 2;
    }
}

// A point of the singular quadrature: dd = xe - X(l1, l2), returns the
// Jacobian, summed as the reference sums it (nodal shape functions, N the
// shape values at (l1, l2)), so that K follows the reference's rounding.
template <int NEN>
__device__ __forceinline__ double sing_point(const double (*X)[3], const double *xe, double l1, double l2,
                                             const double *N, double *dd)
{
    double XL[3];
    const double J = map_point<NEN>(X, l1, l2, N, XL);
#pragma unroll
    for (int d = 0; d < 3; d++) dd[d] = xe[d] - XL[d];
    return J;
}

// c / r^3 at squared distance rsq, by the reference's division.
template <int NEN>
__device__ __forceinline__ double over_r3(double c, double rsq)
{
    if (NEN == 3) return c / (rsq * sqrt(rsq));
    const double dr = sqrt(rsq);
    return c / (dr * dr * dr);
}

// Warp-cooperative weakly singular G: out[k] (lane 0 valid after the call,
// every lane holds the reduced value) = sum over 8 x 8 (x2) points of
// w1 w2 J B N_k / r, B = 1/8 (one sub-triangle) or 1/16 (two).
template <int NEN>
__device__ void warp_singular_G(int s, const double (*X)[3], const double *xe, double *out)
{
    const int lane = threadIdx.x & 31;
    double La[2], Lb[2], N[6], dd[3];
    double acc[NEN];
#pragma unroll
    for (int k = 0; k < NEN; k++) acc[k] = 0.0;
    const int T = duffy<NEN>(s, 0.0, 0.0, La, Lb);
    const double B = T == 1 ? 0.125 : 0.0625;
    for (int p = lane; p < 64 * T; p += 32) {
        int ij = p / T, t = p % T;
        int i = ij / 8, j = ij % 8;
        double u1 = c_gl8[i][0], w1 = c_gl8[i][1];
        double u2 = c_gj8[j][0], w2 = c_gj8[j][1];
        duffy<NEN>(s, u1, u2, La, Lb);
        const double *L = t == 0 ? La : Lb;
        shape<NEN>(L[0], L[1], N);
        const double J = sing_point<NEN>(X, xe, L[0], L[1], N, dd);
        const double dx = dd[0], dy = dd[1], dz = dd[2];
        const double A = w1 * w2 * J * B / sqrt(dx * dx + dy * dy + dz * dz);
#pragma unroll
        for (int k = 0; k < NEN; k++) acc[k] += A * N[k];
    }
#pragma unroll
    for (int k = 0; k < NEN; k++) out[k] = warp_sum(acc[k]);
}

// The subdivision's points at level 0 (level m: times 2^-m, exact): for
// sub-triangle i and point q of the 7-point rule, l[i][q] = (l1, l2); for
// the tria6 mid-side rotations s = 2, 4, 6, ab[s / 2 - 1][i][q] = the two
// mapped points (a1, a2, b1, b2).  The same sums as warp_singular_H takes
// per point, evaluated once at compile time (the table of the double-FP32
// form, dsc_singular_df.cuh).
struct SubdivPts {
    double l[3][kTriPts][2];
    double ab[3][3][kTriPts][4];
};

constexpr SubdivPts make_subdiv_pts()
{
    SubdivPts t{};
    const double xs[3][3][2] = {{{1.0, 0.0}, {0.5, 0.5}, {0.5, 0.0}},
                                {{0.5, 0.0}, {0.5, 0.5}, {0.0, 0.5}},
                                {{0.5, 0.5}, {0.0, 1.0}, {0.0, 0.5}}};
    for (int i = 0; i < 3; i++)
        for (int q = 0; q < kTriPts; q++) {
            const double M1 = kTri7.v[q][0], M2 = kTri7.v[q][1], M3 = 1.0 - M1 - M2;
            t.l[i][q][0] = xs[i][0][0] * M1 + xs[i][1][0] * M2 + xs[i][2][0] * M3;
            t.l[i][q][1] = xs[i][0][1] * M1 + xs[i][1][1] * M2 + xs[i][2][1] * M3;
            for (int r = 0; r < 3; r++) {
                double U1 = 0.0, U2 = 0.0, V1 = 0.0, V2 = 0.0;
                if (r == 0) { U1 = 0.5 * M3; U2 = M1 + 0.5 * M3; V1 = M1 + 0.5 * M3; V2 = M3; }
                else if (r == 1) { U1 = M1; U2 = 0.5 * M3; V1 = M1; V2 = M2 + 0.5 * M3; }
                else { U1 = 0.5 * M3; U2 = M1; V1 = M1 + 0.5 * M3; V2 = M2; }
                const double U3 = 1.0 - U1 - U2, V3 = 1.0 - V1 - V2;
                t.ab[r][i][q][0] = xs[i][0][0] * U1 + xs[i][1][0] * U2 + xs[i][2][0] * U3;
                t.ab[r][i][q][1] = xs[i][0][1] * U1 + xs[i][1][1] * U2 + xs[i][2][1] * U3;
                t.ab[r][i][q][2] = xs[i][0][0] * V1 + xs[i][1][0] * V2 + xs[i][2][0] * V3;
                t.ab[r][i][q][3] = xs[i][0][1] * V1 + xs[i][1][1] * V2 + xs[i][2][1] * V3;
            }
        }
    return t;
}


// Position p of the rotated element holds original node perm[p]
// (src/kernelIntegrals.c:494-499, :636-647).
template <int NEN>
__device__ __forceinline__ int singular_perm(int s, int p)
{
    if (NEN == 3) {
        if (s == 1) return (p + 1) % 3;
        if (s == 2) return (p + 2) % 3;
        return p;
    }
    if (s == 1) return (p + 2) % 6;
    if (s == 3) return (p + 4) % 6;
    return p;
}

// Warp-cooperative strongly singular H (FLAG = 0: normal derivative with
// the node normal n, out[k]; FLAG = 1: gradient, out[3k + c]; FLAG = 2:
// both from the same points, out[k] and out[NEN + 3k + c], each summed as
// FLAG 0 and FLAG 1 sum it) by 8-level subdivision x 3 sub-triangles x 7
// points towards local (0,0) of the rotated element
// (src/kernelIntegrals.c:472-593 tria3, :611-805 tria6).  For tria6
// mid-side nodes each point is split into two mapped points with weight
// 1/2; the gradient's z-component of the second one uses its y-distance,
// as in the reference (:762).
template <int NEN, int FLAG>
__device__ void warp_singular_H(int s, const double (*X0)[3], const double *xe, const double *n,
                                double *out)
{
    constexpr int NOUT = FLAG == 2 ? 4 * NEN : FLAG ? 3 * NEN : NEN;
    constexpr int G0 = FLAG == 2 ? NEN : 0;  // first gradient accumulator
    const int lane = threadIdx.x & 31;
    double X[NEN][3];
#pragma unroll
    for (int p = 0; p < NEN; p++)
#pragma unroll
        for (int d = 0; d < 3; d++) X[p][d] = X0[singular_perm<NEN>(s, p)][d];
    double acc[NOUT];
#pragma unroll
    for (int k = 0; k < NOUT; k++) acc[k] = 0.0;
    const bool two = (NEN == 6) && (s % 2 == 0);
    // sub-triangle vertices at level 0 (src/kernelIntegrals.c:501-512)
    const double xs0[3][3][2] = {{{1.0, 0.0}, {0.5, 0.5}, {0.5, 0.0}},
                                 {{0.5, 0.0}, {0.5, 0.5}, {0.0, 0.5}},
                                 {{0.5, 0.5}, {0.0, 1.0}, {0.0, 0.5}}};
    double N1[6], N2[6], D1[3], D2[3];
    for (int p = lane; p < kSubdiv * 3 * kTriPts; p += 32) {
        int m = p / (3 * kTriPts), i = (p / kTriPts) % 3, q = p % kTriPts;
        double scale = ldexp(1.0, -m);          // xs halves each level (exact)
        double J = ldexp(1.0, -2 * (m + 1));    // 0.25^(m+1) (exact)
        double M1 = c_tri7[q][0], M2 = c_tri7[q][1];
        double M3 = 1.0 - M1 - M2, W = c_tri7[q][2];
        double x00 = xs0[i][0][0] * scale, x01 = xs0[i][0][1] * scale;
        double x10 = xs0[i][1][0] * scale, x11 = xs0[i][1][1] * scale;
        double x20 = xs0[i][2][0] * scale, x21 = xs0[i][2][1] * scale;
        if (!two) {
            double l1 = x00 * M1 + x10 * M2 + x20 * M3;
            double l2 = x01 * M1 + x11 * M2 + x21 * M3;
            shape<NEN>(l1, l2, N1);
            const double JL = sing_point<NEN>(X, xe, l1, l2, N1, D1);
            const double dx = D1[0], dy = D1[1], dz = D1[2];
            const double A = over_r3<NEN>(J * JL * W, dx * dx + dy * dy + dz * dz);
            if (FLAG != 1) {
                const double An = A * (dx * n[0] + dy * n[1] + dz * n[2]);
#pragma unroll
                for (int k = 0; k < NEN; k++) acc[k] -= An * N1[k];
            }
            if (FLAG != 0) {
#pragma unroll
                for (int k = 0; k < NEN; k++) {
                    acc[G0 + 3 * k + 0] += A * dx * N1[k];
                    acc[G0 + 3 * k + 1] += A * dy * N1[k];
                    acc[G0 + 3 * k + 2] += A * dz * N1[k];
                }
            }
        } else {
            double U1, U2, V1, V2;
            if (s == 2) { U1 = 0.5 * M3; U2 = M1 + 0.5 * M3; V1 = M1 + 0.5 * M3; V2 = M3; }
            else if (s == 4) { U1 = M1; U2 = 0.5 * M3; V1 = M1; V2 = M2 + 0.5 * M3; }
            else { U1 = 0.5 * M3; U2 = M1; V1 = M1 + 0.5 * M3; V2 = M2; }
            double U3 = 1.0 - U1 - U2, V3 = 1.0 - V1 - V2;
            double a1 = x00 * U1 + x10 * U2 + x20 * U3, a2 = x01 * U1 + x11 * U2 + x21 * U3;
            double b1 = x00 * V1 + x10 * V2 + x20 * V3, b2 = x01 * V1 + x11 * V2 + x21 * V3;
            shape<NEN>(a1, a2, N1);
            shape<NEN>(b1, b2, N2);
            const double JL1 = sing_point<NEN>(X, xe, a1, a2, N1, D1);
            const double JL2 = sing_point<NEN>(X, xe, b1, b2, N2, D2);
            const double dx1 = D1[0], dy1 = D1[1], dz1 = D1[2];
            const double dx2 = D2[0], dy2 = D2[1], dz2 = D2[2];
            const double A1 = over_r3<NEN>(0.5 * J * JL1 * W, dx1 * dx1 + dy1 * dy1 + dz1 * dz1);
            const double A2 = over_r3<NEN>(0.5 * J * JL2 * W, dx2 * dx2 + dy2 * dy2 + dz2 * dz2);
            if (FLAG != 1) {
                const double An1 = A1 * (dx1 * n[0] + dy1 * n[1] + dz1 * n[2]);
                const double An2 = A2 * (dx2 * n[0] + dy2 * n[1] + dz2 * n[2]);
#pragma unroll
                for (int k = 0; k < NEN; k++) acc[k] -= An1 * N1[k] + An2 * N2[k];
            }
            if (FLAG != 0) {
#pragma unroll
                for (int k = 0; k < NEN; k++) {
                    acc[G0 + 3 * k + 0] += A1 * dx1 * N1[k] + A2 * dx2 * N2[k];
                    acc[G0 + 3 * k + 1] += A1 * dy1 * N1[k] + A2 * dy2 * N2[k];
                    acc[G0 + 3 * k + 2] += A1 * dz1 * N1[k] + A2 * dy2 * N2[k];
                }
            }
        }
    }
    // reduce, then return each node's value at its original position
    double red[NOUT];
#pragma unroll
    for (int k = 0; k < NOUT; k++) red[k] = warp_sum(acc[k]);
#pragma unroll
    for (int p = 0; p < NEN; p++) {
        int o = singular_perm<NEN>(s, p);
        if (FLAG != 1) out[o] = red[p];
        if (FLAG != 0) {
            out[G0 + 3 * o + 0] = red[G0 + 3 * p + 0];
            out[G0 + 3 * o + 1] = red[G0 + 3 * p + 1];
            out[G0 + 3 * o + 2] = red[G0 + 3 * p + 2];
        }
    }
}

}  // namespace dsc
