// dsc_common.cuh -- shared device definitions of libdepsolver_cuda.
//
// Quadrature rules, shape functions and the isoparametric map of 3- and
// 6-node triangles, as used by depSolver's element integrals
// (src/kernelIntegrals.c, src/shapeFunctions.c, src/globalToLocal.c,
// rules in src/gaussData.h:38-73).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace dsc {

constexpr double kEps0 = 8.854187817E-12;   // src/constants.h:42
constexpr double kPi2 = 6.283185307179586E+00;
constexpr double kPi4 = 1.256637061435917E+01;
constexpr int kTriPts = 7;    // TNGAUSS / TSNGAUSS
constexpr int kLinePts = 8;   // NGAUSS
constexpr int kSubdiv = 8;    // NSUBDIVISIONS

// Published rules written to the 15 significant digits the reference
// tabulates: Dunavant's 7-point degree-5 triangle rule (weights sum 1/2),
// 8-point Gauss-Legendre, and 8-point Gauss-Jacobi for weight (1 + x).
#define DSC_TRI7_ROWS                                                \
    {0.333333333333333, 0.333333333333333, 0.1125},                  \
        {0.470142064105115, 0.470142064105115, 0.066197076394253},   \
        {0.0597158717897700, 0.470142064105115, 0.066197076394253},  \
        {0.470142064105115, 0.0597158717897700, 0.066197076394253},  \
        {0.101286507323456, 0.101286507323456, 0.062969590272414},   \
        {0.797426985353088, 0.101286507323456, 0.062969590272414},   \
    {                                                                \
        0.101286507323456, 0.797426985353088, 0.062969590272414      \
    }
__constant__ __device__ static const double c_tri7[kTriPts][3] = {DSC_TRI7_ROWS};
// the same rule for tables built at compile time
struct Tri7Rule {
    double v[kTriPts][3];
};
constexpr Tri7Rule kTri7{{DSC_TRI7_ROWS}};

__constant__ __device__ static const double c_gl8[kLinePts][2] = {
    {-0.960289856497536, 0.101228536290370}, {-0.796666477413627, 0.222381034453376},
    {-0.525532409916329, 0.313706645877887}, {-0.183434642495650, 0.362683783378362},
    {0.183434642495650, 0.362683783378362},  {0.525532409916329, 0.313706645877887},
    {0.796666477413627, 0.222381034453376},  {0.960289856497536, 0.101228536290370}};

__constant__ __device__ static const double c_gj8[kLinePts][2] = {
    {-0.910732089420060, 0.0131807657689955}, {-0.711267485915709, 0.0713716106239446},
    {-0.426350485711139, 0.181757278018796},  {-0.0903733696068533, 0.316798397969277},
    {0.256135670833455, 0.424189437743720},   {0.571383041208738, 0.450023197883551},
    {0.817352784200412, 0.364476094545495},   {0.964440169705273, 0.178203217446225}};

// Shape functions; node order corner(L1=1), mid, corner(L2=1), mid,
// corner(L3=1), mid.
template <int NEN>
__host__ __device__ __forceinline__ void shape(double l1, double l2, double *N)
{
    double l3 = 1.0 - l1 - l2;
    if (NEN == 3) {
        N[0] = l1;
        N[1] = l2;
        N[2] = l3;
    } else {
        N[0] = l1 * (2.0 * l1 - 1.0);
        N[1] = 4.0 * l1 * l2;
        N[2] = l2 * (2.0 * l2 - 1.0);
        N[3] = 4.0 * l2 * l3;
        N[4] = l3 * (2.0 * l3 - 1.0);
        N[5] = 4.0 * l1 * l3;
    }
}

// Tangent vectors dX/dL1, dX/dL2 of the map X(L) = sum N_k(L) X_k.
template <int NEN>
__host__ __device__ __forceinline__ void tangents(const double (*X)[3], double l1, double l2,
                                                  double *t1, double *t2)
{
#pragma unroll
    for (int d = 0; d < 3; d++) {
        if (NEN == 3) {
            t1[d] = X[0][d] - X[2][d];
            t2[d] = X[1][d] - X[2][d];
        } else {
            double a = X[1][d] - X[3][d] + X[4][d] - X[5][d];
            t1[d] = 4.0 * (l1 * (X[0][d] + X[4][d] - 2.0 * X[5][d]) + l2 * a + X[5][d]) - X[0][d] -
                    3.0 * X[4][d];
            t2[d] = 4.0 * (l1 * a + l2 * (X[2][d] + X[4][d] - 2.0 * X[3][d]) + X[3][d]) - X[2][d] -
                    3.0 * X[4][d];
        }
    }
}

// Point X(L) and surface Jacobian |t1 x t2|.
template <int NEN>
__host__ __device__ __forceinline__ double map_point(const double (*X)[3], double l1, double l2,
                                                     const double *N, double *XL)
{
    double t1[3], t2[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < NEN; k++) s += N[k] * X[k][d];
        XL[d] = s;
    }
    tangents<NEN>(X, l1, l2, t1, t2);
    double j1 = t1[1] * t2[2] - t2[1] * t1[2];
    double j2 = t2[0] * t1[2] - t1[0] * t2[2];
    double j3 = t1[0] * t2[1] - t2[0] * t1[1];
    return sqrt(j1 * j1 + j2 * j2 + j3 * j3);
}

template <int NEN>
__host__ __device__ __forceinline__ void local_normal(const double (*X)[3], double l1, double l2,
                                                      double *n)
{
    double t1[3], t2[3];
    tangents<NEN>(X, l1, l2, t1, t2);
    n[0] = t1[1] * t2[2] - t2[1] * t1[2];
    n[1] = t2[0] * t1[2] - t1[0] * t2[2];
    n[2] = t1[0] * t2[1] - t2[0] * t1[1];
    double inv = 1.0 / sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    n[0] *= inv;
    n[1] *= inv;
    n[2] *= inv;
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace dsc
