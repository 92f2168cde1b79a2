/*
 * quadrature.c -- rules, shape functions and the isoparametric map
 * (oracle restatement; test infrastructure).
 *
 * The three rules are standard published ones, written to the same 15
 * significant digits the reference tabulates (src/gaussData.h:38-73) so that
 * the oracle reproduces the reference's sums to rounding:
 *   - 8-point Gauss-Legendre on [-1, 1];
 *   - 8-point Gauss-Jacobi on [-1, 1] with weight (1 + x) (alpha 0, beta 1);
 *   - Dunavant's 7-point degree-5 triangle rule, weights summing to 1/2:
 *     centroid 9/80, points a = (6 -+ sqrt 15)/21 with weights
 *     (155 -+ sqrt 15)/2400.
 */
#include <math.h>
#include "oracle.h"

const double orc_gauss_legendre8[ORC_NGAUSS][2] = {
    {-0.960289856497536, 0.101228536290370},
    {-0.796666477413627, 0.222381034453376},
    {-0.525532409916329, 0.313706645877887},
    {-0.183434642495650, 0.362683783378362},
    { 0.183434642495650, 0.362683783378362},
    { 0.525532409916329, 0.313706645877887},
    { 0.796666477413627, 0.222381034453376},
    { 0.960289856497536, 0.101228536290370}};

const double orc_gauss_jacobi8[ORC_NGAUSS][2] = {
    {-0.910732089420060, 0.0131807657689955},
    {-0.711267485915709, 0.0713716106239446},
    {-0.426350485711139, 0.181757278018796},
    {-0.0903733696068533, 0.316798397969277},
    { 0.256135670833455, 0.424189437743720},
    { 0.571383041208738, 0.450023197883551},
    { 0.817352784200412, 0.364476094545495},
    { 0.964440169705273, 0.178203217446225}};

/* (L1, L2, weight); L3 = 1 - L1 - L2. */
const double orc_triangle7[ORC_TNGAUSS][3] = {
    {0.333333333333333, 0.333333333333333, 0.1125},
    {0.470142064105115, 0.470142064105115, 0.066197076394253},
    {0.0597158717897700, 0.470142064105115, 0.066197076394253},
    {0.470142064105115, 0.0597158717897700, 0.066197076394253},
    {0.101286507323456, 0.101286507323456, 0.062969590272414},
    {0.797426985353088, 0.101286507323456, 0.062969590272414},
    {0.101286507323456, 0.797426985353088, 0.062969590272414}};

/* Node order 1..6 = corner(L1=1), mid, corner(L2=1), mid, corner(L3=1), mid
 * (src/shapeFunctions.c:53-87). */
void orc_shape(int nen, const double L[2], double *N)
{
    double l1 = L[0], l2 = L[1], l3 = 1.0 - l1 - l2;
    if (nen == 3) {
        N[0] = l1;
        N[1] = l2;
        N[2] = l3;
        return;
    }
    N[0] = l1 * (2.0 * l1 - 1.0);
    N[1] = 4.0 * l1 * l2;
    N[2] = l2 * (2.0 * l2 - 1.0);
    N[3] = 4.0 * l2 * l3;
    N[4] = l3 * (2.0 * l3 - 1.0);
    N[5] = 4.0 * l1 * l3;
}

/* Tangent vectors dX/dL1, dX/dL2 of the isoparametric map, from the
 * derivatives of the shape functions above. */
static void tangents(int nen, const double *X, const double L[2], double t1[3], double t2[3])
{
    if (nen == 3) {
        for (int d = 0; d < 3; d++) {
            t1[d] = X[0 * 3 + d] - X[2 * 3 + d];
            t2[d] = X[1 * 3 + d] - X[2 * 3 + d];
        }
        return;
    }
    double l1 = L[0], l2 = L[1];
    for (int d = 0; d < 3; d++) {
        double x1 = X[0 * 3 + d], x2 = X[1 * 3 + d], x3 = X[2 * 3 + d];
        double x4 = X[3 * 3 + d], x5 = X[4 * 3 + d], x6 = X[5 * 3 + d];
        double a = x2 - x4 + x5 - x6;
        t1[d] = 4.0 * (l1 * (x1 + x5 - 2.0 * x6) + l2 * a + x6) - x1 - 3.0 * x5;
        t2[d] = 4.0 * (l1 * a + l2 * (x3 + x5 - 2.0 * x4) + x4) - x3 - 3.0 * x5;
    }
}

/* Global point XL = sum N_k X_k and surface Jacobian |t1 x t2|
 * (src/globalToLocal.c:75-148). */
double orc_x2l(int nen, const double *X, const double L[2], const double *N, double XL[3])
{
    double t1[3], t2[3];
    for (int d = 0; d < 3; d++) {
        double s = 0.0;
        for (int k = 0; k < nen; k++) s += N[k] * X[k * 3 + d];
        XL[d] = s;
    }
    tangents(nen, X, L, t1, t2);
    double j1 = t1[1] * t2[2] - t2[1] * t1[2];
    double j2 = t2[0] * t1[2] - t1[0] * t2[2];
    double j3 = t1[0] * t2[1] - t2[0] * t1[1];
    return sqrt(j1 * j1 + j2 * j2 + j3 * j3);
}

/* Unit normal t1 x t2 / |t1 x t2| at local point L
 * (src/normals.c:45-112). */
void orc_local_normal(int nen, const double *X, const double L[2], double n[3])
{
    double t1[3], t2[3];
    tangents(nen, X, L, t1, t2);
    n[0] = t1[1] * t2[2] - t2[1] * t1[2];
    n[1] = t2[0] * t1[2] - t1[0] * t2[2];
    n[2] = t1[0] * t2[1] - t2[0] * t1[1];
    double inv = 1.0 / sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    n[0] *= inv;
    n[1] *= inv;
    n[2] *= inv;
}
