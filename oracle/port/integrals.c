/*
 * integrals.c -- element integrals of G = 1/r and its derivative
 * (oracle restatement of src/kernelIntegrals.c; test infrastructure).
 *
 * Int layout: flag 0 -> Int[k] for node k; flag != 0 -> Int[3k + c] for
 * node k, component c of the gradient.
 */
#include <math.h>
#include <string.h>
#include "oracle.h"

/* Regular 7-point rule for sum_q w_q J_q N_k(q) / r_q
 * (intG_tria3 src/kernelIntegrals.c:61-95, intG_tria6 :109-142). */
void orc_intG(int nen, const double *X, const double *Xe, double *Int)
{
    double N[6], XL[3];
    for (int k = 0; k < nen; k++) Int[k] = 0.0;
    for (int q = 0; q < ORC_TNGAUSS; q++) {
        const double L[2] = {orc_triangle7[q][0], orc_triangle7[q][1]};
        orc_shape(nen, L, N);
        double J = orc_x2l(nen, X, L, N, XL);
        double dx = Xe[0] - XL[0], dy = Xe[1] - XL[1], dz = Xe[2] - XL[2];
        double A = orc_triangle7[q][2] * J / sqrt(dx * dx + dy * dy + dz * dz);
        for (int k = 0; k < nen; k++) Int[k] += A * N[k];
    }
}

/* Regular 7-point rule for the normal derivative (flag 0):
 *   Int[k] = - sum_q w J N_k n.(x - y) / r^3
 * or the full gradient (flag != 0): Int[3k+c] = sum_q w J N_k (x - y)_c / r^3
 * (intH_tria3 src/kernelIntegrals.c:160-213, intH_tria6 :231-282). */
void orc_intH(int nen, unsigned flag, const double *X, const double *Xe, double *Int,
              const double *n)
{
    double N[6], XL[3];
    int nout = flag ? 3 * nen : nen;
    for (int k = 0; k < nout; k++) Int[k] = 0.0;
    for (int q = 0; q < ORC_TNGAUSS; q++) {
        const double L[2] = {orc_triangle7[q][0], orc_triangle7[q][1]};
        orc_shape(nen, L, N);
        double J = orc_x2l(nen, X, L, N, XL);
        double dx = Xe[0] - XL[0], dy = Xe[1] - XL[1], dz = Xe[2] - XL[2];
        double rsq = dx * dx + dy * dy + dz * dz;
        double A = J * orc_triangle7[q][2] / pow(rsq, 1.5);
        if (!flag) {
            A *= dx * n[0] + dy * n[1] + dz * n[2];
            for (int k = 0; k < nen; k++) Int[k] -= A * N[k];
        } else {
            for (int k = 0; k < nen; k++) {
                Int[3 * k + 0] += A * dx * N[k];
                Int[3 * k + 1] += A * dy * N[k];
                Int[3 * k + 2] += A * dz * N[k];
            }
        }
    }
}

/* Local coordinates of the collapsed-square (Duffy) maps used for the weakly
 * singular G integral.  Returns the number of sub-triangles (1 or 2); the
 * second map is written to L2 only when two are used
 * (src/kernelIntegrals.c:322-336 for tria3, :391-429 for tria6). */
static int duffy_map(int nen, unsigned s, double u1, double u2, double L1[2], double L2[2])
{
    if (nen == 3) {
        if (s == 1) { L1[0] = 0.5 * (1.0 - u2); L1[1] = 0.25 * (1.0 + u1) * (1.0 + u2); }
        else if (s == 2) { L1[0] = 0.25 * (1.0 - u1) * (1.0 + u2); L1[1] = 0.5 * (1.0 - u2); }
        else { L1[0] = 0.25 * (1.0 + u1) * (1.0 + u2); L1[1] = 0.25 * (1.0 - u1) * (1.0 + u2); }
        return 1;
    }
    switch (s) {
    case 1:
        L1[0] = 0.5 * (1.0 - u2); L1[1] = 0.25 * (1.0 + u1) * (1.0 + u2);
        return 1;
    case 2:
        L1[0] = 0.25 * (1.0 - u2); L1[1] = 0.5 + 0.25 * u1 * (1.0 + u2);
        L2[0] = 0.5 - 0.25 * u1 * (1.0 + u2); L2[1] = 0.25 * (1.0 - u2);
        return 2;
    case 3:
        L1[0] = 0.25 * (1.0 - u1) * (1.0 + u2); L1[1] = 0.5 * (1.0 - u2);
        return 1;
    case 4:
        L1[0] = 0.25 * (1.0 + u1) * (1.0 + u2); L1[1] = 0.5 - 0.25 * u1 * (1.0 + u2);
        L2[0] = 0.25 * (1.0 - u1) * (1.0 + u2); L2[1] = 0.25 * (1.0 - u2);
        return 2;
    case 5:
        L1[0] = 0.25 * (1.0 + u1) * (1.0 + u2); L1[1] = 0.25 * (1.0 - u1) * (1.0 + u2);
        return 1;
    default:
        L1[0] = 0.5 + 0.25 * u1 * (1.0 + u2); L1[1] = 0.25 * (1.0 - u1) * (1.0 + u2);
        L2[0] = 0.25 * (1.0 - u2); L2[1] = 0.25 * (1.0 + u1) * (1.0 + u2);
        return 2;
    }
}

/* Weakly singular G: 8 x 8 Gauss-Legendre x Gauss-Jacobi on the collapsed
 * square, weight 1/8 for one sub-triangle and 1/16 for two
 * (intSingularG_tria3 src/kernelIntegrals.c:299-350, tria6 :367-454). */
void orc_intSingularG(int nen, unsigned sinNode, const double *X, const double *Xe, double *Int)
{
    double N[6], XL[3], La[2], Lb[2];
    for (int k = 0; k < nen; k++) Int[k] = 0.0;
    int T = duffy_map(nen, sinNode, 0.0, 0.0, La, Lb);
    double B = (T == 1) ? 0.125 : 0.0625;
    for (int i = 0; i < ORC_NGAUSS; i++) {
        double u1 = orc_gauss_legendre8[i][0], w1 = orc_gauss_legendre8[i][1];
        for (int j = 0; j < ORC_NGAUSS; j++) {
            double u2 = orc_gauss_jacobi8[j][0], w2 = orc_gauss_jacobi8[j][1];
            duffy_map(nen, sinNode, u1, u2, La, Lb);
            for (int t = 0; t < T; t++) {
                const double *L = t == 0 ? La : Lb;
                orc_shape(nen, L, N);
                double J = orc_x2l(nen, X, L, N, XL);
                double dx = Xe[0] - XL[0], dy = Xe[1] - XL[1], dz = Xe[2] - XL[2];
                double A = w1 * w2 * J * B / sqrt(dx * dx + dy * dy + dz * dz);
                for (int k = 0; k < nen; k++) Int[k] += A * N[k];
            }
        }
    }
}

/* Node rotation of the strongly singular H integral: the element is
 * re-ordered so that the singular node sits at local (0,0) (node 3 of a
 * tria3, node 5 of a tria6); perm[p] is the original index of position p
 * (src/kernelIntegrals.c:494-499 for tria3, :636-647 for tria6; mid-side
 * nodes of a tria6 are not rotated). */
static void singular_perm(int nen, unsigned s, int perm[6])
{
    for (int p = 0; p < 6; p++) perm[p] = p;
    if (nen == 3) {
        if (s == 1) { perm[0] = 1; perm[1] = 2; perm[2] = 0; }
        else if (s == 2) { perm[0] = 2; perm[1] = 0; perm[2] = 1; }
        return;
    }
    if (s == 1) { int p[6] = {2, 3, 4, 5, 0, 1}; memcpy(perm, p, sizeof p); }
    else if (s == 3) { int p[6] = {4, 5, 0, 1, 2, 3}; memcpy(perm, p, sizeof p); }
}

/* The three initial sub-triangles of the unit triangle that exclude the
 * corner at (0,0); each level halves them towards (0,0)
 * (src/kernelIntegrals.c:501-512). */
static const double SUBTRI0[3][3][2] = {
    {{1.0, 0.0}, {0.5, 0.5}, {0.5, 0.0}},
    {{0.5, 0.0}, {0.5, 0.5}, {0.0, 0.5}},
    {{0.5, 0.5}, {0.0, 1.0}, {0.0, 0.5}}};

/* Strongly singular H by 8-level subdivision x 3 sub-triangles x 7 points,
 * the innermost triangle dropped (intSingularH_tria3
 * src/kernelIntegrals.c:472-593, intSingularH_tria6 :611-805).
 *
 * For a tria6 mid-side singular node each point is split into two mapped
 * points with weight 1/2 each (:694-749).  With flag != 0 the z-component of
 * the second point uses its y-distance, exactly as the reference does
 * (:762); this changes the field at particle nodes and is kept for parity. */
void orc_intSingularH(int nen, unsigned flag, unsigned sinNode, const double *X0,
                      const double *Xe, double *Int, const double *n)
{
    int perm[6];
    double X[18], R[18];
    double N1[6], N2[6], XL1[3], XL2[3], La[2], Lb[2];
    double xs[3][3][2];
    int nout = flag ? 3 * nen : nen;

    singular_perm(nen, sinNode, perm);
    for (int p = 0; p < nen; p++)
        for (int d = 0; d < 3; d++) X[p * 3 + d] = X0[perm[p] * 3 + d];
    for (int k = 0; k < nout; k++) R[k] = 0.0;
    memcpy(xs, SUBTRI0, sizeof xs);

    int two = (nen == 6) && (sinNode % 2 == 0);
    double J = 1.0;
    for (int m = 0; m < ORC_NSUBDIV; m++) {
        J *= 0.25;
        for (int i = 0; i < 3; i++) {
            for (int q = 0; q < ORC_TNGAUSS; q++) {
                double M1 = orc_triangle7[q][0], M2 = orc_triangle7[q][1];
                double M3 = 1.0 - M1 - M2, W = orc_triangle7[q][2];
                if (!two) {
                    La[0] = xs[i][0][0] * M1 + xs[i][1][0] * M2 + xs[i][2][0] * M3;
                    La[1] = xs[i][0][1] * M1 + xs[i][1][1] * M2 + xs[i][2][1] * M3;
                    orc_shape(nen, La, N1);
                    double JL = orc_x2l(nen, X, La, N1, XL1);
                    double dx = Xe[0] - XL1[0], dy = Xe[1] - XL1[1], dz = Xe[2] - XL1[2];
                    double dr;
                    double A;
                    if (nen == 3) {
                        A = J * JL * W / pow(dx * dx + dy * dy + dz * dz, 1.5);
                    } else {
                        dr = sqrt(dx * dx + dy * dy + dz * dz);
                        A = J * JL * W / (dr * dr * dr);
                    }
                    if (!flag) {
                        A *= dx * n[0] + dy * n[1] + dz * n[2];
                        for (int k = 0; k < nen; k++) R[k] -= A * N1[k];
                    } else {
                        for (int k = 0; k < nen; k++) {
                            R[3 * k + 0] += A * dx * N1[k];
                            R[3 * k + 1] += A * dy * N1[k];
                            R[3 * k + 2] += A * dz * N1[k];
                        }
                    }
                } else {
                    /* Two affine maps of the (M1, M2, M3) point, then the
                     * sub-triangle interpolation (:696-715). */
                    double U1, U2, U3, V1, V2, V3;
                    if (sinNode == 2) {
                        U1 = 0.5 * M3; U2 = M1 + 0.5 * M3;
                        V1 = M1 + 0.5 * M3; V2 = M3;
                    } else if (sinNode == 4) {
                        U1 = M1; U2 = 0.5 * M3;
                        V1 = M1; V2 = M2 + 0.5 * M3;
                    } else {
                        U1 = 0.5 * M3; U2 = M1;
                        V1 = M1 + 0.5 * M3; V2 = M2;
                    }
                    U3 = 1.0 - U1 - U2;
                    V3 = 1.0 - V1 - V2;
                    La[0] = xs[i][0][0] * U1 + xs[i][1][0] * U2 + xs[i][2][0] * U3;
                    La[1] = xs[i][0][1] * U1 + xs[i][1][1] * U2 + xs[i][2][1] * U3;
                    Lb[0] = xs[i][0][0] * V1 + xs[i][1][0] * V2 + xs[i][2][0] * V3;
                    Lb[1] = xs[i][0][1] * V1 + xs[i][1][1] * V2 + xs[i][2][1] * V3;
                    orc_shape(nen, La, N1);
                    orc_shape(nen, Lb, N2);
                    double JL1 = orc_x2l(nen, X, La, N1, XL1);
                    double JL2 = orc_x2l(nen, X, Lb, N2, XL2);
                    double dx1 = Xe[0] - XL1[0], dy1 = Xe[1] - XL1[1], dz1 = Xe[2] - XL1[2];
                    double dx2 = Xe[0] - XL2[0], dy2 = Xe[1] - XL2[1], dz2 = Xe[2] - XL2[2];
                    double dr1 = sqrt(dx1 * dx1 + dy1 * dy1 + dz1 * dz1);
                    double dr2 = sqrt(dx2 * dx2 + dy2 * dy2 + dz2 * dz2);
                    double A1 = 0.5 * J * JL1 * W / (dr1 * dr1 * dr1);
                    double A2 = 0.5 * J * JL2 * W / (dr2 * dr2 * dr2);
                    if (!flag) {
                        A1 *= dx1 * n[0] + dy1 * n[1] + dz1 * n[2];
                        A2 *= dx2 * n[0] + dy2 * n[1] + dz2 * n[2];
                        for (int k = 0; k < nen; k++) R[k] -= A1 * N1[k] + A2 * N2[k];
                    } else {
                        for (int k = 0; k < nen; k++) {
                            R[3 * k + 0] += A1 * dx1 * N1[k] + A2 * dx2 * N2[k];
                            R[3 * k + 1] += A1 * dy1 * N1[k] + A2 * dy2 * N2[k];
                            R[3 * k + 2] += A1 * dz1 * N1[k] + A2 * dy2 * N2[k];
                        }
                    }
                }
            }
        }
        for (int i = 0; i < 3; i++)
            for (int v = 0; v < 3; v++) {
                xs[i][v][0] *= 0.5;
                xs[i][v][1] *= 0.5;
            }
    }

    /* Return each node's value at its original position (:777-803). */
    for (int p = 0; p < nen; p++) {
        if (!flag) Int[perm[p]] = R[p];
        else
            for (int c = 0; c < 3; c++) Int[3 * perm[p] + c] = R[3 * p + c];
    }
}
