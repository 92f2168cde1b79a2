/*
 * quad8.c -- the quad8 element family (test infrastructure).
 *
 * The reference has no quad8 integrals (it recognises the element type,
 * src/preProcess.c:142-146, and its driver rejects it), so this is the
 * oracle of the GPU library's quad8 extension, written independently in
 * plain loops from the same definitions:
 *   - serendipity element on [-1, 1]^2, nodes 1-4 the corners (-1,-1),
 *     (1,-1), (1,1), (-1,1), nodes 5-8 the mid-sides of edges 1-2, 2-3,
 *     3-4, 4-1;
 *   - regular integrals by the 3 x 3 Gauss-Legendre product rule;
 *   - singular integrals (the collocation point is node s of the element)
 *     on the triangles of the parent square with their apex at node s (two
 *     for a corner, three for a mid-side node): G by the Duffy map with
 *     8 x 8 Gauss-Legendre / Gauss-Jacobi points (as the reference does for
 *     triangles, src/kernelIntegrals.c:311-345), H and the field's gradient
 *     by 8 levels of subdivision towards the apex with the 7-point rule
 *     and the innermost triangle left out (src/kernelIntegrals.c:472-593);
 *   - the field on a node takes the jump sigma / (2 eps0) n once, with
 *     that node's sigma and normal.
 * Parity unpinned: there is no reference output to pin these to; the
 * tests compare them with the GPU library and with analytic fields.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

static const double GL3[3][2] = {{-0.7745966692414834, 0.5555555555555556},
                                 {0.0, 0.8888888888888888},
                                 {0.7745966692414834, 0.5555555555555556}};
static const double Q8N[8][2] = {{-1.0, -1.0}, {1.0, -1.0}, {1.0, 1.0}, {-1.0, 1.0},
                                 {0.0, -1.0},  {1.0, 0.0},  {0.0, 1.0}, {-1.0, 0.0}};

void orc_q8_shape(double xi, double eta, double N[8], double Nx[8], double Ne[8])
{
    for (int k = 0; k < 8; k++) {
        const double px = Q8N[k][0], py = Q8N[k][1];
        if (k < 4) {
            const double a = xi * px, b = eta * py;
            N[k] = 0.25 * (1.0 + a) * (1.0 + b) * (a + b - 1.0);
            Nx[k] = 0.25 * px * (1.0 + b) * (2.0 * a + b);
            Ne[k] = 0.25 * py * (1.0 + a) * (a + 2.0 * b);
        } else if (px == 0.0) {
            const double b = eta * py;
            N[k] = 0.5 * (1.0 - xi * xi) * (1.0 + b);
            Nx[k] = -xi * (1.0 + b);
            Ne[k] = 0.5 * py * (1.0 - xi * xi);
        } else {
            const double a = xi * px;
            N[k] = 0.5 * (1.0 + a) * (1.0 - eta * eta);
            Nx[k] = 0.5 * px * (1.0 - eta * eta);
            Ne[k] = -eta * (1.0 + a);
        }
    }
}

/* X(xi, eta) into XL, shape values into N, unit normal into n (may be
 * NULL); returns the surface Jacobian.  X is 8 x 3. */
double orc_q8_map(const double *X, double xi, double eta, double XL[3], double N[8], double *n)
{
    double Nx[8], Ne[8], t1[3] = {0, 0, 0}, t2[3] = {0, 0, 0};
    orc_q8_shape(xi, eta, N, Nx, Ne);
    for (int d = 0; d < 3; d++) {
        XL[d] = 0.0;
        for (int k = 0; k < 8; k++) {
            XL[d] += N[k] * X[3 * k + d];
            t1[d] += Nx[k] * X[3 * k + d];
            t2[d] += Ne[k] * X[3 * k + d];
        }
    }
    const double c0 = t1[1] * t2[2] - t2[1] * t1[2];
    const double c1 = t2[0] * t1[2] - t1[0] * t2[2];
    const double c2 = t1[0] * t2[1] - t2[0] * t1[1];
    const double J = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
    if (n) {
        n[0] = c0 / J;
        n[1] = c1 / J;
        n[2] = c2 / J;
    }
    return J;
}

/* Triangles (apex, P1, P2) of the parent square with the apex at node s
 * (0-based); returns their number. */
static int apex_triangles(int s, double tri[3][3][2])
{
    const int c = s < 4 ? s : s - 4, count = s < 4 ? 2 : 3;
    for (int t = 0; t < count; t++) {
        const int a = (c + 1 + t) % 4, b = (c + 2 + t) % 4;
        tri[t][0][0] = Q8N[s][0];
        tri[t][0][1] = Q8N[s][1];
        tri[t][1][0] = Q8N[a][0];
        tri[t][1][1] = Q8N[a][1];
        tri[t][2][0] = Q8N[b][0];
        tri[t][2][1] = Q8N[b][1];
    }
    return count;
}

/* Regular G: Int[k] = sum over the 3 x 3 points of w J N_k / r. */
void orc_q8_intG(const double *X, const double *Xe, double Int[8])
{
    double XL[3], N[8];
    for (int k = 0; k < 8; k++) Int[k] = 0.0;
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            const double J = orc_q8_map(X, GL3[a][0], GL3[b][0], XL, N, NULL);
            const double dx = Xe[0] - XL[0], dy = Xe[1] - XL[1], dz = Xe[2] - XL[2];
            const double w = GL3[a][1] * GL3[b][1] * J / sqrt(dx * dx + dy * dy + dz * dz);
            for (int k = 0; k < 8; k++) Int[k] += w * N[k];
        }
}

/* Regular H: flag 0: Int[k] = sum of w J (d . n) / r^3 N_k; flag 1:
 * Int[3k + c] = sum of w J d_c / r^3 N_k (d = Xe - X). */
void orc_q8_intH(int flag, const double *X, const double *Xe, double *Int, const double *n)
{
    double XL[3], N[8];
    const int nout = flag ? 24 : 8;
    for (int k = 0; k < nout; k++) Int[k] = 0.0;
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            const double J = orc_q8_map(X, GL3[a][0], GL3[b][0], XL, N, NULL);
            const double dx = Xe[0] - XL[0], dy = Xe[1] - XL[1], dz = Xe[2] - XL[2];
            const double r = sqrt(dx * dx + dy * dy + dz * dz);
            const double w = GL3[a][1] * GL3[b][1] * J / (r * r * r);
            for (int k = 0; k < 8; k++) {
                if (flag == 0) {
                    Int[k] += w * (dx * n[0] + dy * n[1] + dz * n[2]) * N[k];
                } else {
                    Int[3 * k] += w * dx * N[k];
                    Int[3 * k + 1] += w * dy * N[k];
                    Int[3 * k + 2] += w * dz * N[k];
                }
            }
        }
}

/* Singular G at node s (0-based): Int[k] = int N_k / r. */
void orc_q8_intSingularG(int s, const double *X, const double *Xe, double Int[8])
{
    double tri[3][3][2], XL[3], N[8];
    const int nt = apex_triangles(s, tri);
    for (int k = 0; k < 8; k++) Int[k] = 0.0;
    for (int t = 0; t < nt; t++) {
        const double a1 = tri[t][1][0] - tri[t][0][0], a2 = tri[t][1][1] - tri[t][0][1];
        const double b1 = tri[t][2][0] - tri[t][0][0], b2 = tri[t][2][1] - tri[t][0][1];
        const double det = a1 * b2 - a2 * b1;
        for (int i = 0; i < ORC_NGAUSS; i++)
            for (int j = 0; j < ORC_NGAUSS; j++) {
                const double u1 = orc_gauss_legendre8[i][0], u2 = orc_gauss_jacobi8[j][0];
                /* Duffy map of the unit triangle with its vertex (0, 0) at u2 = -1 */
                const double l1 = 0.25 * (1.0 + u1) * (1.0 + u2), l2 = 0.25 * (1.0 - u1) * (1.0 + u2);
                const double xi = tri[t][0][0] + l1 * a1 + l2 * b1, eta = tri[t][0][1] + l1 * a2 + l2 * b2;
                const double J = orc_q8_map(X, xi, eta, XL, N, NULL);
                const double dx = Xe[0] - XL[0], dy = Xe[1] - XL[1], dz = Xe[2] - XL[2];
                const double w = orc_gauss_legendre8[i][1] * orc_gauss_jacobi8[j][1] * 0.125 * det * J /
                                 sqrt(dx * dx + dy * dy + dz * dz);
                for (int k = 0; k < 8; k++) Int[k] += w * N[k];
            }
    }
}

/* Singular H at node s: flag 0 Int[k] = -int (d . n) / r^3 N_k (the
 * assembly's sign, as the triangles' singular H); flag 1 Int[3k + c] =
 * int d_c / r^3 N_k. */
void orc_q8_intSingularH(int flag, int s, const double *X, const double *Xe, double *Int, const double *n)
{
    static const double XS[3][3][2] = {{{1.0, 0.0}, {0.5, 0.5}, {0.5, 0.0}},
                                       {{0.5, 0.0}, {0.5, 0.5}, {0.0, 0.5}},
                                       {{0.5, 0.5}, {0.0, 1.0}, {0.0, 0.5}}};
    double tri[3][3][2], XL[3], N[8];
    const int nt = apex_triangles(s, tri), nout = flag ? 24 : 8;
    for (int k = 0; k < nout; k++) Int[k] = 0.0;
    for (int t = 0; t < nt; t++) {
        const double a1 = tri[t][1][0] - tri[t][0][0], a2 = tri[t][1][1] - tri[t][0][1];
        const double b1 = tri[t][2][0] - tri[t][0][0], b2 = tri[t][2][1] - tri[t][0][1];
        const double det = a1 * b2 - a2 * b1;
        double scale = 1.0, Js = 0.25;
        for (int m = 0; m < ORC_NSUBDIV; m++) {
            for (int i = 0; i < 3; i++)
                for (int q = 0; q < ORC_TNGAUSS; q++) {
                    const double M1 = orc_triangle7[q][0], M2 = orc_triangle7[q][1], M3 = 1.0 - M1 - M2;
                    const double l1 = (XS[i][0][0] * M1 + XS[i][1][0] * M2 + XS[i][2][0] * M3) * scale;
                    const double l2 = (XS[i][0][1] * M1 + XS[i][1][1] * M2 + XS[i][2][1] * M3) * scale;
                    const double xi = tri[t][0][0] + l1 * a1 + l2 * b1, eta = tri[t][0][1] + l1 * a2 + l2 * b2;
                    const double J = orc_q8_map(X, xi, eta, XL, N, NULL);
                    const double dx = Xe[0] - XL[0], dy = Xe[1] - XL[1], dz = Xe[2] - XL[2];
                    const double r2 = dx * dx + dy * dy + dz * dz;
                    const double A = Js * orc_triangle7[q][2] * det * J / (r2 * sqrt(r2));
                    for (int k = 0; k < 8; k++) {
                        if (flag == 0) {
                            Int[k] -= A * (dx * n[0] + dy * n[1] + dz * n[2]) * N[k];
                        } else {
                            Int[3 * k] += A * dx * N[k];
                            Int[3 * k + 1] += A * dy * N[k];
                            Int[3 * k + 2] += A * dz * N[k];
                        }
                    }
                }
            scale *= 0.5;
            Js *= 0.25;
        }
    }
}

static void coords8(const double *nodes, const unsigned *el, double *X)
{
    for (int k = 0; k < 8; k++)
        for (int d = 0; d < 3; d++) X[3 * k + d] = nodes[3 * (size_t)(el[k] - 1) + d];
}

/* Averaged unit normal at 1-based node `node1`: the sum over the elements
 * containing it (first position in each) of the unit normal there. */
void orc_q8_node_normal(unsigned E, const double *nodes, const unsigned *elems, unsigned node1, double n[3])
{
    double acc[3] = {0.0, 0.0, 0.0}, X[24], XL[3], N[8], ln[3];
    for (unsigned e = 0; e < E; e++) {
        const unsigned *el = elems + (size_t)e * 8;
        int pos = -1;
        for (int k = 0; k < 8; k++)
            if (el[k] == node1) {
                pos = k;
                break;
            }
        if (pos < 0) continue;
        coords8(nodes, el, X);
        orc_q8_map(X, Q8N[pos][0], Q8N[pos][1], XL, N, ln);
        for (int d = 0; d < 3; d++) acc[d] += ln[d];
    }
    const double inv = 1.0 / sqrt(acc[0] * acc[0] + acc[1] * acc[1] + acc[2] * acc[2]);
    for (int d = 0; d < 3; d++) n[d] = acc[d] * inv;
}

/* The compact (full = 0, N rows of 2N) or full (2N rows) system, rows
 * formed as orc_assemble forms them (conductor rows C int G N_k, the other
 * rows the interface coefficients times -int dG/dn N_k, -1/(2 eps0) on the
 * diagonal).  A zeroed by the caller; returns 1 on an undefined boundary
 * type. */
int orc_q8_assemble(int full, unsigned N, unsigned E, unsigned nIf, const double *nodes, const unsigned *elems,
                    const unsigned *bctype, const unsigned *ifaces, const double *mat, double freq,
                    const double *mbc, double *A, size_t lda, double *B)
{
    const double C = 1.0 / (ORC_PI4 * ORC_EPS0);
    double *Ak = (double *)calloc(nIf ? nIf : 1, sizeof(double));
    double *Bk = (double *)calloc(nIf ? nIf : 1, sizeof(double));
    if (nIf) orc_interface_coeffs(nIf, ifaces, mat, freq, Ak, Bk);
    double X[24], Sub[8], nrm[3] = {0, 0, 0};
    int bad = 0;
    for (unsigned i = 0; i < N; i++) {
        const unsigned t = bctype[i];
        if (t != 0 && t != 1 && t != 6) {
            bad = 1;
            continue;
        }
        double *Ai = A + (size_t)i * lda, *Aim = full ? A + (size_t)(i + N) * lda : NULL;
        const double *Xe = nodes + 3 * (size_t)i;
        unsigned ifc = 0;
        if (t != 1) {
            ifc = (unsigned)mbc[3 * (size_t)i + 1] - 1;
            orc_q8_node_normal(E, nodes, elems, i + 1, nrm);
            Ai[i] -= 0.5 / ORC_EPS0;
            if (full) Aim[i + N] -= 0.5 / ORC_EPS0;
        }
        for (unsigned e = 0; e < E; e++) {
            const unsigned *el = elems + (size_t)e * 8;
            int sin = -1;
            for (int k = 0; k < 8; k++)
                if (el[k] - 1 == i) sin = k;
            coords8(nodes, el, X);
            if (t == 1) {
                if (sin < 0) orc_q8_intG(X, Xe, Sub);
                else orc_q8_intSingularG(sin, X, Xe, Sub);
                for (int k = 0; k < 8; k++) {
                    const unsigned c = el[k] - 1;
                    Ai[c] += C * Sub[k];
                    if (full) Aim[c + N] += C * Sub[k];
                }
            } else {
                if (sin < 0) {
                    orc_q8_intH(0, X, Xe, Sub, nrm);
                    for (int k = 0; k < 8; k++) Sub[k] = -Sub[k];
                } else {
                    orc_q8_intSingularH(0, sin, X, Xe, Sub, nrm);
                }
                for (int k = 0; k < 8; k++) {
                    const unsigned c = el[k] - 1;
                    Ai[c] += Ak[ifc] * Sub[k];
                    Ai[c + N] += Bk[ifc] * Sub[k];
                    if (full) {
                        Aim[c] -= Bk[ifc] * Sub[k];
                        Aim[c + N] += Ak[ifc] * Sub[k];
                    }
                }
            }
        }
        B[i] = mbc[3 * (size_t)i];
        B[i + N] = mbc[3 * (size_t)(i + N)];
    }
    free(Ak);
    free(Bk);
    return bad;
}

/* Field (6 values) at Xin: regular gradient sums, the singular ones for the
 * elements with a node at exactly Xin (first such position), and the jump
 * sigma / (2 eps0) n of the lowest-numbered node at Xin once. */
void orc_q8_field(unsigned N, unsigned E, const double *nodes, const unsigned *elems, const double *vB,
                  const double *Xin, double mE[6])
{
    const double A = 1.0 / (ORC_PI4 * ORC_EPS0);
    double X[24], Sub[24], nrm[3];
    unsigned first = 0;
    for (int i = 0; i < 6; i++) mE[i] = 0.0;
    for (unsigned e = 0; e < E; e++) {
        const unsigned *el = elems + (size_t)e * 8;
        coords8(nodes, el, X);
        int sin = -1;
        for (int k = 0; k < 8 && sin < 0; k++)
            if (X[3 * k] == Xin[0] && X[3 * k + 1] == Xin[1] && X[3 * k + 2] == Xin[2]) sin = k;
        if (sin >= 0) orc_q8_intSingularH(1, sin, X, Xin, Sub, NULL);
        else orc_q8_intH(1, X, Xin, Sub, NULL);
        for (int k = 0; k < 8; k++) {
            const unsigned c = el[k] - 1;
            for (int d = 0; d < 3; d++) {
                mE[2 * d] += A * Sub[3 * k + d] * vB[c];
                mE[2 * d + 1] += A * Sub[3 * k + d] * vB[c + N];
            }
        }
    }
    for (unsigned v = 0; v < N; v++)
        if (nodes[3 * (size_t)v] == Xin[0] && nodes[3 * (size_t)v + 1] == Xin[1] &&
            nodes[3 * (size_t)v + 2] == Xin[2]) {
            first = v + 1;
            break;
        }
    if (first) {
        orc_q8_node_normal(E, nodes, elems, first, nrm);
        const double B = 0.5 / ORC_EPS0;
        for (int d = 0; d < 3; d++) {
            mE[2 * d] += B * vB[first - 1] * nrm[d];
            mE[2 * d + 1] += B * vB[first - 1 + N] * nrm[d];
        }
    }
}

/* Potential (2 values) at Xin. */
void orc_q8_potential(unsigned N, unsigned E, const double *nodes, const unsigned *elems, const double *vB,
                      const double *Xin, double mPot[2])
{
    const double A = 1.0 / (ORC_PI4 * ORC_EPS0);
    double X[24], Sub[8];
    mPot[0] = mPot[1] = 0.0;
    for (unsigned e = 0; e < E; e++) {
        const unsigned *el = elems + (size_t)e * 8;
        coords8(nodes, el, X);
        int sin = -1;
        for (int k = 0; k < 8 && sin < 0; k++)
            if (X[3 * k] == Xin[0] && X[3 * k + 1] == Xin[1] && X[3 * k + 2] == Xin[2]) sin = k;
        if (sin >= 0) orc_q8_intSingularG(sin, X, Xin, Sub);
        else orc_q8_intG(X, Xin, Sub);
        for (int k = 0; k < 8; k++) {
            const unsigned c = el[k] - 1;
            mPot[0] += A * Sub[k] * vB[c];
            mPot[1] += A * Sub[k] * vB[c + N];
        }
    }
}

/* Maxwell-stress force on the elements whose first node has type 6: Re(E)
 * at the type-6 nodes, 3 x 3 points of eps / 2 [E (E.n) - |E|^2 n / 2] with
 * the element's unit normal, Xce = X(0, 0), Xcm the mean of the type-6
 * nodes. */
void orc_q8_forceMST(unsigned N, unsigned E, const double *nodes, const unsigned *elems, const unsigned *bctype,
                     const double *vB, double eps, double *Fce, double *Xce, double Fcm[3], double Xcm[3])
{
    double *Ef = (double *)calloc((size_t)N * 3, sizeof(double));
    double mE[6], X[24], XL[3], Nv[8], n[3];
    unsigned np = 0;
    for (int d = 0; d < 3; d++) Fcm[d] = Xcm[d] = 0.0;
    for (unsigned i = 0; i < N; i++) {
        if (bctype[i] != 6) continue;
        orc_q8_field(N, E, nodes, elems, vB, nodes + 3 * (size_t)i, mE);
        for (int d = 0; d < 3; d++) {
            Ef[3 * (size_t)i + d] = mE[2 * d];
            Xcm[d] += nodes[3 * (size_t)i + d];
        }
        np++;
    }
    if (np == 0) {
        free(Ef);
        return;
    }
    for (int d = 0; d < 3; d++) Xcm[d] /= np;
    for (unsigned e = 0; e < E; e++) {
        const unsigned *el = elems + (size_t)e * 8;
        if (bctype[el[0] - 1] != 6) continue;
        coords8(nodes, el, X);
        double I[3] = {0.0, 0.0, 0.0};
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                const double J = orc_q8_map(X, GL3[a][0], GL3[b][0], XL, Nv, n);
                double Ev[3] = {0.0, 0.0, 0.0};
                for (int k = 0; k < 8; k++)
                    for (int d = 0; d < 3; d++) Ev[d] += Ef[3 * (size_t)(el[k] - 1) + d] * Nv[k];
                const double NE = Ev[0] * n[0] + Ev[1] * n[1] + Ev[2] * n[2];
                const double Esq = Ev[0] * Ev[0] + Ev[1] * Ev[1] + Ev[2] * Ev[2];
                const double w = GL3[a][1] * GL3[b][1] * J;
                for (int d = 0; d < 3; d++) I[d] += w * (Ev[d] * NE - 0.5 * Esq * n[d]);
            }
        orc_q8_map(X, 0.0, 0.0, XL, Nv, NULL);
        for (int d = 0; d < 3; d++) {
            Fce[3 * (size_t)e + d] = 0.5 * eps * I[d];
            Xce[3 * (size_t)e + d] = XL[d];
            Fcm[d] += Fce[3 * (size_t)e + d];
        }
    }
    free(Ef);
}
