/*
 * postproc.c -- field, potential and Maxwell-stress force
 * (oracle restatement of src/field.c, src/potential.c, src/force.c and
 * src/forceIntegrals.c; test infrastructure).
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include "oracle.h"

static void element_coords(int nen, const double *nodes, const unsigned *el, double *X)
{
    for (int k = 0; k < nen; k++) {
        const double *x = nodes + 3 * (size_t)(el[k] - 1);
        X[k * 3 + 0] = x[0];
        X[k * 3 + 1] = x[1];
        X[k * 3 + 2] = x[2];
    }
}

/* E(x) = 1/(4 pi eps0) sum_e sum_k Int_k sigma_k, with the singular
 * integral for every element that has a node at exactly x (coordinate
 * equality).  For each such element the jump term sigma / (2 eps0) n is
 * added once, with sigma taken at the element's FIRST node and n the
 * averaged normal of the matching node -- the reference's behaviour
 * (src/field.c:137-200, jump term :189-195), kept for parity. */
void orc_field(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
               const double *vB, const double *Xin, double *mE)
{
    const double B = 0.5 / ORC_EPS0;
    const double A = B / ORC_PI2;
    double X[18], Sub[18], nrm[3] = {0, 0, 0};
    for (int i = 0; i < 6; i++) mE[i] = 0.0;
    for (unsigned e = 0; e < E; e++) {
        const unsigned *el = elems + (size_t)e * nen;
        element_coords(nen, nodes, el, X);
        int test = 0;
        unsigned sin = 0;
        for (int j = 0; j < nen; j++) {
            double dx = Xin[0] - X[j * 3], dy = Xin[1] - X[j * 3 + 1], dz = Xin[2] - X[j * 3 + 2];
            if (dx == 0 && dy == 0.0 && dz == 0.0 && test == 0) {
                test = 1;
                sin = (unsigned)j + 1;
                orc_node_normal(nen, E, nodes, elems, el[j], nrm);
            }
        }
        if (test) orc_intSingularH(nen, 1, sin, X, Xin, Sub, nrm);
        else orc_intH(nen, 1, X, Xin, Sub, nrm);
        for (int j = 0; j < nen; j++) {
            unsigned c = el[j] - 1;
            for (int k = 0; k < 3; k++) {
                mE[k * 2] += A * Sub[j * 3 + k] * vB[c];
                mE[k * 2 + 1] += A * Sub[j * 3 + k] * vB[c + N];
            }
            if (test == 1) {
                for (int k = 0; k < 3; k++) {
                    mE[k * 2] += B * vB[c] * nrm[k];
                    mE[k * 2 + 1] += B * vB[c + N] * nrm[k];
                }
                test = 2;
            }
        }
    }
}

/* phi(x) = 1/(4 pi eps0) sum_e sum_k Int_k sigma_k (src/potential.c:126-179). */
void orc_potential(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
                   const double *vB, const double *Xin, double *mPot)
{
    const double A = 1.0 / (ORC_PI4 * ORC_EPS0);
    double X[18], Sub[6];
    mPot[0] = mPot[1] = 0.0;
    for (unsigned e = 0; e < E; e++) {
        const unsigned *el = elems + (size_t)e * nen;
        element_coords(nen, nodes, el, X);
        unsigned sin = 0;
        for (int j = 0; j < nen; j++) {
            double dx = X[j * 3] - Xin[0], dy = X[j * 3 + 1] - Xin[1], dz = X[j * 3 + 2] - Xin[2];
            if (dx == 0 && dy == 0.0 && dz == 0.0 && sin == 0) sin = (unsigned)j + 1;
        }
        if (sin) orc_intSingularG(nen, sin, X, Xin, Sub);
        else orc_intG(nen, X, Xin, Sub);
        for (int j = 0; j < nen; j++) {
            unsigned c = el[j] - 1;
            mPot[0] += A * Sub[j] * vB[c];
            mPot[1] += A * Sub[j] * vB[c + N];
        }
    }
}

struct fp_pool {
    int nen;
    unsigned N, E, npts, next;
    const double *nodes, *vB, *pts;
    const unsigned *elems;
    double *mE;
};

static void *fp_thread(void *p)
{
    struct fp_pool *pl = (struct fp_pool *)p;
    for (;;) {
        unsigned i = __atomic_fetch_add(&pl->next, 1u, __ATOMIC_RELAXED);
        if (i >= pl->npts) break;
        orc_field(pl->nen, pl->N, pl->E, pl->nodes, pl->elems, pl->vB, pl->pts + 3 * (size_t)i,
                  pl->mE + 6 * (size_t)i);
    }
    return NULL;
}

void orc_field_points(int nen, unsigned N, unsigned E, const double *nodes,
                      const unsigned *elems, const double *vB, unsigned npts,
                      const double *pts, double *mE, int nthreads)
{
    struct fp_pool pl = {nen, N, E, npts, 0, nodes, vB, pts, elems, mE};
    if (nthreads <= 1) {
        fp_thread(&pl);
        return;
    }
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof *th);
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, fp_thread, &pl);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th);
}

/* 7-point integral of T.n = E (E.n) - |E|^2 n / 2 over one element, with the
 * field interpolated from the nodal values and the local normal at each
 * point (intF_tria3 src/forceIntegrals.c:632-671, intF_tria6 :684-723). */
void orc_intF(int nen, const double *X, const double *En, double Int[3])
{
    double N[6], XL[3], n[3];
    Int[0] = Int[1] = Int[2] = 0.0;
    for (int q = 0; q < ORC_TNGAUSS; q++) {
        const double L[2] = {orc_triangle7[q][0], orc_triangle7[q][1]};
        orc_shape(nen, L, N);
        double J = orc_x2l(nen, X, L, N, XL);
        orc_local_normal(nen, X, L, n);
        double Ex = 0, Ey = 0, Ez = 0;
        for (int k = 0; k < nen; k++) {
            Ex += En[k * 3] * N[k];
            Ey += En[k * 3 + 1] * N[k];
            Ez += En[k * 3 + 2] * N[k];
        }
        double NE = Ex * n[0] + Ey * n[1] + Ez * n[2];
        double Esq = Ex * Ex + Ey * Ey + Ez * Ez;
        double A = J * orc_triangle7[q][2];
        Int[0] += A * (Ex * NE - 0.5 * Esq * n[0]);
        Int[1] += A * (Ey * NE - 0.5 * Esq * n[1]);
        Int[2] += A * (Ez * NE - 0.5 * Esq * n[2]);
    }
}

/* Maxwell-stress force on every element whose first node has boundary type
 * 6, using Re(E) at the type-6 nodes; Xcm is the mean of those nodes
 * (forceMST_tria3 src/force.c:348-437, forceMST_tria6 :463-552). */
int orc_forceMST(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
                 const unsigned *bctype, const double *vB, double eps,
                 double *Fce, double *Xce, double *Fcm, double *Xcm, int nthreads)
{
    const double A = 0.5 * eps;
    double *Ef = (double *)calloc((size_t)N * 3, sizeof(double));
    unsigned np = 0;
    for (unsigned i = 0; i < N; i++) np += bctype[i] == 6;
    unsigned *ids = (unsigned *)malloc((np ? np : 1) * sizeof(unsigned));
    double *pts = (double *)calloc((np ? np : 1) * 3, sizeof(double));
    double *mE = (double *)malloc((np ? np : 1) * 6 * sizeof(double));
    Xcm[0] = Xcm[1] = Xcm[2] = 0.0;
    Fcm[0] = Fcm[1] = Fcm[2] = 0.0;
    unsigned p = 0;
    for (unsigned i = 0; i < N; i++) {
        if (bctype[i] != 6) continue;
        ids[p] = i;
        for (int d = 0; d < 3; d++) {
            pts[3 * p + d] = nodes[3 * (size_t)i + d];
            Xcm[d] += nodes[3 * (size_t)i + d];
        }
        p++;
    }
    orc_field_points(nen, N, E, nodes, elems, vB, np, pts, mE, nthreads);
    for (unsigned q = 0; q < np; q++) {
        Ef[3 * (size_t)ids[q] + 0] = mE[6 * q + 0];
        Ef[3 * (size_t)ids[q] + 1] = mE[6 * q + 2];
        Ef[3 * (size_t)ids[q] + 2] = mE[6 * q + 4];
    }
    Xcm[0] /= np;
    Xcm[1] /= np;
    Xcm[2] /= np;
    double X[18], En[18], mF[3], M[6], XL[3];
    const double Lc[2] = {0.25, 0.25};
    for (unsigned e = 0; e < E; e++) {
        const unsigned *el = elems + (size_t)e * nen;
        if (bctype[el[0] - 1] != 6) continue;
        element_coords(nen, nodes, el, X);
        for (int k = 0; k < nen; k++)
            for (int d = 0; d < 3; d++) En[k * 3 + d] = Ef[3 * (size_t)(el[k] - 1) + d];
        orc_intF(nen, X, En, mF);
        orc_shape(nen, Lc, M);
        orc_x2l(nen, X, Lc, M, XL);
        for (int d = 0; d < 3; d++) {
            Fce[3 * (size_t)e + d] = A * mF[d];
            Xce[3 * (size_t)e + d] = XL[d];
            Fcm[d] += Fce[3 * (size_t)e + d];
        }
    }
    free(Ef); free(ids); free(pts); free(mE);
    return 0;
}
