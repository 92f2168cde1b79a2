/*
 * ref_harness.c -- test infrastructure only.
 *
 * Flat-array entry points around the UNMODIFIED depSolver reference objects
 * (compiled from the reference tree by oracle/Makefile into oracle/_ref/).
 * The reference keeps its matrices as row-pointer arrays and reads its sizes
 * from globals defined by its own driver (src/depSolver.c:46-50); this file
 * defines those globals, builds row-pointer views over contiguous buffers and
 * calls the reference functions, so that tests can compare the GPU library
 * and the C restatement (oracle/port) against the reference itself.
 *
 * Nothing in the product links this file.  It is built only where the
 * reference sources are present.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* The reference's quadrature tables are defined by including gaussData.h in
 * exactly one translation unit (src/depSolver.c:40 does the same). */
#include "gaussData.h"

/* Globals the reference reads (defined in src/depSolver.c:46-50). */
FILE *file_log;
char cElemType[6];
unsigned int nDim, nElems, nElemType, nFPoints, nInternalPoints, nInterfaces,
             nMats, nNodes, nNodesAux, nNodesInElem, nCols, nColType, NX, NY, NZ;
double deltaX, deltaY, deltaZ;

/* Reference prototypes (src/assembly_el.h:29-67, src/gaussBksb.h:29,
 * src/gmres_el.h:29, src/field.h:30-41, src/potential.h:29-40,
 * src/force.h:54-73, src/kernelIntegrals.h:29-71). */
int electricFormA_tria3(double**, unsigned**, unsigned*, unsigned**, double**, double*, double**, double**, double*);
int electricFormA_tria6(double**, unsigned**, unsigned*, unsigned**, double**, double*, double**, double**, double*);
int electricFormFullA_tria3(double**, unsigned**, unsigned*, unsigned**, double**, double*, double**, double**, double*);
int electricFormFullA_tria6(double**, unsigned**, unsigned*, unsigned**, double**, double*, double**, double**, double*);
int gaussBksb(unsigned, double**, double*);
void solverGMRES_el(unsigned, unsigned, double**, double*);
void solverGMRES_el_tight(unsigned, unsigned, double**, double*);
int field_tria3(double*, double**, unsigned**, double*, double*);
int field_tria6(double*, double**, unsigned**, double*, double*);
int potential_tria3(double*, double**, unsigned**, double*, double*);
int potential_tria6(double*, double**, unsigned**, double*, double*);
int forceMST_tria3(double**, unsigned**, unsigned*, double*, double, double**, double**, double*, double*);
int forceMST_tria6(double**, unsigned**, unsigned*, double*, double, double**, double**, double*, double*);
int intG_tria3(double X[3][3], double*, double*);
int intG_tria6(double X[6][3], double*, double*);
int intH_tria3(const unsigned, double X[3][3], double*, double*, double*);
int intH_tria6(const unsigned, double X[6][3], double*, double*, double*);
int intSingularG_tria3(unsigned, double X[3][3], double*, double*);
int intSingularG_tria6(unsigned, double X[6][3], double*, double*);
int intSingularH_tria3(const unsigned, unsigned, double X[3][3], double*, double*, double*);
int intSingularH_tria6(const unsigned, unsigned, double X[6][3], double*, double*, double*);
int getNormal_tria3(unsigned, double**, unsigned**, double*);
int getNormal_tria6(unsigned, double**, unsigned**, double*);
int forceMultipole_tria3(unsigned, double, double*, double**, unsigned**, double*, double**, double*, double*);
int forceMultipole_tria6(unsigned, double, double*, double**, unsigned**, double*, double**, double*, double*);
int forceEllipsoid_tria3(unsigned, unsigned, double*, double*, double**, unsigned**, double*, double**, double*, double*);
int forceEllipsoid_tria6(unsigned, unsigned, double*, double*, double**, unsigned**, double*, double**, double*, double*);

static double **rows_d(double *base, unsigned nrows, unsigned ld)
{
    double **r = (double **)malloc((nrows ? nrows : 1) * sizeof(double *));
    for (unsigned i = 0; i < nrows; i++) r[i] = base + (size_t)i * ld;
    return r;
}

static unsigned **rows_u(unsigned *base, unsigned nrows, unsigned ld)
{
    unsigned **r = (unsigned **)malloc((nrows ? nrows : 1) * sizeof(unsigned *));
    for (unsigned i = 0; i < nrows; i++) r[i] = base + (size_t)i * ld;
    return r;
}

static void open_log(void)
{
    if (!file_log) file_log = fopen("bem.log", "a");
}

/* Sets the reference's size globals.  nen = 3 (tria3) or 6 (tria6). */
void ref_set_sizes(unsigned N, unsigned E, unsigned nIf)
{
    nNodes = N;
    nElems = E;
    nInterfaces = nIf;
    nDim = 3;
    open_log();
}

/* electricFormA_* (full = 0, A is N x 2N) or electricFormFullA_* (full = 1,
 * A is 2N x 2N).  A must be zeroed by the caller (the reference's caller
 * passes calloc'ed rows, src/depSolver.c:276-277). */
int ref_assemble(int nen, int full, unsigned N, unsigned E, unsigned nIf,
                 double *nodes, unsigned *elems, unsigned *bctype,
                 unsigned *ifaces, double *mat, double freq, double *mbc,
                 double *A, double *B)
{
    ref_set_sizes(N, E, nIf);
    double **mNodes = rows_d(nodes, N, 3);
    unsigned **mElems = rows_u(elems, E, (unsigned)nen);
    unsigned **vIf = nIf ? rows_u(ifaces, nIf, 2) : NULL;
    unsigned nmat = 0;
    for (unsigned i = 0; i < nIf; i++) {
        if (ifaces[2 * i] > nmat) nmat = ifaces[2 * i];
        if (ifaces[2 * i + 1] > nmat) nmat = ifaces[2 * i + 1];
    }
    double **vMat = rows_d(mat, nmat ? nmat : 1, 2);
    double **mBC = rows_d(mbc, 2 * N, 3);
    double **mA = rows_d(A, full ? 2 * N : N, 2 * N);
    double prob[1] = {freq};
    int rc;
    if (nen == 3)
        rc = full ? electricFormFullA_tria3(mNodes, mElems, bctype, vIf, vMat, prob, mA, mBC, B)
                  : electricFormA_tria3(mNodes, mElems, bctype, vIf, vMat, prob, mA, mBC, B);
    else
        rc = full ? electricFormFullA_tria6(mNodes, mElems, bctype, vIf, vMat, prob, mA, mBC, B)
                  : electricFormA_tria6(mNodes, mElems, bctype, vIf, vMat, prob, mA, mBC, B);
    free(mNodes); free(mElems); free(vIf); free(vMat); free(mBC); free(mA);
    return rc;
}

int ref_gauss(unsigned n, double *A, double *B)
{
    open_log();
    double **mA = rows_d(A, n, n);
    int rc = gaussBksb(n, mA, B);
    free(mA);
    return rc;
}

/* solverGMRES_el on the compact N x 2N form.  tight = 1 calls the copy built
 * with a tighter TOLERANCE (see oracle/Makefile).  Writes gmres.log in the
 * current directory, exactly as the reference does. */
void ref_gmres(int tight, unsigned preCond, unsigned N, double *A, double *B)
{
    nNodes = N;
    open_log();
    double **mA = rows_d(A, N, 2 * N);
    if (tight) solverGMRES_el_tight(preCond, 0, mA, B);
    else solverGMRES_el(preCond, 0, mA, B);
    free(mA);
}

int ref_field(int nen, unsigned N, unsigned E, double *nodes, unsigned *elems,
              double *vB, double *Xin, double *mE)
{
    ref_set_sizes(N, E, nInterfaces);
    double **mNodes = rows_d(nodes, N, 3);
    unsigned **mElems = rows_u(elems, E, (unsigned)nen);
    double x[3] = {Xin[0], Xin[1], Xin[2]};
    int rc = nen == 3 ? field_tria3(x, mNodes, mElems, vB, mE)
                      : field_tria6(x, mNodes, mElems, vB, mE);
    free(mNodes); free(mElems);
    return rc;
}

int ref_potential(int nen, unsigned N, unsigned E, double *nodes, unsigned *elems,
                  double *vB, double *Xin, double *mPot)
{
    ref_set_sizes(N, E, nInterfaces);
    double **mNodes = rows_d(nodes, N, 3);
    unsigned **mElems = rows_u(elems, E, (unsigned)nen);
    double x[3] = {Xin[0], Xin[1], Xin[2]};
    int rc = nen == 3 ? potential_tria3(x, mNodes, mElems, vB, mPot)
                      : potential_tria6(x, mNodes, mElems, vB, mPot);
    free(mNodes); free(mElems);
    return rc;
}

int ref_forceMST(int nen, unsigned N, unsigned E, double *nodes, unsigned *elems,
                 unsigned *bctype, double *vB, double eps, double *Fce,
                 double *Xce, double *Fcm, double *Xcm)
{
    ref_set_sizes(N, E, nInterfaces);
    double **mNodes = rows_d(nodes, N, 3);
    unsigned **mElems = rows_u(elems, E, (unsigned)nen);
    double **mFce = rows_d(Fce, E, 3);
    double **mXce = rows_d(Xce, E, 3);
    int rc = nen == 3 ? forceMST_tria3(mNodes, mElems, bctype, vB, eps, mFce, mXce, Fcm, Xcm)
                      : forceMST_tria6(mNodes, mElems, bctype, vB, eps, mFce, mXce, Fcm, Xcm);
    free(mNodes); free(mElems); free(mFce); free(mXce);
    return rc;
}

/* forceMultipole_* (src/force.c:572,709) at Xeval for a sphere of radius R:
 * mat holds the medium's and the particle's (sigma, eps_r) rows. */
int ref_forceMultipole(int nen, unsigned N, unsigned E, double *nodes, unsigned *elems,
                       double *vB, unsigned order, double R, double *Xeval, double *mat,
                       double freq, double *F)
{
    ref_set_sizes(N, E, nInterfaces);
    double **mNodes = rows_d(nodes, N, 3);
    unsigned **mElems = rows_u(elems, E, (unsigned)nen);
    double m[4] = {mat[0], mat[1], mat[2], mat[3]};
    double **vMat = rows_d(m, 2, 2);
    double prob[1] = {freq};
    double x[3] = {Xeval[0], Xeval[1], Xeval[2]};
    int rc = nen == 3 ? forceMultipole_tria3(order, R, x, mNodes, mElems, vB, vMat, prob, F)
                      : forceMultipole_tria6(order, R, x, mNodes, mElems, vB, vMat, prob, F);
    free(mNodes); free(mElems); free(vMat);
    return rc;
}

/* forceEllipsoid_* (src/force.c:65,204): analysis 10 (homogeneous) or 11
 * (shelled); the reference rescales the particle's row of vMatParam in place
 * for 11, so it works on a copy here. */
int ref_forceEllipsoid(int nen, unsigned N, unsigned E, double *nodes, unsigned *elems,
                       double *vB, unsigned analysis, double *axis, double *Xeval, double *mat,
                       double freq, double *F)
{
    ref_set_sizes(N, E, nInterfaces);
    double **mNodes = rows_d(nodes, N, 3);
    unsigned **mElems = rows_u(elems, E, (unsigned)nen);
    double m[4] = {mat[0], mat[1], mat[2], mat[3]};
    double **vMat = rows_d(m, 2, 2);
    double prob[1] = {freq};
    double x[3] = {Xeval[0], Xeval[1], Xeval[2]};
    double ax[3] = {axis[0], axis[1], axis[2]};
    int rc = nen == 3 ? forceEllipsoid_tria3(analysis, 1, ax, x, mNodes, mElems, vB, vMat, prob, F)
                      : forceEllipsoid_tria6(analysis, 1, ax, x, mNodes, mElems, vB, vMat, prob, F);
    free(mNodes); free(mElems); free(vMat);
    return rc;
}

/* Single-element integrals: X is nen x 3 (copied, because the singular H
 * routines reorder their X argument in place). */
int ref_int(int which, int nen, unsigned flag, unsigned sinNode,
            const double *X, double *Xeval, double *Int, double *normal)
{
    double X3[3][3], X6[6][3];
    for (int k = 0; k < nen; k++)
        for (int d = 0; d < 3; d++) {
            if (nen == 3) X3[k][d] = X[k * 3 + d];
            else X6[k][d] = X[k * 3 + d];
        }
    switch (which) {
    case 0: return nen == 3 ? intG_tria3(X3, Xeval, Int) : intG_tria6(X6, Xeval, Int);
    case 1: return nen == 3 ? intH_tria3(flag, X3, Xeval, Int, normal) : intH_tria6(flag, X6, Xeval, Int, normal);
    case 2: return nen == 3 ? intSingularG_tria3(sinNode, X3, Xeval, Int) : intSingularG_tria6(sinNode, X6, Xeval, Int);
    default: return nen == 3 ? intSingularH_tria3(flag, sinNode, X3, Xeval, Int, normal)
                             : intSingularH_tria6(flag, sinNode, X6, Xeval, Int, normal);
    }
}

int ref_node_normal(int nen, unsigned N, unsigned E, double *nodes, unsigned *elems,
                    unsigned node1, double *normal)
{
    ref_set_sizes(N, E, nInterfaces);
    double **mNodes = rows_d(nodes, N, 3);
    unsigned **mElems = rows_u(elems, E, (unsigned)nen);
    int rc = nen == 3 ? getNormal_tria3(node1, mNodes, mElems, normal)
                      : getNormal_tria6(node1, mNodes, mElems, normal);
    free(mNodes); free(mElems);
    return rc;
}
