/*
 * oracle.h -- CPU restatement of depSolver's BEM hot path (test infrastructure).
 *
 * This library is the oracle for the GPU library and the CPU baseline of the
 * benchmark.  It is NOT part of the product: only tests, the smoke check and
 * the benchmark's CPU leg load it.  Every function restates one reference
 * function (cited by file:line in the reference tree) in plain C99 on flat
 * arrays, keeping the reference's arithmetic, loop order and quirks:
 *
 *   nodes  : N x 3 doubles, row-major
 *   elems  : E x nen unsigned, 1-based node ids (as read from elems.bem)
 *   bctype : 2N unsigned (rows N..2N-1 describe the imaginary equations)
 *   mbc    : 2N x 3 doubles (value, interface id, unused)
 *   ifaces : nIf x 2 unsigned material ids (1-based)
 *   mat    : nMat x 2 doubles (sigma, eps_r)
 *
 * nen is 3 (tria3) or 6 (tria6).
 */
#ifndef DSC_ORACLE_H
#define DSC_ORACLE_H

#include <stddef.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Physical constants and rule sizes (reference src/constants.h:42-55). */
#define ORC_EPS0 8.854187817E-12
#define ORC_PI2 6.283185307179586E+00
#define ORC_PI4 1.256637061435917E+01
#define ORC_NGAUSS 8
#define ORC_TNGAUSS 7
#define ORC_NSUBDIV 8

extern const double orc_gauss_legendre8[ORC_NGAUSS][2];
extern const double orc_gauss_jacobi8[ORC_NGAUSS][2];
extern const double orc_triangle7[ORC_TNGAUSS][3];

/* Shape functions and isoparametric map (src/shapeFunctions.c:53-87,
 * src/globalToLocal.c:75-148). */
void orc_shape(int nen, const double L[2], double *N);
double orc_x2l(int nen, const double *X, const double L[2], const double *N, double XL[3]);
void orc_local_normal(int nen, const double *X, const double L[2], double n[3]);

/* Element integrals (src/kernelIntegrals.c).  X is nen x 3 and is not
 * modified (the reference reorders its argument in place; the port works on
 * a copy). */
void orc_intG(int nen, const double *X, const double *Xe, double *Int);
void orc_intH(int nen, unsigned flag, const double *X, const double *Xe, double *Int, const double *n);
void orc_intSingularG(int nen, unsigned sinNode, const double *X, const double *Xe, double *Int);
void orc_intSingularH(int nen, unsigned flag, unsigned sinNode, const double *X, const double *Xe,
                      double *Int, const double *n);

/* Averaged unit normal at 1-based node `node1` (src/normals.c:120-319). */
void orc_node_normal(int nen, unsigned E, const double *nodes, const unsigned *elems,
                     unsigned node1, double n[3]);

/* Dense assembly (src/assembly_el.c).  full = 0: electricFormA (A is N rows
 * of 2N); full = 1: electricFormFullA (A is 2N rows of 2N).  Only rows
 * i in [row0, row1) are formed (full form: rows i and i + N); A must be
 * zeroed by the caller.  lda is the row stride of A in doubles.
 * nthreads > 1 splits the row range over POSIX threads; each row is
 * computed exactly as in the sequential loop.  Returns 0, or 1 if a row has
 * a boundary-condition type the assembly does not define (anything but
 * 0, 1 or 6), which the reference would silently mis-assemble. */
int orc_assemble(int nen, int full, unsigned N, unsigned E, unsigned nIf,
                 const double *nodes, const unsigned *elems, const unsigned *bctype,
                 const unsigned *ifaces, const double *mat, double freq,
                 const double *mbc, unsigned row0, unsigned row1,
                 double *A, size_t lda, double *B, int nthreads);

/* Interface coefficients A_k, B_k of the reference (src/assembly_el.c:223-239). */
void orc_interface_coeffs(unsigned nIf, const unsigned *ifaces, const double *mat,
                          double freq, double *Ak, double *Bk);

/* Un-pivoted Gauss elimination with back-substitution
 * (src/gaussBksb.c:39-108).  Returns 0, or 1 where the reference would
 * print "Singularity ..." and exit. */
int orc_gauss(unsigned n, double *A, double *B);

/* GMRES on the compact N x 2N form (src/gmres_el.c:66-260).
 * tol_rel replaces the compile-time TOLERANCE (1e-6 in the reference),
 * max_iters replaces MAX_ITERS (600).  x0 (2N, may be NULL) is the initial
 * guess.  log (may be NULL) receives gmres.log in the reference's format.
 * nthreads > 1 splits the matrix-vector product rows over threads.
 * Returns 0 converged, 1 not converged, 2 "CONVERGENCE RATE TOO SLOW";
 * *iters receives the iteration count; the solution is returned in B. */
int orc_gmres(unsigned N, unsigned preCond, double tol_rel, unsigned max_iters,
              double *A, double *B, const double *x0, FILE *log, int nthreads,
              unsigned *iters);

/* Rows [r0, r1) of y = (A1 - i A2) x on the compact form; A holds the
 * rows from r0 on (row r at A + (r - r0) * 2N), y is 2N long. */
void orc_matvec_rows(unsigned N, const double *A, const double *x, double *y, unsigned r0,
                     unsigned r1, int nthreads);

/* Field and potential at a point (src/field.c:57-200,
 * src/potential.c:55-179).  mE[0..5] = Re Ex, Im Ex, Re Ey, Im Ey, Re Ez,
 * Im Ez; mPot[0..1] = Re, Im. */
void orc_field(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
               const double *vB, const double *Xin, double *mE);
void orc_potential(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
                   const double *vB, const double *Xin, double *mPot);

/* Field at many points, split over nthreads (each point as orc_field). */
void orc_field_points(int nen, unsigned N, unsigned E, const double *nodes,
                      const unsigned *elems, const double *vB, unsigned npts,
                      const double *pts, double *mE, int nthreads);

/* Maxwell-stress force on the type-6 surface (src/force.c:348-552,
 * src/forceIntegrals.c:632-723).  Fce and Xce are E x 3; only rows of
 * particle elements are written.  nthreads splits the nodal field loop. */
int orc_forceMST(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
                 const unsigned *bctype, const double *vB, double eps,
                 double *Fce, double *Xce, double *Fcm, double *Xcm, int nthreads);

/* Per-element MST integral (src/forceIntegrals.c:632-723). */
void orc_intF(int nen, const double *X, const double *Enodes, double Int[3]);

/* The quad8 extension (quad8.c; no reference counterpart): element
 * integrals (X 8 x 3, s the 0-based singular node), node normals, the
 * assembled rows as orc_assemble forms them, field, potential and
 * Maxwell-stress force. */
void orc_q8_shape(double xi, double eta, double N[8], double Nx[8], double Ne[8]);
double orc_q8_map(const double *X, double xi, double eta, double XL[3], double N[8], double *n);
void orc_q8_intG(const double *X, const double *Xe, double Int[8]);
void orc_q8_intH(int flag, const double *X, const double *Xe, double *Int, const double *n);
void orc_q8_intSingularG(int s, const double *X, const double *Xe, double Int[8]);
void orc_q8_intSingularH(int flag, int s, const double *X, const double *Xe, double *Int, const double *n);
void orc_q8_node_normal(unsigned E, const double *nodes, const unsigned *elems, unsigned node1, double n[3]);
int orc_q8_assemble(int full, unsigned N, unsigned E, unsigned nIf, const double *nodes, const unsigned *elems,
                    const unsigned *bctype, const unsigned *ifaces, const double *mat, double freq,
                    const double *mbc, double *A, size_t lda, double *B);
void orc_q8_field(unsigned N, unsigned E, const double *nodes, const unsigned *elems, const double *vB,
                  const double *Xin, double mE[6]);
void orc_q8_potential(unsigned N, unsigned E, const double *nodes, const unsigned *elems, const double *vB,
                      const double *Xin, double mPot[2]);
void orc_q8_forceMST(unsigned N, unsigned E, const double *nodes, const unsigned *elems, const unsigned *bctype,
                     const double *vB, double eps, double *Fce, double *Xce, double Fcm[3], double Xcm[3]);

#ifdef __cplusplus
}
#endif
#endif
