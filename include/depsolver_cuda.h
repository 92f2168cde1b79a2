/*
 * depsolver_cuda.h -- C ABI of libdepsolver_cuda, the GB300 (sm_103a)
 * implementation of depSolver's boundary-element hot path.
 *
 * Two layers:
 *
 *  1. Drop-in entry points with the reference's exact names, signatures and
 *     error behaviour.  A depSolver build links libdepsolver_cuda.so in place
 *     of assembly_el.o, kernelIntegrals.o, gaussBksb.o, gmres_el.o, field.o,
 *     potential.o, force.o (MST part) and forceIntegrals.o; the driver, input
 *     parsing, normals and post-processing stay the reference's C code and
 *     input decks and output files are unchanged.  Like the reference they
 *     read the globals nNodes, nElems and nInterfaces and report fatal
 *     errors on stderr and in bem.log before exit(1).
 *
 *  2. dsc_* entry points on flat row-major arrays that return a status
 *     code (0 = success, see dsc_last_error()) instead of exiting.  Meshes
 *     are passed as in the reference's input files: elems are 1-based node
 *     ids, bctype and mbc have 2N rows.
 *
 * No torch or CUDA types appear in any signature.
 */
#ifndef DEPSOLVER_CUDA_H
#define DEPSOLVER_CUDA_H

#include <stddef.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ globals
 * Read by the drop-in entry points exactly where the reference reads them
 * (defined in src/depSolver.c:46-50).  The library carries its own
 * definitions; when linked into the depSolver executable, the executable's
 * definitions take precedence. */
extern unsigned int nNodes, nElems, nInterfaces;
extern FILE *file_log;

/* --------------------------------------------------------- drop-in: assembly
 * Replace src/assembly_el.c:63 / :197 / :329 / :470 (declared in
 * src/assembly_el.h:29-67).  Compact form (electricFormA_*): mA has nNodes
 * rows of 2*nNodes; full form (electricFormFullA_*): 2*nNodes rows.  The
 * assembled values are ADDED to mA (the reference accumulates into a
 * zeroed matrix); vB receives the boundary values.  Boundary types other
 * than 0, 1 and 6 (which the reference assembles with stale interface data)
 * are reported as a fatal error. */
int electricFormA_tria3(double **mNodes, unsigned int **mElems, unsigned int *vBCType,
                        unsigned int **vInterfaces, double **vMatParam, double *vProbParam,
                        double **mA, double **mBC, double *vB);
int electricFormA_tria6(double **mNodes, unsigned int **mElems, unsigned int *vBCType,
                        unsigned int **vInterfaces, double **vMatParam, double *vProbParam,
                        double **mA, double **mBC, double *vB);
int electricFormFullA_tria3(double **mNodes, unsigned int **mElems, unsigned int *vBCType,
                            unsigned int **vInterfaces, double **vMatParam, double *vProbParam,
                            double **mA, double **mBC, double *vB);
int electricFormFullA_tria6(double **mNodes, unsigned int **mElems, unsigned int *vBCType,
                            unsigned int **vInterfaces, double **vMatParam, double *vProbParam,
                            double **mA, double **mBC, double *vB);

/* ----------------------------------------------------------- drop-in: solve
 * gaussBksb replaces src/gaussBksb.c:39 (src/gaussBksb.h:29): N x N system,
 * solution returned in B.  A's contents after the call are unspecified (the
 * reference leaves its eliminated matrix there; no caller reads it).
 * solverGMRES_el replaces src/gmres_el.c:66 (src/gmres_el.h:29): compact
 * nNodes x 2nNodes system, Jacobi scaling when preCond == 1, initial guess
 * from solution.init when nInit != 0, gmres.log written in the working
 * directory in the reference's format, solution returned in B. */
int gaussBksb(unsigned int N, double **A, double *B);
void solverGMRES_el(unsigned int preCond, unsigned int nInit, double **A, double *B);

/* ---------------------------------------------------- drop-in: post-process
 * field_* replace src/field.c:57 / :137 (src/field.h:30-41):
 *   mE = {Re Ex, Im Ex, Re Ey, Im Ey, Re Ez, Im Ez} at Xin.
 * potential_* replace src/potential.c:55 / :126 (src/potential.h:29-40):
 *   mPot = {Re, Im}.
 * forceMST_* replace src/force.c:348 / :463 (src/force.h:54-73): Maxwell
 * stress force on the elements whose first node has boundary type 6
 * (rows of Fce / Xce written for those elements only), total Fcm and the
 * mean Xcm of the type-6 nodes. */
int field_tria3(double *Xin, double **mNodes, unsigned int **mElems, double *vB, double *mE);
int field_tria6(double *Xin, double **mNodes, unsigned int **mElems, double *vB, double *mE);
int potential_tria3(double *Xin, double **mNodes, unsigned int **mElems, double *vB, double *mPot);
int potential_tria6(double *Xin, double **mNodes, unsigned int **mElems, double *vB, double *mPot);
int forceMST_tria3(double **mNodes, unsigned int **mElems, unsigned int *vBCType, double *vB,
                   double Eps, double **Fce, double **Xce, double *Fcm, double *Xcm);
int forceMST_tria6(double **mNodes, unsigned int **mElems, unsigned int *vBCType, double *vB,
                   double Eps, double **Fce, double **Xce, double *Fcm, double *Xcm);
/* forceMultipole_* replace src/force.c:572 / :709 (src/force.h): the DEP
 * force on a sphere of radius R centred at Xeval by the multipole expansion
 * of order nOrder (the reference adds the terms up to order 3; orders 4
 * and 5 give the order-3 force), from Re(E) and its derivatives at Xeval;
 * vMatParam rows 0 (medium) and 1 (particle), vProbParam[0] the frequency.
 * forceEllipsoid_* replace src/force.c:65 / :204: the dipole force on an
 * ellipsoid of semi-axes `axis` (ANALYSIS 10 homogeneous, 11 single-shell;
 * for 11 the reference scales vMatParam[1] in place, and so does this). */
int forceMultipole_tria3(unsigned int nOrder, double R, double *Xeval, double **mNodes,
                         unsigned int **mElems, double *vB, double **vMatParam, double *vProbParam,
                         double *F);
int forceMultipole_tria6(unsigned int nOrder, double R, double *Xeval, double **mNodes,
                         unsigned int **mElems, double *vB, double **vMatParam, double *vProbParam,
                         double *F);
int forceEllipsoid_tria3(unsigned int ANALYSIS, unsigned int nOrder, double *axis, double *Xeval,
                         double **mNodes, unsigned int **mElems, double *vB, double **vMatParam,
                         double *vProbParam, double *F);
int forceEllipsoid_tria6(unsigned int ANALYSIS, unsigned int nOrder, double *axis, double *Xeval,
                         double **mNodes, unsigned int **mElems, double *vB, double **vMatParam,
                         double *vProbParam, double *F);

/* ------------------------------------------------------------ flat dsc_ API */

/* Status codes. */
#define DSC_OK 0
#define DSC_ERR_CUDA 1
#define DSC_ERR_ARG 2
#define DSC_ERR_BCTYPE 3
#define DSC_ERR_SINGULAR 4
#define DSC_ERR_NOCONVERGE 5
#define DSC_ERR_STAGNATION 6
#define DSC_ERR_MEMORY 7

/* Message of the last failure on this thread. */
const char *dsc_last_error(void);

/* Number of CUDA devices visible (0 when none; no error). */
int dsc_device_count(void);

/* Running total of kernels this library has launched in this process. */
unsigned long long dsc_kernel_launches(void);

/* Flat form of electricFormA_* (full = 0; A is N x 2N) and
 * electricFormFullA_* (full = 1; A is 2N x 2N); rows of A are lda doubles
 * apart and receive A += assembled values; B (2N) = boundary values.
 * nen = 3 or 6 (tria3, tria6) or 8 (quad8, an extension: the reference
 * has no quad8 integrals; see dsc_field_points); elems 1-based (E x nen);
 * bctype 2N; ifaces nIf x 2; mat
 * has at least max(ifaces) rows of (sigma, eps_r); mbc 2N x 3. */
int dsc_assemble(int nen, int full, unsigned N, unsigned E, unsigned nIf, const double *nodes,
                 const unsigned *elems, const unsigned *bctype, const unsigned *ifaces,
                 const double *mat, double freq, const double *mbc, double *A, size_t lda,
                 double *B);

/* Flat form of gaussBksb: row-major n x n (stride lda), B overwritten with
 * the solution; A is left unchanged. */
int dsc_gauss(unsigned n, const double *A, size_t lda, double *B);

/* How gaussBksb and dsc_gauss solve (process-wide; no counterpart in the
 * reference, whose gaussBksb is the FP64 elimination of src/gaussBksb.c):
 *   DSC_GAUSS_MIXED (default) -- block LU without pivoting in FP32 tiles,
 *     its trailing updates as 3xFP16 products on the tensor cores, then FP64
 *     iterative refinement (residual b - A x with A in FP64) until the
 *     correction is at FP64's rounding level of x; if the residual stops
 *     falling first (factors too inaccurate for the matrix), the solve is
 *     redone with the FP64 LU;
 *   DSC_GAUSS_FP64 -- blocked FP64 LU without pivoting.
 * Both report a pivot within 1e-9 of zero as the reference does
 * ("Singularity in row"; DSC_ERR_SINGULAR for dsc_gauss).
 * dsc_gauss_info gives the last mixed solve's refinement steps, final
 * relative residual |b - A x| / |b|, whether it fell back to the FP64 LU,
 * and in ms[0..1] (may be NULL) the device time of the factorisation
 * (conversion to FP32 included) and of the refinement; it returns the mode.
 * Any pointer may be NULL. */
#define DSC_GAUSS_MIXED 0
#define DSC_GAUSS_FP64 1
int dsc_set_gauss_mode(int mode);

/* Host matrices of gaussBksb / dsc_gauss and solverGMRES_el / dsc_gmres
 * (row pointers or flat rows) reach the device through one gather kernel
 * that reads them in place when the device can read pageable host memory
 * (Grace-Blackwell, through the host's page tables), else through pinned
 * staging by host threads.  mode 0: staged copies both ways; 1 (default):
 * host matrices read in place, the assembled rows of electricFormA_* /
 * dsc_assemble staged; 2: the assembled rows also added into the caller's
 * rows by the device.  Every mode gives the same bytes. */
int dsc_set_host_direct(int mode);
int dsc_gauss_info(int *refinements, double *rel_residual, int *fell_back, double *ms);

/* Flat form of solverGMRES_el with the tolerance (relative to |B|, the
 * reference compiles 1e-6) and the iteration cap (600) as arguments.
 * A (N x 2N, stride lda) is left unchanged; B is overwritten with the
 * solution on success; x0 (2N) may be NULL; log_path may be NULL (no log);
 * *iters receives the iteration count. */
int dsc_gmres(unsigned N, unsigned preCond, double tol, unsigned max_iters, const double *A,
              size_t lda, double *B, const double *x0, const char *log_path, unsigned *iters);

/* Field (mE: npts x 6) or potential (mPot: npts x 2) at npts points
 * (pts: npts x 3), from the nodal solution vB (2N).  nen = 3, 6 or 8.
 * quad8 (nen = 8) is this library's extension of the element families:
 * serendipity element on [-1, 1]^2, nodes 1-4 the corners (-1,-1),
 * (1,-1), (1,1), (-1,1), nodes 5-8 the mid-sides of edges 1-2, 2-3, 3-4,
 * 4-1; 3 x 3 Gauss points for regular pairs; singular pairs on triangles
 * with their apex at the collocation node, with the triangle path's Duffy
 * and subdivision schemes; on a node the field adds the jump
 * sigma / (2 eps0) n once with that node's sigma (the triangle families
 * keep the reference's jump per singular element). */
int dsc_field_points(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
                     const double *vB, unsigned npts, const double *pts, double *mE);
int dsc_potential_points(int nen, unsigned N, unsigned E, const double *nodes,
                         const unsigned *elems, const double *vB, unsigned npts,
                         const double *pts, double *mPot);

/* Flat forms of forceMultipole_* and forceEllipsoid_* at npts points (pts
 * npts x 3, F npts x 3); mat = {sigma_m, eps_m, sigma_p, eps_p}.  Unlike the
 * reference's forceEllipsoid (ANALYSIS 11), the flat form leaves mat
 * unchanged.  dsc_depolarization gives the ellipsoid's depolarisation
 * factors (src/depolarization.c:44-115). */
int dsc_force_multipole(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
                        const double *vB, unsigned npts, const double *pts, unsigned order, double R,
                        const double *mat, double freq, double *F);
int dsc_force_ellipsoid(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
                        const double *vB, unsigned npts, const double *pts, unsigned analysis,
                        const double *axis, const double *mat, double freq, double *F);
int dsc_depolarization(const double *axis, double *Ld);

/* Flat form of forceMST_*: Fce, Xce are E x 3 (may be NULL); nen = 3, 6
 * or 8 (quad8: the 3 x 3 Gauss points, Xce at the element's centre). */
int dsc_force_mst(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
                  const unsigned *bctype, const double *vB, double eps, double *Fce, double *Xce,
                  double *Fcm, double *Xcm);

/* ------------------------------------------------------- sessions / sweeps
 * No counterpart call in the reference: depSolver solves one (geometry,
 * frequency) system per process run (src/depSolver.c:52-427) and a position
 * sweep is many runs of depSolver-sft (src/depSolver-shift.c:212-217).  A
 * session keeps one geometry in GPU memory: the frequency-independent
 * geometric matrix is assembled once and every frequency only rescales its
 * rows (the interface coefficients of src/assembly_el.c:223-239), so a
 * sweep solves many systems per assembly.
 *
 * Modes:
 *   DSC_MODE_FP64  -- the reference's algorithm in FP64: its GMRES (real
 *                     2N form, Jacobi scaling, modified Gram-Schmidt, at
 *                     tolerance `tol`) one frequency at a time, FP64 field
 *                     and Maxwell-stress force.
 *   DSC_MODE_MIXED -- all frequencies at once: complex GMRES whose matrix
 *                     products run on the tensor cores (3xFP16 on a scaled
 *                     fp16 pair of the matrix: about FP32 accuracy),
 *                     double-FP32 Arnoldi, right preconditioning by the
 *                     electrodes' blocks, iterative refinement on an
 *                     FP64-accurate residual to `tol` (relative residual),
 *                     batched field and force.
 * forces receives 9 doubles per frequency: Fcm[3], Xcm[3] and the sum over
 * particle elements of |Fce| per component (the scale of the net force).
 * sigma (may be NULL) receives 2N doubles per frequency (Re then Im).
 * iters (may be NULL) receives the iteration count per frequency.
 * max_iters caps each system's GMRES iterations: per frequency in the FP64
 * mode (the reference's MAX_ITERS, src/gmres_el.c:42-50), and the inner
 * iterations summed over the refinement steps in the mixed mode.
 *
 * A system that does not converge does not stop the sweep: its sigma and
 * forces are NaN, the others are returned as usual, and the call returns
 * DSC_ERR_NOCONVERGE (the reference's GMRES exits instead,
 * src/gmres_el.c:123-126,233-236).  dsc_session_status gives each system's
 * outcome: DSC_SYS_CONVERGED, DSC_SYS_CAPPED (max_iters reached) or
 * DSC_SYS_STAGNATED (the FP64 GMRES's "CONVERGENCE RATE TOO SLOW", or the
 * mixed mode's refinement steps used up). */
#define DSC_MODE_FP64 1
#define DSC_MODE_MIXED 2

typedef struct dsc_session dsc_session;

int dsc_session_create(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
                       const unsigned *bctype, const double *mbc, unsigned nIf,
                       const unsigned *ifaces, unsigned nMat, const double *mat,
                       dsc_session **out);
/* A session's device memory comes from the device's default memory pool in
 * stream order; on destroy it goes back to the pool, which keeps it for the
 * next session of the process instead of returning it to the device. */
void dsc_session_destroy(dsc_session *s);
/* Assembles the geometric matrix now, again if it already exists
 * (otherwise the first solve assembles it and later solves reuse it).
 * mode DSC_MODE_FP64: regular pairs in FP64, the reference's arithmetic;
 * DSC_MODE_MIXED: regular pairs in the arithmetic dsc_session_set_mixed_
 * assembly chose, and the fp16 copies for the tensor cores.  Singular pairs
 * are FP64 in the FP64 mode and double-FP32 (about 1e-13 of FP64) in the
 * mixed mode.  An FP64 solve on a matrix assembled for the mixed mode
 * assembles it again in FP64; a mixed solve keeps a more accurate matrix. */
int dsc_session_assemble(dsc_session *s, int mode);
/* Arithmetic of the mixed mode's regular (non-singular) pairs:
 *   DSC_ASM_FP32 (default) -- FP32, with each element's quadrature points
 *     as offsets from its centroid (about 1e-7 of each entry: the far-field
 *     assembly in FP32; the solution follows that matrix to ~1e-7, the
 *     Maxwell-stress force to ~1e-9 of the sum of |Fce| on the 12k-node
 *     scene);
 *   DSC_ASM_DF32 -- double-FP32 on the FP32 pipes (about 2^-46 per
 *     operation, entries within ~1e-13 of FP64; the mixed solution then
 *     matches the FP64 one to ~1e-10). */
#define DSC_ASM_FP32 2
#define DSC_ASM_DF32 1
int dsc_session_set_mixed_assembly(dsc_session *s, int prec);
/* Mixed mode's batched field at the force points: on (default) takes the
 * far element-point pairs on the tensor cores (the kernel 1/r^2 generated
 * into shared memory as fp16 pairs, 3xFP16 products read back into FP32
 * every 64 quadrature points) and the near ones on the FP32 pipes; off
 * takes all of them on the FP32 pipes. */
int dsc_session_set_field_tensor(dsc_session *s, int on);
/* FP64 mode's Jacobi scaling.  The reference scales row i of the compact
 * matrix and B[i] by 1 / A[i][i] but leaves B[N + i], the imaginary
 * right-hand side, unscaled (src/gmres_el.c:87-93): with a complex boundary
 * value (a phase-shifted electrode, e.g. a rotating-field trap) it solves
 * for an imaginary part off by the factor A[i][i].  full = 0 (default)
 * keeps that behaviour (parity with the reference); full = 1 scales B[N + i]
 * as well, which solves the assembled system itself (what the mixed mode
 * does).  With real boundary values the two are identical. */
int dsc_session_set_fp64_jacobi(dsc_session *s, int full);
/* Mixed mode's first FP64-accurate residual r = b - M x: K x either from
 * K's eight fixed-point row digits on the tensor cores (exact integer digit
 * products; the digits take 16 bytes per entry of K beside it) or by an
 * FP64 GEMV over the FP64 K for each system (K read once per system).
 * DSC_RESIDUAL_AUTO (default) keeps the digits when they fill at most a
 * quarter of the device's memory (so a 100k-node scene takes the GEMV). */
#define DSC_RESIDUAL_AUTO 0
#define DSC_RESIDUAL_DIGITS 1
#define DSC_RESIDUAL_FP64 2
int dsc_session_set_residual(dsc_session *s, int how);
/* The geometric matrix K (N x N) as assembled for `mode` (assembling it if
 * needed): K[c * ldk + i] = entry (row i, node c), i.e. C * int G N_c for
 * conductor rows and int H N_c for interface rows (src/assembly_el.c). */
int dsc_session_geometric_matrix(dsc_session *s, int mode, double *K, size_t ldk);
int dsc_session_solve(dsc_session *s, int mode, unsigned nfreq, const double *freqs, double tol,
                      unsigned max_iters, double *sigma, double *forces, unsigned *iters);
#define DSC_SYS_CONVERGED 0
#define DSC_SYS_CAPPED 1
#define DSC_SYS_STAGNATED 2
/* Outcome of each system of the session's last solve: writes up to n of
 * them to status (may be NULL) and returns how many systems it solved. */
int dsc_session_status(dsc_session *s, int *status, unsigned n);
/* Maxwell-stress results per particle of the last solve (the reference
 * sums every type-6 element into one force, src/force.c:516-547; the
 * per-particle force is that sum over one particle's elements, i.e. its
 * forceMST_* with vBCType masked to that particle).  A particle is a
 * connected set of type-6 elements (elements sharing a node), numbered by
 * their lowest node id.  Returns the number of particles P and writes, for
 * the first n systems of the last solve, P x 12 doubles each to out (may be
 * NULL): force[3], centre[3] (the mean of its type-6 nodes, as Xcm),
 * sum |Fce|[3] over its elements, torque[3] about the centre: sum over its
 * elements of (Xce - centre) x Fce, Xce the point X(1/4, 1/4) where the
 * reference reports an element's force (an extension: the reference has no
 * torque; like the force it is the stress of Re(E) only).  NaN for systems
 * that did not converge. */
int dsc_session_particles(dsc_session *s, double *out, unsigned n);
/* CUDA-event timing of kernel classes (off by default).  Since the last
 * call: ms[k] the summed time of class k, count[k] its timed scopes and
 * work[k] its algorithmic work (any of the three may be NULL; n entries):
 *   k = 0 assembly regular pairs   work: (row, element) pairs
 *       1 assembly fix-up                0
 *       2 assembly singular pairs        0
 *       3 FP64 K GEMV                    bytes of K read
 *       4 K GEMM (mixed, tensor cores)   flops of the three fp16 products
 *       5 field                          (particle node, element) pairs x systems
 *       6 Maxwell stress                 0
 *       7 FP64-accurate residual         digit multiply-adds (tensor cores)
 *       8 other Krylov kernels           0
 *       9 Gram-Schmidt passes            bytes the kernels read and wrote
 *      10 K to its fp16 pair and digits  bytes read and written
 *      11 conductor-block inverses       flops of the Gauss-Jordan updates
 *      12 conductor-block products       flops of the three fp16 products */
int dsc_session_set_timing(dsc_session *s, int on);
/* The mixed mode's right preconditioner (on by default): the rows of each
 * connected electrode (boundary type 1, a fixed potential) form a
 * frequency-independent first-kind block whose inverse (Gauss-Jordan on
 * the device after each assembly of K) is applied on the right, so GMRES
 * converges in a few iterations while the solution stays that of the
 * unpreconditioned system.  on = 0 solves with the complex Jacobi scaling
 * alone.  dsc_session_preconditioner_blocks returns the number of blocks
 * and writes up to n of their row counts to rows (may be NULL). */
int dsc_session_set_preconditioner(dsc_session *s, int on);
int dsc_session_preconditioner_blocks(dsc_session *s, int *rows, int n);
/* The CUDA stream (cudaStream_t) all of the session's work runs on, so a
 * caller can record its own events around a solve. */
void *dsc_session_stream(dsc_session *s);
int dsc_session_timing(dsc_session *s, double *ms, int *count, double *work, int n);

/* Tensor-core product of host FP64 matrices, the kernel behind the mixed
 * sweep's matrix products (no counterpart call in the reference, whose
 * GMRES product is the scalar loop of src/gmres_el.c:323-337):
 * Y (M x Nc) = A (M x Kd) * B^T (B is Nc x Kd), all row-major; each operand
 * is split into a pair of 11-bit halves and three products hi*hi + hi*lo +
 * lo*hi are accumulated in FP32 per split of k and in FP64 across splits
 * (about FP32 accuracy).  Nc <= 160; splits <= 0 picks the split count.
 * a_in_smem = 0 stores A as the tf32 pair; 1 stores A as plain FP32 and
 * splits it inside the kernel (half the reads of A); 2 does the same on A
 * stored in a biased encoding whose truncation to tf32 is the rounded hi;
 * 3 (the mixed sweep's mode) scales each row of A and of B by a power of two
 * and splits it into an fp16 pair, products on the fp16 tensor path (twice
 * the tf32 rate), the scales multiplied back out in the epilogue; 4 is the
 * digit product of the mixed sweep's first residual: A and B rounded to
 * fp16 and one product per split of at most 4096 k, exact for integer
 * entries |A| <= 32 and |B| <= 128 (Nc <= 384, splits ignored). */
int dsc_tc_gemm(int M, int Nc, int Kd, const double *A, const double *B, double *Y, int splits,
                int a_in_smem);

/* The same product on caller-owned device memory, allocating nothing (no
 * counterpart in the reference, which has no GPU code).  For callers that
 * cannot let a library allocate: one that sized its device memory up front
 * (the FP32 matrix, the Krylov vectors) and keeps none free, and one that
 * runs work on other streams while it calls, since cudaFree synchronises
 * the whole device and cudaMalloc may as well.  This call makes no
 * cudaMalloc/cudaFree or other allocating call: its scratch is one static
 * device array of DSC_NOALLOC_SCRATCH_BYTES (32 MiB) per device, reserved
 * when the library's module holding it loads there.
 *
 * Y (M x Nc, FP64, row stride ldy) = A (M x Kd, FP32, row stride lda) *
 * B^T (B: Nc x Kd, FP64, row stride ldb); A, B, Y on the current device.
 * A's base is 16-byte aligned and lda a multiple of 4 (the tensor-memory
 * copy engine's rule).  Same 3xTF32 products, split of k and split order as
 * dsc_tc_gemm: for A holding FP32 values the two give identical Y.
 * splits <= 0 picks dsc_tc_gemm's split count, lowered until the scratch
 * fits; a shape (or an explicit splits) needing more than the scratch,
 * about 4 * Nc * (2 * round_up(Kd, 32) + splits * M) bytes, is rejected
 * with DSC_ERR_ARG and a message naming both sizes.
 *
 * The call is synchronous: it queues its kernels on `stream` (a
 * cudaStream_t; NULL = the default stream), then copies the kernels' status
 * word back and synchronises `stream` on the host, so it returns only once
 * Y is written, with the status of the kernels' bounded waits.  The first
 * call on each device also looks up the scratch's address
 * (cudaGetSymbolAddress) and keeps it: make that first call during set-up,
 * and do not call again on a device after cudaDeviceReset.  All calls on a device share its scratch, so two calls
 * that overlapped would race on it; the library prevents that with a
 * process-wide lock held until a call's work has finished. */
#define DSC_NOALLOC_SCRATCH_BYTES 33554432u /* 32 MiB */
int dsc_tc_gemm_noalloc(int M, int Nc, int Kd, const float *A, size_t lda, const double *B,
                        size_t ldb, double *Y, size_t ldy, int splits, void *stream);

/* ------------------------------------------------------- position sweeps
 * Replaces a series of depSolver-sft runs, each of which shifts nodes
 * pNodes..nNodes-1 (the particle) rigidly by the REPOSITION vector and
 * solves the whole system again (src/depSolver-shift.c:129-133,212-217).
 * A position-sweep object holds a fixed part of the scene -- N nodes, E
 * elements, bctype (2N), mbc (2N x 3), materials and interfaces, in the
 * reference's input model as for dsc_session_create -- and particle meshes
 * added with dsc_positions_add_particle (any number of nodes each, node
 * coordinates about the particle's own origin, elements 1-based within the
 * particle, one interface id; its nodes get boundary type 6, so its
 * Maxwell-stress force is computed).
 *
 * dsc_positions_solve solves, for each of npos positions q (particle
 * tmpl[q] with its origin at centres[3q..3q+2]), the scene "fixed part's
 * nodes, then the particle's nodes + centre" at nfreq frequencies, every
 * system in the mixed mode to relative residual tol (DSC_MODE_MIXED of
 * dsc_session_solve).  The fixed part's conductor-block inverses are
 * computed once and reused by every position.  Outputs, position-major:
 * forces (npos x nfreq x 9, as dsc_session_solve), iters (npos x nfreq, may
 * be NULL), status (npos x nfreq, DSC_SYS_*), crossover_hz (npos, may be
 * NULL: the frequency where the force's component along its lowest-
 * frequency direction first changes sign, interpolated in log f; NaN when
 * it keeps its sign), sigma (may be NULL: for each position in turn
 * nfreq x 2N_q doubles, N_q its node count).  Systems that do not converge
 * get NaN results and a status, and the call returns DSC_ERR_NOCONVERGE
 * after solving all the others.  Positions run on a pool of host workers
 * (dsc_positions_set_workers, default 4), each with its own CUDA stream,
 * largest systems first. */
typedef struct dsc_positions dsc_positions;
int dsc_positions_create(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
                         const unsigned *bctype, const double *mbc, unsigned nIf,
                         const unsigned *ifaces, unsigned nMat, const double *mat,
                         dsc_positions **out);
void dsc_positions_destroy(dsc_positions *p);
/* Returns the particle's index (>= 0), or minus a status code. */
int dsc_positions_add_particle(dsc_positions *p, unsigned N, unsigned E, const double *nodes,
                               const unsigned *elems, unsigned iface);
int dsc_positions_set_workers(dsc_positions *p, int workers);
int dsc_positions_set_mixed_assembly(dsc_positions *p, int prec);
/* Timing of kernel classes summed over the positions' solves, as
 * dsc_session_set_timing / dsc_session_timing (resets on read). */
int dsc_positions_set_timing(dsc_positions *p, int on);
int dsc_positions_timing(dsc_positions *p, double *ms, int *count, double *work, int n);
/* How many positions inverted the conductor blocks themselves (at most the
 * number of workers; the others copied the shared inverses). */
int dsc_positions_inversions(dsc_positions *p);
int dsc_positions_solve(dsc_positions *p, unsigned npos, const unsigned *tmpl, const double *centres,
                        unsigned nfreq, const double *freqs, double tol, unsigned max_iters,
                        double *forces, unsigned *iters, int *status, double *crossover_hz,
                        double *sigma);

/* The crossover_hz of dsc_positions_solve for one force spectrum (forces:
 * nfreq x 9 as dsc_session_solve writes them, freqs ascending; status may
 * be NULL, else a system that did not converge gives NaN).  Host only. */
double dsc_force_crossover(unsigned nfreq, const double *freqs, const double *forces,
                           const int *status);

/* Autotuner of the mixed sweep's tensor-core product (no counterpart in the
 * reference): the product of K with the 2F Krylov columns is split along k
 * into partial tiles; the split count is chosen by timing the candidates
 * around the built-in rule (about eleven waves of one CTA per SM) as the
 * product plus the epilogue that sums the tiles, with CUDA events, the
 * first time a solve meets a (device, N, 2F) size; the choice is kept for
 * the process.  dsc_set_autotune(0) uses the rule alone (default on).
 * dsc_autotune_table writes up to n rows of (N, columns, splits) to rows
 * (3 ints each, may be NULL) and returns the number of tuned sizes. */
int dsc_set_autotune(int on);
int dsc_autotune_table(int *rows, int n);

/* ---------------------------------------------------------- input decks
 * The reference's input deck as a library call (host only): input.bem in
 * directory dir and the node, element, boundary-condition, internal-point
 * and force-point files it names, parsed as src/depSolver.c:98-252 and
 * src/depSolver-shift.c:120-140,205-217 do ("//" comments stripped as
 * comFilter does, src/preProcess.c:48-81; "C<k>" boundary types read as
 * k + 5).  A REPOSITION section (depSolver-sft decks) shifts nodes pNodes..
 * (0-based) by dr, as that driver does.  Element types other than tria3 and
 * tria6 are rejected, as the reference's driver rejects them
 * (src/depSolver.c:180-183).
 *
 * dsc_bem_info returns the sizes and scalars (any pointer may be NULL;
 * analysis is the ANALYSIS type, gmres 1 for the GMRES solver with preCond
 * and nInit, axis the sphere radius in axis[0] or the ellipsoid's
 * semi-axes); dsc_bem_arrays copies the arrays (any may be NULL): nodes
 * N x 3, elems E x nen (1-based), bctype 2N, mbc 2N x 3, mat nMat x 2,
 * ifaces nIf x 2, internal points and force points nPoints x 3. */
typedef struct dsc_bem dsc_bem;
int dsc_bem_read(const char *dir, dsc_bem **out);
void dsc_bem_free(dsc_bem *b);
int dsc_bem_info(const dsc_bem *b, int *nen, unsigned *N, unsigned *E, unsigned *nMat, unsigned *nIf,
                 double *freq, int *analysis, int *gmres, unsigned *preCond, unsigned *nInit,
                 unsigned *nInternal, unsigned *nForcePoints, int *reposition, unsigned *pNodes,
                 double *dr, double *axis);
int dsc_bem_arrays(const dsc_bem *b, double *nodes, unsigned *elems, unsigned *bctype, double *mbc,
                   double *mat, unsigned *ifaces, double *internal, double *force_points);

/* Averaged unit normal at every node (normals: N x 3), replacing the
 * reference's getNormal_tria3/6 (src/normals.c:120-319), which scans every
 * element per node: the average over the elements containing the node of
 * their local normals at it, normalised (host threads, O(N + E)); nen = 3,
 * 6 or 8. */
int dsc_node_normals(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
                     double *normals);

/* One-call sweep from host arrays (session created and destroyed inside). */
int dsc_sweep(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
              const unsigned *bctype, const double *mbc, unsigned nIf, const unsigned *ifaces,
              unsigned nMat, const double *mat, int mode, unsigned nfreq, const double *freqs,
              double tol, unsigned max_iters, double *sigma, double *forces, unsigned *iters);

#ifdef __cplusplus
}
#endif
#endif
