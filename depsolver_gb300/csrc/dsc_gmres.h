// dsc_gmres.h -- solver entry points inside libdepsolver_cuda (not exported).
#pragma once

#include <cuda_runtime.h>
#include <stdio.h>

namespace dsc {

// A real linear operator of dimension n on the device: y = Op x.
struct RealOp {
    virtual ~RealOp() = default;
    virtual int apply(const double *x, double *y, cudaStream_t st) = 0;
    // device flag (may be null): when set, the kernels of apply return at
    // once (a GMRES that runs iterations ahead of its host stops them so)
    const int *skip = nullptr;
};

// The reference's GMRES iteration (src/gmres_el.c:149-260) on any real
// operator: dB (n) in, solution out; preconditioning, if any, is already
// folded into op and dB by the caller.
int gmres_real_fp64(int n, RealOp &op, double *dB, const double *dx0, double tol_rel,
                    unsigned max_iters, FILE *log, unsigned *iters, cudaStream_t st);

// Reference-faithful FP64 GMRES on the compact form (device A, N x 2N with
// row stride lda, scaled in place when preCond == 1; device B overwritten
// with the solution on success).  log (may be null) receives gmres.log.
int gmres_compact_fp64(int N, double *dA, size_t lda, double *dB, const double *dx0,
                       unsigned preCond, double tol_rel, unsigned max_iters, FILE *log,
                       unsigned *iters, cudaStream_t st);

// Un-pivoted blocked LU solve of a dense row-major FP64 system on the
// device.  dA is n x (n + 1) with stride lda >= n + 1 and the right-hand
// side in column n; on success column n holds the solution.  A pivot within
// 1e-9 of zero stops the solve with kErrSingular (*bad_row receives it).
int lu_solve_augmented_fp64(int n, double *dA, size_t lda, int *bad_row, cudaStream_t st);
int lu_extract_solution(int n, const double *dA, size_t lda, double *dB, cudaStream_t st);

// The same solve as a low-precision block LU on the tensor cores (3xFP16
// trailing updates, FP32 factors) with FP64-residual iterative refinement:
// dA as above (n x (n + 1), B in column n, left unchanged), dx (n) receives
// the solution.  Stops when |b - A x| <= tol |b| or the correction falls to
// the rounding level of x; kErrStagnation when the residual stops falling
// first (the factors too inaccurate for the matrix's conditioning: the
// caller falls back to the FP64 LU); kErrSingular for a pivot within 1e-9
// of zero (*bad_row).
struct LuMixedInfo {
    bool factor_done = false;
    int refinements = 0;
    double rel_residual = 0.0, last_correction = 0.0;
    // CUDA-event times on the solve's stream: the conversion to FP32 and the
    // factorisation, and the refinement (triangular solves and residuals)
    float factor_ms = 0.0f, refine_ms = 0.0f;
};
int lu_solve_mixed(int n, const double *dA, size_t lda, double *dx, double tol, LuMixedInfo *info, int *bad_row,
                   cudaStream_t st);

}  // namespace dsc
