// dsc_gmres.cu -- FP64 GMRES on the compact N x 2N form, following the
// reference's algorithm step for step (solverGMRES_el / iterGMRES_el,
// src/gmres_el.c:66-260):
//   * optional Jacobi scaling of row i of A and of B[i] only (:87-93);
//   * absolute tolerance |B| * tol;
//   * Arnoldi with modified Gram-Schmidt in the same order, the reference's
//     Givens form (:202-220) and stagnation test (:233-236);
//   * triangular solve and x += sum y_j v_j.
// The O(N^2) matrix-vector products and the O(N) Gram-Schmidt updates run on
// the GPU; the Hessenberg matrix and rotations (a few hundred scalars) are
// kept on the host, exactly as small as in the reference.
#include <math.h>
#include <stdio.h>

#include <vector>

#include "dsc_blas.cuh"
#include "dsc_gmres.h"
#include "dsc_internal.h"

namespace dsc {

// y = (A1 - i A2) x on the compact row-major form: one warp per row, lanes
// stride over the columns (matVectProd_el src/gmres_el.c:323-337).
__global__ void k_matvec_compact(const double *__restrict__ A, size_t lda, int N,
                                 const double *__restrict__ x, double *__restrict__ y)
{
    const int i = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= N) return;
    const double *a1 = A + (size_t)i * lda, *a2 = a1 + N;
    const double *xr = x, *xi = x + N;
    double yr = 0.0, yi = 0.0;
    for (int c = lane; c < N; c += 32) {
        double p = a1[c], q = a2[c], u = xr[c], v = xi[c];
        yr += p * u + q * v;
        yi += p * v - q * u;
    }
    yr = warp_sum(yr);
    yi = warp_sum(yi);
    if (lane == 0) {
        y[i] = yr;
        y[i + N] = yi;
    }
}

// Jacobi scaling: row i of A and B[i] times 1 / A[i][i] (real diagonal).
__global__ void k_jacobi_scale(double *__restrict__ A, size_t lda, int N, double *__restrict__ B)
{
    const int i = blockIdx.x;
    double *a = A + (size_t)i * lda;
    const double diag = 1.0 / a[i];
    __syncthreads();
    for (int c = threadIdx.x; c < 2 * N; c += blockDim.x) a[c] = diag * a[c];
    if (threadIdx.x == 0) B[i] = B[i] * diag;
}

__global__ void __launch_bounds__(kRedThreads) k_dot(const double *__restrict__ a,
                                                     const double *__restrict__ b, int n,
                                                     RedWork rw, double *out)
{
    __shared__ double sh[32];
    double s = 0.0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
        s += a[t] * b[t];
    finish_reduction(s, rw, out, sh);
}

// One modified Gram-Schmidt step: w -= h[j-1] v_{j-1} (j > 0), then
// h[j] = v_j . w (v_j = nullptr: h[j] = w . w for the final norm).
__global__ void __launch_bounds__(kRedThreads) k_mgs_step(double *__restrict__ w,
                                                          const double *__restrict__ vprev,
                                                          const double *__restrict__ vcur, int n,
                                                          const double *hprev, RedWork rw,
                                                          double *hout)
{
    __shared__ double sh[32];
    const double h = vprev ? *hprev : 0.0;
    double s = 0.0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        double v = w[t];
        if (vprev) {
            v = v - h * vprev[t];
            w[t] = v;
        }
        s += (vcur ? vcur[t] : v) * v;
    }
    finish_reduction(s, rw, hout, sh);
}

// w /= sqrt(*ss) when the norm is not zero (the norm is written to *norm).
__global__ void k_normalize(double *__restrict__ w, int n, const double *ss, double *norm,
                            int set_norm)
{
    const double nr = sqrt(*ss);
    if (set_norm && blockIdx.x == 0 && threadIdx.x == 0) *norm = nr;
    if (nr == 0.0) return;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
        w[t] = w[t] / nr;
}

__global__ void k_residual0(const double *__restrict__ B, const double *__restrict__ y,
                            double *__restrict__ r, int n, int use_y)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
        r[t] = use_y ? B[t] - y[t] : B[t];
}

// x[k] += sum_j res[j] V[j][k], j in increasing order.
__global__ void k_update_x(double *__restrict__ x, const double *__restrict__ V, size_t ldv,
                           const double *__restrict__ res, int it, int n)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        double acc = x[k];
        for (int j = 0; j < it; j++) acc += res[j] * V[(size_t)j * ldv + k];
        x[k] = acc;
    }
}

// The compact N x 2N matrix as an operator.
struct CompactOp : RealOp {
    const double *A;
    size_t lda;
    int N;
    int apply(const double *x, double *y, cudaStream_t st) override
    {
        DSC_LAUNCH(k_matvec_compact<<<(N * 32 + 255) / 256, 256, 0, st>>>(A, lda, N, x, y));
        DSC_CUDA(cudaGetLastError());
        return kOk;
    }
};

int gmres_compact_fp64(int N, double *dA, size_t lda, double *dB, const double *dx0,
                       unsigned preCond, double tol_rel, unsigned max_iters, FILE *log,
                       unsigned *iters_out, cudaStream_t st)
{
    if (preCond == 1) {
        DSC_LAUNCH(k_jacobi_scale<<<N, 256, 0, st>>>(dA, lda, N, dB));
        DSC_CUDA(cudaGetLastError());
    }
    CompactOp op;
    op.A = dA;
    op.lda = lda;
    op.N = N;
    return gmres_real_fp64(2 * N, op, dB, dx0, tol_rel, max_iters, log, iters_out, st);
}

int gmres_real_fp64(int n, RealOp &op, double *dB, const double *dx0, double tol_rel,
                    unsigned max_iters, FILE *log, unsigned *iters_out, cudaStream_t st)
{
    const unsigned M = max_iters;
    DevBuf<double> V, x, y, scal, part, resd;
    DevBuf<unsigned> cnt;
    DSC_TRY(V.alloc((size_t)(M + 1) * n));
    DSC_TRY(x.alloc(n));
    DSC_TRY(y.alloc(n));
    DSC_TRY(scal.alloc(M + 8));      // h column, then aux scalars
    DSC_TRY(part.alloc(kRedBlocks));
    DSC_TRY(resd.alloc(M + 2));
    DSC_TRY(cnt.alloc(1));
    DSC_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned), st));
    RedWork rw{part.p, cnt.p};
    const dim3 rg(kRedBlocks), rt(kRedThreads);
    const int vblocks = 2 * 152;
    double *hcol = scal.p;            // h[0..i+1] of the current column
    double *aux = scal.p + M + 2;     // aux[0] |w|^2 before MGS, [1] |B|^2 or |x|^2, [2] |r0|, [3] |w|^2 after

    if (dx0) DSC_CUDA(cudaMemcpyAsync(x.p, dx0, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    else DSC_CUDA(cudaMemsetAsync(x.p, 0, n * sizeof(double), st));
    DSC_LAUNCH(k_dot<<<rg, rt, 0, st>>>(dB, dB, n, rw, aux + 1));
    double bb;
    DSC_CUDA(cudaMemcpyAsync(&bb, aux + 1, sizeof(double), cudaMemcpyDeviceToHost, st));
    DSC_CUDA(cudaStreamSynchronize(st));
    const double tolerance = sqrt(bb) * tol_rel;
    if (log) {
        fprintf(log, "\n\nRELATIVE TOLERANCE = %10.4e\n", tolerance);
        fprintf(log, "\n%10s%21s\n", "ITER #    ", "RELATIVE RESIDUAL");
        fprintf(log, "%10s%21s\n", "***************", "*******************");
        fflush(log);
    }
    // initial residual (initRes_el src/gmres_el.c:272-294)
    double xx = 0.0;
    if (dx0) {
        DSC_LAUNCH(k_dot<<<rg, rt, 0, st>>>(x.p, x.p, n, rw, aux + 1));
        DSC_CUDA(cudaMemcpyAsync(&xx, aux + 1, sizeof(double), cudaMemcpyDeviceToHost, st));
        DSC_CUDA(cudaStreamSynchronize(st));
    }
    if (sqrt(xx) != 0.0) DSC_TRY(op.apply(x.p, y.p, st));
    DSC_LAUNCH(k_residual0<<<vblocks, 256, 0, st>>>(dB, y.p, V.p, n, sqrt(xx) != 0.0));
    DSC_LAUNCH(k_dot<<<rg, rt, 0, st>>>(V.p, V.p, n, rw, aux + 1));
    DSC_LAUNCH(k_normalize<<<vblocks, 256, 0, st>>>(V.p, n, aux + 1, aux + 2, 1));
    DSC_CUDA(cudaGetLastError());
    double r0;
    DSC_CUDA(cudaMemcpyAsync(&r0, aux + 2, sizeof(double), cudaMemcpyDeviceToHost, st));
    DSC_CUDA(cudaStreamSynchronize(st));

    std::vector<double> h((size_t)(M + 2) * (M + 2), 0.0), c(M + 1, 0.0), s(M + 1, 0.0),
        res(M + 2, 0.0), col(M + 3);
    auto H = [&](unsigned r, unsigned q) -> double & { return h[(size_t)r * (M + 2) + q]; };
    res[0] = r0;
    double err0 = r0, err1 = r0;
    int status = 1;
    unsigned it = 0;
    if (err0 < tolerance) {
        status = 0;
    } else {
        for (unsigned i = 0; i < M; i++) {
            it++;
            double *vi = V.p + (size_t)i * n, *w = V.p + (size_t)(i + 1) * n;
            DSC_TRY(op.apply(vi, w, st));
            DSC_LAUNCH(k_dot<<<rg, rt, 0, st>>>(w, w, n, rw, aux));
            for (unsigned j = 0; j <= i; j++)
                DSC_LAUNCH(k_mgs_step<<<rg, rt, 0, st>>>(w, j ? V.p + (size_t)(j - 1) * n : nullptr,
                                              V.p + (size_t)j * n, n, hcol + (j ? j - 1 : 0), rw,
                                              hcol + j));
            DSC_LAUNCH(k_mgs_step<<<rg, rt, 0, st>>>(w, V.p + (size_t)i * n, nullptr, n, hcol + i, rw,
                                          aux + 3));
            DSC_LAUNCH(k_normalize<<<vblocks, 256, 0, st>>>(w, n, aux + 3, hcol + i + 1, 1));
            DSC_CUDA(cudaGetLastError());
            DSC_CUDA(cudaMemcpyAsync(col.data(), hcol, (i + 2) * sizeof(double),
                                     cudaMemcpyDeviceToHost, st));
            double ww;
            DSC_CUDA(cudaMemcpyAsync(&ww, aux, sizeof(double), cudaMemcpyDeviceToHost, st));
            DSC_CUDA(cudaStreamSynchronize(st));
            const double norm = sqrt(ww);
            for (unsigned j = 0; j <= i + 1; j++) H(j, i) = col[j];
            for (unsigned j = 0; j + 1 <= i; j++) {
                double h1 = c[j] * H(j, i) + s[j] * H(j + 1, i);
                double h2 = -s[j] * H(j, i) + c[j] * H(j + 1, i);
                H(j, i) = h1;
                H(j + 1, i) = h2;
            }
            double htmp = H(i + 1, i) / H(i, i);
            if (norm != 0.0) {
                c[i] = 1.0 / sqrt(1.0 + htmp * htmp);
                s[i] = c[i] * htmp;
                H(i, i) = c[i] * H(i, i) + s[i] * H(i + 1, i);
                H(i + 1, i) = 0.0;
                res[i + 1] = -s[i] * res[i];
                res[i] = c[i] * res[i];
            }
            err1 = fabs(res[i + 1]);
            if (log) {
                fprintf(log, "%8d%25.4e\n", (int)it, err1);
                fflush(log);
            }
            if (err1 < tolerance) { status = 0; break; }
            if (fabs((err1 - err0) / err0) < 1.0e-6 * tolerance) { status = 2; break; }
            err0 = err1;
        }
        if (status != 2) {
            for (int i = (int)it - 1; i >= 0; i--) {
                for (unsigned j = (unsigned)i + 1; j <= it; j++) res[i] -= H(i, j) * res[j];
                res[i] = res[i] / H(i, i);
            }
            DSC_CUDA(cudaMemcpyAsync(resd.p, res.data(), it * sizeof(double),
                                     cudaMemcpyHostToDevice, st));
            DSC_LAUNCH(k_update_x<<<vblocks, 256, 0, st>>>(x.p, V.p, n, resd.p, (int)it, n));
            DSC_CUDA(cudaGetLastError());
        }
    }
    if (status == 0) {
        if (log) fprintf(log, "\n\n***PROBLEM CONVERGES IN %d ITERATIONS***\n\n", (int)it);
        DSC_CUDA(cudaMemcpyAsync(dB, x.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    } else if (status == 1 && log) {
        fprintf(log, "Problem fails to vonverge to given tolerance in %d iterations\n\n", (int)M);
    }
    DSC_CUDA(cudaStreamSynchronize(st));
    if (iters_out) *iters_out = it;
    if (status == 1) {
        set_error("GMRES did not reach the tolerance in %u iterations", M);
        return kErrNoConverge;
    }
    if (status == 2) {
        set_error("CONVERGENCE RATE TOO SLOW");
        return kErrStagnation;
    }
    return kOk;
}

}  // namespace dsc
