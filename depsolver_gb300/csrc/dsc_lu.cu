// dsc_lu.cu -- dense FP64 solve without pivoting (gaussBksb,
// src/gaussBksb.c:39-108), as a blocked right-looking LU on the device.
//
// The reference eliminates column by column on [A | B] and never pivots
// unless a pivot is within 1e-9 of zero.  Here the system is stored as an
// n x (n + 1) row-major block with B as the last column, factored in panels
// of kNB columns: unblocked elimination inside the panel, a unit-lower
// triangular solve for the panel's rows to the right, and an FP64 GEMM
// update of the trailing matrix (B column included), then a blocked back
// substitution.  Same arithmetic up to the order of the rounding; a pivot
// within 1e-9 of zero stops the solve with kErrSingular (the reference
// would try to swap rows there -- only reachable for matrices some 19
// orders of magnitude below the BEM scale).
#include <math.h>

#include "dsc_common.cuh"
#include "dsc_gmres.h"
#include "dsc_internal.h"

namespace dsc {

constexpr int kNB = 64;
constexpr double kPivTol = 1.0E-9;

// Column j of the panel [j0, j1): scale the sub-column by the pivot and
// update the rest of the panel for rows below j.
__global__ void k_panel_col(double *__restrict__ A, size_t lda, int n, int j, int j1, int *bad)
{
    const int r = j + 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const double p = A[(size_t)j * lda + j];
    if (blockIdx.x == 0 && threadIdx.x == 0 && !(fabs(p) > kPivTol) && *bad < 0) *bad = j;
    if (r >= n) return;
    double *ar = A + (size_t)r * lda;
    const double *aj = A + (size_t)j * lda;
    const double l = ar[j] / p;
    ar[j] = l;
    for (int c = j + 1; c < j1; c++) ar[c] -= l * aj[c];
}

// Rows [j0, j1) of the columns right of the panel (B column included):
// U12 = L11^{-1} A12 with L11 unit lower; one thread per column.
__global__ void k_trsm_rows(double *__restrict__ A, size_t lda, int ncols, int j0, int j1)
{
    __shared__ double L[kNB][kNB + 1];
    const int kb = j1 - j0;
    for (int t = threadIdx.x; t < kb * kb; t += blockDim.x) {
        int r = t / kb, c = t % kb;
        L[r][c] = A[(size_t)(j0 + r) * lda + j0 + c];
    }
    __syncthreads();
    const int c = j1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncols) return;
    double u[kNB];
    for (int r = 0; r < kb; r++) {
        double v = A[(size_t)(j0 + r) * lda + c];
        for (int t = 0; t < r; t++) v -= L[r][t] * u[t];
        u[r] = v;
        A[(size_t)(j0 + r) * lda + c] = v;
    }
}

// Trailing update A22 -= L21 U12 for rows >= j1 and columns in [j1, ncols).
// 64 x 64 output tile per CTA, 256 threads with 4 x 4 outputs each.
__global__ void __launch_bounds__(256) k_gemm_update(double *__restrict__ A, size_t lda, int n,
                                                     int ncols, int j0, int j1)
{
    __shared__ double Ls[kNB][64 + 1];  // [t][row]
    __shared__ double Us[kNB][64 + 1];  // [t][col]
    const int kb = j1 - j0;
    const int r0 = j1 + blockIdx.y * 64, c0 = j1 + blockIdx.x * 64;
    for (int t = threadIdx.x; t < 64 * kb; t += 256) {
        int rr = t / kb, tt = t % kb;
        int r = r0 + rr;
        Ls[tt][rr] = r < n ? A[(size_t)r * lda + j0 + tt] : 0.0;
    }
    for (int t = threadIdx.x; t < kb * 64; t += 256) {
        int tt = t / 64, cc = t % 64;
        int c = c0 + cc;
        Us[tt][cc] = c < ncols ? A[(size_t)(j0 + tt) * lda + c] : 0.0;
    }
    __syncthreads();
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    double acc[4][4] = {};
    for (int t = 0; t < kb; t++) {
        double a[4], b[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            a[u] = Ls[t][ty + 16 * u];
            b[u] = Us[t][tx + 16 * u];
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
            for (int v = 0; v < 4; v++) acc[u][v] += a[u] * b[v];
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
        int r = r0 + ty + 16 * u;
        if (r >= n) continue;
#pragma unroll
        for (int v = 0; v < 4; v++) {
            int c = c0 + tx + 16 * v;
            if (c < ncols) A[(size_t)r * lda + c] -= acc[u][v];
        }
    }
}

// Back substitution, block [j0, j1): x_r = (y_r - sum_{c>r} U_rc x_c) / U_rr
// inside the block (one CTA), after the rows above have been updated.
__global__ void k_back_block(double *__restrict__ A, size_t lda, int n, int j0, int j1)
{
    __shared__ double x[kNB];
    const int kb = j1 - j0;
    for (int r = kb - 1; r >= 0; r--) {
        const double *ar = A + (size_t)(j0 + r) * lda;
        double s = 0.0;
        for (int c = r + 1 + threadIdx.x; c < kb; c += blockDim.x) s += ar[j0 + c] * x[c];
        s = warp_sum(s);
        if (threadIdx.x == 0) x[r] = (ar[n] - s) / ar[j0 + r];
        __syncthreads();
    }
    for (int r = threadIdx.x; r < kb; r += blockDim.x) A[(size_t)(j0 + r) * lda + n] = x[r];
}

// y_r -= sum_{c in [j0, j1)} U_rc x_c for the rows above the block.
__global__ void k_back_update(double *__restrict__ A, size_t lda, int n, int j0, int j1)
{
    const int r = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (r >= j0) return;
    const double *ar = A + (size_t)r * lda;
    double s = 0.0;
    for (int c = j0 + lane; c < j1; c += 32) s += ar[c] * A[(size_t)c * lda + n];
    s = warp_sum(s);
    if (lane == 0) A[(size_t)r * lda + n] -= s;
}

__global__ void k_copy_col(const double *__restrict__ A, size_t lda, int n, double *__restrict__ B)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) B[r] = A[(size_t)r * lda + n];
}

// dA: n x (n + 1) row-major (stride lda >= n + 1) with B in column n.
int lu_solve_augmented_fp64(int n, double *dA, size_t lda, int *bad_row, cudaStream_t st)
{
    DevBuf<int> bad;
    DSC_TRY(bad.alloc(1));
    int minus1 = -1;
    DSC_CUDA(cudaMemcpyAsync(bad.p, &minus1, sizeof(int), cudaMemcpyHostToDevice, st));
    const int ncols = n + 1;
    for (int j0 = 0; j0 < n; j0 += kNB) {
        const int j1 = std::min(n, j0 + kNB);
        for (int j = j0; j < j1; j++) {
            int rows = n - j - 1;
            DSC_LAUNCH(k_panel_col<<<std::max(1, (rows + 255) / 256), 256, 0, st>>>(dA, lda, n, j, j1, bad.p));
        }
        DSC_LAUNCH(k_trsm_rows<<<(ncols - j1 + 127) / 128, 128, 0, st>>>(dA, lda, ncols, j0, j1));
        if (j1 < n) {
            dim3 g((ncols - j1 + 63) / 64, (n - j1 + 63) / 64);
            DSC_LAUNCH(k_gemm_update<<<g, 256, 0, st>>>(dA, lda, n, ncols, j0, j1));
        }
        DSC_CUDA(cudaGetLastError());
    }
    int hbad = -1;
    DSC_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    DSC_CUDA(cudaStreamSynchronize(st));
    if (hbad >= 0) {
        if (bad_row) *bad_row = hbad;
        set_error("Singularity in row %d in system matrix", hbad);
        return kErrSingular;
    }
    for (int j1 = n; j1 > 0; j1 -= kNB) {
        const int j0 = std::max(0, j1 - kNB);
        DSC_LAUNCH(k_back_block<<<1, 32, 0, st>>>(dA, lda, n, j0, j1));
        if (j0 > 0) DSC_LAUNCH(k_back_update<<<(j0 * 32 + 255) / 256, 256, 0, st>>>(dA, lda, n, j0, j1));
        DSC_CUDA(cudaGetLastError());
    }
    return kOk;
}

int lu_extract_solution(int n, const double *dA, size_t lda, double *dB, cudaStream_t st)
{
    DSC_LAUNCH(k_copy_col<<<(n + 255) / 256, 256, 0, st>>>(dA, lda, n, dB));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

}  // namespace dsc
