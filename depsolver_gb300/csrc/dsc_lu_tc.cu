// dsc_lu_tc.cu -- the dense direct solve (gaussBksb, src/gaussBksb.c:39-108)
// as a low-precision block LU on the tensor cores with FP64-residual
// iterative refinement.
//
// Factorisation, without pivoting like the reference (which only swaps rows
// when a pivot is within 1e-9 of zero), in 128 x 128 tiles of an FP32
// working copy W of A (column-major, padded with the identity to a multiple
// of 128).  Step k of the block LU A = L U (L unit lower by blocks, U upper
// by blocks with the Schur complement's diagonal tiles):
//   P_k = W_kk^-1                 Gauss-Jordan of the tile in registers of one
//                                 CTA (gj_invert_tile); a pivot within 1e-9 of
//                                 zero is reported with its row, as the
//                                 reference's "Singularity in row" exit
//   R_kJ = P_k W_kJ  (J > k)      FP32 pipes; R replaces row block k
//   W_IJ -= W_Ik R_kJ (I, J > k)  the trailing update: one 3xFP16 product on
//                                 the tensor cores (k_tc_gemm3's read-modify-
//                                 write epilogue on the trailing sub-matrix),
//                                 operands as row-scaled fp16 pairs
// so that L_Ik = W_Ik P_k, U_kk = P_k^-1, U_kJ = P_k^-1 R_kJ, and a solve is
//   forward:  z_k = P_k (r_k - sum_{j<k} W_kj z_j)
//   backward: x_k = z_k - sum_{J>k} R_kJ x_J
// (one kernel per tile step, FP32, each updating the remaining rows with the
// finished tile's values).  The FP32-accurate factors solve the correction
// equation of an FP64 iterative refinement: x = 0, r = b; d = LU^-1 r (on r
// scaled to unit norm), x += d, r = b - A x with A in FP64; until |r| <=
// tol |b|, the correction is below 1e-14 |x|, or the residual stops falling.
#include <math.h>

#include <algorithm>
#include <vector>

#include "dsc_async.cuh"
#include "dsc_blas.cuh"
#include "dsc_common.cuh"
#include "dsc_gjtile.cuh"
#include "dsc_gmres.h"
#include "dsc_internal.h"
#include "dsc_tcgemm.h"

namespace dsc {

constexpr float kLuPivTol = 1.0E-9f;  // the reference's singular-pivot threshold (src/gaussBksb.c:46)
constexpr int kLuMaxRefine = 30;

// W (column-major FP32, np x np) = A (row-major FP64, n x n, stride lda),
// the identity on the padding; 32 x 32 tiles through shared memory.
__global__ void k_lu_load(const double *__restrict__ A, size_t lda, int n, float *__restrict__ W, int np)
{
    __shared__ float t[32][33];
    const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int r = r0 + y, c = c0 + threadIdx.x;
        t[y][threadIdx.x] = (r < n && c < n) ? (float)A[(size_t)r * lda + c] : (r == c ? 1.0f : 0.0f);
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) W[(size_t)(c0 + y) * np + r0 + threadIdx.x] = t[threadIdx.x][y];
}

// P_k = the inverse of the diagonal tile of step k (and its transpose).
__global__ void __launch_bounds__(kGjThreads) k_lu_pivot(const float *__restrict__ W, int np, int k, float *__restrict__ P,
                                                   float *__restrict__ PT, int *bad)
{
    grid_dep_wait();  // a programmatic dependent of the previous step's update
    gj_invert_tile(W + (size_t)k * kPB * np + k * kPB, np, P + (size_t)k * kPB * kPB, PT + (size_t)k * kPB * kPB,
                   kLuPivTol, bad, k * kPB);
}

// Step k, tile J = k + 1 + blockIdx.x: blockIdx.y < 4: columns 32 y ..
// 32 y + 31 of R_kJ = P_k W_kJ (PT: every step's P transposed, tile k at
// PT + k * 128 * 128) written into row block k and, transposed, as the
// update's B rows (the tile's columns, 128 k-values each, at Bh + (J - k -
// 1) * 128 * 128); blockIdx.y = 4: the column block's tile I = J as the
// update's A rows.  256 threads.
__global__ void __launch_bounds__(256) k_lu_row(float *__restrict__ W, int np, int k, const float *__restrict__ PT,
                                                __half *__restrict__ Ah, __half *__restrict__ Al,
                                                float *__restrict__ ra, __half *__restrict__ Bh,
                                                __half *__restrict__ Bl, float *__restrict__ rb)
{
    grid_dep_wait();  // a programmatic dependent of the pivot inversion
    const int J = k + 1 + blockIdx.x, o = blockIdx.x * kPB;
    extern __shared__ __align__(16) float sm[];
    const int warp = threadIdx.x >> 5;
    if (blockIdx.y == 4) {
        // A row i of tile I = J: A[i][kk] = W(J*128 + i, k*128 + kk)
        gj_load_rows(W + (size_t)k * kPB * np + J * kPB, (size_t)np, sm);
        for (int i = warp; i < kPB; i += 8)
            pre_row_pair(&sm[i * 129], Ah + (size_t)(o + i) * kPB, Al + (size_t)(o + i) * kPB, &ra[o + i]);
        return;
    }
    const int j0 = 32 * blockIdx.y;
    const float *T =
        gj_row_product(PT + (size_t)k * kPB * kPB, W + (size_t)J * kPB * np + k * kPB, (size_t)np, j0, sm);
    for (int t = threadIdx.x; t < 32 * kPB; t += blockDim.x) {
        const int jj = t >> 7, kk = t & 127;
        W[(size_t)(J * kPB + j0 + jj) * np + k * kPB + kk] = T[jj * 129 + kk];
    }
    for (int jj = warp; jj < 32; jj += 8)
        pre_row_pair(&T[jj * 129], Bh + (size_t)(o + j0 + jj) * kPB, Bl + (size_t)(o + j0 + jj) * kPB,
                     &rb[o + j0 + jj]);
}

// Forward step k: z_k = P_k y_k (every block forms it from the finished y_k;
// block 0 stores it), then y_r -= sum_c W(r, k*128 + c) z_k[c] for the rows
// r >= (k + 1) * 128 of this block.
__global__ void __launch_bounds__(256) k_lu_fwd(const float *__restrict__ W, int np, int k,
                                                const float *__restrict__ P, float *__restrict__ y,
                                                float *__restrict__ z)
{
    grid_dep_wait();
    __shared__ float yk[kPB], zk[kPB];
    const int kb = k * kPB;
    if (threadIdx.x < kPB) yk[threadIdx.x] = y[kb + threadIdx.x];
    __syncthreads();
    const float *Pk = P + (size_t)k * kPB * kPB;
    {
        // row i of P_k by two threads (halves of the row), then a shuffle
        const int i = threadIdx.x >> 1, h = threadIdx.x & 1;
        float s = 0.0f;
        const float *pr = Pk + (size_t)i * kPB + 64 * h;
#pragma unroll 8
        for (int q = 0; q < 64; q++) s = fmaf(pr[q], yk[64 * h + q], s);
        s += __shfl_xor_sync(0xffffffffu, s, 1);
        if (h == 0) zk[i] = s;
    }
    __syncthreads();
    if (blockIdx.x == 0 && threadIdx.x < kPB) z[kb + threadIdx.x] = zk[threadIdx.x];
    const int r = (k + 1) * kPB + blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= np) return;
    float s = 0.0f;
    const float *w = W + (size_t)kb * np + r;
#pragma unroll 8
    for (int c = 0; c < kPB; c++) s = fmaf(w[(size_t)c * np], zk[c], s);
    y[r] -= s;
}

// Backward step k: x_k = z_k is final; z_r -= sum_c R(r, k*128 + c) x_k[c]
// for the rows r < k * 128 of this block.
__global__ void __launch_bounds__(256) k_lu_bwd(const float *__restrict__ W, int np, int k, float *__restrict__ z)
{
    grid_dep_wait();
    __shared__ float xk[kPB];
    const int kb = k * kPB;
    if (threadIdx.x < kPB) xk[threadIdx.x] = z[kb + threadIdx.x];
    __syncthreads();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= kb) return;
    float s = 0.0f;
    const float *w = W + (size_t)kb * np + r;
#pragma unroll 8
    for (int c = 0; c < kPB; c++) s = fmaf(w[(size_t)c * np], xk[c], s);
    z[r] -= s;
}

// ---- the triangular sweeps in one cooperative launch each (CTA k: tile
// row k, every CTA resident at once).  A tile's values are published with
// a release store of the sweep's epoch into its flag; a CTA that needs them
// waits (thread 0, an acquire load; bounded: after kSpin cycles, or once
// another CTA has given up, it sets *err and returns) and reads them past
// L1.  Rows by two threads, on the two halves of each tile's 128 columns.

__device__ __forceinline__ int lu_ld_acquire(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void lu_st_release(int *p, int v)
{
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Thread 0 waits for flag == epoch; true for the whole CTA when it came.
__device__ __forceinline__ bool lu_wait(const int *flag, int epoch, int *err, int code)
{
    __shared__ int ok;
    if (threadIdx.x == 0) {
        const long long t0 = clock64();
        int good = 1;
        while (lu_ld_acquire(flag) != epoch) {
            if (clock64() - t0 > kSpin || *(volatile int *)err) {
                atomicCAS(err, 0, code);
                good = 0;
                break;
            }
            __nanosleep(32);
        }
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// acc[r] += sum over the 16 columns c0 .. c0+15 of tile column block (at
// col, leading dimension ld: element (row, c) at col[c * ld + row]) of
// element (4 lane + r, c) times v[c - c0]: 16 float4 loads issued together.
// GLOBAL_V: v is a published vector in global memory, read past L1; else v
// is in shared memory.
template <bool GLOBAL_V>
__device__ __forceinline__ void lu_tile_mv16(const float *__restrict__ col, size_t ld, int lane,
                                             const float *__restrict__ v, float (&acc)[4])
{
    float4 w[16];
#pragma unroll
    for (int c = 0; c < 16; c++) w[c] = *(const float4 *)(col + (size_t)c * ld + 4 * lane);
    float x[16];
#pragma unroll
    for (int c = 0; c < 16; c += 4) {
        const float4 q = GLOBAL_V ? __ldcg((const float4 *)(v + c)) : *(const float4 *)(v + c);
        x[c] = q.x;
        x[c + 1] = q.y;
        x[c + 2] = q.z;
        x[c + 3] = q.w;
    }
#pragma unroll
    for (int c = 0; c < 16; c++) {
        acc[0] = fmaf(w[c].x, x[c], acc[0]);
        acc[1] = fmaf(w[c].y, x[c], acc[1]);
        acc[2] = fmaf(w[c].z, x[c], acc[2]);
        acc[3] = fmaf(w[c].w, x[c], acc[3]);
    }
}

// The 8 column groups' partial sums of rows 4 lane .. 4 lane + 3 (thread
// group g = threadIdx.x >> 5) summed into out[128] (shared), g order.
__device__ __forceinline__ void lu_reduce8(const float (&acc)[4], float (*red)[kPB], float *out)
{
    const int g = threadIdx.x >> 5, lane = threadIdx.x & 31;
    *(float4 *)&red[g][4 * lane] = make_float4(acc[0], acc[1], acc[2], acc[3]);
    __syncthreads();
    if (threadIdx.x < kPB) {
        float s = 0.0f;
#pragma unroll
        for (int q = 0; q < 8; q++) s += red[q][threadIdx.x];
        out[threadIdx.x] = s;
    }
    __syncthreads();
}

// Forward: y_k -= sum_{j < k} W_kj z_j as each z_j is published, then
// z_k = P_k y_k (PT: every step's P transposed), published.  Thread (g,
// lane): rows 4 lane .. 4 lane + 3 of the tile row, columns 16 g .. 16 g + 15
// of each tile.
__global__ void __launch_bounds__(256, 1) k_lu_fwd_all(const float *__restrict__ W, int np,
                                                    const float *__restrict__ PT, const float *__restrict__ y,
                                                    float *__restrict__ z, int *flags, int epoch, int *err)
{
    __shared__ __align__(16) float red[8][kPB];
    __shared__ __align__(16) float yk[kPB];
    const int k = blockIdx.x, g = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int j = 0; j < k; j++) {
        if (!lu_wait(&flags[j], epoch, err, 11)) return;
        lu_tile_mv16<true>(W + (size_t)(j * kPB + 16 * g) * np + (size_t)k * kPB, (size_t)np, lane,
                           z + (size_t)j * kPB + 16 * g, acc);
    }
    lu_reduce8(acc, red, yk);
    if (threadIdx.x < kPB) yk[threadIdx.x] = y[(size_t)k * kPB + threadIdx.x] - yk[threadIdx.x];
    __syncthreads();
    float a2[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    lu_tile_mv16<false>(PT + (size_t)k * kPB * kPB + (size_t)(16 * g) * kPB, kPB, lane, yk + 16 * g, a2);
    lu_reduce8(a2, red, yk);
    if (threadIdx.x < kPB) z[(size_t)k * kPB + threadIdx.x] = yk[threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        lu_st_release(&flags[k], epoch);
    }
}

// Backward, in place on z: x_k = z_k - sum_{J > k} R_kJ x_J as each x_J is
// published (R: row block k of W), then x_k published over z_k.
__global__ void __launch_bounds__(256, 1) k_lu_bwd_all(const float *__restrict__ W, int np, int nb,
                                                    float *__restrict__ z, int *flags, int epoch, int *err)
{
    __shared__ __align__(16) float red[8][kPB];
    __shared__ __align__(16) float s[kPB];
    const int k = blockIdx.x, g = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int J = nb - 1; J > k; J--) {
        if (!lu_wait(&flags[J], epoch, err, 12)) return;
        lu_tile_mv16<true>(W + (size_t)(J * kPB + 16 * g) * np + (size_t)k * kPB, (size_t)np, lane,
                           z + (size_t)J * kPB + 16 * g, acc);
    }
    lu_reduce8(acc, red, s);
    if (threadIdx.x < kPB) z[(size_t)k * kPB + threadIdx.x] -= s[threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        lu_st_release(&flags[k], epoch);
    }
}

// y = r / scale (FP32), zero on the padding.
__global__ void k_lu_scale_in(const double *__restrict__ r, int n, int np, const double *__restrict__ nrm2,
                              float *__restrict__ y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const double s = sqrt(*nrm2);
    y[i] = (i < n && s > 0.0) ? (float)(r[i] / s) : 0.0f;
}

// x += scale * z; dn2 partial = |scale z|^2 (reduction as k_dot)
__global__ void k_lu_update(double *__restrict__ x, const float *__restrict__ z, int n,
                            const double *__restrict__ nrm2, RedWork rw, double *__restrict__ dn2)
{
    __shared__ double sh[32];
    const double s = sqrt(*nrm2);
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double d = s * (double)z[i];
        x[i] += d;
        acc += d * d;
    }
    finish_reduction(acc, rw, dn2, sh);
}

// r = b - A x (A row-major FP64, stride lda); one warp per row.
__global__ void k_lu_residual(const double *__restrict__ A, size_t lda, int n, const double *__restrict__ b,
                              const double *__restrict__ x, double *__restrict__ r)
{
    const int row = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (row >= n) return;
    const double *a = A + (size_t)row * lda;
    double s = 0.0;
    for (int c = lane; c < n; c += 32) s = fma(a[c], x[c], s);
    s = warp_sum(s);
    if (lane == 0) r[row] = b[row] - s;
}

__global__ void k_lu_dot(const double *__restrict__ a, int n, RedWork rw, double *__restrict__ out)
{
    __shared__ double sh[32];
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) acc += a[i] * a[i];
    finish_reduction(acc, rw, out, sh);
}

__global__ void k_lu_copy_b(const double *__restrict__ A, size_t lda, int n, double *__restrict__ b)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = A[(size_t)i * lda + n];
}

int lu_solve_mixed(int n, const double *dA, size_t lda, double *dx, double tol, LuMixedInfo *info, int *bad_row,
                   cudaStream_t st)
{
    const int np = (n + kPB - 1) / kPB * kPB, nb = np / kPB;
    DevBuf<float> W, P, PT, y, z;
    DevBuf<__half> gAh, gAl, gBh, gBl;
    DevBuf<float> ra, rb;
    DevBuf<int> bad, err;
    DevBuf<double> b, r, scal, part;
    DevBuf<unsigned> cnt;
    DSC_TRY(W.alloc((size_t)np * np));
    DSC_TRY(P.alloc((size_t)nb * kPB * kPB));
    DSC_TRY(PT.alloc((size_t)nb * kPB * kPB));
    // the update operands: two halves, alternating by the parity of the step
    const size_t oh = (size_t)np * kPB;
    DSC_TRY(gAh.alloc(2 * oh));
    DSC_TRY(gAl.alloc(2 * oh));
    DSC_TRY(gBh.alloc(2 * oh));
    DSC_TRY(gBl.alloc(2 * oh));
    DSC_TRY(ra.alloc(2 * (size_t)np));
    DSC_TRY(rb.alloc(2 * (size_t)np));
    DSC_TRY(bad.alloc(1));
    DSC_TRY(err.alloc(1));
    DSC_TRY(y.alloc(np));
    DSC_TRY(z.alloc(np));
    DSC_TRY(b.alloc(n));
    DSC_TRY(r.alloc(n));
    DSC_TRY(scal.alloc(4));
    DSC_TRY(part.alloc(kRedBlocks));
    DSC_TRY(cnt.alloc(1));
    const int big = 0x7FFFFFFF;
    DSC_CUDA(cudaMemcpyAsync(bad.p, &big, sizeof(int), cudaMemcpyHostToDevice, st));
    DSC_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    DSC_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned), st));
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    struct EvGuard {
        cudaEvent_t *e;
        ~EvGuard()
        {
            for (int q = 0; q < 3; q++)
                if (e[q]) cudaEventDestroy(e[q]);
        }
    } evg{ev};
    for (int q = 0; q < 3; q++) DSC_CUDA(cudaEventCreate(&ev[q]));
    DSC_CUDA(cudaEventRecord(ev[0], st));
    DSC_LAUNCH(k_lu_load<<<dim3(np / 32, np / 32), dim3(32, 8), 0, st>>>(dA, lda, n, W.p, np));
    DSC_CUDA(cudaGetLastError());
    // ---- factorisation
    const size_t rsmem = std::max(kGjRowSmem, sizeof(float) * kPB * 129);
    DSC_TRY(raise_smem_limit((const void *)k_lu_row, (int)rsmem));
    // Step k on a high-priority stream (hp, forked from st): the pivot
    // inverse and row block k, then (after the rest of step k - 1) the cross
    // of the trailing matrix's first tile -- the next pivot tile, row block
    // and column block -- and on a side stream the rest of the trailing
    // update (after row block k) on all but kGjReserveSms SMs, which step
    // k + 1's pivot and row block have to themselves.  The operands of step
    // k + 1 go to the other half of the buffers.
    struct OwnStream {
        cudaStream_t s = nullptr;
        ~OwnStream()
        {
            if (s) cudaStreamDestroy(s);
        }
    } side, hp;
    {
        int least = 0, greatest = 0;
        DSC_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        DSC_CUDA(cudaStreamCreateWithPriority(&side.s, cudaStreamNonBlocking, least));
        DSC_CUDA(cudaStreamCreateWithPriority(&hp.s, cudaStreamNonBlocking, greatest));
    }
    SideJoin hj;
    DSC_TRY(hj.fork(st, hp.s));
    EventPair evs;  // a: row block k is done; b: the rest of the last update is
    DSC_TRY(evs.create());
    int nsm = 0;
    DSC_TRY(current_sm_count(&nsm));
    const int rest_ctas = std::max(1, nsm - kGjReserveSms);
    bool rest_pending = false;
    for (int k = 0; k < nb; k++) {
        DSC_TRY(launch_dependent(k_lu_pivot, dim3(1), dim3(kGjThreads), 0, hp.s, (const float *)W.p, np, k, P.p, PT.p,
                                 bad.p));
        if (k + 1 == nb) break;
        const int rest = nb - k - 1, k1 = (k + 1) * kPB, m = np - k1;
        const size_t h = (size_t)(k & 1);
        __half *Ah = gAh.p + h * oh, *Al = gAl.p + h * oh, *Bh = gBh.p + h * oh, *Bl = gBl.p + h * oh;
        float *rah = ra.p + h * np, *rbh = rb.p + h * np;
        DSC_TRY(launch_dependent(k_lu_row, dim3(rest, 5), dim3(256), rsmem, hp.s, W.p, np, k, (const float *)PT.p,
                                 Ah, Al, rah, Bh, Bl, rbh));
        DSC_CUDA(cudaEventRecord(evs.a, hp.s));
        if (rest_pending) DSC_CUDA(cudaStreamWaitEvent(hp.s, evs.b, 0));
        // W_IJ -= A_I B_J^T on the trailing sub-matrix (no tile excluded)
        TcGjPlan plan;
        DSC_TRY(tc_gj_plan(plan, Ah, Al, kPB, Bh, Bl, kPB, m, m, W.p + (size_t)k1 * np + k1, (size_t)np, err.p,
                           rah, rbh));
        if (rest >= 2) {
            DSC_TRY(tc_gj_run(plan, big, hp.s, 1, 0));
            DSC_CUDA(cudaStreamWaitEvent(side.s, evs.a, 0));
            DSC_TRY(tc_gj_run(plan, big, side.s, 2, 0, rest_ctas));
            DSC_CUDA(cudaEventRecord(evs.b, side.s));
            rest_pending = true;
        } else {
            DSC_TRY(tc_gj_run(plan, big, hp.s));
            rest_pending = false;
        }
    }
    if (rest_pending) DSC_CUDA(cudaStreamWaitEvent(hp.s, evs.b, 0));
    DSC_TRY(hj.done(hp.s));
    DSC_TRY(hj.join());
    DSC_CUDA(cudaEventRecord(ev[1], st));
    int hbad = big, herr = 0;
    DSC_CUDA(cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    DSC_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    DSC_CUDA(cudaStreamSynchronize(st));
    if (herr) {
        set_error("block LU: a pipeline wait of the tensor-core update gave up (code %d)", herr);
        return kErrCuda;
    }
    if (hbad < n) {
        if (bad_row) *bad_row = hbad;
        set_error("Singularity in row %d in system matrix", hbad);
        return kErrSingular;
    }
    if (info) info->factor_done = true;
    // ---- refinement: x = 0, r = b
    RedWork rw{part.p, cnt.p};
    DSC_LAUNCH(k_lu_copy_b<<<(n + 255) / 256, 256, 0, st>>>(dA, lda, n, b.p));
    DSC_CUDA(cudaMemcpyAsync(r.p, b.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    DSC_CUDA(cudaMemsetAsync(dx, 0, n * sizeof(double), st));
    double *rn2 = scal.p, *dn2 = scal.p + 1;
    DSC_LAUNCH(k_lu_dot<<<kRedBlocks, kRedThreads, 0, st>>>(b.p, n, rw, rn2));
    double h[2];
    DSC_CUDA(cudaMemcpyAsync(h, rn2, sizeof(double), cudaMemcpyDeviceToHost, st));
    DSC_CUDA(cudaStreamSynchronize(st));
    const double bnorm = sqrt(h[0]);
    double rprev = bnorm;
    int it = 0, status = 1;  // 1 running, 0 converged, 2 the residual stopped falling
    if (bnorm == 0.0) status = 0;
    const int vg = (np + 255) / 256;
    // the one-launch sweeps need every tile row's CTA resident at once
    bool coop = false;
    DevBuf<int> flags;
    int epoch = 0;
    {
        int dev = 0, can = 0, per = 0, nsm = 0;
        DSC_CUDA(cudaGetDevice(&dev));
        DSC_CUDA(cudaDeviceGetAttribute(&can, cudaDevAttrCooperativeLaunch, dev));
        DSC_TRY(current_sm_count(&nsm));
        int per_b = 0;
        DSC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_lu_fwd_all, 256, 0));
        DSC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_b, k_lu_bwd_all, 256, 0));
        coop = can && (long long)std::min(per, per_b) * nsm >= nb;
        if (coop) {
            DSC_TRY(flags.alloc(nb));
            DSC_CUDA(cudaMemsetAsync(flags.p, 0, nb * sizeof(int), st));
        }
    }
    while (status == 1 && it < kLuMaxRefine) {
        it++;
        // d = LU^-1 (r / |r|) |r|
        DSC_LAUNCH(k_lu_scale_in<<<vg, 256, 0, st>>>(r.p, n, np, rn2, y.p));
        if (coop) {
            // one cooperative launch per sweep, tiles handed on by flags
            const float *Wc = W.p, *Pc = PT.p, *yc = y.p;
            float *zc = z.p;
            int *fl = flags.p, *er = err.p;
            int ef = ++epoch;
            void *fa[] = {(void *)&Wc, (void *)&np, (void *)&Pc, (void *)&yc, (void *)&zc, (void *)&fl, (void *)&ef,
                          (void *)&er};
            note_launch();
            DSC_CUDA(cudaLaunchCooperativeKernel((const void *)k_lu_fwd_all, dim3(nb), dim3(256), fa, 0, st));
            int eb = ++epoch;
            void *ba[] = {(void *)&Wc, (void *)&np, (void *)&nb, (void *)&zc, (void *)&fl, (void *)&eb, (void *)&er};
            note_launch();
            DSC_CUDA(cudaLaunchCooperativeKernel((const void *)k_lu_bwd_all, dim3(nb), dim3(256), ba, 0, st));
        } else {
            for (int k = 0; k < nb; k++) {
                const int rows = np - (k + 1) * kPB;
                DSC_TRY(launch_dependent(k_lu_fwd, dim3(std::max(1, (rows + 255) / 256)), dim3(256), 0, st,
                                         (const float *)W.p, np, k, (const float *)P.p, y.p, z.p));
            }
            for (int k = nb - 1; k >= 0; k--)
                if (k > 0)
                    DSC_TRY(launch_dependent(k_lu_bwd, dim3((k * kPB + 255) / 256), dim3(256), 0, st,
                                             (const float *)W.p, np, k, z.p));
        }
        DSC_LAUNCH(k_lu_update<<<kRedBlocks, kRedThreads, 0, st>>>(dx, z.p, n, rn2, rw, dn2));
        DSC_LAUNCH(k_lu_residual<<<(n * 32 + 255) / 256, 256, 0, st>>>(dA, lda, n, b.p, dx, r.p));
        DSC_LAUNCH(k_lu_dot<<<kRedBlocks, kRedThreads, 0, st>>>(r.p, n, rw, rn2));
        DSC_LAUNCH(k_lu_dot<<<kRedBlocks, kRedThreads, 0, st>>>(dx, n, rw, scal.p + 2));
        DSC_CUDA(cudaGetLastError());
        double hv[3];
        int herr_s = 0;
        DSC_CUDA(cudaMemcpyAsync(hv, scal.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
        if (coop) DSC_CUDA(cudaMemcpyAsync(&herr_s, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        DSC_CUDA(cudaStreamSynchronize(st));
        if (herr_s) {
            set_error("block LU: a triangular sweep's wait for a tile gave up (code %d)", herr_s);
            return kErrCuda;
        }
        const double rnorm = sqrt(hv[0]), dnorm = sqrt(hv[1]), xnorm = sqrt(hv[2]);
        // converged: the residual is below the tolerance or the correction
        // at the rounding level of x (1e-14 |x|); a residual that stops
        // falling is accepted once the corrections are within 1e-12 |x|
        // (the FP64 residual's own rounding), else the factors are too
        // inaccurate for this matrix
        if (rnorm <= tol * bnorm || dnorm <= 1e-14 * xnorm) status = 0;
        else if (it >= 3 && rnorm > 0.5 * rprev) status = dnorm <= 1e-12 * xnorm ? 0 : 2;
        if (info) {
            info->refinements = it;
            info->rel_residual = rnorm / bnorm;
            info->last_correction = xnorm > 0.0 ? dnorm / xnorm : dnorm;
        }
        rprev = rnorm;
    }
    if (status == 1) status = 2;
    DSC_CUDA(cudaEventRecord(ev[2], st));
    DSC_CUDA(cudaEventSynchronize(ev[2]));
    if (info) {
        DSC_CUDA(cudaEventElapsedTime(&info->factor_ms, ev[0], ev[1]));
        DSC_CUDA(cudaEventElapsedTime(&info->refine_ms, ev[1], ev[2]));
    }
    if (status != 0) {
        set_error("block LU refinement: relative residual %.3e after %d steps (tolerance %.1e)",
                  info ? info->rel_residual : 0.0, it, tol);
        return kErrStagnation;
    }
    return kOk;
}

}  // namespace dsc
