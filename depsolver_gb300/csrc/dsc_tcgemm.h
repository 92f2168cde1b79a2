// dsc_tcgemm.h -- tensor-core GEMM of libdepsolver_cuda (not exported).
#pragma once

#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stddef.h>

namespace dsc {

// Fixed-point digits of the FP64-accurate product K x (the mixed sweep's
// first residual): K as kKDigits balanced digits of kKDigitBits bits per
// row (|q| <= 32), x as kXDigits digits of kXDigitBits bits per column
// (|q| <= 128): every digit product is at most 2^12 and a 4096-long sum of
// them at most 2^24.
constexpr int kKDigits = 8, kKDigitBits = 6;
constexpr int kXDigits = 3, kXDigitBits = 8;
// The x digits taken with K digit i: those whose weight is within 2^-48 of
// the largest, kKDigitBits i + kXDigitBits j <= 48.
constexpr int x_digits_for(int i)
{
    return (48 - kKDigitBits * i) / kXDigitBits + 1 < kXDigits ? (48 - kKDigitBits * i) / kXDigitBits + 1
                                                               : kXDigits;
}

// Y[s][n][m] (split s, column n, row m; stride ldy per column and ldy * Nc
// per split) = partial sums over split s's share of k of
//   (Ah + Al)[m][k] * (Bh + Bl)[n][k]  with the three products hh + hl + lh.
// A: M x Kd, B: Nc x Kd, both K-major FP32 holding tf32 pairs, row strides
// lda / ldb (multiples of 4 elements, 16-byte aligned bases).  Nc <= 160.
// *d_err (device, zero on entry) is set when a wait inside the kernel gives
// up.  The caller adds the splits.  Al = null: A is plain FP32 (split in
// shared memory), or with a_biased in the encoding split_transpose_K(...,
// biased = true) writes.
int tc_gemm_3xtf32(const float *Ah, const float *Al, size_t lda, const float *Bh, const float *Bl,
                   size_t ldb, int M, int Nc, int Kd, float *Y, size_t ldy, int splits, int *d_err,
                   cudaStream_t st, bool a_biased = false);
int tc_gemm_splits_for(int M, int Kd);

// The same three products in fp16 (kind::f16, twice the tf32 rate) on
// scaled fp16 pairs: A = 2^s_m (Ah + Al) per row, B = 2^t_n (Bh + Bl) per
// column, each row's / column's largest entry in [2^14, 2^15).  Y is the
// unscaled product: the epilogue multiplies row m by rsc[m] = 2^-s_m and
// column n by csc[n] = 2^-t_n (either null: 1).  Row strides lda / ldb in
// elements (multiples of 8, 16-byte aligned bases).
int tc_gemm_3xf16(const __half *Ah, const __half *Al, size_t lda, const __half *Bh, const __half *Bl,
                  size_t ldb, int M, int Nc, int Kd, float *Y, size_t ldy, int splits, int *d_err,
                  cudaStream_t st, const float *rsc, const float *csc);
int tc_gemm_f16_splits_for(int M, int Kd);
// The split count tc_gemm_3xf16 actually uses when asked for `splits` (the
// k-blocks dealt evenly: the number of partial tiles it writes).
int tc_gemm_f16_splits_norm(int Kd, int splits);
// One fp16 product per split, for integer-valued operands ("digits"):
// Y[s][n][m] = sum over split s's k-range of A[m][k] * B[n][k], each split
// at most 4096 k long, so that with |A| <= 32 and |B| <= 128 (or any pair
// whose product stays within 2^12) every partial sum is an integer of at
// most 2^24 and exact in the FP32 accumulator.  Nc <= 384; row strides in
// elements (multiples of 8, 16-byte aligned bases).  tc_digit_splits(Kd)
// is the split count, S, the partial tiles Y holds (stride ldy * Nc).
int tc_gemm_digits(const __half *A, size_t lda, const __half *B, size_t ldb, int M, int Nc, int Kd, float *Y,
                   size_t ldy, int *d_err, cudaStream_t st);
int tc_digit_splits(int Kd);
// Tensor map of a row-major matrix of FP32 (esize 4) or fp16 (esize 2)
// values, rows x k (k contiguous, row stride ld elements, 16-byte aligned),
// boxes of one 128-byte swizzle row of k by box_rows rows, zero fill.
int tc_make_map(CUtensorMap *map, const void *base, int esize, int rows, int k, size_t ld, int box_rows);
// The Gauss-Jordan update of step k (3xFP16, K = 128): for every 128 x 128
// tile (I, J) of C (column-major, M x Nc, stride ldc a multiple of 4, C
// 16-byte aligned) with I != k: C_IJ -= A_I B_J^T (C_Ik = -A_I B_k^T); A
// (M x 128) and B (Nc x 128) K-major scaled fp16 pairs with row factors
// rsc, csc.  The tensor maps are encoded once (tc_gj_plan) for all steps.
constexpr int kTcGjMaxProblems = 4;
struct TcGjPlan {
    struct Maps;
    Maps *maps = nullptr;
    int M = 0, Nc = 0;
    float *C = nullptr;
    size_t ldc = 0;
    int *err = nullptr;
    const float *rsc = nullptr, *csc = nullptr;
    TcGjPlan() = default;
    TcGjPlan(const TcGjPlan &) = delete;
    TcGjPlan &operator=(const TcGjPlan &) = delete;
    ~TcGjPlan();
};
int tc_gj_plan(TcGjPlan &p, const __half *Ah, const __half *Al, size_t lda, const __half *Bh,
               const __half *Bl, size_t ldb, int M, int Nc, float *C, size_t ldc, int *d_err,
               const float *rsc, const float *csc);
// sel = 0: every tile of the update; sel = 1: only the cross of tile la
// (row tile la and column tile la, la != k), sel = 2: every other tile --
// so that the next step's pivot tile, row block and column block (la = k +
// 1) can be ready while the rest is updated.  max_ctas > 0 sets the
// persistent grid (below the SM count: SMs left for kernels of other
// streams).
int tc_gj_run(const TcGjPlan &p, int k, cudaStream_t st, int sel = 0, int la = 0, int max_ctas = 0);
// The same step of up to kTcGjMaxProblems plans (sharing one error word) in
// one launch.
int tc_gj_run_batch(const TcGjPlan *const *plans, int np, int k, cudaStream_t st, int sel = 0, int la = 0,
                    int max_ctas = 0);
// Row scales of column-major FP64 K (stride ld): rowE (N ints) the biased
// exponent of each row's largest entry, rsK = 2^-s_i.
int k16_row_scales(const double *K, size_t ld, int N, int *rowE, float *rsK, cudaStream_t st);
// K to the row-major scaled fp16 pair of fl32(K) (Th, Tl) and, with Dg not
// null, to K's kKDigits row digits (digit d at Dg + d * dstride: fp16
// integers, K[i][c] ~ 2^(rowE[i] - 1069) sum_d q_d 2^(kKDigitBits
// (kKDigits - 1 - d))), after k16_row_scales.
int split_transpose_K16(const double *K, size_t ld, int N, const int *rowE, __half *Th, __half *Tl,
                        __half *Dg, size_t dstride, size_t ldt, cudaStream_t st);
// Columns of X (ncol, N entries each, stride ldx) to their kXDigits digits
// (digit j of column c: fp16 row j * ncol + c of Xd, stride ldd;
// X[c][i] = 2^(colE[c] - 1045) sum_j q_j 2^(kXDigitBits (kXDigits - 1 - j))
// + Xr[c][i], the remainder exact in FP64, stride ldr).
int x_digits(const double *X, size_t ldx, int N, int ncol, __half *Xd, size_t ldd, double *Xr, size_t ldr,
             int *colE, cudaStream_t st);
// Y (FP64, column c at c * ldy; first: =, else +=) gets the product of K
// digit i with the first nj x digits from tc_gemm_digits' S partial tiles
// P (column j * ncol + c at stride ldp), weighted by the digits' places.
int digit_accumulate(const float *P, int S, size_t ldp, int ncol, int nj, int i, int N, double *Y, size_t ldy,
                     bool first, cudaStream_t st);
// Y *= the units of K's rows and x's columns: Y = K x (digit parts).
int digit_finish(const int *rowE, const int *colE, int N, int ncol, double *Y, size_t ldy, cudaStream_t st);
// Columns (N entries each, stride ldx) to scaled fp16 pairs (stride ldh),
// csc[n] = the column's 2^-t_n.
int split_cols_f16(const double *x, size_t ldx, int N, int ncol, __half *h, __half *l, size_t ldh,
                   float *csc, cudaStream_t st);
int split_cols_f16(const float *x, size_t ldx, int N, int ncol, __half *h, __half *l, size_t ldh,
                   float *csc, cudaStream_t st);

// Column-major FP64 N x N matrix (stride ld) to row-major FP32: the tf32
// pair of each entry (Th, Tl), the entry rounded to FP32 (Th; plain or in
// the biased tf32 encoding), or the biased FP32 entry (Th) and the biased
// FP32 rounding of the rest (Tl: a - (double)(float)a).
enum { kTransposePair = 0, kTransposePlain = 1, kTransposeBiased = 2, kTransposeBiasedRem = 3 };
int split_transpose_K(const double *K, size_t ld, int N, float *Th, float *Tl, size_t ldt,
                      cudaStream_t st, int mode);
// FP32 array to tf32 pairs, elementwise.
int f32_to_tf32_pair(const float *x, float *h, float *l, size_t n, cudaStream_t st);
// Y[n * ldy + m] += the S partial tiles of tc_gemm_3xtf32 (tile s, column n,
// row m at s * split_stride + n * ldp + m), in split order.
int add_splits(const float *P, int S, size_t split_stride, size_t ldp, int M, int Nc, double *Y,
               size_t ldy, cudaStream_t st);
// FP64 array to tf32 pairs, elementwise.
int split_vec(const double *x, float *h, float *l, size_t n, cudaStream_t st);
// Row-major FP64 rows x k (row stride ld) to tf32 pairs (row stride ldh).
int split_rows(const double *x, size_t ld, int rows, int k, float *h, float *l, size_t ldh,
               cudaStream_t st);
// Y[m * ldy + n] = sum over S partial tiles of tc_gemm_3xtf32 (tile s,
// column n, row m at s * split_stride + n * ldp + m), in split order.
int sum_splits(const float *P, int S, size_t split_stride, size_t ldp, int M, int Nc, double *Y,
               size_t ldy, cudaStream_t st);
// The number of partial tiles tc_gemm_3xtf32 writes for `splits` (>= 1).
int tc_gemm_splits_used(int Kd, int splits);

}  // namespace dsc
