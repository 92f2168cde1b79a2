// dsc_tcgemm.cu -- split-K three-product GEMM on the 5th-generation tensor
// cores, in tf32 or in fp16.
//
//   Y[s] (Nc x M, per split s) = sum over the k-range of split s of
//       A (M x Kd) * B^T,   A = Ah + Al,  B = Bh + Bl
//   with the three products Ah Bh + Ah Bl + Al Bh: about FP32 accuracy.
//
// tf32 (3xTF32): A and B are K-major FP32 tf32 pairs, or A plain FP32 split
// in shared memory.  fp16 (3xFP16): A and B are K-major fp16 pairs of
// operands scaled by powers of two (per row of A, per column of B) so that
// each row's / column's largest entry lies in [2^14, 2^15); the epilogue
// multiplies the scales back out (exact).  Both halves of a pair carry 11
// significant bits, as tf32 does, and kind::f16 issues at twice the
// kind::tf32 rate.
//
// Persistent kernel: one CTA per SM walks the units (128-row tile, split of
// k) u = blockIdx.x, + gridDim.x, ...  Warp 0 lane 0 streams k-blocks (one
// 128-byte swizzle row: 32 tf32 or 64 fp16 values) of A and Bh, Bl into a
// 3-stage shared-memory ring with TMA (128B swizzle) without pausing between
// units; warps 2-5 split a plain FP32 A in shared memory; warp 1 lane 0
// issues tcgen05.mma (M = 128, 32 bytes of k per instruction: K = 8 tf32 or
// K = 16 fp16) into one of two FP32 accumulator buffers in tensor memory and
// releases each stage with tcgen05.commit; warps 6-9 read the finished
// buffer back (tcgen05.ld, one TMEM lane per row) and store the partial tile
// while the next unit accumulates in the other buffer.  Every wait on an
// mbarrier gives up after ~2 s of clock, sets *err and lets the CTA drain
// and free its tensor memory.  The Gauss-Jordan / block-LU update is a
// kernel of its own on the same building blocks (k_tc_gj, below).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>

#include "dsc_async.cuh"
#include "dsc_tc.cuh"
#include "dsc_df32.cuh"
#include "dsc_internal.h"
#include "dsc_tcgemm.h"

namespace dsc {

constexpr int kTcBM = 128;
// k-blocks of kTcRowBytes (dsc_tc.cuh).  Measured at the 12k-node scene:
// 128-byte rows in 3 stages 32.5 ms per sweep's products, 64-byte rows in
// 6 stages 47.1 ms (twice the barrier hand-offs per byte).
constexpr int kTcBK = kTcRowBytes / 4;    // fp32 elements per k-block
constexpr int kTcBK16 = kTcRowBytes / 2;  // fp16 elements per k-block
constexpr int kTcStages = 3;
// warps: 0 TMA producer, 1 MMA issuer, 2 .. 2 + kTcSplitWarps - 1 split A,
// the last 4 read the accumulators back
constexpr int kTcSplitWarps = 4;
constexpr int kTcSplitters = 32 * kTcSplitWarps;
constexpr int kTcThreads = 32 * (2 + kTcSplitWarps + 4);
// 3 stages of 2 x 16 KB (A) + 2 x BN x 128 B (B) fit the 227 KB of shared
// memory a CTA may use for BN <= 160
constexpr int kTcMaxNc = 160;
constexpr long long kTcSpin = kSpin;  // clock cycles before a wait gives up
// digit products: at most 64 k-blocks (4096 k) per split, and up to 384
// columns (3 stages of a 16 KB A tile and a 48 KB B tile)
constexpr int kTcDigitKBlocks = 64;
constexpr int kTcMaxDigitCols = 384;
// The Gauss-Jordan update (rank 128 on 128 x 128 tiles: two k-blocks per
// unit) keeps one stage of operands and a ring of kGjXSlots half tiles (128
// rows x 64 columns, FP32) of the old values, which the producer fetches by
// TMA when it starts a unit; each epilogue warp rewrites its 32 x 64 box in
// place and stores it back by TMA.  Four slots are two units: the old
// values of the next unit stream in while this one is formed.
constexpr int kGjStages = 1;
constexpr int kGjXSlots = 4;
constexpr int kGjXBoxRows = 32, kGjXBoxCols = 64;
constexpr uint32_t kGjXBoxBytes = kGjXBoxRows * kGjXBoxCols * 4;
constexpr uint32_t kGjXHalfBytes = 4 * kGjXBoxBytes;

// The tf32 value the tensor core reads from an FP32 word: the top 19 bits
// (the low 13 mantissa bits are ignored).
__device__ __forceinline__ float tf32_trunc(float v)
{
    return __uint_as_float(__float_as_uint(v) & 0xFFFFE000u);
}

__device__ __forceinline__ float tf32_rna(float v)
{
    uint32_t h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
    return __uint_as_float(h);
}

// lo of the split a = trunc(a) + lo, itself rounded to tf32 so that the
// tensor core's truncation of it loses nothing more
__device__ __forceinline__ float tf32_lo(float v)
{
    return tf32_rna(v - tf32_trunc(v));
}

// Half a tf32 unit in the last place of t (t's sign; 0 for tiny t).
__device__ __forceinline__ float tf32_half_ulp(float t)
{
    const uint32_t u = __float_as_uint(t);
    const uint32_t e = u & 0x7F800000u;
    return e > (11u << 23) ? __uint_as_float((u & 0x80000000u) | (e - (11u << 23))) : 0.0f;
}

// Biased encoding of an FP32 value a for the tensor core: s = a + half-ulp
// of h = rna_tf32(a), with a's sign, so that the truncation the tensor core
// applies to s gives h (the round-to-nearest hi) and the low part can be
// recovered as s - trunc(s) - half-ulp, |lo| <= half a tf32 ulp.
__device__ __forceinline__ float tf32_bias_encode(float a)
{
    return __fadd_rn(a, tf32_half_ulp(tf32_rna(a)));
}

// trunc(s) + half-ulp is s's top 19 bits with mantissa bit 12 set (for
// normal s), so the low part is one exact subtraction.
__device__ __forceinline__ float tf32_lo_biased(float s)
{
    const float mid = __uint_as_float((__float_as_uint(s) & 0xFFFFE000u) | 0x00001000u);
    return tf32_rna(__fsub_rn(s, mid));
}

// AMODE 0: A arrives as a tf32 pair (tmAh, tmAl).
// AMODE 1: A arrives as plain FP32 through tmAh into the hi slot; the tensor
// core reads it as its truncated tf32 value, and the splitter warps write the
// remainder a - trunc(a), rounded to tf32, into the lo slot before the
// products with lo may read the stage.
// AMODE 2: as 1, with A in the biased encoding (tf32_bias_encode): the
// truncation gives the round-to-nearest hi, so |lo| is half as large and the
// dropped lo*lo product is at 2^-22 instead of 2^-21.
// AMODE 3: A and B arrive as scaled fp16 pairs (kind::f16); the epilogue
// multiplies row m by rsc[m] and column n by csc[n] (null: 1).
// AMODE 4 (digits): one product A B^T of single fp16 operands (no pairs),
// BN up to 384 columns (two MMAs of BN / 2 when BN > 256; one accumulator
// buffer when two do not fit the 512 TMEM columns).  With small-integer
// operands and short enough splits every partial sum is an integer below
// 2^24, which the FP32 accumulator holds exactly whatever its rounding.
// COMB (BN a multiple of 32, at most 128): Ah*Bh and Ah*Bl are one MMA of
// N = 2 BN against the adjacent Bh and Bl tiles, into accumulator columns
// [0, BN) and [BN, 2 BN); Al*Bh adds into [BN, 2 BN) too; the epilogue adds
// the two.  This reads Ah once instead of twice, and keeps the small
// products out of the main accumulator: the tensor core's FP32 accumulation
// truncates (sums of positive products come out low), so every MMA added
// into an accumulator costs up to one of its units in the last place.
// Row and column tile of unit u of the Gauss-Jordan update.  sel = 0: row
// tile u % tiles, column tile (u / tiles) % ntn.  sel = 1 takes the cross of tile la: row tile la with every
// column tile (u < ntn), then column tile la with every row tile other than
// la and gk; with sel = 2 every other tile (row tiles other than la and gk,
// column tiles other than la).  A gk outside [0, tiles) excludes nothing.
// Together sel 1 and sel 2 cover the tiles of sel 0 but row tile gk (which
// the update leaves alone).
__device__ __forceinline__ void unit_tile(int u, int tiles, int ntn, int sel, int la, int gk, int &tm, int &tn)
{
    if (sel == 0) {
        tm = u % tiles;
        tn = (u / tiles) % ntn;
        return;
    }
    const bool gv = gk >= 0 && gk < tiles && gk != la;
    const int e1 = gv ? min(la, gk) : la, e2 = gv ? max(la, gk) : 0x7FFFFFFF;
    if (sel == 1 && u < ntn) {
        tm = la;
        tn = u;
        return;
    }
    const int nr = tiles - 1 - (gv ? 1 : 0);
    int i = sel == 1 ? u - ntn : u % nr;  // the i-th row tile other than e1, e2
    if (i >= e1) i++;
    if (i >= e2) i++;
    tm = i;
    if (sel == 1) {
        tn = la;
    } else {
        const int c = u / nr;
        tn = c >= la ? c + 1 : c;
    }
}

// Units of the update's tile selection sel (see unit_tile).
__host__ __device__ inline int gj_sel_units(int tiles, int ntn, int sel, int la, int gk)
{
    if (sel == 0) return tiles * ntn;
    const bool gv = gk >= 0 && gk < tiles && gk != la;
    const int nr = tiles - 1 - (gv ? 1 : 0);
    return sel == 1 ? ntn + nr : nr * (ntn - 1);
}

template <int AMODE>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_tc_gemm3(const __grid_constant__ CUtensorMap tmAh, const __grid_constant__ CUtensorMap tmAl,
               const __grid_constant__ CUtensorMap tmBh, const __grid_constant__ CUtensorMap tmBl,
               int M, int Nc, int BN, int ntn, int nkb_total, int kb_per_split, int nsplit,
               float *__restrict__ Y, size_t ldy, size_t split_stride, int tmem_cols,
               uint32_t acc_stride, const float *__restrict__ rsc, const float *__restrict__ csc,
               int *err)
{
    grid_dep_wait();  // launched as a programmatic dependent of the kernel before
    // ntn: column tiles of BN columns
    // acc_stride: TMEM columns of one accumulator buffer, a power of two of
    // at least the columns it holds (so each buffer's MMAs start aligned)
    constexpr bool SPLIT_A = AMODE == 1 || AMODE == 2;
    constexpr bool DIG = AMODE == 4;
    constexpr bool F16 = AMODE == 3 || DIG;
    constexpr int BK = F16 ? kTcBK16 : kTcBK;  // elements per k-block
    const bool comb = !DIG && BN <= 128 && BN % 32 == 0;
    // B rows per TMA box and per MMA (a box and an MMA take at most 256)
    const int bsub = BN > 256 ? BN / 2 : BN;
    // accumulator buffers: two unless they do not fit the allocation
    const int nbuf = 2 * (int)acc_stride <= tmem_cols ? 2 : 1;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t a_bytes = kTcBM * kTcRowBytes, b_bytes = (uint32_t)BN * kTcRowBytes;
    const uint32_t stage_bytes = DIG ? a_bytes + b_bytes : 2 * a_bytes + 2 * b_bytes;
    uint64_t *full = (uint64_t *)(smem + kTcStages * stage_bytes);
    uint64_t *empty = full + kTcStages;
    uint64_t *splitb = empty + kTcStages;
    uint64_t *acc_full = splitb + kTcStages;  // [2]
    uint64_t *acc_empty = acc_full + 2;       // [2]
    uint64_t *done = acc_empty + 2;
    uint32_t *tmem_slot = (uint32_t *)(done + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tiles = (M + kTcBM - 1) / kTcBM;
    // unit u: row tile u % tiles, then column tile, then split
    const int units = tiles * ntn * nsplit;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kTcStages; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
            mbar_init(&splitb[s], kTcSplitters);  // the threads of warps 2 .. 2 + kTcSplitWarps - 1
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 4);  // one lane of each epilogue warp
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         su32(tmem_slot)),
                     "r"(tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    // Every role walks the same sequence: units u = blockIdx.x, + gridDim.x,
    // ... (unit = row tile + tiles * split), and within a unit its k-blocks;
    // g counts k-blocks over all units (stage g % kTcStages, use g / kTcStages).
    if (warp == 0) {
        if (lane == 0) {
            // ---- producer
            uint32_t g = 0;
            bool ok = true;
            for (int u = blockIdx.x; ok && u < units; u += gridDim.x) {
                const int m0 = (u % tiles) * kTcBM, n0 = ((u / tiles) % ntn) * BN;
                const int kb0 = (u / tiles / ntn) * kb_per_split;
                const int nkb = min(nkb_total, kb0 + kb_per_split) - kb0;
                for (int i = 0; i < nkb; i++, g++) {
                    const uint32_t s = g % kTcStages, n = g / kTcStages;
                    if (n > 0 && !mbar_wait(&empty[s], (n - 1) & 1, err, 1)) {
                        ok = false;
                        break;
                    }
                    uint8_t *st = smem + s * stage_bytes;
                    mbar_expect_tx(&full[s], SPLIT_A ? stage_bytes - a_bytes : stage_bytes);
                    const int kx = (kb0 + i) * BK;
                    tma_load_2d(st, &tmAh, &full[s], kx, m0);
                    if (DIG) {
                        for (int r = 0; r < BN; r += bsub)
                            tma_load_2d(st + a_bytes + (uint32_t)r * kTcRowBytes, &tmBh, &full[s], kx, n0 + r);
                        continue;
                    }
                    if (!SPLIT_A) tma_load_2d(st + a_bytes, &tmAl, &full[s], kx, m0);
                    tma_load_2d(st + 2 * a_bytes, &tmBh, &full[s], kx, n0);
                    tma_load_2d(st + 2 * a_bytes + b_bytes, &tmBl, &full[s], kx, n0);
                }
            }
            // drain: the last loads of every stage have landed before the CTA
            // may exit (immediate in the normal path, bounded otherwise)
            for (uint32_t h = g > (uint32_t)kTcStages ? g - kTcStages : 0; h < g; h++)
                mbar_drain(&full[h % kTcStages], (h / kTcStages) & 1);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---- MMA issuer
            const uint32_t idesc = F16 ? idesc_f16(DIG ? bsub : BN, kTcBM) : idesc_tf32(BN, kTcBM);
            const uint32_t idesc2 = F16 ? idesc_f16(2 * BN, kTcBM) : idesc_tf32(2 * BN, kTcBM);
            uint32_t g = 0;
            bool ok = true;
            int j = 0;
            for (int u = blockIdx.x; ok && u < units; u += gridDim.x, j++) {
                const int kb0 = (u / tiles / ntn) * kb_per_split;
                const int nkb = min(nkb_total, kb0 + kb_per_split) - kb0;
                const uint32_t buf = j % nbuf, q = j / nbuf;
                if (q > 0 && !mbar_wait(&acc_empty[buf], (q - 1) & 1, err, 5)) break;
                tc_fence_after();
                const uint32_t acc = tmem + buf * acc_stride;
                for (int i = 0; i < nkb; i++, g++) {
                    const uint32_t s = g % kTcStages, n = g / kTcStages;
                    if (!mbar_wait(&full[s], n & 1, err, 2)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    uint8_t *st = smem + s * stage_bytes;
                    if (DIG) {
                        const uint64_t da = sw_desc(st);
#pragma unroll
                        for (int kk = 0; kk < kTcRowBytes / 32; kk++) {
                            const uint64_t off = (uint64_t)(kk * 32) >> 4;
                            for (int r = 0; r < BN; r += bsub)
                                mma_op<true>(acc + (uint32_t)r, da + off,
                                             sw_desc(st + a_bytes + (uint32_t)r * kTcRowBytes) + off, idesc,
                                             (i | kk) != 0);
                        }
                        mma_commit(&empty[s]);
                        continue;
                    }
                    const uint64_t dah = sw_desc(st), dal = sw_desc(st + a_bytes);
                    const uint64_t dbh = sw_desc(st + 2 * a_bytes);
                    const uint64_t dbl = sw_desc(st + 2 * a_bytes + b_bytes);
                    // products with Ah: the stage as it landed
#pragma unroll
                    for (int kk = 0; kk < kTcRowBytes / 32; kk++) {
                        // 32 bytes of k per MMA: 8 tf32 or 16 fp16
                        const uint64_t off = (uint64_t)(kk * 32) >> 4;
                        if (comb) {
                            mma_op<F16>(acc, dah + off, dbh + off, idesc2, (i | kk) != 0);
                        } else {
                            mma_op<F16>(acc, dah + off, dbh + off, idesc, (i | kk) != 0);
                            mma_op<F16>(acc, dah + off, dbl + off, idesc, 1);
                        }
                    }
                    // products with Al: after the split
                    if (SPLIT_A) {
                        if (!mbar_wait(&splitb[s], n & 1, err, 2)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                    }
#pragma unroll
                    for (int kk = 0; kk < kTcRowBytes / 32; kk++) {
                        const uint64_t off = (uint64_t)(kk * 32) >> 4;
                        mma_op<F16>(comb ? acc + BN : acc, dal + off, dbh + off, idesc, 1);
                    }
                    mma_commit(&empty[s]);
                }
                if (ok) mma_commit(&acc_full[buf]);
            }
            mma_commit(done);  // arrives when every MMA issued above has completed
        }
    } else if (warp < 2 + kTcSplitWarps) {
        if (SPLIT_A) {
            // ---- splitters: the lo slot of each stage
            const int tid = threadIdx.x - 64;
            uint32_t g = 0;
            bool ok = true;
            for (int u = blockIdx.x; ok && u < units; u += gridDim.x) {
                const int kb0 = (u / tiles / ntn) * kb_per_split;
                const int nkb = min(nkb_total, kb0 + kb_per_split) - kb0;
                for (int i = 0; i < nkb; i++, g++) {
                    const uint32_t s = g % kTcStages, n = g / kTcStages;
                    if (!mbar_wait(&full[s], n & 1, err, 4)) {
                        ok = false;
                        break;
                    }
                    const float4 *hi = (const float4 *)(smem + s * stage_bytes);
                    float4 *lo = (float4 *)(smem + s * stage_bytes + a_bytes);
                    for (int t = tid; t < (int)(a_bytes / 16); t += kTcSplitters) {
                        const float4 v = hi[t];
                        float4 l;
                        if (AMODE == 2) {
                            l.x = tf32_lo_biased(v.x);
                            l.y = tf32_lo_biased(v.y);
                            l.z = tf32_lo_biased(v.z);
                            l.w = tf32_lo_biased(v.w);
                        } else {
                            l.x = tf32_lo(v.x);
                            l.y = tf32_lo(v.y);
                            l.z = tf32_lo(v.z);
                            l.w = tf32_lo(v.w);
                        }
                        lo[t] = l;
                    }
                    // generic-proxy writes must be visible to the tensor core's reads
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    mbar_arrive(&splitb[s]);
                }
            }
        }
    } else {
        // ---- epilogue (the last 4 warps: TMEM lanes 32 (warp % 4) .. + 31 =
        // rows)
        const int ew = warp & 3;
        int j = 0;
        for (int u = blockIdx.x; u < units; u += gridDim.x, j++) {
            const int split = u / tiles / ntn;
            const int m0 = (u % tiles) * kTcBM, n0 = ((u / tiles) % ntn) * BN;
            const uint32_t buf = j % nbuf, q = j / nbuf;
            bool have = mbar_wait(&acc_full[buf], q & 1, err, 3);
            // tcgen05.ld is warp-collective: the whole warp reads or none of it
            if (!__all_sync(0xffffffffu, have)) break;
            tc_fence_after();
            const uint32_t acc = tmem + ((uint32_t)(ew * 32) << 16) + buf * acc_stride;
            const int m = m0 + ew * 32 + lane;
            const float rs = (rsc && m < M) ? rsc[m] : 1.0f;
            float *Ys = Y + (size_t)split * split_stride;
            for (int c0 = 0; c0 < BN; c0 += 32) {
                uint32_t r[32];
                tmem_ld32(acc + (uint32_t)c0, r);
                if (comb) {
                    uint32_t r2[32];
                    tmem_ld32(acc + (uint32_t)(BN + c0), r2);
#pragma unroll
                    for (int t = 0; t < 32; t++) r[t] = __float_as_uint(__uint_as_float(r[t]) + __uint_as_float(r2[t]));
                }
                if (m < M) {
#pragma unroll
                    for (int t = 0; t < 32; t++) {
                        const int n = n0 + c0 + t;
                        if (n < Nc) {
                            // powers of two: the scaling is exact
                            const float cn = csc ? csc[n] : 1.0f;
                            Ys[(size_t)n * ldy + m] = __uint_as_float(r[t]) * rs * cn;
                        }
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[buf]);
        }
    }
    __syncwarp();
    if (warp == 0) {
        // every MMA has completed before the accumulator memory is freed
        if (lane == 0) {
            const long long t0 = clock64();
            while (!mbar_try(done, 0) && clock64() - t0 < kTcSpin) {
            }
        }
        __syncwarp();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmem_cols)
                     : "memory");
}

// ------------------------------------------------ the Gauss-Jordan update
//
// C -= A B^T on 128 x 128 tiles of up to kTcGjMaxProblems column-major FP32
// matrices C in one launch (rank 128: A = the old column block, B = the
// row block, scaled fp16 pairs, 3xFP16 with the two Ah products in one
// MMA of N = 256); per problem: row tile gk left alone, column tile gk
// overwritten with -A B^T, tiles chosen by sel / la (unit_tile).  The units
// of the problems follow one another; one persistent CTA per SM walks them.
// Warp 0 lane 0 streams each unit's old values into a ring of kGjXSlots
// half tiles (TMA, 4 boxes of 32 rows x 64 columns each) and its two
// k-blocks of operands through one stage; warp 1 lane 0 issues the MMAs
// into one of two TMEM accumulators; warps 2 .. 9 (two per TMEM lane
// group, one per half of the columns) rewrite their 32 x 64 box of old
// values in shared memory and store it back by TMA.

struct TcGjProblem {
    CUtensorMap ah, al, bh, bl, c;  // A, B: rows x 128 k; c: the matrix in 32 x 64 boxes
    float *C;
    const float *rsc, *csc;  // power-of-two row scales of A and B
    int M, Nc, tiles, ntn;
    int gk, sel, la, units;
};

struct TcGjBatch {
    TcGjProblem p[kTcGjMaxProblems];
    int np, units;
};

// problem and tiles of unit u of the batch
__device__ __forceinline__ const TcGjProblem &gj_locate(const TcGjBatch &B, int u, int &tm, int &tn)
{
    int pi = 0;
    while (pi + 1 < B.np && u >= B.p[pi].units) u -= B.p[pi++].units;
    const TcGjProblem &P = B.p[pi];
    unit_tile(u, P.tiles, P.ntn, P.sel, P.la, P.gk, tm, tn);
    return P;
}

__global__ void __launch_bounds__(kTcThreads, 1) k_tc_gj(const __grid_constant__ TcGjBatch B, int *err)
{
    grid_dep_wait();  // launched as a programmatic dependent of the kernel before
    constexpr int BN = 128;
    constexpr uint32_t a_bytes = kTcBM * kTcRowBytes, b_bytes = BN * kTcRowBytes;
    constexpr uint32_t stage_bytes = 2 * a_bytes + 2 * b_bytes;
    constexpr uint32_t acc_stride = 2 * BN;  // Ah [Bh | Bl] in [0, 2 BN); Al Bh added to [BN, 2 BN)
    constexpr int nkb = 128 / kTcBK16;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *xbuf = smem + kGjStages * stage_bytes;
    uint64_t *full = (uint64_t *)(xbuf + kGjXSlots * kGjXHalfBytes);
    uint64_t *empty = full + kGjStages;
    uint64_t *acc_full = empty + kGjStages;  // [2]
    uint64_t *acc_empty = acc_full + 2;      // [2]
    uint64_t *done = acc_empty + 2;
    uint64_t *xfull = done + 1;            // [kGjXSlots]
    uint64_t *xempty = xfull + kGjXSlots;  // [kGjXSlots]
    uint32_t *tmem_slot = (uint32_t *)(xempty + kGjXSlots);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int units = B.units;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kGjStages; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 8);  // one lane of each epilogue warp
        }
        mbar_init(done, 1);
        for (int s = 0; s < kGjXSlots; s++) {
            mbar_init(&xfull[s], 1);
            mbar_init(&xempty[s], 4);  // the four warps on that half of the columns
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         su32(tmem_slot)),
                     "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    // Every role walks the same units u = blockIdx.x, + gridDim.x, ...; g
    // counts k-blocks (stage g % kGjStages), xh half-tile slot uses (slot
    // xh % kGjXSlots; unit j of this CTA takes uses 2 j and 2 j + 1).
    if (warp == 0) {
        if (lane == 0) {
            // ---- producer
            uint32_t g = 0, xh = 0;
            bool ok = true;
            for (int u = blockIdx.x; ok && u < units; u += gridDim.x) {
                int tm, tn;
                const TcGjProblem &P = gj_locate(B, u, tm, tn);
                const int m0 = tm * kTcBM, n0 = tn * BN;
                // the old values (none in row tile gk, which stays, nor in
                // column tile gk, which is overwritten)
                const bool old = tm != P.gk && tn != P.gk;
                for (int h = 0; h < 2; h++, xh++) {
                    const uint32_t s = xh % kGjXSlots, n = xh / kGjXSlots;
                    if (n > 0 && !mbar_wait(&xempty[s], (n - 1) & 1, err, 6)) {
                        ok = false;
                        break;
                    }
                    if (!old) {
                        mbar_arrive(&xfull[s]);
                        continue;
                    }
                    uint8_t *xb = xbuf + s * kGjXHalfBytes;
                    mbar_expect_tx(&xfull[s], kGjXHalfBytes);
                    for (int r = 0; r < 4; r++)
                        tma_load_2d(xb + r * kGjXBoxBytes, &P.c, &xfull[s], m0 + r * kGjXBoxRows, n0 + h * kGjXBoxCols);
                }
                if (!ok) break;
                // and those of the unit after it into L2
                if (u + (int)gridDim.x < units) {
                    int tm2, tn2;
                    const TcGjProblem &P2 = gj_locate(B, u + (int)gridDim.x, tm2, tn2);
                    if (tm2 != P2.gk && tn2 != P2.gk)
                        for (int b = 0; b < 8; b++)
                            tma_prefetch_2d(&P2.c, tm2 * kTcBM + (b & 3) * kGjXBoxRows, tn2 * BN + (b >> 2) * kGjXBoxCols);
                }
                for (int i = 0; i < nkb; i++, g++) {
                    const uint32_t s = g % kGjStages, n = g / kGjStages;
                    if (n > 0 && !mbar_wait(&empty[s], (n - 1) & 1, err, 1)) {
                        ok = false;
                        break;
                    }
                    uint8_t *st = smem + s * stage_bytes;
                    mbar_expect_tx(&full[s], stage_bytes);
                    const int kx = i * kTcBK16;
                    tma_load_2d(st, &P.ah, &full[s], kx, m0);
                    tma_load_2d(st + a_bytes, &P.al, &full[s], kx, m0);
                    tma_load_2d(st + 2 * a_bytes, &P.bh, &full[s], kx, n0);
                    tma_load_2d(st + 2 * a_bytes + b_bytes, &P.bl, &full[s], kx, n0);
                }
            }
            // drain: the last loads of every stage and slot have landed
            // before the CTA may exit (immediate in the normal path, bounded
            // otherwise)
            for (uint32_t h = g > (uint32_t)kGjStages ? g - kGjStages : 0; h < g; h++)
                mbar_drain(&full[h % kGjStages], (h / kGjStages) & 1);
            for (uint32_t h = xh > (uint32_t)kGjXSlots ? xh - kGjXSlots : 0; h < xh; h++)
                mbar_drain(&xfull[h % kGjXSlots], (h / kGjXSlots) & 1);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---- MMA issuer
            const uint32_t idesc = idesc_f16(BN, kTcBM), idesc2 = idesc_f16(2 * BN, kTcBM);
            uint32_t g = 0;
            bool ok = true;
            int j = 0;
            for (int u = blockIdx.x; ok && u < units; u += gridDim.x, j++) {
                const uint32_t buf = j & 1, q = j >> 1;
                if (q > 0 && !mbar_wait(&acc_empty[buf], (q - 1) & 1, err, 5)) break;
                tc_fence_after();
                const uint32_t acc = tmem + buf * acc_stride;
                for (int i = 0; i < nkb; i++, g++) {
                    const uint32_t s = g % kGjStages, n = g / kGjStages;
                    if (!mbar_wait(&full[s], n & 1, err, 2)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    uint8_t *st = smem + s * stage_bytes;
                    const uint64_t dah = sw_desc(st), dal = sw_desc(st + a_bytes);
                    const uint64_t dbh = sw_desc(st + 2 * a_bytes);
#pragma unroll
                    for (int kk = 0; kk < kTcRowBytes / 32; kk++) {
                        // 32 bytes of k per MMA (16 fp16): Ah against Bh and
                        // the adjacent Bl, then Al against Bh
                        const uint64_t off = (uint64_t)(kk * 32) >> 4;
                        mma_op<true>(acc, dah + off, dbh + off, idesc2, (i | kk) != 0);
                    }
#pragma unroll
                    for (int kk = 0; kk < kTcRowBytes / 32; kk++) {
                        const uint64_t off = (uint64_t)(kk * 32) >> 4;
                        mma_op<true>(acc + BN, dal + off, dbh + off, idesc, 1);
                    }
                    mma_commit(&empty[s]);
                }
                if (ok) mma_commit(&acc_full[buf]);
            }
            mma_commit(done);  // arrives when every MMA issued above has completed
        }
    } else {
        // ---- epilogue (warps 2 .. 9: TMEM lanes 32 (warp % 4) .. + 31 =
        // rows, the first four on columns 0 .. 63, the others on 64 .. 127):
        // C = old - the product (-the product in column tile gk), row tile
        // gk left alone.  The warp's 32 x 64 box of the unit's half-tile
        // slot is column-major (a column's 32 rows are 128 contiguous
        // bytes, lane = row); the TMA store drops rows >= M and columns >=
        // Nc.
        const int ew = warp & 3, hh = warp >= 6 ? 1 : 0;
        const int cbeg = hh * kGjXBoxCols;
        int j = 0;
        for (int u = blockIdx.x; u < units; u += gridDim.x, j++) {
            int tm, tn;
            const TcGjProblem &P = gj_locate(B, u, tm, tn);
            const int m0 = tm * kTcBM, n0 = tn * BN;
            const uint32_t buf = j & 1, q = j >> 1;
            const uint32_t xs = (2 * j + hh) % kGjXSlots, xn = (2 * j + hh) / kGjXSlots;
            // the row's scale and (lane t) those of columns t and t + 32 of
            // this half, read before the waits
            const int m = m0 + ew * 32 + lane;
            const float rs = (P.rsc && m < P.M) ? P.rsc[m] : 1.0f;
            float cl[2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int n = n0 + cbeg + 32 * h + lane;
                cl[h] = (P.csc && n < P.Nc) ? P.csc[n] : 1.0f;
            }
            bool have = mbar_wait(&acc_full[buf], q & 1, err, 3);
            have = have && mbar_wait(&xfull[xs], xn & 1, err, 7);
            // tcgen05.ld is warp-collective: the whole warp reads or none of it
            if (!__all_sync(0xffffffffu, have)) break;
            tc_fence_after();
            if (tm != P.gk) {
                float *xw = (float *)(xbuf + xs * kGjXHalfBytes + ew * kGjXBoxBytes) + lane;
                const uint32_t acc = tmem + ((uint32_t)(ew * 32) << 16) + buf * acc_stride;
                const bool keep = tn != P.gk;
#pragma unroll
                for (int c0 = 0; c0 < kGjXBoxCols; c0 += 32) {
                    uint32_t r[32], r2[32];
                    tmem_ld32(acc + (uint32_t)(cbeg + c0), r);
                    tmem_ld32(acc + (uint32_t)(BN + cbeg + c0), r2);
#pragma unroll
                    for (int t = 0; t < 32; t++) {
                        // powers of two: the scaling is exact
                        const float cn = __shfl_sync(0xffffffffu, cl[c0 / 32], t);
                        const float v = (__uint_as_float(r[t]) + __uint_as_float(r2[t])) * rs * cn;
                        float *x = xw + (c0 + t) * kGjXBoxRows;
                        *x = (keep ? *x : 0.0f) - v;
                    }
                }
                // the box's generic writes before the TMA engine reads it
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) {
                    tma_store_2d(&P.c, xw, m0 + ew * kGjXBoxRows, n0 + cbeg);
                    bulk_commit();
                    bulk_wait_read0();  // the slot may be refilled once the store has read it
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&acc_empty[buf]);
                mbar_arrive(&xempty[xs]);
            }
        }
        if (lane == 0) bulk_wait0();  // the stores are complete before the CTA exits
    }
    __syncwarp();
    if (warp == 0) {
        // every MMA has completed before the accumulator memory is freed
        if (lane == 0) mbar_drain(done, 0);
        __syncwarp();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
}

// ---------------------------------------------------------------- host

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    // looked up once (a function-local static is initialised exactly once,
    // whichever thread gets here first)
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return (PFN_cuTensorMapEncodeTiled_v12000)p;
        cudaGetLastError();
        return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
    }();
    return fn;
}

// 2-D tensor of FP32 (esize 4) or fp16 (esize 2) values: rows x k (k
// contiguous, row stride ld elements), boxes of one swizzle row of k x
// box_rows rows, kTcRowBytes-byte swizzle, zero fill outside.
static int make_map(CUtensorMap *map, const void *base, int esize, int rows, int k, size_t ld,
                    int box_rows)
{
    auto fn = encode_fn();
    if (!fn) {
        set_error("cuTensorMapEncodeTiled is not available");
        return kErrCuda;
    }
    if (((uintptr_t)base & 15) || ((ld * esize) & 15)) {
        set_error("TMA operand not 16-byte aligned");
        return kErrArg;
    }
    cuuint64_t dims[2] = {(cuuint64_t)k, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(ld * esize)};
    cuuint32_t box[2] = {(cuuint32_t)(kTcRowBytes / esize), (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, esize == 2 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                    (void *)base, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE,
                    kTcRowBytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return kErrCuda;
    }
    return kOk;
}

// Column-major FP32 matrix (rows x cols, entry (r, c) at c * ld + r) in
// unswizzled boxes of box_rows x box_cols (rows innermost); loads fill zeros
// outside, stores drop what falls outside.
static int make_box_map(CUtensorMap *map, const float *base, int rows, int cols, size_t ld, int box_rows,
                        int box_cols)
{
    auto fn = encode_fn();
    if (!fn) {
        set_error("cuTensorMapEncodeTiled is not available");
        return kErrCuda;
    }
    if (((uintptr_t)base & 15) || ((ld * 4) & 15)) {
        set_error("TMA matrix not 16-byte aligned (base and column stride)");
        return kErrArg;
    }
    cuuint64_t dims[2] = {(cuuint64_t)rows, (cuuint64_t)cols};
    cuuint64_t strides[1] = {(cuuint64_t)(ld * 4)};
    cuuint32_t box[2] = {(cuuint32_t)box_rows, (cuuint32_t)box_cols};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)base, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return kErrCuda;
    }
    return kOk;
}

int tc_make_map(CUtensorMap *map, const void *base, int esize, int rows, int k, size_t ld, int box_rows)
{
    return make_map(map, base, esize, rows, k, ld, box_rows);
}

// Split counts: at least one k-block per split, normalised so that every
// split has one (callers size their partial-tile buffers by this count).
static int splits_norm(int nkb, int splits)
{
    splits = std::max(1, std::min(splits, nkb));
    const int kps = (nkb + splits - 1) / splits;
    return (nkb + kps - 1) / kps;
}

// about eleven waves of one CTA per SM, at least four k-blocks per split
static int splits_for_bk(int M, int Kd, int bk)
{
    const int tiles = (M + kTcBM - 1) / kTcBM;
    const int nkb = (Kd + bk - 1) / bk;
    int s = std::max(1, (11 * 152) / std::max(1, tiles));
    s = std::max(1, std::min(s, nkb / 4));
    return splits_norm(nkb, s);
}

// Launch of the persistent kernel on encoded maps (bk: elements per k-block).
static int tc_launch(int amode, const CUtensorMap &ah, const CUtensorMap &al, const CUtensorMap &bh,
                     const CUtensorMap &bl, int M, int Nc, int Kd, int bk, float *Y, size_t ldy, int splits,
                     int *d_err, cudaStream_t st, const float *rsc, const float *csc)
{
    // one column tile of all Nc columns; above 256 columns (digits) a
    // multiple of 32 (two halves)
    int BN = (Nc + 15) / 16 * 16;
    if (BN > 256) BN = (Nc + 31) / 32 * 32;
    const int ntn = (Nc + BN - 1) / BN;
    // two accumulator buffers of 2 BN (COMB) or BN columns, each rounded up
    // to a power of two; one when two would pass the 512 TMEM columns
    const bool comb = amode != 4 && BN <= 128 && BN % 32 == 0;
    uint32_t acc_stride = 32;
    while (acc_stride < (uint32_t)(comb ? 2 * BN : BN)) acc_stride *= 2;
    const int tmem_cols = std::min(2 * (int)acc_stride, 512);
    const int nkb = (Kd + bk - 1) / bk;
    splits = splits_norm(nkb, splits);
    const int kps = (nkb + splits - 1) / splits;
    const size_t smem = 1024 + (size_t)kTcStages * (amode == 4 ? kTcBM + BN : 2 * kTcBM + 2 * BN) * kTcRowBytes + 256;
    // persistent: one CTA per SM walks the (row tile, split) units
    int nsm = 0;
    DSC_TRY(current_sm_count(&nsm));
    const int units = (M + kTcBM - 1) / kTcBM * ntn * splits;
    const dim3 grid(std::min(units, nsm));
    // the shared-memory limit of each instantiation is raised to the largest
    // request seen on the device (once per size, not per launch)
    auto launch = [&](auto kern, int slot) -> int {
        (void)slot;
        DSC_TRY(raise_smem_limit((const void *)kern, (int)smem));
        DSC_TRY(launch_dependent(kern, grid, dim3(kTcThreads), smem, st, ah, al, bh, bl, M, Nc, BN, ntn, nkb, kps,
                                 splits, Y, ldy, ldy * (size_t)Nc, tmem_cols, acc_stride, rsc, csc, d_err));
        return kOk;
    };
    switch (amode) {
    case 0: DSC_TRY(launch(k_tc_gemm3<0>, 0)); break;
    case 1: DSC_TRY(launch(k_tc_gemm3<1>, 1)); break;
    case 2: DSC_TRY(launch(k_tc_gemm3<2>, 2)); break;
    case 4: DSC_TRY(launch(k_tc_gemm3<4>, 5)); break;
    default: DSC_TRY(launch(k_tc_gemm3<3>, 3)); break;
    }
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

int tc_gemm_3xtf32(const float *Ah, const float *Al, size_t lda, const float *Bh, const float *Bl,
                   size_t ldb, int M, int Nc, int Kd, float *Y, size_t ldy, int splits, int *d_err,
                   cudaStream_t st, bool a_biased)
{
    if (Nc < 1 || Nc > kTcMaxNc || M < 1 || Kd < 1 || ldy < (size_t)M) {
        set_error("tc_gemm_3xtf32: unsupported shape M %d Nc %d Kd %d (Nc <= %d)", M, Nc, Kd, kTcMaxNc);
        return kErrArg;
    }
    const int BN = (Nc + 15) / 16 * 16;
    const bool split_a = Al == nullptr;  // plain FP32 A, split in shared memory
    CUtensorMap ah, al, bh, bl;
    DSC_TRY(make_map(&ah, Ah, 4, M, Kd, lda, kTcBM));
    if (split_a) al = ah;
    else DSC_TRY(make_map(&al, Al, 4, M, Kd, lda, kTcBM));
    DSC_TRY(make_map(&bh, Bh, 4, Nc, Kd, ldb, BN));
    DSC_TRY(make_map(&bl, Bl, 4, Nc, Kd, ldb, BN));
    const int amode = !split_a ? 0 : a_biased ? 2 : 1;
    return tc_launch(amode, ah, al, bh, bl, M, Nc, Kd, kTcBK, Y, ldy, splits, d_err, st, nullptr, nullptr);
}

int tc_gemm_3xf16(const __half *Ah, const __half *Al, size_t lda, const __half *Bh, const __half *Bl,
                  size_t ldb, int M, int Nc, int Kd, float *Y, size_t ldy, int splits, int *d_err,
                  cudaStream_t st, const float *rsc, const float *csc)
{
    if (Nc < 1 || Nc > kTcMaxNc || M < 1 || Kd < 1 || ldy < (size_t)M || !Al) {
        set_error("tc_gemm_3xf16: unsupported shape M %d Nc %d Kd %d (Nc <= %d)", M, Nc, Kd, kTcMaxNc);
        return kErrArg;
    }
    const int BN = (Nc + 15) / 16 * 16;
    CUtensorMap ah, al, bh, bl;
    DSC_TRY(make_map(&ah, Ah, 2, M, Kd, lda, kTcBM));
    DSC_TRY(make_map(&al, Al, 2, M, Kd, lda, kTcBM));
    DSC_TRY(make_map(&bh, Bh, 2, Nc, Kd, ldb, BN));
    DSC_TRY(make_map(&bl, Bl, 2, Nc, Kd, ldb, BN));
    return tc_launch(3, ah, al, bh, bl, M, Nc, Kd, kTcBK16, Y, ldy, splits, d_err, st, rsc, csc);
}

int tc_gemm_digits(const __half *A, size_t lda, const __half *B, size_t ldb, int M, int Nc, int Kd, float *Y,
                   size_t ldy, int *d_err, cudaStream_t st)
{
    if (Nc < 1 || Nc > kTcMaxDigitCols || M < 1 || Kd < 1 || ldy < (size_t)M) {
        set_error("tc_gemm_digits: unsupported shape M %d Nc %d Kd %d (Nc <= %d)", M, Nc, Kd, kTcMaxDigitCols);
        return kErrArg;
    }
    int BN = (Nc + 15) / 16 * 16;
    if (BN > 256) BN = (Nc + 31) / 32 * 32;
    CUtensorMap a, b;
    DSC_TRY(make_map(&a, A, 2, M, Kd, lda, kTcBM));
    DSC_TRY(make_map(&b, B, 2, Nc, Kd, ldb, BN > 256 ? BN / 2 : BN));
    return tc_launch(4, a, a, b, b, M, Nc, Kd, kTcBK16, Y, ldy, tc_digit_splits(Kd), d_err, st, nullptr, nullptr);
}

int tc_digit_splits(int Kd)
{
    const int nkb = (Kd + kTcBK16 - 1) / kTcBK16;
    return splits_norm(nkb, (nkb + kTcDigitKBlocks - 1) / kTcDigitKBlocks);
}

struct TcGjPlan::Maps {
    TcGjProblem pr;  // the maps, matrix and scales; the step's fields set per launch
};

TcGjPlan::~TcGjPlan() { delete maps; }

int tc_gj_plan(TcGjPlan &p, const __half *Ah, const __half *Al, size_t lda, const __half *Bh,
               const __half *Bl, size_t ldb, int M, int Nc, float *C, size_t ldc, int *d_err,
               const float *rsc, const float *csc)
{
    if (M < 1 || Nc < 1 || ldc < (size_t)M) {
        set_error("tc_gj_plan: unsupported shape M %d Nc %d", M, Nc);
        return kErrArg;
    }
    if (!p.maps) p.maps = new TcGjPlan::Maps();
    TcGjProblem &pr = p.maps->pr;
    DSC_TRY(make_map(&pr.ah, Ah, 2, M, 128, lda, kTcBM));
    DSC_TRY(make_map(&pr.al, Al, 2, M, 128, lda, kTcBM));
    DSC_TRY(make_map(&pr.bh, Bh, 2, Nc, 128, ldb, 128));
    DSC_TRY(make_map(&pr.bl, Bl, 2, Nc, 128, ldb, 128));
    DSC_TRY(make_box_map(&pr.c, C, M, Nc, ldc, kGjXBoxRows, kGjXBoxCols));
    pr.C = C;
    pr.rsc = rsc;
    pr.csc = csc;
    pr.M = M;
    pr.Nc = Nc;
    pr.tiles = (M + kTcBM - 1) / kTcBM;
    pr.ntn = (Nc + 127) / 128;
    p.M = M;
    p.Nc = Nc;
    p.C = C;
    p.ldc = ldc;
    p.err = d_err;
    p.rsc = rsc;
    p.csc = csc;
    return kOk;
}

int tc_gj_run_batch(const TcGjPlan *const *plans, int np, int k, cudaStream_t st, int sel, int la, int max_ctas)
{
    if (np < 1 || np > kTcGjMaxProblems || k < 0 || sel < 0 || sel > 2) {
        set_error("tc_gj_run: %d problems (at most %d), step %d, tile selection %d", np, kTcGjMaxProblems, k, sel);
        return kErrArg;
    }
    TcGjBatch B{};
    B.np = np;
    for (int q = 0; q < np; q++) {
        const TcGjPlan &p = *plans[q];
        if (!p.maps || p.err != plans[0]->err) {
            set_error("tc_gj_run: problem %d has no plan or another error word", q);
            return kErrArg;
        }
        TcGjProblem &pr = B.p[q];
        pr = p.maps->pr;
        if (sel && (la < 0 || la >= pr.tiles || la >= pr.ntn || la == k)) {
            set_error("tc_gj_run: look-ahead tile %d outside the update", la);
            return kErrArg;
        }
        pr.gk = k;
        pr.sel = sel;
        pr.la = la;
        pr.units = gj_sel_units(pr.tiles, pr.ntn, sel, la, k);
        B.units += pr.units;
    }
    if (B.units < 1) return kOk;
    int nsm = 0;
    DSC_TRY(current_sm_count(&nsm));
    const dim3 grid(std::min(B.units, max_ctas > 0 ? std::min(max_ctas, nsm) : nsm));
    const size_t smem = 1024 + (size_t)kGjStages * 4 * kTcBM * kTcRowBytes + (size_t)kGjXSlots * kGjXHalfBytes + 256;
    DSC_TRY(raise_smem_limit((const void *)k_tc_gj, (int)smem));
    DSC_TRY(launch_dependent(k_tc_gj, grid, dim3(kTcThreads), smem, st, B, plans[0]->err));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

int tc_gj_run(const TcGjPlan &p, int k, cudaStream_t st, int sel, int la, int max_ctas)
{
    const TcGjPlan *pl = &p;
    return tc_gj_run_batch(&pl, 1, k, st, sel, la, max_ctas);
}

int tc_gemm_splits_for(int M, int Kd) { return splits_for_bk(M, Kd, kTcBK); }

int tc_gemm_f16_splits_for(int M, int Kd) { return splits_for_bk(M, Kd, kTcBK16); }

int tc_gemm_f16_splits_norm(int Kd, int splits) { return splits_norm((Kd + kTcBK16 - 1) / kTcBK16, splits); }

// ---------------------------------------------------------- operand split
// tf32 pair of a value: hi = round-to-nearest tf32, lo = value - hi, also
// rounded to tf32 (the tensor core would truncate it).
__device__ __forceinline__ void tf32_split(double v, float &hi, float &lo)
{
    hi = tf32_rna((float)v);
    lo = tf32_rna((float)(v - (double)hi));
}

// Column-major FP64 K (entry (i, c) at c * ld + i) to row-major tf32 pairs
// (entry (i, c) at i * ldt + c): a 32 x 32 shared tile per block.
__global__ void k_split_transpose(const double *__restrict__ K, size_t ld, int N,
                                  float *__restrict__ Th, float *__restrict__ Tl, size_t ldt,
                                  int mode)
{
    __shared__ double t[32][33];
    const int i0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        int c = c0 + k, i = i0 + threadIdx.x;
        t[k][threadIdx.x] = (c < N && i < N) ? K[(size_t)c * ld + i] : 0.0;
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        int i = i0 + k, c = c0 + threadIdx.x;
        if (i < N && c < N) {
            const double a = t[threadIdx.x][k];
            if (mode == kTransposePair) {
                float h, l;
                tf32_split(a, h, l);
                Th[(size_t)i * ldt + c] = h;
                Tl[(size_t)i * ldt + c] = l;
                continue;
            }
            const float v = (float)a;
            Th[(size_t)i * ldt + c] = mode == kTransposePlain ? v : tf32_bias_encode(v);
            if (mode == kTransposeBiasedRem)  // the part of a below FP32, biased too
                Tl[(size_t)i * ldt + c] = tf32_bias_encode((float)(a - (double)v));
        }
    }
}

// ------------------------------------------------ fp16 operand preparation

// 2^k as FP32, exact, for -126 <= k <= 127.
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((127 + k) << 23); }

// Shift s with 2^s * max in [2^14, 2^15) from the biased exponent E of the
// largest magnitude (FP64: bias 1023, FP32: bias 127; E = 0: all zero, no
// shift), clamped so that 2^s and 2^(s + 24) stay normal FP32 values.
__device__ __forceinline__ int scale_shift(int E, int bias)
{
    return E == 0 ? 0 : max(-100, min(100, 14 - (E - bias)));
}

// rowE[i] = max over the row's entries of the biased FP64 exponent of
// column-major K (entry (i, c) at c * ld + i); rowE zero on entry.  Block
// (row block, column chunk); the exponent comes from the high word of each
// double (integer work only).
__global__ void k_row_exponent(const double *__restrict__ K, size_t ld, int N, int cols, int *rowE)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const int c0 = blockIdx.y * cols, c1 = min(N, c0 + cols);
    int e = 0;
#pragma unroll 8
    for (int c = c0; c < c1; c++) e = max(e, (__double2hiint(K[(size_t)c * ld + i]) >> 20) & 0x7FF);
    atomicMax(&rowE[i], e);
}

// The epilogue's row factors: rsK[i] = 2^-s_i for K's fp16 pair.
__global__ void k_row_scales(const int *__restrict__ rowE, int N, float *__restrict__ rsK)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    rsK[i] = pow2f(-scale_shift(rowE[i], 1023));
}

// ---------------------------------------------------------------- digits
// Fixed-point digits for exact products on the tensor cores.  A value a
// with |a| < 2^(E - 1022) (E: the biased FP64 exponent of the largest
// magnitude in its row or column) is rounded to the integer V = round(a *
// 2^(B - E + 1022)), |V| <= 2^B, and V is written in balanced digits of b
// bits, q_0 2^(b (n - 1)) + ... + q_(n-1), |q| <= 2^(b - 1) (bn = B + 1).
// The work is integer only: the 53-bit significand shifted right by the
// exponent difference, rounded half up in magnitude; the digits of |V|,
// negated for a < 0.  An fp16 holds the small integers exactly: the value
// 1536 + q has the bits 0x6600 + q (1536 <= 1536 + q < 2048, one binade of
// integer steps), and the subtraction of 1536 is exact.

// |V| for a's significand M (53 bits): V = M 2^(E - 1075 + B - (Erow -
// 1022)), a right shift by sh = Erow - E + off with off = 53 - B; 0 for
// zeros, subnormals and shifts of 54 or more
__device__ __forceinline__ unsigned long long digit_magnitude(double a, int Erow, int off)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(a);
    const int E = (int)((b >> 52) & 0x7FF);
    const int sh = Erow - E + off;
    if (E == 0 || sh >= 54) return 0;
    const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    return (m + (1ull << (sh - 1))) >> sh;
}

__device__ __forceinline__ __half digit_f16(int q)
{
    return __hsub(__ushort_as_half((unsigned short)(0x6600 + q)), __ushort_as_half((unsigned short)0x6600));
}

// The kKDigits = 8 base-64 digits of a K entry (row exponent Erow): B =
// 47, |q| <= 32.  Adding 32 to every 6-bit field of the signed V (the
// constant 0x820820820820) makes each field minus 32 a balanced digit, so
// the digits are plain bit fields of w = V + that constant (w >= 0; the top
// field, bits 42 and up, reaches 64 for V = 2^47).  The fp16 of q is 0x65E0
// + (q + 32) minus 1536, exact.
static_assert(kKDigits == 8 && kKDigitBits == 6, "k_digit_fields extracts 8 fields of 6 bits");
__device__ __forceinline__ __half2 digit_pair_f16(unsigned fa, unsigned fb)
{
    const __half2 h = __halves2half2(__ushort_as_half((unsigned short)(0x65E0u + fa)),
                                     __ushort_as_half((unsigned short)(0x65E0u + fb)));
    return __hsub2(h, __halves2half2(__ushort_as_half((unsigned short)0x6600u),
                                     __ushort_as_half((unsigned short)0x6600u)));
}

// f[d] = digit d + 32, most significant first
__device__ __forceinline__ void k_digit_fields(double a, int Erow, unsigned *f)
{
    const unsigned long long u = digit_magnitude(a, Erow, 53 - (kKDigits * kKDigitBits - 1));
    const long long V = __double_as_longlong(a) < 0 ? -(long long)u : (long long)u;
    const unsigned long long w = (unsigned long long)(V + 0x820820820820ll);
    const unsigned lo = (unsigned)w, hi = (unsigned)(w >> 32);
    f[7] = lo & 63u;
    f[6] = (lo >> 6) & 63u;
    f[5] = (lo >> 12) & 63u;
    f[4] = (lo >> 18) & 63u;
    f[3] = (lo >> 24) & 63u;
    f[2] = __funnelshift_r(lo, hi, 30) & 63u;
    f[1] = (hi >> 4) & 63u;
    f[0] = hi >> 10;
}

// Column-major FP64 K to row-major fp16 pairs (entry (i, c) at i * ldt + c)
// of 2^s_i fl32(K) (Th, Tl; hi = rn_fp16(x), lo = rn_fp16(x - hi)) and,
// with Dg not null, to the kKDigits digit matrices of K (digit d at Dg + d *
// dstride, same layout).  Each row's largest entry scales below 2^15, so
// the pair stays below fp16's largest finite value (65504).  Block: 32 rows
// x 64 columns through a shared tile; each thread writes two adjacent
// columns of a row (4-byte stores; ldt is even, and the column after N - 1
// is the row's padding, written with zeros).
__global__ void k_split_transpose_f16(const double *__restrict__ K, size_t ld, int N,
                                      const int *__restrict__ rowE, __half *__restrict__ Th,
                                      __half *__restrict__ Tl, __half *__restrict__ Dg, size_t dstride,
                                      size_t ldt)
{
    __shared__ double t[64][33];
    const int i0 = blockIdx.x * 32, c0 = blockIdx.y * 64;
    for (int k = threadIdx.y; k < 64; k += blockDim.y) {
        const int c = c0 + k, i = i0 + threadIdx.x;
        t[k][threadIdx.x] = (c < N && i < N) ? K[(size_t)c * ld + i] : 0.0;
    }
    __syncthreads();
    const int c = c0 + 2 * threadIdx.x;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int i = i0 + k;
        if (i >= N || c >= N) continue;
        const double a0 = t[2 * threadIdx.x][k], a1 = t[2 * threadIdx.x + 1][k];
        const int Er = rowE[i];
        const float sc = pow2f(scale_shift(Er, 1023));
        const float x0 = (float)a0 * sc, x1 = (float)a1 * sc;
        const __half2 h = __floats2half2_rn(x0, x1);
        const size_t o = (size_t)i * ldt + c;
        *(__half2 *)(Th + o) = h;
        *(__half2 *)(Tl + o) = __floats2half2_rn(x0 - __low2float(h), x1 - __high2float(h));
        if (Dg) {
            unsigned f0[kKDigits], f1[kKDigits];
            k_digit_fields(a0, Er, f0);
            k_digit_fields(a1, Er, f1);
#pragma unroll
            for (int d = 0; d < kKDigits; d++) *(__half2 *)(Dg + d * dstride + o) = digit_pair_f16(f0[d], f1[d]);
        }
    }
}

template <typename T>
__device__ __forceinline__ float to_f32(T v) { return (float)v; }

// Columns of x (column n: N entries at n * ldx) to fp16 pairs of
// 2^t_n x (rows of h / l: n * ldh), t_n from the column's largest FP32
// exponent; csc[n] = 2^-t_n.  One block per column.
template <typename T>
__global__ void __launch_bounds__(256) k_split_cols_f16(const T *__restrict__ x, size_t ldx, int N,
                                                        __half *__restrict__ h, __half *__restrict__ l,
                                                        size_t ldh, float *__restrict__ csc)
{
    __shared__ int emax;
    if (threadIdx.x == 0) emax = 0;
    __syncthreads();
    const T *col = x + (size_t)blockIdx.x * ldx;
    int e = 0;
    for (int i = threadIdx.x; i < N; i += blockDim.x)
        e = max(e, (__float_as_int(to_f32(col[i])) >> 23) & 0xFF);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&emax, e);
    __syncthreads();
    const int sh = scale_shift(emax, 127);
    const float f = pow2f(sh);
    __half *hc = h + (size_t)blockIdx.x * ldh, *lc = l + (size_t)blockIdx.x * ldh;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const float v = to_f32(col[i]) * f;
        const __half a = __float2half_rn(v);
        hc[i] = a;
        lc[i] = __float2half_rn(v - __half2float(a));
    }
    if (threadIdx.x == 0) csc[blockIdx.x] = pow2f(-sh);
}

int k16_row_scales(const double *K, size_t ld, int N, int *rowE, float *rsK, cudaStream_t st)
{
    DSC_CUDA(cudaMemsetAsync(rowE, 0, (size_t)N * sizeof(int), st));
    const int chunks = 64, cols = (N + chunks - 1) / chunks;
    DSC_LAUNCH(k_row_exponent<<<dim3((N + 255) / 256, (N + cols - 1) / cols), 256, 0, st>>>(K, ld, N, cols, rowE));
    DSC_LAUNCH(k_row_scales<<<(N + 255) / 256, 256, 0, st>>>(rowE, N, rsK));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

int split_transpose_K16(const double *K, size_t ld, int N, const int *rowE, __half *Th, __half *Tl,
                        __half *Dg, size_t dstride, size_t ldt, cudaStream_t st)
{
    if (ldt % 2 || ldt < (size_t)N + (N & 1) || (Dg && dstride % 2)) {
        set_error("split_transpose_K16: strides must be even and the row stride cover N rounded up to even");
        return kErrArg;
    }
    dim3 g((N + 31) / 32, (N + 63) / 64), b(32, 8);
    DSC_LAUNCH(k_split_transpose_f16<<<g, b, 0, st>>>(K, ld, N, rowE, Th, Tl, Dg, dstride, ldt));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

// Columns of X (column c: N entries at c * ldx) to kXDigits digits of
// kXDigitBits bits each (B = 23, |q| <= 128), written as fp16 rows j * ncol
// + c of Xd (stride ldd), colE[c] = the column's largest biased exponent,
// and the remainder X - (the digits' value) (FP64, exact) at Xr.  One block
// per column.
__global__ void __launch_bounds__(256) k_x_digits(const double *__restrict__ X, size_t ldx, int N, int ncol,
                                                  __half *__restrict__ Xd, size_t ldd, double *__restrict__ Xr,
                                                  size_t ldr, int *__restrict__ colE)
{
    __shared__ int emax;
    if (threadIdx.x == 0) emax = 0;
    __syncthreads();
    const int c = blockIdx.x;
    const double *col = X + (size_t)c * ldx;
    int e = 0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) e = max(e, (__double2hiint(col[i]) >> 20) & 0x7FF);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&emax, e);
    __syncthreads();
    const int Ec = emax;
    constexpr int B = kXDigits * kXDigitBits - 1;
    const unsigned half = 1u << (kXDigitBits - 1), mask = (1u << kXDigitBits) - 1;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const double a = col[i];
        // V = round(a 2^(B - Ec + 1022)): shift Ec - E + 1075 - 1022 - B
        const unsigned long long u0 = digit_magnitude(a, Ec, 53 - B);
        const bool neg = __double_as_longlong(a) < 0;
        unsigned long long u = u0;
#pragma unroll
        for (int d = kXDigits - 1; d > 0; d--) {
            const int t = (int)((unsigned)(u + half) & mask) - (int)half;
            u = (u + half) >> kXDigitBits;
            Xd[((size_t)d * ncol + c) * ldd + i] = digit_f16(neg ? -t : t);
        }
        Xd[(size_t)c * ldd + i] = digit_f16(neg ? -(int)u : (int)u);
        const double v = ldexp(neg ? -(double)u0 : (double)u0, Ec - 1022 - B);
        Xr[(size_t)c * ldr + i] = a - v;
    }
    if (threadIdx.x == 0) colE[c] = Ec;
}

int x_digits(const double *X, size_t ldx, int N, int ncol, __half *Xd, size_t ldd, double *Xr, size_t ldr,
             int *colE, cudaStream_t st)
{
    DSC_LAUNCH(k_x_digits<<<ncol, 256, 0, st>>>(X, ldx, N, ncol, Xd, ldd, Xr, ldr, colE));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

// Y[c * ldy + m] (+)= 2^(kKDigitBits (kKDigits - 1 - i)) * sum over x digits
// j < nj of 2^(kXDigitBits (kXDigits - 1 - j)) * (the S partial tiles of the
// product of K digit i with x digit j; column j * ncol + c of the tiles).
// The tiles hold integers below 2^24: they are summed as integers (exact),
// then added in FP64.  Four rows per thread (ldp a multiple of 4: float4
// loads, all S nj of them issued before the sums).
__global__ void k_digit_accumulate(const float *__restrict__ P, int S, size_t ldp, int ncol, int nj, int i,
                                   int N, double *__restrict__ Y, size_t ldy, int first)
{
    grid_dep_wait();  // a programmatic dependent of the digit product
    const int m0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int c = blockIdx.y;
    if (m0 >= N) return;
    const size_t split_stride = ldp * (size_t)(nj * ncol);
    long long t[4] = {0, 0, 0, 0};
    for (int j = 0; j < nj; j++) {
        int sum[4] = {0, 0, 0, 0};
        const float *pj = P + (size_t)(j * ncol + c) * ldp + m0;
#pragma unroll 4
        for (int k = 0; k < S; k++) {
            const float4 v = __ldg((const float4 *)(pj + k * split_stride));
            sum[0] += __float2int_rn(v.x);
            sum[1] += __float2int_rn(v.y);
            sum[2] += __float2int_rn(v.z);
            sum[3] += __float2int_rn(v.w);
        }
        const long long w = 1ll << (kXDigitBits * (kXDigits - 1 - j));
#pragma unroll
        for (int r = 0; r < 4; r++) t[r] += (long long)sum[r] * w;
    }
    double *y = Y + (size_t)c * ldy + m0;
#pragma unroll
    for (int r = 0; r < 4; r++) {
        if (m0 + r >= N) break;
        const double v = ldexp((double)t[r], kKDigitBits * (kKDigits - 1 - i));
        y[r] = first ? v : y[r] + v;
    }
}

int digit_accumulate(const float *P, int S, size_t ldp, int ncol, int nj, int i, int N, double *Y, size_t ldy,
                     bool first, cudaStream_t st)
{
    if (ldp % 4 || ((uintptr_t)P & 15)) {
        set_error("digit_accumulate: the partial tiles' stride must be a multiple of 4 floats, 16-byte aligned");
        return kErrArg;
    }
    dim3 g((N + 1023) / 1024, ncol);
    DSC_TRY(launch_dependent(k_digit_accumulate, g, dim3(256), 0, st, P, S, ldp, ncol, nj, i, N, Y, ldy,
                             first ? 1 : 0));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

// Y[c * ldy + m] *= the units of K's row m and x's column c:
// 2^(rowE[m] - 1022 - 47) * 2^(colE[c] - 1022 - 23)
__global__ void k_digit_finish(const int *__restrict__ rowE, const int *__restrict__ colE, int N,
                               double *__restrict__ Y, size_t ldy)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (m >= N) return;
    double *y = Y + (size_t)c * ldy + m;
    *y = ldexp(*y, rowE[m] + colE[c] - 2044 - (kKDigits * kKDigitBits - 1) - (kXDigits * kXDigitBits - 1));
}

int digit_finish(const int *rowE, const int *colE, int N, int ncol, double *Y, size_t ldy, cudaStream_t st)
{
    dim3 g((N + 255) / 256, ncol);
    DSC_LAUNCH(k_digit_finish<<<g, 256, 0, st>>>(rowE, colE, N, Y, ldy));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

int split_cols_f16(const double *x, size_t ldx, int N, int ncol, __half *h, __half *l, size_t ldh,
                   float *csc, cudaStream_t st)
{
    DSC_LAUNCH(k_split_cols_f16<double><<<ncol, 256, 0, st>>>(x, ldx, N, h, l, ldh, csc));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

int split_cols_f16(const float *x, size_t ldx, int N, int ncol, __half *h, __half *l, size_t ldh,
                   float *csc, cudaStream_t st)
{
    DSC_LAUNCH(k_split_cols_f16<float><<<ncol, 256, 0, st>>>(x, ldx, N, h, l, ldh, csc));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

// FP64 vectors (any layout) to tf32 pairs, elementwise.
__global__ void k_split_vec(const double *__restrict__ x, float *__restrict__ h,
                            float *__restrict__ l, size_t n)
{
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n;
         t += (size_t)gridDim.x * blockDim.x) {
        float a, b;
        tf32_split(x[t], a, b);
        h[t] = a;
        l[t] = b;
    }
}

int split_transpose_K(const double *K, size_t ld, int N, float *Th, float *Tl, size_t ldt,
                      cudaStream_t st, int mode)
{
    dim3 g((N + 31) / 32, (N + 31) / 32), b(32, 8);
    DSC_LAUNCH(k_split_transpose<<<g, b, 0, st>>>(K, ld, N, Th, Tl, ldt, mode));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

int split_vec(const double *x, float *h, float *l, size_t n, cudaStream_t st)
{
    DSC_LAUNCH(k_split_vec<<<4 * 152, 256, 0, st>>>(x, h, l, n));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

__global__ void k_to_f32_plain(const double *__restrict__ x, float *__restrict__ y, size_t n,
                               bool biased)
{
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n;
         t += (size_t)gridDim.x * blockDim.x)
        y[t] = biased ? tf32_bias_encode((float)x[t]) : (float)x[t];
}

// Y (M x Nc, row-major FP64) = sum over splits of the partial tiles.
__global__ void k_sum_splits(const float *__restrict__ P, int S, size_t split_stride, size_t ldy,
                             int M, int Nc, double *__restrict__ Y)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = blockIdx.y;
    if (m >= M) return;
    double s = 0.0;
    for (int k = 0; k < S; k++) s += (double)P[(size_t)k * split_stride + (size_t)n * ldy + m];
    Y[(size_t)m * Nc + n] = s;
}

// Rows of a row-major FP64 matrix (rows x k, row stride ld) to tf32 pairs
// with row stride ldh; only the first k entries of each row are read and
// written.
__global__ void k_split_rows(const double *__restrict__ x, size_t ld, int rows, int k,
                             float *__restrict__ h, float *__restrict__ l, size_t ldh)
{
    const size_t n = (size_t)rows * k;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n;
         t += (size_t)gridDim.x * blockDim.x) {
        const size_t r = t / k, c = t % k;
        float a, b;
        tf32_split(x[r * ld + c], a, b);
        h[r * ldh + c] = a;
        l[r * ldh + c] = b;
    }
}

int split_rows(const double *x, size_t ld, int rows, int k, float *h, float *l, size_t ldh,
               cudaStream_t st)
{
    DSC_LAUNCH(k_split_rows<<<4 * 152, 256, 0, st>>>(x, ld, rows, k, h, l, ldh));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

// Y[m * ldy + n] (FP64) = sum over the S partial tiles, in split order.
__global__ void k_sum_splits_ld(const float *__restrict__ P, int S, size_t split_stride,
                                size_t ldp, int M, int Nc, double *__restrict__ Y, size_t ldy)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = blockIdx.y;
    if (m >= M) return;
    double s = 0.0;
    for (int k = 0; k < S; k++) s += (double)P[(size_t)k * split_stride + (size_t)n * ldp + m];
    Y[(size_t)m * ldy + n] = s;
}

int sum_splits(const float *P, int S, size_t split_stride, size_t ldp, int M, int Nc, double *Y,
               size_t ldy, cudaStream_t st)
{
    dim3 g((M + 255) / 256, Nc);
    DSC_LAUNCH(k_sum_splits_ld<<<g, 256, 0, st>>>(P, S, split_stride, ldp, M, Nc, Y, ldy));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

int tc_gemm_splits_used(int Kd, int splits) { return splits_norm((Kd + kTcBK - 1) / kTcBK, splits); }

// FP32 array to tf32 pairs (hi = rna(x), lo = rna(x - hi)), elementwise.
__global__ void k_f32_to_tf32_pair(const float *__restrict__ x, float *__restrict__ h,
                                   float *__restrict__ l, size_t n)
{
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n;
         t += (size_t)gridDim.x * blockDim.x) {
        const float a = x[t], hi = tf32_rna(a);
        h[t] = hi;
        l[t] = tf32_rna(a - hi);
    }
}

int f32_to_tf32_pair(const float *x, float *h, float *l, size_t n, cudaStream_t st)
{
    DSC_LAUNCH(k_f32_to_tf32_pair<<<4 * 152, 256, 0, st>>>(x, h, l, n));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

// Y[n * ldy + m] (FP64, column n) += the S partial tiles, in split order,
// summed in double-FP32 (about 2^-48 of the largest partial; the FP64 pipe
// only for the final addition).
__global__ void k_add_splits(const float *__restrict__ P, int S, size_t split_stride, size_t ldp,
                             int M, double *__restrict__ Y, size_t ldy)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = blockIdx.y;
    if (m >= M) return;
    float2 s = make_float2(0.0f, 0.0f);
    for (int k = 0; k < S; k++) s = df_add(s, make_float2(P[(size_t)k * split_stride + (size_t)n * ldp + m], 0.0f));
    Y[(size_t)n * ldy + m] += df_to(s);
}

int add_splits(const float *P, int S, size_t split_stride, size_t ldp, int M, int Nc, double *Y,
               size_t ldy, cudaStream_t st)
{
    dim3 g((M + 255) / 256, Nc);
    DSC_LAUNCH(k_add_splits<<<g, 256, 0, st>>>(P, S, split_stride, ldp, M, Y, ldy));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

}  // namespace dsc

using namespace dsc;

namespace dsc {
__global__ void k_f64_to_f16(const double *__restrict__ x, __half *__restrict__ y, size_t n)
{
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        y[t] = __float2half_rn((float)x[t]);  // exact for integers below 2048 in magnitude
}
}  // namespace dsc

// Host-array entry point of the tensor-core product (row-major FP64 in and
// out): Y (M x Nc) = A (M x Kd) * B^T (B: Nc x Kd) with 3xTF32 products
// (a_in_smem 0: A as a tf32 pair, 1: plain FP32 A split in shared memory,
// 2: the same in the biased encoding), 3xFP16 products on per-row scaled
// fp16 pairs (a_in_smem 3), or the digit product of A and B rounded to
// fp16 (a_in_smem 4: exact for integer entries |A| <= 32, |B| <= 128;
// Nc <= 384; `splits` ignored).
extern "C" int dsc_tc_gemm(int M, int Nc, int Kd, const double *A, const double *B, double *Y,
                           int splits, int a_in_smem)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        set_error("no CUDA device available");
        return kErrCuda;
    }
    if (M < 1 || Kd < 1 || Nc < 1 || Nc > (a_in_smem == 4 ? kTcMaxDigitCols : kTcMaxNc)) {
        set_error("dsc_tc_gemm: unsupported shape (1 <= Nc <= %d)", a_in_smem == 4 ? kTcMaxDigitCols : kTcMaxNc);
        return kErrArg;
    }
    if (a_in_smem < 0 || a_in_smem > 4) {
        set_error("dsc_tc_gemm: unknown operand mode %d (0 .. 4)", a_in_smem);
        return kErrArg;
    }
    cudaStream_t st = 0;
    const size_t lda = ((size_t)Kd + 31) / 32 * 32;
    DevBuf<double> dA, dB, dY;
    DevBuf<float> Ah, Al, Bh, Bl, P;
    DevBuf<int> err;
    DSC_TRY(dA.alloc((size_t)M * lda));
    DSC_TRY(dB.alloc((size_t)Nc * lda));
    DSC_CUDA(cudaMemset(dA.p, 0, (size_t)M * lda * sizeof(double)));
    DSC_CUDA(cudaMemset(dB.p, 0, (size_t)Nc * lda * sizeof(double)));
    DSC_CUDA(cudaMemcpy2D(dA.p, lda * sizeof(double), A, Kd * sizeof(double), Kd * sizeof(double), M,
                          cudaMemcpyHostToDevice));
    DSC_CUDA(cudaMemcpy2D(dB.p, lda * sizeof(double), B, Kd * sizeof(double), Kd * sizeof(double), Nc,
                          cudaMemcpyHostToDevice));
    if (a_in_smem == 4) {
        DevBuf<__half> a16, b16;
        DSC_TRY(a16.alloc((size_t)M * lda));
        DSC_TRY(b16.alloc((size_t)Nc * lda));
        DSC_LAUNCH(k_f64_to_f16<<<4 * 152, 256, 0, st>>>(dA.p, a16.p, (size_t)M * lda));
        DSC_LAUNCH(k_f64_to_f16<<<4 * 152, 256, 0, st>>>(dB.p, b16.p, (size_t)Nc * lda));
        const int S = tc_digit_splits(Kd);
        DSC_TRY(P.alloc((size_t)S * Nc * M));
        DSC_TRY(err.alloc(1));
        DSC_CUDA(cudaMemset(err.p, 0, sizeof(int)));
        DSC_TRY(tc_gemm_digits(a16.p, lda, b16.p, lda, M, Nc, Kd, P.p, (size_t)M, err.p, st));
        DSC_TRY(dY.alloc((size_t)M * Nc));
        dim3 g((M + 255) / 256, Nc);
        DSC_LAUNCH(k_sum_splits<<<g, 256, 0, st>>>(P.p, S, (size_t)M * Nc, (size_t)M, M, Nc, dY.p));
        DSC_CUDA(cudaGetLastError());
        int herr = 0;
        DSC_CUDA(cudaMemcpy(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (herr) {
            set_error("tensor-core GEMM: a pipeline wait gave up (code %d)", herr);
            return kErrCuda;
        }
        DSC_CUDA(cudaMemcpy(Y, dY.p, (size_t)M * Nc * sizeof(double), cudaMemcpyDeviceToHost));
        return kOk;
    }
    if (a_in_smem == 3) {
        // 3xFP16: rows of A and of B to scaled fp16 pairs (row factors of A
        // and of B as the epilogue's row and column factors)
        DevBuf<__half> h16[4];
        DevBuf<float> ra, cb;
        for (auto &b16 : h16) DSC_TRY(b16.alloc((size_t)std::max(M, Nc) * lda));
        DSC_TRY(ra.alloc(M));
        DSC_TRY(cb.alloc(Nc));
        DSC_TRY(split_cols_f16(dA.p, lda, Kd, M, h16[0].p, h16[1].p, lda, ra.p, st));
        DSC_TRY(split_cols_f16(dB.p, lda, Kd, Nc, h16[2].p, h16[3].p, lda, cb.p, st));
        if (splits <= 0) splits = tc_gemm_f16_splits_for(M, Kd);
        const int S = splits_norm((Kd + kTcBK16 - 1) / kTcBK16, splits);
        DSC_TRY(P.alloc((size_t)S * Nc * M));
        DSC_TRY(err.alloc(1));
        DSC_CUDA(cudaMemset(err.p, 0, sizeof(int)));
        DSC_TRY(tc_gemm_3xf16(h16[0].p, h16[1].p, lda, h16[2].p, h16[3].p, lda, M, Nc, Kd, P.p, (size_t)M, S,
                              err.p, st, ra.p, cb.p));
        DSC_TRY(dY.alloc((size_t)M * Nc));
        dim3 g((M + 255) / 256, Nc);
        DSC_LAUNCH(k_sum_splits<<<g, 256, 0, st>>>(P.p, S, (size_t)M * Nc, (size_t)M, M, Nc, dY.p));
        DSC_CUDA(cudaGetLastError());
        int herr = 0;
        DSC_CUDA(cudaMemcpy(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (herr) {
            set_error("tensor-core GEMM: a pipeline wait gave up (code %d)", herr);
            return kErrCuda;
        }
        DSC_CUDA(cudaMemcpy(Y, dY.p, (size_t)M * Nc * sizeof(double), cudaMemcpyDeviceToHost));
        return kOk;
    }
    DSC_TRY(Ah.alloc((size_t)M * lda));
    DSC_TRY(Al.alloc((size_t)M * lda));
    DSC_TRY(Bh.alloc((size_t)Nc * lda));
    DSC_TRY(Bl.alloc((size_t)Nc * lda));
    if (a_in_smem)
        DSC_LAUNCH(k_to_f32_plain<<<4 * 152, 256, 0, st>>>(dA.p, Ah.p, (size_t)M * lda, a_in_smem == 2));
    else DSC_TRY(split_vec(dA.p, Ah.p, Al.p, (size_t)M * lda, st));
    DSC_TRY(split_vec(dB.p, Bh.p, Bl.p, (size_t)Nc * lda, st));
    if (splits <= 0) splits = tc_gemm_splits_for(M, Kd);
    const int nkb = (Kd + kTcBK - 1) / kTcBK;
    const int S = std::min(splits, nkb);
    DSC_TRY(P.alloc((size_t)S * Nc * M));
    DSC_TRY(err.alloc(1));
    DSC_CUDA(cudaMemset(err.p, 0, sizeof(int)));
    DSC_CUDA(cudaMemset(P.p, 0, (size_t)S * Nc * M * sizeof(float)));
    DSC_TRY(tc_gemm_3xtf32(Ah.p, a_in_smem ? nullptr : Al.p, lda, Bh.p, Bl.p, lda, M, Nc, Kd, P.p,
                           (size_t)M, S, err.p, st, a_in_smem == 2));
    DSC_TRY(dY.alloc((size_t)M * Nc));
    dim3 g((M + 255) / 256, Nc);
    DSC_LAUNCH(k_sum_splits<<<g, 256, 0, st>>>(P.p, S, (size_t)M * Nc, (size_t)M, M, Nc, dY.p));
    DSC_CUDA(cudaGetLastError());
    int herr = 0;
    DSC_CUDA(cudaMemcpy(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) {
        set_error("tensor-core GEMM: a pipeline wait gave up (code %d)", herr);
        return kErrCuda;
    }
    DSC_CUDA(cudaMemcpy(Y, dY.p, (size_t)M * Nc * sizeof(double), cudaMemcpyDeviceToHost));
    return kOk;
}
