// dsc_field_tc.cu -- far-field part of the batched field on the tensor cores.
//
// For points p (the force points) and quadrature points q (element e, rule
// point k: q = 8 e + k, the eighth slot of each element empty, so that one
// 16-byte chunk of a tile row is one element) the far field is
// E(p, f) = sum_q G(p, q) c(q, f),
// G = (x_p - y_q) / |x_p - y_q|^3 (3 components), c the charge weights of
// system f.  Per CTA a tile of 128 points and a range of q:
//   * warps 2-9 generate G for 128 points x 64 q (one k-block) in FP32 from
//     centroid-relative coordinates (as the FP32 pass does), scale it by a
//     power of two that keeps every far value below 2^15 and write it as
//     fp16 pairs (hi = rn16(x), lo = rn16(x - hi)), three components, into
//     shared memory in the 128-byte swizzled K-major layout the MMA reads;
//     near pairs (the point within 4 quadrature radii of the element's
//     centroid, which includes the singular elements) and padding get 0 --
//     the FP32 pass takes them;
//   * warp 0 streams the charges' fp16 pairs (64 systems x 64 q per
//     k-block, scaled per system) with TMA into one buffer (the products of
//     a k-block finish long before the next one is generated), and each
//     k-block's geometry (8 centroids, 64 point offsets: 1280 contiguous
//     bytes) with bulk copies into two buffers, one k-block ahead;
//   * warp 1 issues tcgen05.mma kind::f16, hi*hi + hi*lo + lo*hi per
//     component, into one of two TMEM buffers (3 x 64 columns);
//   * warps 2-9, after generating the next k-block, read the finished
//     buffer back and add it into FP32 registers (round to nearest): the
//     tensor core's truncating FP32 accumulation never spans more than one
//     k-block of 64 terms.
// Two stages of 96 KB for G; every mbarrier wait is bounded (codes 21-26).
#include <cuda.h>
#include <cuda_fp16.h>

#include <algorithm>

#include "dsc_async.cuh"
#include "dsc_common.cuh"
#include "dsc_field_tc.h"
#include "dsc_internal.h"
#include "dsc_tc.cuh"
#include "dsc_tcgemm.h"

namespace dsc {

constexpr int kFtM = 128;                     // points per tile (TMEM lanes)
constexpr int kFtK = kTcRowBytes / 2;         // quadrature points per k-block (64 fp16)
constexpr int kFtN = 64;                      // systems per product
constexpr int kFtGen = 8;                     // generator / reader warps
constexpr int kFtThreads = 32 * (2 + kFtGen);
constexpr uint32_t kFtATile = kFtM * kTcRowBytes;   // one (component, half) of G: 16 KB
constexpr uint32_t kFtBTile = kFtN * kTcRowBytes;   // one half of the charges: 8 KB
constexpr uint32_t kFtStage = 6 * kFtATile;   // the generated G of one k-block
constexpr int kFtStages = 2;
constexpr uint32_t kFtGeo = 8 * 32 + kFtK * 16;  // one k-block's centroids and point offsets
constexpr uint32_t kFtAcc = 256;              // TMEM columns per accumulator buffer (192 used)
constexpr size_t kFtSmem = 1024 + (size_t)kFtStages * kFtStage + 2 * kFtBTile + kFtStages * kFtGeo + 256;

struct FieldTcArgs {
    const float *phl;    // P x 6: point hi (3), lo (3)
    const float *ecent;  // E x 8: centroid hi (3), lo (3), squared near radius, 0
    const float4 *q8;    // 8E: quadrature points relative to their centroid (x, y, z, 0), slot 7 unused
    const float *gsc;    // [0]: the power of two applied to G; [1]: its inverse
    const float *csc;    // per system: the inverse of the charges' factor
    float *part;         // [split][f][p][3]
    int P, E, F;
    int nkb, kb_per_split, nsplit, tiles;
    int *err;
};

__device__ __forceinline__ uint32_t pack_half2(__half a, __half b)
{
    return (uint32_t)__half_as_ushort(a) | ((uint32_t)__half_as_ushort(b) << 16);
}

__global__ void __launch_bounds__(kFtThreads, 1)
    k_field_far_tc(const __grid_constant__ CUtensorMap tmBh, const __grid_constant__ CUtensorMap tmBl,
                   FieldTcArgs a)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *btile = smem + kFtStages * kFtStage;        // charges (hi, lo), one buffer
    uint8_t *geo = btile + 2 * kFtBTile;                 // kFtStages x kFtGeo
    uint64_t *a_full = (uint64_t *)(geo + kFtStages * kFtGeo);
    uint64_t *geo_full = a_full + kFtStages;
    uint64_t *st_free = geo_full + kFtStages;
    uint64_t *b_full = st_free + kFtStages;              // [1]
    uint64_t *b_free = b_full + 1;                       // [1]
    uint64_t *acc_full = b_free + 1;
    uint64_t *acc_empty = acc_full + 2;
    uint64_t *done = acc_empty + 2;
    uint32_t *tmem_slot = (uint32_t *)(done + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int units = a.tiles * a.nsplit;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kFtStages; s++) {
            mbar_init(&a_full[s], 32 * kFtGen);
            mbar_init(&geo_full[s], 1);
            mbar_init(&st_free[s], 1);
        }
        mbar_init(b_full, 1);
        mbar_init(b_free, 1);
        for (int b = 0; b < 2; b++) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], kFtGen);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tmem_slot)),
                     "r"(2 * kFtAcc)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    // every role walks units u = blockIdx.x, + gridDim.x, ... (tile u % tiles,
    // split u / tiles) and their k-blocks; g counts k-blocks over the units
    if (warp == 0) {
        if (lane == 0) {
            // ---- geometry (bulk copies) and charges (TMA)
            uint32_t g = 0;
            bool ok = true;
            for (int u = blockIdx.x; ok && u < units; u += gridDim.x) {
                const int kb0 = (u / a.tiles) * a.kb_per_split, kb1 = min(a.nkb, kb0 + a.kb_per_split);
                for (int kb = kb0; kb < kb1; kb++, g++) {
                    const uint32_t s = g % kFtStages, n = g / kFtStages;
                    if (n > 0 && !mbar_wait(&st_free[s], (n - 1) & 1, a.err, 21)) {
                        ok = false;
                        break;
                    }
                    uint8_t *gs_ = geo + s * kFtGeo;
                    mbar_expect_tx(&geo_full[s], kFtGeo);
                    bulk_g2s(gs_, a.ecent + (size_t)kb * 8 * 8, 8 * 32, &geo_full[s]);
                    bulk_g2s(gs_ + 8 * 32, a.q8 + (size_t)kb * kFtK, kFtK * 16, &geo_full[s]);
                    if (g > 0 && !mbar_wait(b_free, (g - 1) & 1, a.err, 26)) {
                        ok = false;
                        break;
                    }
                    mbar_expect_tx(b_full, 2 * kFtBTile);
                    tma_load_2d(btile, &tmBh, b_full, kb * kFtK, 0);
                    tma_load_2d(btile + kFtBTile, &tmBl, b_full, kb * kFtK, 0);
                }
            }
            // drain: the last copies have landed before the CTA may exit
            if (g > 0) {
                const long long t0 = clock64();
                while (!mbar_try(b_full, (g - 1) & 1) && clock64() - t0 < kSpin) {
                }
            }
            for (uint32_t h = g > (uint32_t)kFtStages ? g - kFtStages : 0; h < g; h++) {
                const long long t0 = clock64();
                while (!mbar_try(&geo_full[h % kFtStages], (h / kFtStages) & 1) && clock64() - t0 < kSpin) {
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---- MMA issuer
            const uint32_t idesc = idesc_f16(kFtN, kFtM);
            uint32_t g = 0;
            bool ok = true;
            for (int u = blockIdx.x; ok && u < units; u += gridDim.x) {
                const int kb0 = (u / a.tiles) * a.kb_per_split, kb1 = min(a.nkb, kb0 + a.kb_per_split);
                for (int kb = kb0; kb < kb1; kb++, g++) {
                    const uint32_t s = g % kFtStages, n = g / kFtStages;
                    const uint32_t buf = g & 1, q = g >> 1;
                    if (!mbar_wait(&a_full[s], n & 1, a.err, 22) || !mbar_wait(b_full, g & 1, a.err, 22) ||
                        (q > 0 && !mbar_wait(&acc_empty[buf], (q - 1) & 1, a.err, 23))) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    uint8_t *st = smem + s * kFtStage;
                    const uint64_t dbh = sw_desc(btile), dbl = sw_desc(btile + kFtBTile);
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        const uint32_t acc = tmem + buf * kFtAcc + (uint32_t)(c * kFtN);
                        const uint64_t dah = sw_desc(st + (2 * c) * kFtATile);
                        const uint64_t dal = sw_desc(st + (2 * c + 1) * kFtATile);
#pragma unroll
                        for (int kk = 0; kk < kTcRowBytes / 32; kk++) {
                            const uint64_t off = (uint64_t)(kk * 32) >> 4;
                            mma_f16(acc, dah + off, dbh + off, idesc, kk != 0);
                            mma_f16(acc, dah + off, dbl + off, idesc, 1);
                            mma_f16(acc, dal + off, dbh + off, idesc, 1);
                        }
                    }
                    mma_commit(&st_free[s]);
                    mma_commit(b_free);
                    mma_commit(&acc_full[buf]);
                }
            }
            mma_commit(done);
        }
    } else {
        // ---- generators, then readers of the previous k-block's products
        const int gt = threadIdx.x - 64;  // 0 .. 255
        const int r = gt & (kFtM - 1), h = gt >> 7;
        const int quarter = warp & 3, chalf = (warp - 2) >> 2;
        const float gs = a.gsc[0];
        float acc[96];
#pragma unroll
        for (int j = 0; j < 96; j++) acc[j] = 0.0f;
        uint32_t g = 0;
        bool ok = true;
        // read k-block gg's products into acc (the whole warp)
        auto drain = [&](uint32_t gg) -> bool {
            const uint32_t buf = gg & 1;
            const bool have = mbar_wait(&acc_full[buf], (gg >> 1) & 1, a.err, 24);
            if (!__all_sync(0xffffffffu, have)) return false;
            tc_fence_after();
            const uint32_t base = tmem + ((uint32_t)(quarter * 32) << 16) + buf * kFtAcc + (uint32_t)(96 * chalf);
#pragma unroll
            for (int c0 = 0; c0 < 96; c0 += 32) {
                uint32_t v[32];
                tmem_ld32(base + (uint32_t)c0, v);
#pragma unroll
                for (int t = 0; t < 32; t++) acc[c0 + t] += __uint_as_float(v[t]);
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[buf]);
            return true;
        };
        for (int u = blockIdx.x; ok && u < units; u += gridDim.x) {
            const int tm = u % a.tiles, sp = u / a.tiles;
            const int kb0 = sp * a.kb_per_split, kb1 = min(a.nkb, kb0 + a.kb_per_split);
            const int p = min(tm * kFtM + r, a.P - 1);
            const float ph[3] = {a.phl[(size_t)p * 6], a.phl[(size_t)p * 6 + 1], a.phl[(size_t)p * 6 + 2]};
            const float pl[3] = {a.phl[(size_t)p * 6 + 3], a.phl[(size_t)p * 6 + 4], a.phl[(size_t)p * 6 + 5]};
            for (int kb = kb0; kb < kb1; kb++, g++) {
                const uint32_t s = g % kFtStages, n = g / kFtStages;
                if ((n > 0 && !mbar_wait(&st_free[s], (n - 1) & 1, a.err, 25)) ||
                    !mbar_wait(&geo_full[s], n & 1, a.err, 25)) {
                    ok = false;
                    break;
                }
                uint8_t *st = smem + s * kFtStage;
                const float *gce = (const float *)(geo + s * kFtGeo);           // [8][8]
                const float4 *gq8 = (const float4 *)(geo + s * kFtGeo + 8 * 32);  // [64]
                // the thread's four elements: one 16-byte chunk each of row r
#pragma unroll 1
                for (int j = 0; j < 4; j++) {
                    const int el = 4 * h + j, e = kb * 8 + el;
                    const float4 c0 = ((const float4 *)(gce + el * 8))[0];
                    const float4 c1 = ((const float4 *)(gce + el * 8))[1];
                    const float d0x = (ph[0] - c0.x) + (pl[0] - c0.w);
                    const float d0y = (ph[1] - c0.y) + (pl[1] - c1.x);
                    const float d0z = (ph[2] - c0.z) + (pl[2] - c1.y);
                    // near pairs (and the padding past E) to the FP32 pass; the
                    // squared distance rounded as that pass rounds it
                    const float dd = __fmaf_rn(d0z, d0z, __fmaf_rn(d0y, d0y, __fmul_rn(d0x, d0x)));
                    const bool far = e < a.E && dd >= c1.z;
                    uint32_t w[6][4];
                    if (far) {
                        float4 o[kTriPts];
#pragma unroll
                        for (int k = 0; k < kTriPts; k++) o[k] = gq8[el * 8 + k];
                        const float2 dx0 = make_float2(d0x, d0x), dy0 = make_float2(d0y, d0y),
                                     dz0 = make_float2(d0z, d0z);
                        const float2 g2 = make_float2(gs, gs), half2c = make_float2(-0.5f, -0.5f),
                                     th2 = make_float2(1.5f, 1.5f);
                        // two quadrature points (k, k + 1) per step in packed FP32x2
#pragma unroll
                        for (int k = 0; k < 8; k += 2) {
                            const float4 ob = k + 1 < kTriPts ? o[k + 1] : o[k];  // slot 7: zeroed below
                            const float2 dx = __fadd2_rn(dx0, make_float2(-o[k].x, -ob.x));
                            const float2 dy = __fadd2_rn(dy0, make_float2(-o[k].y, -ob.y));
                            const float2 dz = __fadd2_rn(dz0, make_float2(-o[k].z, -ob.z));
                            const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
                            float2 inv = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
                            // one Newton step: inv (1.5 - 0.5 r2 inv^2)
                            inv = __fmul2_rn(inv, __ffma2_rn(half2c, __fmul2_rn(__fmul2_rn(r2, inv), inv), th2));
                            float2 i3 = __fmul2_rn(__fmul2_rn(__fmul2_rn(inv, inv), inv), g2);
                            if (k + 1 >= kTriPts) i3.y = 0.0f;
                            const float2 gv[3] = {__fmul2_rn(dx, i3), __fmul2_rn(dy, i3), __fmul2_rn(dz, i3)};
#pragma unroll
                            for (int c = 0; c < 3; c++) {
                                const __half2 hi = __floats2half2_rn(gv[c].x, gv[c].y);
                                const float2 hb = __half22float2(hi);
                                const float2 rem = __fadd2_rn(gv[c], make_float2(-hb.x, -hb.y));
                                const __half2 lo = __floats2half2_rn(rem.x, rem.y);
                                w[2 * c][k / 2] = *(const uint32_t *)&hi;
                                w[2 * c + 1][k / 2] = *(const uint32_t *)&lo;
                            }
                        }
                    } else {
#pragma unroll
                        for (int t = 0; t < 6; t++) w[t][0] = w[t][1] = w[t][2] = w[t][3] = 0u;
                    }
                    // swizzled K-major: row r, 16-byte chunk (4 h + j) ^ (r % 8)
                    const uint32_t off = (uint32_t)r * kTcRowBytes + (uint32_t)(((4 * h + j) ^ (r & 7)) * 16);
#pragma unroll
                    for (int t = 0; t < 6; t++)
                        *(uint4 *)(st + t * kFtATile + off) = make_uint4(w[t][0], w[t][1], w[t][2], w[t][3]);
                }
                // generic-proxy writes must be visible to the tensor core's reads
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_arrive(&a_full[s]);
                if (kb > kb0 && !drain(g - 1)) {
                    ok = false;
                    break;
                }
            }
            if (!ok || kb1 <= kb0) break;
            if (!drain(g - 1)) {
                ok = false;
                break;
            }
            // the unit's sums: row 32 quarter + lane, columns 96 chalf + j = c * 64 + f
            const int pr = tm * kFtM + quarter * 32 + lane;
            if (pr < a.P) {
                const float ig = a.gsc[1];
#pragma unroll
                for (int j = 0; j < 96; j++) {
                    const int col = 96 * chalf + j, c = col >> 6, f = col & 63;
                    if (f < a.F) a.part[(((size_t)sp * a.F + f) * a.P + pr) * 3 + c] = acc[j] * ig * a.csc[f];
                }
            }
#pragma unroll
            for (int j = 0; j < 96; j++) acc[j] = 0.0f;
        }
    }
    __syncwarp();
    if (warp == 1) {
        if (lane == 0) {
            const long long t0 = clock64();
            while (!mbar_try(done, 0) && clock64() - t0 < kSpin) {
            }
        }
        __syncwarp();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * kFtAcc)
                     : "memory");
}

// The quadrature points relative to their centroid in slots of 8 per
// element (float4 x, y, z, 0; slot 7 and elements past E zero).
__global__ void k_q8(const float *__restrict__ qoff, int E, int Epad, float4 *__restrict__ q8)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= Epad * 8) return;
    const int e = t >> 3, k = t & 7;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (e < E && k < kTriPts) {
        const float *o = qoff + ((size_t)e * kTriPts + k) * 3;
        v = make_float4(o[0], o[1], o[2], 0.f);
    }
    q8[t] = v;
}

// The charges as fp16 pairs for the far-field products: row f (f < 64; rows
// F .. 63, slot 7 of each element and columns past E zero) of Ch, Cl
// (stride ldq, slot 8 e + k) = the pair of
// 2^t_f c(q, f), t_f from the largest FP32 exponent of system f (emax[f],
// filled by k_charge_emax); csc[f] = 2^-t_f.
__global__ void k_charge_emax(const float *__restrict__ cT, int E7p, int F, int E7, int *__restrict__ emax)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    int e = 0;
    if (q < E7 && f < F) e = (__float_as_int(cT[((size_t)(f >> 5) * E7p + q) * 32 + (f & 31)]) >> 23) & 0xFF;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
    if ((threadIdx.x & 31) == 0 && e) atomicMax(&emax[f], e);
}

__global__ void k_charge_pairs(const float *__restrict__ cT, int E7p, int F, int E7, const int *__restrict__ emax,
                               __half *__restrict__ Ch, __half *__restrict__ Cl, size_t ldq, float *__restrict__ csc)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;  // slot 8 e + k
    const int f = blockIdx.y;
    if ((size_t)q >= ldq) return;
    const int E = f < F ? emax[f] : 0;
    const int sh = E == 0 ? 0 : max(-100, min(100, 14 - (E - 127)));
    const int qe = (q >> 3) * kTriPts + (q & 7);  // the charge's index 7 e + k
    float x = 0.0f;
    if ((q & 7) < kTriPts && qe < E7 && f < F)
        x = cT[((size_t)(f >> 5) * E7p + qe) * 32 + (f & 31)] * __int_as_float((127 + sh) << 23);
    const __half hh = __float2half_rn(x);
    Ch[(size_t)f * ldq + q] = hh;
    Cl[(size_t)f * ldq + q] = __float2half_rn(x - __half2float(hh));
    if (q == 0) csc[f] = __int_as_float((127 - sh) << 23);
}

// gsc[0] = 2^s with 2^s * (largest far |G|) below 2^15: far pairs have the
// point at least 4 quadrature radii from the centroid (squared near radius
// 16 rq^2), so |x_p - y_q| >= 3 rq and |G| <= 1 / (9 rq^2); gsc[1] = 2^-s.
__global__ void k_far_gscale(const float *__restrict__ ecent, int E, float *__restrict__ gsc)
{
    __shared__ float sm[32];
    float m = 3.0e38f;
    for (int e = threadIdx.x; e < E; e += blockDim.x) {
        const float v = ecent[(size_t)e * 8 + 6];
        if (v > 0.0f) m = fminf(m, v);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        float mm = sm[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) mm = fminf(mm, sm[w]);
        const float gmax = 16.0f / (9.0f * mm);  // bound on far |G|
        int ex = 0;
        frexpf(gmax, &ex);                       // gmax < 2^ex
        const int s = max(-100, min(100, 15 - ex));
        gsc[0] = __int_as_float((127 + s) << 23);
        gsc[1] = __int_as_float((127 - s) << 23);
    }
}

int field_far_tc(const float *phl, int P, const float *ecent, const float *qoff, int E, const float *cT, int E7p,
                 int F, FieldTcWork &w, float *part, int nsplit_max, int *d_err, cudaStream_t st, int *nsplit_out)
{
    if (F < 1 || F > kFtN || P < 1 || E < 1) {
        set_error("field_far_tc: unsupported sizes P %d E %d F %d (F <= %d)", P, E, F, kFtN);
        return kErrArg;
    }
    const int E7 = E * kTriPts;
    const int Epad = (E + 7) / 8 * 8;
    const size_t ldq = (size_t)Epad * 8;  // 8 slots per element: k-blocks of 8 elements
    const int nkb = (int)(ldq / kFtK);
    DSC_TRY(w.q8.alloc(ldq));
    DSC_LAUNCH(k_q8<<<(unsigned)((ldq + 255) / 256), 256, 0, st>>>(qoff, E, Epad, w.q8.p));
    DSC_TRY(w.Ch.alloc((size_t)kFtN * ldq));
    DSC_TRY(w.Cl.alloc((size_t)kFtN * ldq));
    DSC_TRY(w.csc.alloc(kFtN));
    DSC_TRY(w.emax.alloc(kFtN));
    DSC_TRY(w.gsc.alloc(2));
    DSC_CUDA(cudaMemsetAsync(w.emax.p, 0, kFtN * sizeof(int), st));
    DSC_LAUNCH(k_charge_emax<<<dim3((E7 + 255) / 256, F), 256, 0, st>>>(cT, E7p, F, E7, w.emax.p));
    DSC_LAUNCH(k_charge_pairs<<<dim3((unsigned)((ldq + 255) / 256), kFtN), 256, 0, st>>>(cT, E7p, F, E7, w.emax.p,
                                                                                      w.Ch.p, w.Cl.p, ldq, w.csc.p));
    DSC_LAUNCH(k_far_gscale<<<1, 1024, 0, st>>>(ecent, E, w.gsc.p));
    CUtensorMap bh, bl;
    DSC_TRY(tc_make_map(&bh, w.Ch.p, 2, kFtN, (int)ldq, ldq, kFtN));
    DSC_TRY(tc_make_map(&bl, w.Cl.p, 2, kFtN, (int)ldq, ldq, kFtN));
    int nsm = 0;
    DSC_TRY(current_sm_count(&nsm));
    const int tiles = (P + kFtM - 1) / kFtM;
    int nsplit = std::max(1, std::min(nsplit_max, (4 * nsm + tiles - 1) / tiles));
    const int kps = (nkb + nsplit - 1) / nsplit;
    nsplit = (nkb + kps - 1) / kps;
    DSC_TRY(raise_smem_limit((const void *)k_field_far_tc, (int)kFtSmem));
    FieldTcArgs a{phl, ecent, w.q8.p, w.gsc.p, w.csc.p, part, P, E, F, nkb, kps, nsplit, tiles, d_err};
    const int units = tiles * nsplit;
    DSC_LAUNCH(k_field_far_tc<<<std::min(units, nsm), kFtThreads, kFtSmem, st>>>(bh, bl, a));
    DSC_CUDA(cudaGetLastError());
    *nsplit_out = nsplit;
    return kOk;
}

}  // namespace dsc
