// dsc_mixed.cu -- mixed-precision batched frequency sweep.
//
// All frequencies of a sweep share K.  With complex Jacobi scaling
// p_i = 1 / (s_i K_ii + d_i), s_i = a_i - i b_i, each system is
//     (diag(cs_f) K + diag(cd_f)) x_f = bt_f,   cs = p s, cd = p d, bt = p b.
// Outer loop (FP64): iterative refinement on the FP64 residual
//     r_f = bt_f - (cs_f o (K64 x_f) + cd_f o x_f)
// until |r_f| <= tol |bt_f|.  Inner solve (per outer step, all systems at
// once): complex GMRES whose products K v run as ONE matrix product over
// every system's Krylov vector (N x 2F right-hand sides) on an FP32 copy of
// K, with Arnoldi (classical Gram-Schmidt, two passes) in FP64 and Givens
// rotations per system.  Then Re(sigma_f) at the particle nodes for every
// frequency in one batched FP64 field pass and the Maxwell-stress force.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <limits>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "../../include/depsolver_cuda.h"
#include "dsc_async.cuh"
#include "dsc_blas.cuh"
#include "dsc_common.cuh"
#include "dsc_df32.cuh"
#include "dsc_field.h"
#include "dsc_field_tc.h"
#include "dsc_internal.h"
#include "dsc_session.h"
#include "dsc_singular.cuh"
#include "dsc_tcgemm.h"

namespace dsc {

constexpr int kMaxBatch = 64;   // frequencies per batch
constexpr int kInnerMax = 80;   // Krylov dimension of one inner solve
constexpr int kOuterMax = 6;    // refinement steps
// Floor of the inner tolerance: near the accuracy of the FP32 products.
// Measured on the 12k-node scene (64 frequencies to 1e-10): 1e-6 took 110
// products per sweep (the slowest systems needed a third refinement step),
// 3e-7 took 89, 1e-7 took 93.
constexpr double kInnerTol = 3e-7;

// r_f = bt_f - (cs_f o Y_f + cd_f o x_f)
__global__ void k_residual(const double *__restrict__ Y, const double *__restrict__ X,
                           const double2 *__restrict__ cs, const double2 *__restrict__ cd,
                           const double2 *__restrict__ bt, double *__restrict__ R, int N, size_t ld,
                           int F)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (i >= N || f >= F) return;
    const double yr = Y[(size_t)(2 * f) * ld + i], yi = Y[(size_t)(2 * f + 1) * ld + i];
    const double xr = X[(size_t)(2 * f) * ld + i], xi = X[(size_t)(2 * f + 1) * ld + i];
    const double2 s = cs[(size_t)f * N + i], d = cd[(size_t)f * N + i], b = bt[(size_t)f * N + i];
    R[(size_t)(2 * f) * ld + i] = b.x - (s.x * yr - s.y * yi + d.x * xr - d.y * xi);
    R[(size_t)(2 * f + 1) * ld + i] = b.y - (s.x * yi + s.y * yr + d.x * xi + d.y * xr);
}

// y{re,im}[i] = the sum of k_gemv_K2's S split partials (FP64, in split order).
__global__ void k_gemv_parts(const double *__restrict__ part, int S, int N, double *__restrict__ yr,
                             double *__restrict__ yi)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    double tr = 0.0, ti = 0.0;
    for (int s = 0; s < S; s++) {
        tr += part[((size_t)s * 2) * N + i];
        ti += part[((size_t)s * 2 + 1) * N + i];
    }
    yr[i] = tr;
    yi[i] = ti;
}

// ---- Givens rotations and triangular solves on the device, one thread per
// system (complex GMRES; c real, s complex; G = [[c, s], [-conj(s), c]]).
__device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double cabs2(double2 a) { return hypot(a.x, a.y); }
__device__ __forceinline__ double2 cdiv(double2 a, double2 b)
{
    const double d = b.x * b.x + b.y * b.y;
    return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

struct GivensState {
    double2 *H;   // [f][k][j], (kInnerMax + 1) x kInnerMax per system
    double *c;    // [f][j]
    double2 *s;   // [f][j]
    double2 *g;   // [f][k], kInnerMax + 1 per system
};

__global__ void k_givens_init(GivensState gs, const double *__restrict__ beta, int F,
                              int *__restrict__ mcount)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    double2 *g = gs.g + (size_t)f * (kInnerMax + 1);
    for (int k = 0; k <= kInnerMax; k++) g[k] = make_double2(0.0, 0.0);
    g[0] = make_double2(beta[f], 0.0);
    mcount[f] = 0;
}

// Column j of every active system: h[0..j] (complex, from the two Gram-
// Schmidt passes) and h[j+1] = |w|; applies the previous rotations, forms
// the new one, updates g, decides convergence (|g[j+1]| <= itol * beta)
// and the scale of the next basis vector; a system also stops once it has
// taken icap[f] steps.
__global__ void k_givens_step(GivensState gs, const double2 *__restrict__ hacc,
                              const double *__restrict__ hn, int j, int F,
                              const double *__restrict__ beta, const double *__restrict__ itol,
                              const int *__restrict__ icap, int *__restrict__ active,
                              double *__restrict__ scale, int *__restrict__ mcount)
{
    grid_dep_wait();
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    if (!active[f]) {
        scale[f] = 0.0;
        return;
    }
    double2 *H = gs.H + (size_t)f * (kInnerMax + 1) * kInnerMax;
    double *cr = gs.c + (size_t)f * kInnerMax;
    double2 *sr = gs.s + (size_t)f * kInnerMax;
    double2 *g = gs.g + (size_t)f * (kInnerMax + 1);
    double2 prev = hacc[f];  // running entry k
    for (int k = 0; k < j; k++) {
        const double2 nxt = hacc[(size_t)(k + 1) * F + f];
        const double2 t1 = cadd(cscale(prev, cr[k]), cmul(sr[k], nxt));
        const double2 t2 = cadd(cscale(cmul(cconj(sr[k]), prev), -1.0), cscale(nxt, cr[k]));
        H[(size_t)k * kInnerMax + j] = t1;
        prev = t2;
    }
    const double2 a = prev;
    const double b = hn[f];
    const double aa = cabs2(a), nu = hypot(aa, b);
    double c;
    double2 s, top;
    if (aa == 0.0) {
        c = 0.0;
        s = make_double2(1.0, 0.0);
        top = make_double2(b, 0.0);
    } else {
        const double2 sgn = cscale(a, 1.0 / aa);
        c = aa / nu;
        s = cscale(sgn, b / nu);  // sgn * conj(b) / nu with b real
        top = cscale(sgn, nu);
    }
    cr[j] = c;
    sr[j] = s;
    H[(size_t)j * kInnerMax + j] = top;
    const double2 gj = g[j];
    g[j + 1] = cscale(cmul(cconj(s), gj), -1.0);
    g[j] = cscale(gj, c);
    mcount[f] = j + 1;
    const double est = cabs2(g[j + 1]);
    // icap[f]: the system's share of the caller's iteration cap left for
    // this inner solve
    if (est <= itol[f] * beta[f] || b == 0.0 || j + 1 >= icap[f]) {
        active[f] = 0;
        scale[f] = 0.0;
    } else {
        scale[f] = 1.0 / b;
    }
}

// y = R^{-1} g[0..m) for the systems of this inner solve (act0).
__global__ void k_backsolve(GivensState gs, const int *__restrict__ mcount,
                            const int *__restrict__ act0, int F, double2 *__restrict__ y)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    const int m = act0[f] ? mcount[f] : 0;
    const double2 *H = gs.H + (size_t)f * (kInnerMax + 1) * kInnerMax;
    const double2 *g = gs.g + (size_t)f * (kInnerMax + 1);
    for (int k = m - 1; k >= 0; k--) {
        double2 t = g[k];
        for (int q = k + 1; q < m; q++) t = csub(t, cmul(H[(size_t)k * kInnerMax + q], y[(size_t)q * F + f]));
        y[(size_t)k * F + f] = cdiv(t, H[(size_t)k * kInnerMax + k]);
    }
}

// X += D (all 2F columns)
__global__ void k_axpy_blocks(double *__restrict__ X, const double *__restrict__ D, int N, size_t ld,
                              int F)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (i >= N) return;
    X[(size_t)(2 * f) * ld + i] += D[(size_t)(2 * f) * ld + i];
    X[(size_t)(2 * f + 1) * ld + i] += D[(size_t)(2 * f + 1) * ld + i];
}

// r_f -= cs_f o (sum of split partials of K d)_f + cd_f o d_f
__global__ void k_residual_update(const float *__restrict__ P, int S, size_t split_stride,
                                  const double *__restrict__ D, const double2 *__restrict__ cs,
                                  const double2 *__restrict__ cd, double *__restrict__ R, int N,
                                  size_t ld, int F)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (i >= N || f >= F) return;
    double yr = 0.0, yi = 0.0;
    for (int s = 0; s < S; s++) {
        yr += (double)P[(size_t)s * split_stride + (size_t)(2 * f) * ld + i];
        yi += (double)P[(size_t)s * split_stride + (size_t)(2 * f + 1) * ld + i];
    }
    const double dr = D[(size_t)(2 * f) * ld + i], di = D[(size_t)(2 * f + 1) * ld + i];
    const double2 s = cs[(size_t)f * N + i], d = cd[(size_t)f * N + i];
    R[(size_t)(2 * f) * ld + i] -= s.x * yr - s.y * yi + d.x * dr - d.y * di;
    R[(size_t)(2 * f + 1) * ld + i] -= s.x * yi + s.y * yr + d.x * di + d.y * dr;
}

// Gram-Schmidt over the basis in two launches per pass, both without block
// barriers: every warp works alone on units taken in a grid-stride loop
// over the warps of one resident wave.
//
// Dots: unit (row chunk of kDotRows rows, system f, vector k); the warp
// forms the chunk's <V_k,f, W_f> = sum conj(v) w in double-FP32 (two rows
// per lane and step, kDotBatch steps' loads issued together) and lane 0
// writes the double-FP32 pair; k_cgs_dots_reduce adds the chunks in order
// (FP64).  k runs fastest over the units, so the warps of a block share
// their W chunk through the caches.
constexpr int kDotRows = 512;
constexpr int kDotBatch = 4;
static_assert(kDotRows % (64 * kDotBatch) == 0, "a chunk is whole batches of 64-row steps");

__global__ void __launch_bounds__(256) k_cgs_dots(const float2 *__restrict__ Vb, size_t vstride,
                                                  const float2 *__restrict__ W, int N, size_t ld, int F,
                                                  int nk, const int *__restrict__ active,
                                                  float4 *__restrict__ part,
                                                  unsigned long long *__restrict__ bytes)
{
    grid_dep_wait();
    const int lane = threadIdx.x & 31;
    const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nw = (int)((gridDim.x * blockDim.x) >> 5);
    const int nchunk = (N + kDotRows - 1) / kDotRows;
    const int units = nchunk * F * nk;
    for (int un = gw; un < units; un += nw) {
        const int k = un % nk, cf = un / nk, chunk = cf % nchunk, f = cf / nchunk;
        if (!active[f]) continue;  // uniform over the warp
        const int r0 = chunk * kDotRows, nr = min(kDotRows, N - r0);
        // rows up to the even count np2 <= ld exist in V and W (ld is a
        // multiple of 32); the padding row N of both holds zero
        const int np2 = (nr + 1) & ~1;
        if (bytes && lane == 0) atomicAdd(bytes, (unsigned long long)nr * 16u * (k == 0 ? 2 : 1));
        const float2 *vr = Vb + (size_t)k * vstride + (size_t)(2 * f) * ld + r0, *vi = vr + ld;
        const float2 *wr = W + (size_t)(2 * f) * ld + r0, *wi = wr + ld;
        float2 sr = make_float2(0.f, 0.f), si = make_float2(0.f, 0.f);
        // two rows per lane and step (16-byte loads: r0 and ld are even)
        for (int t0 = 2 * lane; t0 < np2; t0 += 64 * kDotBatch) {
            float4 a[kDotBatch], b[kDotBatch], c[kDotBatch], d[kDotBatch];
#pragma unroll
            for (int u = 0; u < kDotBatch; u++) {
                const int t = t0 + 64 * u < np2 ? t0 + 64 * u : 0;  // past the chunk: row 0, unused
                a[u] = __ldcs((const float4 *)(vr + t));
                b[u] = __ldcs((const float4 *)(vi + t));
                c[u] = __ldg((const float4 *)(wr + t));
                d[u] = __ldg((const float4 *)(wi + t));
            }
#pragma unroll
            for (int u = 0; u < kDotBatch; u++) {
                if (t0 + 64 * u >= np2) break;
                const float2 a0 = make_float2(a[u].x, a[u].y), a1 = make_float2(a[u].z, a[u].w);
                const float2 b0 = make_float2(b[u].x, b[u].y), b1 = make_float2(b[u].z, b[u].w);
                const float2 c0 = make_float2(c[u].x, c[u].y), c1 = make_float2(c[u].z, c[u].w);
                const float2 d0 = make_float2(d[u].x, d[u].y), d1 = make_float2(d[u].z, d[u].w);
                df_mac(sr, a0, c0);
                df_mac(sr, b0, d0);
                df_mac(si, a0, d0);
                df_mac(si, df_neg(b0), c0);
                df_mac(sr, a1, c1);
                df_mac(sr, b1, d1);
                df_mac(si, a1, d1);
                df_mac(si, df_neg(b1), c1);
            }
        }
        sr = df_warp_sum(sr);
        si = df_warp_sum(si);
        if (lane == 0) part[((size_t)chunk * nk + k) * F + f] = make_float4(sr.x, sr.y, si.x, si.y);
    }
}

// h[k][f] = the sum of the chunk partials, hacc[k][f] += h[k][f] (the
// Hessenberg column sums the passes' coefficients), hdf[k][f] = the
// update's coefficients (-Re h, Im h) in double-FP32.  One warp per (k, f):
// lane-strided double-FP32 sums over the chunks, then a fixed shuffle tree
// (FP32 pipes; FP64 only for the warp's final h).
__global__ void k_cgs_dots_reduce(const float4 *__restrict__ part, int nchunk, int nk, int F,
                                  const int *__restrict__ active, double2 *__restrict__ h,
                                  double2 *__restrict__ hacc, float4 *__restrict__ hdf)
{
    grid_dep_wait();
    const int t = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (t >= nk * F) return;  // uniform over the warp
    const int f = t % F;
    if (!active[f]) return;
    float2 sr = make_float2(0.f, 0.f), si = make_float2(0.f, 0.f);
    for (int c = lane; c < nchunk; c += 32) {
        const float4 v = part[(size_t)c * nk * F + t];  // double-FP32 (re, im) of chunk c
        sr = df_add(sr, make_float2(v.x, v.y));
        si = df_add(si, make_float2(v.z, v.w));
    }
    sr = df_norm(df_warp_sum(sr));
    si = df_norm(df_warp_sum(si));
    if (lane == 0) {
        const double hr = df_to(sr), hi = df_to(si);
        h[t] = make_double2(hr, hi);
        const double2 a = hacc[t];
        hacc[t] = make_double2(a.x + hr, a.y + hi);
        hdf[t] = make_float4(-sr.x, -sr.y, si.x, si.y);
    }
}

// Update: unit (block of 64 rows, system f); each lane takes two rows and
// W_f -= sum_k h[k][f] V_k,f in double-FP32 with the coefficients of
// k_cgs_dots_reduce, then lane 0 writes the unit's share of |w_f|^2 to
// npart[f][unit] (nb = ceil(N / 64) per system).
constexpr int kUpdRows = 64;

__global__ void __launch_bounds__(256) k_cgs_update(const float2 *__restrict__ Vb, size_t vstride,
                                                    float2 *__restrict__ W, int N, size_t ld, int F,
                                                    int nk, const int *__restrict__ active,
                                                    const float4 *__restrict__ hdf,
                                                    double *__restrict__ npart,
                                                    unsigned long long *__restrict__ bytes)
{
    grid_dep_wait();
    const int lane = threadIdx.x & 31;
    const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nw = (int)((gridDim.x * blockDim.x) >> 5);
    const int nrb = (N + kUpdRows - 1) / kUpdRows;
    for (int un = gw; un < nrb * F; un += nw) {
        const int rb = un % nrb, f = un / nrb;
        if (!active[f]) continue;  // uniform over the warp
        if (bytes && lane == 0)
            atomicAdd(bytes, (unsigned long long)min(kUpdRows, N - rb * kUpdRows) * 16u * (nk + 2));
        // rows i and i + 1 (row N, when i + 1 == N, is a padding row: it is
        // read, updated and not stored)
        const int i = rb * kUpdRows + 2 * lane;
        float2 n2 = make_float2(0.f, 0.f);
        if (i < N) {
            float2 *wrp = W + (size_t)(2 * f) * ld + i, *wip = wrp + ld;
            const float2 *vr = Vb + (size_t)(2 * f) * ld + i, *vi = vr + ld;
            const float4 a = *(const float4 *)wrp, b = *(const float4 *)wip;
            float2 wr0 = make_float2(a.x, a.y), wr1 = make_float2(a.z, a.w);
            float2 wi0 = make_float2(b.x, b.y), wi1 = make_float2(b.z, b.w);
#pragma unroll 4
            for (int k = 0; k < nk; k++) {
                const float4 p = __ldcs((const float4 *)(vr + (size_t)k * vstride));
                const float4 q = __ldcs((const float4 *)(vi + (size_t)k * vstride));
                const float4 c = __ldg(hdf + (size_t)k * F + f);
                const float2 p0 = make_float2(p.x, p.y), p1 = make_float2(p.z, p.w);
                const float2 q0 = make_float2(q.x, q.y), q1 = make_float2(q.z, q.w);
                const float2 a_r = make_float2(c.x, c.y), a_i = make_float2(c.z, c.w), a_in = df_neg(a_i);
                df_mac(wr0, a_r, p0);   // wr -= hr vr - hi vi
                df_mac(wr0, a_i, q0);
                df_mac(wi0, a_r, q0);   // wi -= hr vi + hi vr
                df_mac(wi0, a_in, p0);
                df_mac(wr1, a_r, p1);
                df_mac(wr1, a_i, q1);
                df_mac(wi1, a_r, q1);
                df_mac(wi1, a_in, p1);
            }
            wr0 = df_norm(wr0);
            wi0 = df_norm(wi0);
            df_mac(n2, wr0, wr0);
            df_mac(n2, wi0, wi0);
            if (i + 1 < N) {
                wr1 = df_norm(wr1);
                wi1 = df_norm(wi1);
                *(float4 *)wrp = make_float4(wr0.x, wr0.y, wr1.x, wr1.y);
                *(float4 *)wip = make_float4(wi0.x, wi0.y, wi1.x, wi1.y);
                df_mac(n2, wr1, wr1);
                df_mac(n2, wi1, wi1);
            } else {
                *wrp = wr0;
                *wip = wi0;
            }
        }
        n2 = df_warp_sum(n2);
        if (lane == 0) npart[(size_t)f * nrb + rb] = df_to(n2);
    }
}

// nrm[f] = sqrt(sum of the nb block partials of |w_f|^2) for the systems
// in mask, one warp per system (lane-strided sums, then a fixed shuffle
// tree).  With n0 (not null): also act2[f], whether the system needs the
// second Gram-Schmidt pass, by the DGKS test (its vector lost more than
// 1 - 1/sqrt(2) of its norm n0[f] in the first pass).
__global__ void k_norm_finish(const double *__restrict__ npart, int nb, int F,
                              const int *__restrict__ mask, double *__restrict__ nrm,
                              const double *__restrict__ n0, int *__restrict__ act2)
{
    grid_dep_wait();
    const int f = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (f >= F) return;  // uniform over the warp
    if (!mask[f]) {
        if (n0 && lane == 0) act2[f] = 0;
        return;
    }
    double t = 0.0;
    for (int b = lane; b < nb; b += 32) t += npart[(size_t)f * nb + b];
    t = warp_sum(t);
    if (lane == 0) {
        const double n = sqrt(t);
        nrm[f] = n;
        if (n0) act2[f] = n < 0.7071067811865476 * n0[f];
    }
}

// nrm[f] = |R_f| for FP64 vectors (one block per system)
__global__ void __launch_bounds__(256) k_norms(const double *__restrict__ W, int N, size_t ld, int F,
                                               double *__restrict__ nrm)
{
    __shared__ double sh[32];
    const int f = blockIdx.x;
    const double *wr = W + (size_t)(2 * f) * ld, *wi = wr + ld;
    double s = 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) s += wr[i] * wr[i] + wi[i] * wi[i];
    double t = block_sum(s, sh);
    if (threadIdx.x == 0) nrm[f] = sqrt(t);
}

// The GEMM operand of a Krylov vector v = hi + lo (|v| <= 1: a unit
// vector): the fp16 pair of 2^14 v (the product's column factor is 2^-14).
constexpr float kVScale = 16384.0f;
__device__ __forceinline__ void f16_pair(float2 v, __half &h, __half &l)
{
    const float x = v.x * kVScale;  // exact
    h = __float2half_rn(x);
    l = __float2half_rn(__fadd_rn(__fsub_rn(x, __half2float(h)), v.y * kVScale));
}

// V_f = R_f * scale[f] (R in FP64) as double-FP32, and its fp16 pair for the
// next tensor-core product (Bh, Bl: same layout).
__global__ void k_scale_from64(const double *__restrict__ R, float2 *__restrict__ V,
                               __half *__restrict__ Bh, __half *__restrict__ Bl, int N, size_t ld,
                               int F, const double *__restrict__ scale,
                               const int *__restrict__ active)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (i >= N) return;
    const double s = active[f] ? scale[f] : 0.0;
#pragma unroll
    for (int c = 0; c < 2; c++) {
        const size_t o = (size_t)(2 * f + c) * ld + i;
        const float2 v = df_from(R[o] * s);
        __half th, tl;
        f16_pair(v, th, tl);
        V[o] = v;
        Bh[o] = th;
        Bl[o] = tl;
    }
}

// V_f = W_f * scale[f] (double-FP32), and its fp16 pair.
__global__ void k_scale_df(const float2 *__restrict__ W, float2 *__restrict__ V,
                           __half *__restrict__ Bh, __half *__restrict__ Bl, int N, size_t ld, int F,
                           const double *__restrict__ scale, const int *__restrict__ active)
{
    grid_dep_wait();
    __shared__ float2 s;
    const int f = blockIdx.y;
    if (threadIdx.x == 0) s = df_from(active[f] ? scale[f] : 0.0);
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
#pragma unroll
    for (int c = 0; c < 2; c++) {
        const size_t o = (size_t)(2 * f + c) * ld + i;
        const float2 v = df_mul(W[o], s);
        __half th, tl;
        f16_pair(v, th, tl);
        V[o] = v;
        Bh[o] = th;
        Bl[o] = tl;
    }
}

// D_f = sum_k y[k][f] V_k,f for k < m[f] (double-FP32 sum, FP64 result)
__global__ void k_update_solution(double *__restrict__ D, const float2 *__restrict__ Vb,
                                  size_t vstride, int N, size_t ld, int F,
                                  const double2 *__restrict__ y, const int *__restrict__ m)
{
    __shared__ float2 yr[kInnerMax], yi[kInnerMax], yin[kInnerMax];
    const int f = blockIdx.y;
    const int mf = m[f];
    for (int k = threadIdx.x; k < mf; k += blockDim.x) {
        const double2 c = y[(size_t)k * F + f];
        yr[k] = df_from(c.x);
        yi[k] = df_from(c.y);
        yin[k] = df_from(-c.y);
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    float2 xr = make_float2(0.f, 0.f), xi = make_float2(0.f, 0.f);
    for (int k = 0; k < mf; k++) {
        const float2 vr = Vb[(size_t)k * vstride + (size_t)(2 * f) * ld + i];
        const float2 vi = Vb[(size_t)k * vstride + (size_t)(2 * f + 1) * ld + i];
        df_mac(xr, yr[k], vr);
        df_mac(xr, yin[k], vi);
        df_mac(xi, yr[k], vi);
        df_mac(xi, yi[k], vr);
    }
    D[(size_t)(2 * f) * ld + i] = df_to(xr);
    D[(size_t)(2 * f + 1) * ld + i] = df_to(xi);
}

// ------------------------------------------------------- batched field
constexpr int kBF = 32;   // frequencies per thread in the batched field
constexpr int kBChunk = 32;
constexpr int kFieldTcSplits = 16;  // at most this many q-ranges in the tensor-core far pass

// Charge weights of Re(sigma_f) at every quadrature point, in FP32 for the
// field pass, grouped by kBF systems with the systems innermost:
// cT[(g * E7p + e*7+q) * kBF + ff] = w_q J_q sum_k N_k(q) Re sigma_f(node k)
// (FP64 sum, rounded), f = g kBF + ff; zero for f >= F and for the rows
// e*7+q >= 7E up to E7p (E rounded up to whole chunks of kBChunk).  Block
// (kBF, 8): a warp writes one row's kBF systems.
template <int NEN>
__global__ void k_charge_batched(const int *__restrict__ elems, int E, const double *__restrict__ qp,
                                 const double *__restrict__ X, size_t ld, int F, int E7p, float *__restrict__ cT)
{
    const int ff = threadIdx.x;
    const int t = blockIdx.x * blockDim.y + threadIdx.y;
    const int g = blockIdx.y, f = g * kBF + ff;
    if (t >= E7p) return;
    float v = 0.0f;
    if (t < E * kTriPts && f < F) {
        const int e = t / kTriPts, q = t % kTriPts;
        double N6[NEN];
        shape<NEN>(c_tri7[q][0], c_tri7[q][1], N6);
        const double *xr = X + (size_t)(2 * f) * ld;
        double sum = 0.0;
#pragma unroll
        for (int k = 0; k < NEN; k++) sum += N6[k] * xr[elems[(size_t)e * NEN + k]];
        v = (float)(qp[(size_t)t * 4 + 3] * sum);
    }
    cT[((size_t)g * E7p + t) * kBF + ff] = v;
}

// ---- FP32 far field with FP64 near field
// Per element: centroid as an FP32 (hi, lo) pair, squared near radius, and
// the 7 quadrature points relative to the centroid.  A (point, element)
// pair is "near" when the point lies within kNearFactor times the element's
// quadrature radius of the centroid; near pairs run in FP64.
constexpr float kNearFactor = 4.0f;

__global__ void k_prepare_far(const double *__restrict__ qp, int E, float *__restrict__ ecent,
                              float *__restrict__ qoff, float2 *__restrict__ qdf)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    double c[3] = {0.0, 0.0, 0.0};
    for (int q = 0; q < kTriPts; q++)
        for (int d = 0; d < 3; d++) c[d] += qp[((size_t)e * kTriPts + q) * 4 + d];
    for (int d = 0; d < 3; d++) c[d] /= kTriPts;
    double r2 = 0.0;
    for (int q = 0; q < kTriPts; q++) {
        double s = 0.0;
        for (int d = 0; d < 3; d++) {
            double o = qp[((size_t)e * kTriPts + q) * 4 + d] - c[d];
            qoff[((size_t)e * kTriPts + q) * 3 + d] = (float)o;
            qdf[((size_t)e * kTriPts + q) * 3 + d] = df_from(qp[((size_t)e * kTriPts + q) * 4 + d]);
            s += o * o;
        }
        r2 = fmax(r2, s);
    }
    float *o = ecent + (size_t)e * 8;
    for (int d = 0; d < 3; d++) {
        float h = (float)c[d];
        o[d] = h;
        o[3 + d] = (float)(c[d] - (double)h);
    }
    o[6] = (float)(r2 * (double)(kNearFactor * kNearFactor));
    o[7] = 0.0f;
}

__global__ void k_points_split(const double *__restrict__ px, const double *__restrict__ py,
                               const double *__restrict__ pz, int P, float *__restrict__ phl)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const double v[3] = {px[p], py[p], pz[p]};
    for (int d = 0; d < 3; d++) {
        float h = (float)v[d];
        phl[(size_t)p * 6 + d] = h;
        phl[(size_t)p * 6 + 3 + d] = (float)(v[d] - (double)h);
    }
}

// near_mask[b * ngroup + g] bit c: some point of block b (128 points) lies
// within the near radius of some element of chunk c of group g (nloop
// chunks of kBChunk elements) -- the near test of k_field_batched_mixed,
// from the centroids, with the same rounding.  One block of 128 threads per
// (point block, group); geometry only: once per session.
__global__ void __launch_bounds__(128) k_near_masks(const float *__restrict__ phl, int P,
                                                    const float *__restrict__ ecent, int E, int nloop,
                                                    unsigned *__restrict__ near_mask)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x, group = blockIdx.y;
    const bool valid = p < P;
    const int pp = valid ? p : 0;
    const float ph[3] = {phl[(size_t)pp * 6], phl[(size_t)pp * 6 + 1], phl[(size_t)pp * 6 + 2]};
    const float pl[3] = {phl[(size_t)pp * 6 + 3], phl[(size_t)pp * 6 + 4], phl[(size_t)pp * 6 + 5]};
    unsigned mask = 0;
    for (int cl = 0; cl < nloop && cl < 32; cl++) {
        const int e0 = (group * nloop + cl) * kBChunk;
        if (e0 >= E) break;
        const int ne = min(kBChunk, E - e0);
        bool any = false;
        if (valid) {
#pragma unroll 8
            for (int e = 0; e < ne; e++) {
                const float4 ca = __ldg((const float4 *)(ecent + (size_t)(e0 + e) * 8));
                const float4 cb = __ldg((const float4 *)(ecent + (size_t)(e0 + e) * 8 + 4));
                const float d0x = (ph[0] - ca.x) + (pl[0] - ca.w);
                const float d0y = (ph[1] - ca.y) + (pl[1] - cb.x);
                const float d0z = (ph[2] - ca.z) + (pl[2] - cb.y);
                any |= __fmaf_rn(d0z, d0z, __fmaf_rn(d0y, d0y, __fmul_rn(d0x, d0x))) < cb.z;
            }
        }
        if (__syncthreads_or(any)) mask |= 1u << cl;
    }
    if (threadIdx.x == 0) near_mask[(size_t)blockIdx.x * gridDim.y + group] = mask;
}

// part[group][f][p][3] (FP32): regular contributions of one group of
// kBLoop x kBChunk elements to the field at point p for system f.  Far
// pairs in FP32 (rsqrt with a Newton step, coordinates as centroid-relative
// offsets); near pairs take the point-to-quadrature-point geometry in
// double-FP32 and the products in FP32.  Each chunk's element data (charges
// of the block's kBF systems, centroids, offsets, points, nodes: contiguous
// slices of arrays padded to whole chunks) arrives in shared memory by bulk
// copies on one mbarrier; a wait that gives up sets *err (code 8) and ends
// the block.
constexpr int kBLoop = 8;   // element chunks per block (all pairs)
constexpr int kBLoopNear = 32;  // the same with the far pairs on the tensor cores: fewer partials
template <int NEN>
__global__ void __launch_bounds__(128) k_field_batched_mixed(
    const float *__restrict__ phl, const int4 *__restrict__ coinc, int P, const int *__restrict__ en_pad,
    int E, int E7p, const float *__restrict__ ecent, const float *__restrict__ qoff,
    const float *__restrict__ cT, const float2 *__restrict__ qdf, int F, float *__restrict__ part, int *err,
    int far_on, int nloop, const unsigned *__restrict__ near_mask)
{
    __shared__ __align__(16) float s_c[kBChunk * kTriPts][kBF];
    __shared__ __align__(16) float s_cent[kBChunk * 8];
    __shared__ __align__(16) float s_off[kBChunk * kTriPts * 3];
    __shared__ __align__(16) float2 s_qdf[kBChunk * kTriPts * 3];  // the points in double-FP32 (near pairs)
    __shared__ __align__(16) int s_en[kBChunk * NEN];
    __shared__ __align__(8) uint64_t bar;
    constexpr uint32_t kBytes = sizeof(s_c) + sizeof(s_cent) + sizeof(s_off) + sizeof(s_qdf) + sizeof(s_en);
    static_assert(sizeof(s_c) % 16 == 0 && sizeof(s_cent) % 16 == 0 && sizeof(s_off) % 16 == 0 &&
                      sizeof(s_qdf) % 16 == 0 && sizeof(s_en) % 16 == 0,
                  "bulk copies move multiples of 16 bytes");
    const int group = blockIdx.y, fg = blockIdx.z;
    const int f0 = fg * kBF, nf = min(kBF, F - f0);
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = p < P;
    const int pp = valid ? p : 0;
    const float ph[3] = {phl[(size_t)pp * 6], phl[(size_t)pp * 6 + 1], phl[(size_t)pp * 6 + 2]};
    const float pl[3] = {phl[(size_t)pp * 6 + 3], phl[(size_t)pp * 6 + 4], phl[(size_t)pp * 6 + 5]};
    const float2 pdf[3] = {make_float2(ph[0], pl[0]), make_float2(ph[1], pl[1]), make_float2(ph[2], pl[2])};
    const int4 c = coinc[pp];
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // accumulators of system pairs (2j, 2j + 1) per component: one packed
    // FP32x2 FMA (two round-to-nearest FMAs, as two FFMAs would give) per
    // pair, half the issue slots
    float2 acc[kBF / 2][3];
#pragma unroll
    for (int j = 0; j < kBF / 2; j++) acc[j][0] = acc[j][1] = acc[j][2] = make_float2(0.0f, 0.0f);
    uint32_t phase = 0;
    for (int cl = 0; cl < nloop; cl++) {
        const int e0 = (group * nloop + cl) * kBChunk;
        if (e0 >= E) break;  // uniform over the block
        const int ne = min(kBChunk, E - e0);
        // the far pairs on the tensor cores: chunks with no element near any
        // of the block's points are skipped (bit cl of the block's mask;
        // uniform over the block)
        if (near_mask && !((near_mask[(size_t)blockIdx.x * gridDim.y + group] >> cl) & 1u)) continue;
        __syncthreads();  // the previous chunk is no longer read (and the barrier is initialised)
        if (threadIdx.x == 0) {
            mbar_expect_tx(&bar, kBytes);
            bulk_g2s(s_c, cT + ((size_t)fg * E7p + (size_t)e0 * kTriPts) * kBF, sizeof(s_c), &bar);
            bulk_g2s(s_cent, ecent + (size_t)e0 * 8, sizeof(s_cent), &bar);
            bulk_g2s(s_off, qoff + (size_t)e0 * kTriPts * 3, sizeof(s_off), &bar);
            bulk_g2s(s_qdf, qdf + (size_t)e0 * kTriPts * 3, sizeof(s_qdf), &bar);
            bulk_g2s(s_en, en_pad + (size_t)e0 * NEN, sizeof(s_en), &bar);
        }
        const bool ok = mbar_wait(&bar, phase & 1, err, 8);
        if (!__syncthreads_and(ok)) {
            if (threadIdx.x == 0) mbar_drain(&bar, phase & 1);  // no copy outlives the block
            return;
        }
        phase++;
        if (!valid) continue;
        for (int e = 0; e < ne; e++) {
            const float *ce = s_cent + e * 8;
            const float d0x = (ph[0] - ce[0]) + (pl[0] - ce[3]);
            const float d0y = (ph[1] - ce[1]) + (pl[1] - ce[4]);
            const float d0z = (ph[2] - ce[2]) + (pl[2] - ce[5]);
            // rounded as the tensor-core far pass rounds it: the two passes
            // split the pairs exactly
            const bool near = __fmaf_rn(d0z, d0z, __fmaf_rn(d0y, d0y, __fmul_rn(d0x, d0x))) < ce[6];
            if (!near && !far_on) continue;  // the far pairs go to the tensor cores
            if (near) {
                // singular elements (the point is one of their nodes) lie
                // within the near radius; the singular pass takes them
                bool sing = false;
#pragma unroll
                for (int k = 0; k < NEN; k++) {
                    const int v = s_en[e * NEN + k];
                    sing |= (v == c.x) | (v == c.y) | (v == c.z) | (v == c.w);
                }
                if (sing && c.x >= 0) continue;
            }
            const float *O = s_off + e * kTriPts * 3;
#pragma unroll
            for (int q = 0; q < kTriPts; q++) {
                float gx, gy, gz;
                if (near) {
                    // the difference of close points in double-FP32
                    const float2 *Q = s_qdf + (e * kTriPts + q) * 3;
                    const float2 dx = df_sub(pdf[0], Q[0]), dy = df_sub(pdf[1], Q[1]), dz = df_sub(pdf[2], Q[2]);
                    const float2 r2 = df_add(df_add(df_sqr(dx), df_sqr(dy)), df_sqr(dz));
                    const float2 inv = df_rsqrt(r2);
                    const float2 i3 = df_mul(df_sqr(inv), inv);
                    gx = df_mul(dx, i3).x;
                    gy = df_mul(dy, i3).x;
                    gz = df_mul(dz, i3).x;
                } else {
                    const float dx = d0x - O[q * 3], dy = d0y - O[q * 3 + 1], dz = d0z - O[q * 3 + 2];
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    float inv = rsqrtf(r2);
                    inv = inv * (1.5f - 0.5f * r2 * inv * inv);
                    const float i3 = inv * inv * inv;
                    gx = dx * i3;
                    gy = dy * i3;
                    gz = dz * i3;
                }
                const float4 *cq4 = (const float4 *)s_c[e * kTriPts + q];  // broadcast reads
                const float2 g2x = make_float2(gx, gx), g2y = make_float2(gy, gy), g2z = make_float2(gz, gz);
#pragma unroll
                for (int f4 = 0; f4 < kBF / 4; f4++) {
                    const float4 cq = cq4[f4];
                    const float2 c01 = make_float2(cq.x, cq.y), c23 = make_float2(cq.z, cq.w);
                    acc[2 * f4][0] = __ffma2_rn(c01, g2x, acc[2 * f4][0]);
                    acc[2 * f4][1] = __ffma2_rn(c01, g2y, acc[2 * f4][1]);
                    acc[2 * f4][2] = __ffma2_rn(c01, g2z, acc[2 * f4][2]);
                    acc[2 * f4 + 1][0] = __ffma2_rn(c23, g2x, acc[2 * f4 + 1][0]);
                    acc[2 * f4 + 1][1] = __ffma2_rn(c23, g2y, acc[2 * f4 + 1][1]);
                    acc[2 * f4 + 1][2] = __ffma2_rn(c23, g2z, acc[2 * f4 + 1][2]);
                }
            }
        }
    }
    if (!valid) return;
#pragma unroll
    for (int ff = 0; ff < kBF; ff++)  // unrolled: acc stays in registers
        if (ff < nf)
#pragma unroll
            for (int d = 0; d < 3; d++)
                part[(((size_t)group * F + f0 + ff) * P + p) * 3 + d] = (ff & 1) ? acc[ff / 2][d].y : acc[ff / 2][d].x;
}

// The singular part of the field at each point for every system: the
// gradient integrals of its singular elements (left by the assembly's
// singular pass: Wg + tmap[t] * 3 NEN for the point's tuple t) applied to
// the solution's charges, plus the jump term of the point's own node.  Warp
// per point, lanes = systems f = lane, lane + 32.
template <int NEN>
__global__ void __launch_bounds__(128) k_field_singular_apply(
    int P, const int *__restrict__ elems, const double *__restrict__ normals, const int *__restrict__ sp_ptr,
    const int4 *__restrict__ sp, const int *__restrict__ tmap, const double *__restrict__ Wg,
    const double *__restrict__ Xs, size_t ld, int F, double *__restrict__ sing)
{
    const int p = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (p >= P) return;
    const double A = 0.5 / kEps0 / kPi2, B = 0.5 / kEps0;
    double acc[2][3] = {{0, 0, 0}, {0, 0, 0}};
    for (int t = sp_ptr[p]; t < sp_ptr[p + 1]; t++) {
        const int4 tu = sp[t];
        int nodes[NEN];
#pragma unroll
        for (int k = 0; k < NEN; k++) nodes[k] = elems[(size_t)tu.x * NEN + k];
        const double n[3] = {normals[3 * (size_t)tu.z], normals[3 * (size_t)tu.z + 1],
                             normals[3 * (size_t)tu.z + 2]};
        const double *w = Wg + (size_t)tmap[t] * 3 * NEN;
        for (int r = 0; r < 2; r++) {
            const int f = lane + 32 * r;
            if (f >= F) continue;
            const double *xr = Xs + (size_t)(2 * f) * ld;
#pragma unroll
            for (int k = 0; k < NEN; k++) {
                const double sr = xr[nodes[k]];
#pragma unroll
                for (int c = 0; c < 3; c++) acc[r][c] += A * w[3 * k + c] * sr;
            }
            const double s0 = xr[nodes[0]];
#pragma unroll
            for (int c = 0; c < 3; c++) acc[r][c] += B * s0 * n[c];
        }
    }
    for (int r = 0; r < 2; r++) {
        const int f = lane + 32 * r;
        if (f < F)
            for (int c = 0; c < 3; c++) sing[((size_t)f * P + p) * 3 + c] = acc[r][c];
    }
}

// Enode[f][node][3] = A * sum_chunks part + sing, scattered to node ids.
__global__ void k_field_batched_reduce(const float *__restrict__ part, int nchunk, int F, int P,
                                       const double *__restrict__ sing, const int *__restrict__ ids,
                                       int N, double *__restrict__ Enode)
{
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= (size_t)F * P * 3) return;
    const int d = (int)(t % 3), p = (int)((t / 3) % P), f = (int)(t / (3 * (size_t)P));
    const double A = 0.5 / kEps0 / kPi2;
    double s = 0.0;
    for (int c = 0; c < nchunk; c++) s += (double)part[(size_t)c * F * P * 3 + t];
    Enode[((size_t)f * N + ids[p]) * 3 + d] = A * s + sing[t];
}

// w J of a particle element's quadrature point and the unit normal there
// (one 32-byte load)
struct alignas(32) MstGeo {
    double wj, nx, ny, nz;
};

// Frequency-independent geometry of the Maxwell-stress integrals: per
// (particle element t, point q) the weight w_q J_q and the unit normal.
template <int NEN>
__global__ void k_mst_geometry(const double *__restrict__ X, const double *__restrict__ Y,
                               const double *__restrict__ Z, const int *__restrict__ elems,
                               const int *__restrict__ pel, int npel, MstGeo *__restrict__ geo)
{
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= npel * kTriPts) return;
    const int t = u / kTriPts, q = u % kTriPts;
    const int e = pel[t];
    double Xe[NEN][3], N6[NEN], XL[3], n[3];
#pragma unroll
    for (int k = 0; k < NEN; k++) {
        const int v = elems[(size_t)e * NEN + k];
        Xe[k][0] = X[v];
        Xe[k][1] = Y[v];
        Xe[k][2] = Z[v];
    }
    const double l1 = c_tri7[q][0], l2 = c_tri7[q][1];
    shape<NEN>(l1, l2, N6);
    const double J = map_point<NEN>(Xe, l1, l2, N6, XL);
    local_normal<NEN>(Xe, l1, l2, n);
    geo[u] = MstGeo{J * c_tri7[q][2], n[0], n[1], n[2]};
}

// Maxwell stress per (particle element, frequency), from the element's
// geometry (k_mst_geometry) and the nodal field of that frequency.
template <int NEN>
__global__ void k_mst_batched(const int *__restrict__ elems, const int *__restrict__ pel, int npel,
                              const MstGeo *__restrict__ geo, const double *__restrict__ Enode, int N, int F,
                              double eps, double *__restrict__ Fce)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (t >= npel) return;
    const int e = pel[t];
    const double *En0 = Enode + (size_t)f * N * 3;
    double En[NEN][3], N6[NEN];
#pragma unroll
    for (int k = 0; k < NEN; k++) {
        const int v = elems[(size_t)e * NEN + k];
        En[k][0] = En0[3 * (size_t)v];
        En[k][1] = En0[3 * (size_t)v + 1];
        En[k][2] = En0[3 * (size_t)v + 2];
    }
    double I0 = 0.0, I1 = 0.0, I2 = 0.0;
#pragma unroll
    for (int q = 0; q < kTriPts; q++) {
        shape<NEN>(c_tri7[q][0], c_tri7[q][1], N6);
        const MstGeo g = geo[(size_t)t * kTriPts + q];
        double Ex = 0.0, Ey = 0.0, Ez = 0.0;
#pragma unroll
        for (int k = 0; k < NEN; k++) {
            Ex += En[k][0] * N6[k];
            Ey += En[k][1] * N6[k];
            Ez += En[k][2] * N6[k];
        }
        const double NE = Ex * g.nx + Ey * g.ny + Ez * g.nz;
        const double Esq = Ex * Ex + Ey * Ey + Ez * Ez;
        I0 += g.wj * (Ex * NE - 0.5 * Esq * g.nx);
        I1 += g.wj * (Ey * NE - 0.5 * Esq * g.ny);
        I2 += g.wj * (Ez * NE - 0.5 * Esq * g.nz);
    }
    const double A = 0.5 * eps;
    double *o = Fce + ((size_t)f * npel + t) * 3;
    o[0] = A * I0;
    o[1] = A * I1;
    o[2] = A * I2;
}

// tot[f][9]: Fcm, Xcm, sum |Fce| (one block of kTotThreads per frequency;
// per-thread strided sums, warp sums, then the warps' sums in order: a
// fixed order)
constexpr int kTotThreads = 256;
__global__ void __launch_bounds__(kTotThreads) k_mst_batched_totals(const double *__restrict__ Fce, int npel, int F,
                                                                    const double *__restrict__ X,
                                                                    const double *__restrict__ Y,
                                                                    const double *__restrict__ Z,
                                                                    const int *__restrict__ ids, int P,
                                                                    double *__restrict__ tot)
{
    __shared__ double sh[kTotThreads / 32][9];
    const int f = blockIdx.x, lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const double *Fc = Fce + (size_t)f * npel * 3;
    double s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int t = threadIdx.x; t < npel; t += kTotThreads)
        for (int d = 0; d < 3; d++) {
            s[d] += Fc[3 * (size_t)t + d];
            s[6 + d] += fabs(Fc[3 * (size_t)t + d]);
        }
    for (int q = threadIdx.x; q < P; q += kTotThreads) {
        s[3] += X[ids[q]];
        s[4] += Y[ids[q]];
        s[5] += Z[ids[q]];
    }
    for (int k = 0; k < 9; k++) s[k] = warp_sum(s[k]);
    if (lane == 0)
        for (int k = 0; k < 9; k++) sh[wp][k] = s[k];
    __syncthreads();
    if (threadIdx.x < 9) {
        const int k = threadIdx.x;
        double t = 0.0;
        for (int w = 0; w < kTotThreads / 32; w++) t += sh[w][k];
        tot[(size_t)f * 9 + k] = (k >= 3 && k < 6) ? t / P : t;
    }
}

// ------------------------------------------------------------ workspace

struct Session::Mixed {
    int F = 0, S = 1;
    DevBuf<float2> Vb;      // (kInnerMax + 1) blocks of N x 2F (double-FP32)
    DevBuf<float2> W;       // the new Krylov vector (double-FP32)
    DevBuf<float2> cs32, cd32;  // FP32 copies of the coefficients
    DevBuf<double> Ak, Bk;      // interface coefficients of the batch (F x nIf)
    // the first residual's digit product: x's digits (fp16 rows j * 2F + c),
    // the rest of x (FP64), its columns' exponents, the digit partial tiles
    DevBuf<__half> Xd;
    DevBuf<double> Xrem;
    DevBuf<int> colE;
    DevBuf<float> Pd;
    DevBuf<__half> Vh, Vl;  // scaled fp16 pair of the current GEMM operand block
    DevBuf<float> cscK;     // column factors of the Krylov blocks' pairs (2^-14)
    DevBuf<float> cscX;     // column factors of the other operands' pairs
    DevBuf<float> Yp;       // split-K partial products, S blocks
    DevBuf<int> err;        // set by the tensor-core kernel when a wait gives up
    DevBuf<double> Xs, R, Y64, D;
    DevBuf<double2> cs, cd, bt, h, hacc, ycoef;
    DevBuf<float4> dpart;   // Gram-Schmidt dot partials per row chunk (double-FP32 re, im)
    DevBuf<float4> hdf;     // the update's coefficients (-Re h, Im h) in double-FP32
    DevBuf<double> nrm, nrm0, scale, betad, itold, gc;
    DevBuf<double2> gH, gsn, gg;  // Givens state per system
    DevBuf<int> active, act0, act2, mcount, icap;
    DevBuf<unsigned long long> cgsb;  // bytes the Gram-Schmidt kernels moved (timing on)
    DevBuf<double> npart;   // per-block partials of |w|^2
    int dots_grid = 0, upd_grid = 0;  // one resident wave of the Gram-Schmidt kernels
    // batched field
    DevBuf<double> sing, Enode, Fce, tot, Xce, ptot;
    DevBuf<double> gpart;  // split partials of the FP64 GEMV residual (no digits)
    DevBuf<MstGeo> mst_geo;  // per (particle element, point): w J and the unit normal
    DevBuf<float> part;  // field partials per element group (FP32)
    // FP32 far-field pass: element centroids / offsets, split points, weights
    bool far_ready = false;
    DevBuf<float> ecent, qoff, phl, cf32;  // cf32: the charges, kBF systems innermost
    DevBuf<unsigned> near_mask;            // per (point block, element group): chunks with near pairs
    DevBuf<int> en_pad;                    // element nodes, padded to whole chunks (-1)
    FieldTcWork ftc;                       // the tensor-core far pass
    DevBuf<float2> qdf;  // quadrature points in double-FP32 (near pairs)
};

int Session::make_k16()
{
    if (k16_ready && k64_ready) return kOk;
    DSC_TRY(assemble64(false));
    // the conductor-block inverses need only K64: they run on side2 (and
    // side) beside the conversion below on st, joined at the end
    const bool pre_par = pre_on && pre && pre->nb > 0 && !pre->ready;
    SideJoin pj;
    if (pre_par) DSC_TRY(pj.fork(st, side2));
    {
        // K's row digits for the tensor-core first residual take 16 bytes
        // per entry: kept when they fill at most a quarter of the device
        // (a 100k-node scene's 173 GB do not), else the first residual is
        // an FP64 GEMV over K64 per system
        digits = residual_mode == kResidDigits;
        if (residual_mode == kResidAuto) {
            size_t fr = 0, tot = 0;
            DSC_CUDA(cudaMemGetInfo(&fr, &tot));
            digits = 2.0 * kKDigits * (double)ld * N <= 0.25 * (double)tot;
        }
        TimerScope ts(&timer, kTConvertK, st);
        DSC_TRY(Kh16.alloc(ld * N));
        DSC_TRY(Kl16.alloc(ld * N));
        if (digits) DSC_TRY(Kdig.alloc(kKDigits * ld * N));
        else Kdig.release();
        DSC_TRY(rowE.alloc(N));
        DSC_TRY(rsK.alloc(N));
        DSC_TRY(k16_row_scales(K64.p, ld, N, rowE.p, rsK.p, st));
        DSC_TRY(split_transpose_K16(K64.p, ld, N, rowE.p, Kh16.p, Kl16.p, digits ? Kdig.p : nullptr, ld * N, ld,
                                    st));
        // bytes: K read (8), the fp16 pair and the digits written (2 each)
        timer.add_work(kTConvertK, (8.0 + 2.0 * (2 + (digits ? kKDigits : 0))) * N * N);
    }
    if (pre_par) {
        {
            AllocStreamScope ps(side2);  // its buffers ordered on the stream that first uses them
            DSC_TRY(precond_build(*this, side2, side));
        }
        DSC_TRY(pj.done(side2));
        DSC_TRY(pj.join());
    } else if (pre_on) {
        DSC_TRY(precond_build(*this));
    }
    k16_ready = true;
    return kOk;
}

// w_f = cs_f o (sum of the split partials of K v)_f + cd_f o v_f, in FP32
// (the product itself is FP32-accurate): the partials are added with
// TwoSum compensation, the coefficients are FP32 copies.  Two rows per
// thread (8-byte loads of the partials, all splits' loads issued four at a
// time ahead of the additions).  W is written as double-FP32 with a zero
// low part; npart[f][block] = the block's share of |w_f|^2 (k_norm_finish
// adds them).  Row N (a padding row, when N is odd) is neither stored nor
// counted.
__global__ void __launch_bounds__(256) k_apply_epilogue_splits(
    const float *__restrict__ P, int S, size_t split_stride, const float2 *__restrict__ V,
    const float2 *__restrict__ cs, const float2 *__restrict__ cd, float2 *__restrict__ W, int N,
    size_t ld, int F, double *__restrict__ npart)
{
    grid_dep_wait();
    __shared__ float2 sh[8];
    const int i = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int f = blockIdx.y;
    float2 n2 = make_float2(0.f, 0.f);
    if (i < N) {
        const float *pr = P + (size_t)(2 * f) * ld + i, *pi = pr + ld;
        float2 yr0 = make_float2(0.f, 0.f), yr1 = yr0, yi0 = yr0, yi1 = yr0;
        for (int s0 = 0; s0 < S; s0 += 4) {
            float2 u[4], v[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const size_t o = (size_t)min(s0 + q, S - 1) * split_stride;
                u[q] = *(const float2 *)(pr + o);
                v[q] = *(const float2 *)(pi + o);
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if (s0 + q >= S) break;
                float2 a = df_two_sum(yr0.x, u[q].x);
                yr0 = make_float2(a.x, yr0.y + a.y);
                a = df_two_sum(yr1.x, u[q].y);
                yr1 = make_float2(a.x, yr1.y + a.y);
                a = df_two_sum(yi0.x, v[q].x);
                yi0 = make_float2(a.x, yi0.y + a.y);
                a = df_two_sum(yi1.x, v[q].y);
                yi1 = make_float2(a.x, yi1.y + a.y);
            }
        }
        const float4 vr = *(const float4 *)(V + (size_t)(2 * f) * ld + i);
        const float4 vi = *(const float4 *)(V + (size_t)(2 * f + 1) * ld + i);
        const bool two = i + 1 < N;
        const float2 s0 = cs[(size_t)f * N + i], d0 = cd[(size_t)f * N + i];
        const float2 s1 = two ? cs[(size_t)f * N + i + 1] : make_float2(0.f, 0.f);
        const float2 d1 = two ? cd[(size_t)f * N + i + 1] : make_float2(0.f, 0.f);
        const float ar0 = yr0.x + yr0.y, ai0 = yi0.x + yi0.y;
        const float ar1 = yr1.x + yr1.y, ai1 = yi1.x + yi1.y;
        const float wr0 = s0.x * ar0 - s0.y * ai0 + d0.x * vr.x - d0.y * vi.x;
        const float wi0 = s0.x * ai0 + s0.y * ar0 + d0.x * vi.x + d0.y * vr.x;
        const float wr1 = s1.x * ar1 - s1.y * ai1 + d1.x * vr.z - d1.y * vi.z;
        const float wi1 = s1.x * ai1 + s1.y * ar1 + d1.x * vi.z + d1.y * vr.z;
        float2 *wr = W + (size_t)(2 * f) * ld + i, *wi = wr + ld;
        df_mac(n2, make_float2(wr0, 0.f), make_float2(wr0, 0.f));
        df_mac(n2, make_float2(wi0, 0.f), make_float2(wi0, 0.f));
        if (two) {
            *(float4 *)wr = make_float4(wr0, 0.f, wr1, 0.f);
            *(float4 *)wi = make_float4(wi0, 0.f, wi1, 0.f);
            df_mac(n2, make_float2(wr1, 0.f), make_float2(wr1, 0.f));
            df_mac(n2, make_float2(wi1, 0.f), make_float2(wi1, 0.f));
        } else {
            *wr = make_float2(wr0, 0.f);
            *wi = make_float2(wi0, 0.f);
        }
    }
    const double t = df_block_sum(n2, sh);
    if (threadIdx.x == 0) npart[(size_t)f * gridDim.x + blockIdx.x] = t;
}

// Per system f and row i, from the interface coefficients of the batch
// (Ak, Bk: F x nIf; src/assembly_el.c:223-239): s = a - i b (1 on conductor
// rows), d = -1/(2 eps0) on interface rows (0 otherwise), the complex Jacobi
// scale p = 1 / (s K_ii + d), and cs = p s, cd = p d, bt = p (boundary value)
// in FP64 and FP32; R (the first residual, x = 0) = bt.
__global__ void k_prepare_systems(const int *__restrict__ iface_row, const double *__restrict__ Kdiag,
                                  const double *__restrict__ bre, const double *__restrict__ bim,
                                  const double *__restrict__ Ak, const double *__restrict__ Bk, int nIf,
                                  int N, size_t ld, int F, double2 *__restrict__ cs,
                                  double2 *__restrict__ cd, double2 *__restrict__ bt,
                                  float2 *__restrict__ cs32, float2 *__restrict__ cd32,
                                  double *__restrict__ R)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (i >= N) return;
    const int k = iface_row[i];
    const double a = k < 0 ? 1.0 : Ak[(size_t)f * nIf + k];
    const double b = k < 0 ? 0.0 : -Bk[(size_t)f * nIf + k];  // s = a + i b
    const double d = k < 0 ? 0.0 : -0.5 / kEps0;
    const double gr = a * Kdiag[i] + d, gi = b * Kdiag[i];      // s K_ii + d
    const double q = 1.0 / (gr * gr + gi * gi);
    const double pr = gr * q, pi = -gi * q;                      // p = 1 / (s K_ii + d)
    const double2 c1 = make_double2(pr * a - pi * b, pr * b + pi * a);
    const double2 c2 = make_double2(pr * d, pi * d);
    const double2 r = make_double2(pr * bre[i] - pi * bim[i], pr * bim[i] + pi * bre[i]);
    const size_t o = (size_t)f * N + i;
    cs[o] = c1;
    cd[o] = c2;
    bt[o] = r;
    cs32[o] = make_float2((float)c1.x, (float)c1.y);
    cd32[o] = make_float2((float)c2.x, (float)c2.y);
    R[(size_t)(2 * f) * ld + i] = r.x;
    R[(size_t)(2 * f + 1) * ld + i] = r.y;
}

// ------------------------------------------------------------ autotuner
// Split count of the sweep's tensor-core product K V (M = k = N, 2F
// columns), chosen by measurement: the candidates around the heuristic
// (tc_gemm_f16_splits_for: about eleven waves of one CTA per SM) are each
// timed as the product plus the epilogue that sums its partial tiles, three
// times with CUDA events on the session's stream, and the fastest median
// wins.  Results are kept per (device, N, columns) for the whole process,
// so a size is tuned once, by the first solve that meets it.
static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, int>, int> g_tuned;
static bool g_autotune = true;

static int tuned_splits(Session &s, int F, int *out)
{
    Session::Mixed &w = *s.mx;
    const int N = s.N, Nc = 2 * F;
    const size_t ld = s.ld, blk = ld * (size_t)Nc;
    const int h = tc_gemm_f16_splits_for(N, N);
    int dev = 0;
    DSC_CUDA(cudaGetDevice(&dev));
    const auto key = std::make_tuple(dev, N, Nc);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        if (!g_autotune) {
            *out = h;
            return kOk;
        }
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) {
            *out = it->second;
            return kOk;
        }
    }
    std::vector<int> cand;
    for (int c : {h / 3, h / 2, (2 * h) / 3, h, (3 * h) / 2, 2 * h, 3 * h}) {
        const int v = tc_gemm_f16_splits_norm(N, std::max(1, c));
        if (std::find(cand.begin(), cand.end(), v) == cand.end()) cand.push_back(v);
    }
    const int smax = *std::max_element(cand.begin(), cand.end());
    DSC_TRY(w.Yp.alloc(blk * smax));
    cudaEvent_t e0, e1;
    DSC_CUDA(cudaEventCreate(&e0));
    DSC_CUDA(cudaEventCreate(&e1));
    int best = h;
    float best_ms = 1e30f;
    int rc = kOk;
    for (int S : cand) {
        float t[3];
        for (int r = 0; r < 4 && rc == kOk; r++) {
            cudaEventRecord(e0, s.st);
            rc = tc_gemm_3xf16(s.Kh16.p, s.Kl16.p, ld, w.Vh.p, w.Vl.p, ld, N, Nc, N, w.Yp.p, ld, S, w.err.p, s.st,
                               s.rsK.p, w.cscK.p);
            if (rc != kOk) break;
            const dim3 eg((N + 511) / 512, F);
            rc = launch_dependent(k_apply_epilogue_splits, eg, dim3(256), 0, s.st, (const float *)w.Yp.p, S,
                                  blk, (const float2 *)w.Vb.p, (const float2 *)w.cs32.p, (const float2 *)w.cd32.p,
                                  w.W.p, N, ld, F, w.npart.p);
            cudaEventRecord(e1, s.st);
            if (rc == kOk && cudaEventSynchronize(e1) != cudaSuccess) rc = kErrCuda;
            if (r > 0 && rc == kOk) cudaEventElapsedTime(&t[r - 1], e0, e1);  // the first run warms up
        }
        if (rc != kOk) break;
        std::sort(t, t + 3);
        if (t[1] < best_ms) {
            best_ms = t[1];
            best = S;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc == kErrCuda) set_error("split autotuner: %s", cudaGetErrorString(cudaGetLastError()));
    DSC_TRY(rc);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tuned[key] = best;
    }
    *out = best;
    return kOk;
}

int autotune_set(int on)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_autotune = on != 0;
    return kOk;
}

// (N, columns, splits) of every tuned size, up to n of them; returns the count.
int autotune_table(int *rows, int n)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    int k = 0;
    for (const auto &kv : g_tuned) {
        if (rows && k < n) {
            rows[3 * k] = std::get<1>(kv.first);
            rows[3 * k + 1] = std::get<2>(kv.first);
            rows[3 * k + 2] = kv.second;
        }
        k++;
    }
    return k;
}

// One batch of F <= kMaxBatch frequencies.  status (F) receives each
// system's outcome (kSysConverged, kSysCapped: max_iters inner iterations
// taken without reaching tol, kSysStagnated: kOuterMax refinement steps
// taken); the solution and forces of a system that did not converge are
// NaN, the others are those of a batch of converged systems alone.
static int mixed_batch(Session &s, int F, const double *freqs, double tol, unsigned max_iters,
                       double *sigma_host, double *tot_host, unsigned *iters, int *status, double *part_host)
{
    Session::Mixed &w = *s.mx;
    const int N = s.N;
    const size_t ld = s.ld;
    const size_t blk = ld * 2 * (size_t)F;  // one N x 2F block
    cudaStream_t st = s.st;
    Timer *tm = &s.timer;
    // the product's split count for this size (measured once per process)
    DSC_TRY(tuned_splits(s, F, &w.S));
    DSC_TRY(w.Yp.alloc(blk * w.S));
    if (s.pre_on) DSC_TRY(precond_build(s));  // no-op when built for this K
    const bool pre = s.pre_on && s.pre && s.pre->nb > 0 && s.pre->ready;
    if (pre) DSC_TRY(precond_reserve(s, F));
    // coefficients, complex Jacobi, scaled right-hand sides: on the device,
    // from the interface coefficients of each frequency
    const int nIfc = std::max(1, (int)s.nIf);
    {
        std::vector<double> Ak((size_t)F * nIfc, 0.0), Bk((size_t)F * nIfc, 0.0);
        for (int f = 0; f < F; f++)
            if (s.nIf)
                interface_coeffs(s.nIf, s.ifaces.data(), s.mat.data(), freqs[f], &Ak[(size_t)f * nIfc],
                                 &Bk[(size_t)f * nIfc]);
        DSC_TRY(w.Ak.upload(Ak, st));
        DSC_TRY(w.Bk.upload(Bk, st));
        DSC_LAUNCH(k_prepare_systems<<<dim3((N + 255) / 256, F), 256, 0, st>>>(
            s.rows.p, s.Kdiag.p, s.bre.p, s.bim.p, w.Ak.p, w.Bk.p, nIfc, N, ld, F, w.cs.p, w.cd.p,
            w.bt.p, w.cs32.p, w.cd32.p, w.R.p));
        DSC_CUDA(cudaStreamSynchronize(st));  // Ak, Bk go out of scope
    }
    // x = 0; |b_f| is the first residual norm
    DSC_CUDA(cudaMemsetAsync(w.Xs.p, 0, blk * sizeof(double), st));
    std::vector<double> bnorm(F, 0.0);
    const dim3 vg((N + 255) / 256, F);
    constexpr int kRunning = -1;
    std::vector<int> stat(F, kRunning), total_it(F, 0);
    std::vector<double> rn(F);
    for (int outer = 0; outer <= kOuterMax; outer++) {
        // residual norms
        DSC_LAUNCH(k_norms<<<F, 256, 0, st>>>(w.R.p, N, ld, F, w.nrm.p));
        DSC_CUDA(cudaMemcpyAsync(rn.data(), w.nrm.p, F * sizeof(double), cudaMemcpyDeviceToHost, st));
        DSC_CUDA(cudaStreamSynchronize(st));
        if (outer == 0) bnorm = rn;
        // a system leaves the batch once it has converged, used up its
        // share of max_iters or the refinement steps; the others go on
        int nact = 0;
        for (int f = 0; f < F; f++) {
            if (stat[f] != kRunning) continue;
            if (rn[f] <= tol * bnorm[f]) stat[f] = kSysConverged;
            else if ((unsigned)total_it[f] >= max_iters) stat[f] = kSysCapped;
            else if (outer == kOuterMax || !(rn[f] == rn[f])) stat[f] = kSysStagnated;
            else nact++;
        }
        if (nact == 0) break;
        // ---- inner GMRES on M e = r for the active systems, each for at
        // most what is left of its max_iters
        std::vector<int> act(F), mf(F, 0), icap(F, 0);
        std::vector<double> beta(F), sc(F), itol(F);
        int jcap = 0;
        for (int f = 0; f < F; f++) {
            act[f] = stat[f] == kRunning;
            if (act[f]) {
                icap[f] = (int)std::min<unsigned>(kInnerMax, max_iters - (unsigned)total_it[f]);
                jcap = std::max(jcap, icap[f]);
            }
            beta[f] = rn[f];
            sc[f] = act[f] && beta[f] > 0 ? 1.0 / beta[f] : 0.0;
            // reduce the residual to a tenth of the target, but not below
            // what FP32-accurate products can deliver
            itol[f] = std::min(1e-2, std::max(kInnerTol, 0.1 * tol * bnorm[f] / std::max(rn[f], 1e-300)));
        }
        DSC_TRY(w.active.upload(act, st));
        DSC_TRY(w.act0.upload(act, st));
        DSC_TRY(w.scale.upload(sc, st));
        DSC_TRY(w.betad.upload(beta, st));
        DSC_TRY(w.itold.upload(itol, st));
        DSC_TRY(w.icap.upload(icap, st));
        DSC_LAUNCH(k_scale_from64<<<vg, 256, 0, st>>>(w.R.p, w.Vb.p, w.Vh.p, w.Vl.p, N, ld, F, w.scale.p,
                                                      w.active.p));
        GivensState gst{w.gH.p, w.gc.p, w.gsn.p, w.gg.p};
        const int gb = (F + 63) / 64;
        DSC_LAUNCH(k_givens_init<<<gb, 64, 0, st>>>(gst, w.betad.p, F, w.mcount.p));
        std::vector<int> hact(F);
        for (int j = 0; j < jcap; j++) {
            const float2 *vj = w.Vb.p + (size_t)j * blk;
            float2 *vn = w.Vb.p + (size_t)(j + 1) * blk;
            const float *csc = w.cscK.p;
            if (pre)  // right preconditioning: the product is K z with z = P^-1 v_j
                DSC_TRY(precond_apply_v(s, vj, F, w.Vh.p, w.Vl.p, w.cscK.p, w.err.p, &csc));
            {
                // without preconditioning the fp16 pair of v_j was written with v_j
                TimerScope ts(tm, kTGemmK, st);
                DSC_TRY(tc_gemm_3xf16(s.Kh16.p, s.Kl16.p, ld, w.Vh.p, w.Vl.p, ld, N, 2 * F, N, w.Yp.p, ld,
                                      w.S, w.err.p, st, s.rsK.p, csc));
                tm->add_work(kTGemmK, 6.0 * N * N * 2 * F);  // three tf32 products
            }
            {
                TimerScope ts(tm, kTKrylov, st);
                const dim3 eg((N + 511) / 512, F);  // two rows per thread
                DSC_TRY(launch_dependent(k_apply_epilogue_splits, eg, dim3(256), 0, st, w.Yp.p, w.S,
                                         ld * 2 * (size_t)F, vj, w.cs32.p, w.cd32.p, w.W.p, N, ld, F, w.npart.p));
                DSC_CUDA(cudaMemsetAsync(w.hacc.p, 0, (size_t)(j + 1) * F * sizeof(double2), st));
                DSC_LAUNCH(k_norm_finish<<<(F * 32 + 255) / 256, 256, 0, st>>>(w.npart.p, (int)eg.x, F, w.active.p,
                                                                                w.nrm0.p, nullptr, nullptr));
            }
            // classical Gram-Schmidt; the second pass only for the systems
            // whose vector lost more than 1 - 1/sqrt(2) of its norm in the
            // first (the DGKS criterion), decided on the device.  The norms
            // come from block partials written by the epilogue and update
            // kernels.
            unsigned long long *cgsb = tm->on ? w.cgsb.p : nullptr;
            const int nrb = (N + kUpdRows - 1) / kUpdRows, wb = (F * 32 + 255) / 256;
            for (int pass = 0; pass < 2; pass++) {
                TimerScope tc(tm, kTCgs, st);
                const int *mask = pass == 0 ? w.active.p : w.act2.p;
                const int nchunk = (N + kDotRows - 1) / kDotRows;
                const int dunits = nchunk * F * (j + 1), uunits = nrb * F;
                // the four kernels of a pass follow one another by
                // programmatic dependent launch (each waits for the one
                // before at its start)
                DSC_TRY(launch_dependent(k_cgs_dots, dim3(std::min((dunits + 7) / 8, w.dots_grid)), dim3(256), 0, st,
                                         w.Vb.p, blk, w.W.p, N, ld, F, j + 1, mask, w.dpart.p, cgsb));
                DSC_TRY(launch_dependent(k_cgs_dots_reduce, dim3(((j + 1) * F + 7) / 8), dim3(256), 0, st, w.dpart.p,
                                         nchunk, j + 1, F, mask, w.h.p, w.hacc.p, w.hdf.p));
                DSC_TRY(launch_dependent(k_cgs_update, dim3(std::min((uunits + 7) / 8, w.upd_grid)), dim3(256), 0,
                                         st, w.Vb.p, blk, w.W.p, N, ld, F, j + 1, mask, w.hdf.p, w.npart.p, cgsb));
                // pass 0: |w| of every active system and the DGKS decision;
                // pass 1: |w| of the systems that took the second pass
                if (pass == 0)
                    DSC_TRY(launch_dependent(k_norm_finish, dim3(wb), dim3(256), 0, st, w.npart.p, nrb, F,
                                             w.active.p, w.nrm.p, w.nrm0.p, w.act2.p));
                else
                    DSC_TRY(launch_dependent(k_norm_finish, dim3(wb), dim3(256), 0, st, w.npart.p, nrb, F,
                                             w.act2.p, w.nrm.p, (const double *)nullptr, (int *)nullptr));
            }
            {
                TimerScope ts(tm, kTKrylov, st);
                DSC_TRY(launch_dependent(k_givens_step, gb, dim3(64), 0, st, gst, w.hacc.p, w.nrm.p, j, F, w.betad.p,
                                         w.itold.p, (const int *)w.icap.p, w.active.p, w.scale.p, w.mcount.p));
            }
            DSC_CUDA(cudaGetLastError());
            if ((j + 1) % 4 == 0 || j + 1 == jcap) {
                // poll the converged systems every few steps only
                DSC_CUDA(cudaMemcpyAsync(hact.data(), w.active.p, F * sizeof(int), cudaMemcpyDeviceToHost, st));
                DSC_CUDA(cudaStreamSynchronize(st));
                int still = 0;
                for (int f = 0; f < F; f++) still += hact[f];
                if (still == 0) break;
            }
            if (j + 1 < jcap) {
                TimerScope ts(tm, kTKrylov, st);
                DSC_TRY(launch_dependent(k_scale_df, vg, dim3(256), 0, st, w.W.p, vn, w.Vh.p, w.Vl.p, N, ld, F,
                                         w.scale.p, w.active.p));
            }
        }
        // triangular solves on the device, then x += V y below
        DSC_LAUNCH(k_backsolve<<<gb, 64, 0, st>>>(gst, w.mcount.p, w.act0.p, F, w.ycoef.p));
        DSC_CUDA(cudaMemcpyAsync(mf.data(), w.mcount.p, F * sizeof(int), cudaMemcpyDeviceToHost, st));
        DSC_CUDA(cudaStreamSynchronize(st));
        for (int f = 0; f < F; f++)
            if (act[f]) total_it[f] += mf[f];
        // correction d = P^-1 V y, then x += d
        DSC_LAUNCH(k_update_solution<<<vg, 256, 0, st>>>(w.D.p, w.Vb.p, blk, N, ld, F, w.ycoef.p, w.mcount.p));
        if (pre) DSC_TRY(precond_apply_d(s, w.D.p, F, w.err.p));
        DSC_LAUNCH(k_axpy_blocks<<<vg, 256, 0, st>>>(w.Xs.p, w.D.p, N, ld, F));
        if (outer == 0 && !s.digits) {
            // the first residual in FP64 without K's digits: K x by an FP64
            // GEMV over K64 for each system (K read once per system)
            TimerScope ts(tm, kTGemvK, st);
            const int rowblocks = (N + 255) / 256;
            const int S = std::max(1, std::min(64, 4 * 152 / rowblocks)), cols = (N + S - 1) / S;
            DSC_TRY(w.gpart.alloc((size_t)S * 2 * N));
            for (int f = 0; f < F; f++) {
                DSC_LAUNCH(k_gemv_K2<double><<<dim3(rowblocks, S), 256, 0, st>>>(
                    s.K64.p, ld, N, w.Xs.p + (size_t)(2 * f) * ld, w.Xs.p + (size_t)(2 * f + 1) * ld, cols, w.gpart.p));
                DSC_LAUNCH(k_gemv_parts<<<(N + 255) / 256, 256, 0, st>>>(w.gpart.p, S, N, w.Y64.p + (size_t)(2 * f) * ld,
                                                                         w.Y64.p + (size_t)(2 * f + 1) * ld));
                tm->add_work(kTGemvK, 8.0 * N * N);  // bytes of K read
            }
            DSC_LAUNCH(k_residual<<<vg, 256, 0, st>>>(w.Y64.p, w.Xs.p, w.cs.p, w.cd.p, w.bt.p, w.R.p, N, ld, F));
        } else if (outer == 0) {
            // the first residual in FP64: r = bt - M x, with K x from
            //   K's row digits times x's column digits (fixed point, the
            //     21 digit products whose weight is within 2^-48 of the
            //     largest), exact integer sums on the tensor cores
            // + K times the rest of x (below 2^-23 of its column's largest
            //     entry: the fp16-pair product's FP32-level accuracy suffices)
            TimerScope ts(tm, kTResidual, st);
            const int ncol = 2 * F, Sd = tc_digit_splits(N);
            DSC_TRY(x_digits(w.Xs.p, ld, N, ncol, w.Xd.p, ld, w.Xrem.p, ld, w.colE.p, st));
            for (int i = 0; i < kKDigits; i++) {
                const int nj = x_digits_for(i);
                DSC_TRY(tc_gemm_digits(s.Kdig.p + (size_t)i * ld * N, ld, w.Xd.p, ld, N, nj * ncol, N, w.Pd.p, ld,
                                       w.err.p, st));
                DSC_TRY(digit_accumulate(w.Pd.p, Sd, ld, ncol, nj, i, N, w.Y64.p, ld, i == 0, st));
                tm->add_work(kTResidual, (double)N * N * nj * ncol);  // digit multiply-adds
            }
            DSC_TRY(digit_finish(s.rowE.p, w.colE.p, N, ncol, w.Y64.p, ld, st));
            DSC_TRY(split_cols_f16(w.Xrem.p, ld, N, ncol, w.Vh.p, w.Vl.p, ld, w.cscX.p, st));
            DSC_TRY(tc_gemm_3xf16(s.Kh16.p, s.Kl16.p, ld, w.Vh.p, w.Vl.p, ld, N, ncol, N, w.Yp.p, ld, w.S,
                                  w.err.p, st, s.rsK.p, w.cscX.p));
            DSC_TRY(add_splits(w.Yp.p, w.S, ld * (size_t)ncol, ld, N, ncol, w.Y64.p, ld, st));
            DSC_LAUNCH(k_residual<<<vg, 256, 0, st>>>(w.Y64.p, w.Xs.p, w.cs.p, w.cd.p, w.bt.p, w.R.p, N, ld, F));
        } else {
            // later residuals are updated, r -= M d: d is small, so the
            // tensor-core product's error is relative to |r|, not to |b|
            TimerScope ts(tm, kTGemmK, st);
            DSC_TRY(split_cols_f16(w.D.p, ld, N, 2 * F, w.Vh.p, w.Vl.p, ld, w.cscX.p, st));
            DSC_TRY(tc_gemm_3xf16(s.Kh16.p, s.Kl16.p, ld, w.Vh.p, w.Vl.p, ld, N, 2 * F, N, w.Yp.p, ld, w.S,
                                  w.err.p, st, s.rsK.p, w.cscX.p));
            tm->add_work(kTGemmK, 6.0 * N * N * 2 * F);
            DSC_LAUNCH(k_residual_update<<<vg, 256, 0, st>>>(w.Yp.p, w.S, ld * 2 * (size_t)F, w.D.p, w.cs.p,
                                                             w.cd.p, w.R.p, N, ld, F));
        }
        DSC_CUDA(cudaGetLastError());
    }
    if (iters)
        for (int f = 0; f < F; f++) iters[f] = (unsigned)total_it[f];
    for (int f = 0; f < F; f++) status[f] = stat[f] == kRunning ? kSysStagnated : stat[f];
    {
        int herr = 0;
        DSC_CUDA(cudaMemcpyAsync(&herr, w.err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        DSC_CUDA(cudaStreamSynchronize(st));
        if (herr) {
            set_error("tensor-core GEMM: a pipeline wait gave up (code %d)", herr);
            return kErrCuda;
        }
    }

    // ---- batched field at the particle nodes and Maxwell-stress force
    DSC_TRY(s.force_wait());
    ForcePlan &fp = s.force;
    if (fp.P > 0) {
        const int E = s.E, P = fp.P;
        const bool tc = s.field_tc && F <= 64;  // far pairs on the tensor cores
        const int nloop = tc ? kBLoopNear : kBLoop;
        const int nchunk = (E + kBChunk * nloop - 1) / (kBChunk * nloop);  // element groups
        DSC_TRY(w.part.alloc((size_t)(nchunk + kFieldTcSplits) * F * P * 3));
        DSC_TRY(w.sing.alloc((size_t)F * P * 3));
        DSC_TRY(w.Enode.alloc((size_t)F * N * 3));
        DSC_TRY(w.Fce.alloc((size_t)F * std::max(fp.npel, 1) * 3));
        {
            TimerScope ts(tm, kTField, st);
            tm->add_work(kTField, (double)P * E * F);  // (particle node, element) pairs x systems
            // element arrays padded to whole chunks for the field pass's bulk copies
            const int Epad = (E + kBChunk - 1) / kBChunk * kBChunk, E7p = Epad * kTriPts;
            const int ngrp = (F + kBF - 1) / kBF;
            DSC_TRY(w.cf32.alloc((size_t)ngrp * E7p * kBF));
            dim3 cg((E7p + 7) / 8, ngrp), cb(kBF, 8);
            if (s.nen == 6)
                DSC_LAUNCH(k_charge_batched<6><<<cg, cb, 0, st>>>(s.dev.elems.p, E, s.dev.qp.p, w.Xs.p, ld, F, E7p,
                                                                  w.cf32.p));
            else
                DSC_LAUNCH(k_charge_batched<3><<<cg, cb, 0, st>>>(s.dev.elems.p, E, s.dev.qp.p, w.Xs.p, ld, F, E7p,
                                                                  w.cf32.p));
            dim3 fg((P + 127) / 128, nchunk, (F + kBF - 1) / kBF);
            if (!w.far_ready) {
                // geometry of the far-field pass (the session's mesh is fixed)
                DSC_TRY(w.ecent.alloc((size_t)Epad * 8));
                DSC_TRY(w.qoff.alloc((size_t)Epad * kTriPts * 3));
                DSC_TRY(w.phl.alloc((size_t)P * 6));
                DSC_TRY(w.qdf.alloc((size_t)Epad * kTriPts * 3));
                DSC_TRY(w.en_pad.alloc((size_t)Epad * s.nen));
                DSC_CUDA(cudaMemsetAsync(w.ecent.p, 0, (size_t)Epad * 8 * sizeof(float), st));
                DSC_CUDA(cudaMemsetAsync(w.qoff.p, 0, (size_t)Epad * kTriPts * 3 * sizeof(float), st));
                DSC_CUDA(cudaMemsetAsync(w.qdf.p, 0, (size_t)Epad * kTriPts * 3 * sizeof(float2), st));
                DSC_CUDA(cudaMemsetAsync(w.en_pad.p, 0xFF, (size_t)Epad * s.nen * sizeof(int), st));
                DSC_CUDA(cudaMemcpyAsync(w.en_pad.p, s.dev.elems.p, (size_t)E * s.nen * sizeof(int),
                                         cudaMemcpyDeviceToDevice, st));
                DSC_LAUNCH(k_prepare_far<<<(E + 127) / 128, 128, 0, st>>>(s.dev.qp.p, E, w.ecent.p, w.qoff.p,
                                                                          w.qdf.p));
                DSC_LAUNCH(k_points_split<<<(P + 127) / 128, 128, 0, st>>>(fp.ps.px.p, fp.ps.py.p, fp.ps.pz.p,
                                                                           P, w.phl.p));
                if (tc && nloop <= 32) {
                    DSC_TRY(w.near_mask.alloc((size_t)fg.x * fg.y));
                    DSC_LAUNCH(k_near_masks<<<dim3(fg.x, fg.y), 128, 0, st>>>(w.phl.p, P, w.ecent.p, E, nloop,
                                                                           w.near_mask.p));
                } else {
                    w.near_mask.release();
                }
                w.far_ready = true;
            }
            // far pairs on the tensor cores (partials after the FP32 pass's
            // nchunk groups), the near ones on the FP32 pipes; or all on the
            // FP32 pipes
            int ntc = 0;
            if (tc)
                DSC_TRY(field_far_tc(w.phl.p, P, w.ecent.p, w.qoff.p, E, w.cf32.p, E7p, F, w.ftc,
                                     w.part.p + (size_t)nchunk * F * P * 3, kFieldTcSplits, w.err.p, st, &ntc));
            if (s.nen == 6)
                DSC_LAUNCH(k_field_batched_mixed<6><<<fg, 128, 0, st>>>(w.phl.p, fp.ps.coinc.p, P, w.en_pad.p, E,
                                                                        E7p, w.ecent.p, w.qoff.p, w.cf32.p,
                                                                        w.qdf.p, F, w.part.p, w.err.p, tc ? 0 : 1,
                                                                        nloop, tc ? w.near_mask.p : nullptr));
            else
                DSC_LAUNCH(k_field_batched_mixed<3><<<fg, 128, 0, st>>>(w.phl.p, fp.ps.coinc.p, P, w.en_pad.p, E,
                                                                        E7p, w.ecent.p, w.qoff.p, w.cf32.p,
                                                                        w.qdf.p, F, w.part.p, w.err.p, tc ? 0 : 1,
                                                                        nloop, tc ? w.near_mask.p : nullptr));
            const int sb = (P * 32 + 127) / 128;
            if (s.nen == 6)
                DSC_LAUNCH(k_field_singular_apply<6><<<sb, 128, 0, st>>>(P, s.dev.elems.p, s.dev.normals.p,
                                                                         fp.ps.sp_ptr.p, fp.ps.sp.p, fp.tmap.p,
                                                                         s.Wsing.p, w.Xs.p, ld, F, w.sing.p));
            else
                DSC_LAUNCH(k_field_singular_apply<3><<<sb, 128, 0, st>>>(P, s.dev.elems.p, s.dev.normals.p,
                                                                         fp.ps.sp_ptr.p, fp.ps.sp.p, fp.tmap.p,
                                                                         s.Wsing.p, w.Xs.p, ld, F, w.sing.p));
            DSC_CUDA(cudaMemsetAsync(w.Enode.p, 0, (size_t)F * N * 3 * sizeof(double), st));
            const size_t nt = (size_t)F * P * 3;
            DSC_LAUNCH(k_field_batched_reduce<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(
                w.part.p, nchunk + ntc, F, P, w.sing.p, fp.ids.p, N, w.Enode.p));
        }
        TimerScope ts(tm, kTMst, st);
        if (fp.npel > 0) {
            DSC_TRY(w.mst_geo.alloc((size_t)fp.npel * kTriPts));
            const int gq = (fp.npel * kTriPts + 127) / 128;
            dim3 mg((fp.npel + 127) / 128, F);
            if (s.nen == 6) {
                DSC_LAUNCH(k_mst_geometry<6><<<gq, 128, 0, st>>>(s.dev.x.p, s.dev.y.p, s.dev.z.p, s.dev.elems.p,
                                                                 fp.pel.p, fp.npel, w.mst_geo.p));
                DSC_LAUNCH(k_mst_batched<6><<<mg, 128, 0, st>>>(s.dev.elems.p, fp.pel.p, fp.npel, w.mst_geo.p,
                                                                w.Enode.p, N, F, s.eps_medium, w.Fce.p));
            } else {
                DSC_LAUNCH(k_mst_geometry<3><<<gq, 128, 0, st>>>(s.dev.x.p, s.dev.y.p, s.dev.z.p, s.dev.elems.p,
                                                                 fp.pel.p, fp.npel, w.mst_geo.p));
                DSC_LAUNCH(k_mst_batched<3><<<mg, 128, 0, st>>>(s.dev.elems.p, fp.pel.p, fp.npel, w.mst_geo.p,
                                                                w.Enode.p, N, F, s.eps_medium, w.Fce.p));
            }
        }
        DSC_LAUNCH(k_mst_batched_totals<<<F, kTotThreads, 0, st>>>(w.Fce.p, fp.npel, F, s.dev.x.p, s.dev.y.p,
                                                                   s.dev.z.p, fp.ids.p, P, w.tot.p));
        DSC_CUDA(cudaGetLastError());
        if (tot_host)
            DSC_CUDA(cudaMemcpyAsync(tot_host, w.tot.p, (size_t)F * 9 * sizeof(double),
                                     cudaMemcpyDeviceToHost, st));
        if (part_host && fp.npart > 0) {
            // per particle: force, centre, scale, torque of every system
            DSC_TRY(w.Xce.alloc((size_t)std::max(fp.npel, 1) * 3));
            DSC_TRY(w.ptot.alloc((size_t)F * fp.npart * kPartVals));
            DSC_TRY(mst_centres(s.dev, fp, w.Xce.p, st));
            DSC_TRY(mst_particles(fp, s.dev.x.p, s.dev.y.p, s.dev.z.p, w.Fce.p, (size_t)fp.npel * 3, w.Xce.p, F,
                                  w.ptot.p, st));
            DSC_CUDA(cudaMemcpyAsync(part_host, w.ptot.p, (size_t)F * fp.npart * kPartVals * sizeof(double),
                                     cudaMemcpyDeviceToHost, st));
        }
    } else if (tot_host) {
        memset(tot_host, 0, (size_t)F * 9 * sizeof(double));
    }
    if (sigma_host) {
        // the solution with Re / Im halves, as the reference's vB: column c
        // of Xs (2f = Re, 2f + 1 = Im of frequency f) is row c of the
        // caller's F x 2N array, so one strided copy moves them all.  The
        // caller's pages are written once on the host first, while the
        // field kernels run: a device-to-host copy into pages never touched
        // (fresh pageable memory) runs several times slower.
        memset(sigma_host, 0, (size_t)F * 2 * N * sizeof(double));
        DSC_CUDA(cudaMemcpy2DAsync(sigma_host, (size_t)N * sizeof(double), w.Xs.p, ld * sizeof(double),
                                   (size_t)N * sizeof(double), (size_t)2 * F, cudaMemcpyDeviceToHost, st));
    }
    int herr = 0;  // the field pass's staging waits
    DSC_CUDA(cudaMemcpyAsync(&herr, w.err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    DSC_CUDA(cudaStreamSynchronize(st));
    if (herr) {
        set_error("batched field: a shared-memory staging wait gave up (code %d)", herr);
        return kErrCuda;
    }
    // no result for a system that did not converge
    const double nan = std::numeric_limits<double>::quiet_NaN();
    for (int f = 0; f < F; f++) {
        if (status[f] == kSysConverged) continue;
        if (tot_host) std::fill(tot_host + (size_t)f * 9, tot_host + (size_t)f * 9 + 9, nan);
        if (part_host && s.force.npart > 0)
            std::fill(part_host + (size_t)f * s.force.npart * kPartVals,
                      part_host + (size_t)(f + 1) * s.force.npart * kPartVals, nan);
        if (sigma_host) std::fill(sigma_host + (size_t)f * 2 * N, sigma_host + (size_t)(f + 1) * 2 * N, nan);
    }
    return kOk;
}

int Session::collect_timing(double *ms, int *count, double *work)
{
    DSC_TRY(timer.collect(ms, count, work));
    if (mx && mx->cgsb.p) {
        unsigned long long b = 0;
        DSC_CUDA(cudaMemcpyAsync(&b, mx->cgsb.p, sizeof b, cudaMemcpyDeviceToHost, st));
        DSC_CUDA(cudaMemsetAsync(mx->cgsb.p, 0, sizeof b, st));
        DSC_CUDA(cudaStreamSynchronize(st));
        work[kTCgs] += (double)b;
    }
    return kOk;
}

int Session::solve_mixed(unsigned nfreq, const double *freqs, double tol, unsigned max_iters,
                         double *sigma_host, double *forces_host, unsigned *iters)
{
    last_status.assign(nfreq, kSysStagnated);
    last_particles.clear();
    if (max_iters == 0) {
        set_error("mixed solve: max_iters must be at least 1");
        return kErrArg;
    }
    DSC_TRY(make_k16());
    // the force plan (its particles) is joined by the assembly
    DSC_TRY(force_wait());
    last_particles.assign((size_t)nfreq * force.npart * kPartVals, std::numeric_limits<double>::quiet_NaN());
    if (!mx) mx = new Mixed();
    Mixed &w = *mx;
    const int Fmax = (int)std::min<unsigned>(nfreq, kMaxBatch);
    if (w.F < Fmax) {
        const size_t blk = ld * 2 * (size_t)Fmax;
        DSC_TRY(w.Vb.alloc(blk * (kInnerMax + 1)));
        w.S = tc_gemm_f16_splits_for(N, N);
        DSC_TRY(w.Vh.alloc(blk));
        DSC_TRY(w.Vl.alloc(blk));
        DSC_TRY(w.cscK.alloc(2 * (size_t)Fmax));
        DSC_TRY(w.cscX.alloc(2 * (size_t)Fmax));
        {
            std::vector<float> c(2 * (size_t)Fmax, 1.0f / kVScale);
            DSC_TRY(w.cscK.upload(c, st));
        }
        DSC_TRY(w.Yp.alloc(blk * w.S));
        DSC_TRY(w.err.alloc(1));
        DSC_CUDA(cudaMemsetAsync(w.err.p, 0, sizeof(int), st));
        DSC_TRY(w.W.alloc(blk));
        DSC_TRY(w.Xd.alloc(kXDigits * blk));
        DSC_TRY(w.Xrem.alloc(blk));
        DSC_TRY(w.colE.alloc(2 * (size_t)Fmax));
        DSC_TRY(w.Pd.alloc((size_t)tc_digit_splits(N) * kXDigits * blk));
        DSC_TRY(w.cs.alloc((size_t)Fmax * N));
        DSC_TRY(w.cd.alloc((size_t)Fmax * N));
        DSC_TRY(w.bt.alloc((size_t)Fmax * N));
        DSC_TRY(w.cs32.alloc((size_t)Fmax * N));
        DSC_TRY(w.cd32.alloc((size_t)Fmax * N));
        DSC_TRY(w.Xs.alloc(blk));
        DSC_TRY(w.R.alloc(blk));
        DSC_TRY(w.Y64.alloc(blk));
        DSC_TRY(w.D.alloc(blk));
        DSC_TRY(w.h.alloc((size_t)(kInnerMax + 1) * Fmax));
        DSC_TRY(w.dpart.alloc((size_t)((N + kDotRows - 1) / kDotRows) * (kInnerMax + 1) * Fmax));
        DSC_TRY(w.hacc.alloc((size_t)(kInnerMax + 1) * Fmax));
        DSC_TRY(w.hdf.alloc((size_t)(kInnerMax + 1) * Fmax));
        DSC_TRY(w.ycoef.alloc((size_t)kInnerMax * Fmax));
        DSC_TRY(w.nrm.alloc(Fmax));
        DSC_TRY(w.scale.alloc(Fmax));
        DSC_TRY(w.active.alloc(Fmax));
        DSC_TRY(w.act0.alloc(Fmax));
        DSC_TRY(w.act2.alloc(Fmax));
        DSC_TRY(w.nrm0.alloc(Fmax));
        DSC_TRY(w.betad.alloc(Fmax));
        DSC_TRY(w.itold.alloc(Fmax));
        DSC_TRY(w.icap.alloc(Fmax));
        DSC_TRY(w.gc.alloc((size_t)Fmax * kInnerMax));
        DSC_TRY(w.gsn.alloc((size_t)Fmax * kInnerMax));
        DSC_TRY(w.gg.alloc((size_t)Fmax * (kInnerMax + 1)));
        DSC_TRY(w.gH.alloc((size_t)Fmax * (kInnerMax + 1) * kInnerMax));
        DSC_TRY(w.mcount.alloc(Fmax));
        DSC_TRY(w.tot.alloc((size_t)Fmax * 9));
        DSC_TRY(w.cgsb.alloc(1));
        {
            int dev = 0, nsm = 0, o1 = 0, o2 = 0;
            DSC_CUDA(cudaGetDevice(&dev));
            DSC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
            DSC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o1, k_cgs_dots, 256, 0));
            DSC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o2, k_cgs_update, 256, 0));
            w.dots_grid = nsm * std::max(1, o1);
            w.upd_grid = nsm * std::max(1, o2);
        }
        DSC_TRY(w.npart.alloc((size_t)Fmax * ((N + kUpdRows - 1) / kUpdRows)));
        DSC_CUDA(cudaMemsetAsync(w.cgsb.p, 0, sizeof(unsigned long long), st));
        // the padding rows of the blocks are never read but keep them finite
        DSC_CUDA(cudaMemsetAsync(w.Vb.p, 0, blk * (kInnerMax + 1) * sizeof(float2), st));
        DSC_CUDA(cudaMemsetAsync(w.W.p, 0, blk * sizeof(float2), st));
        w.F = Fmax;
    }
    for (unsigned f0 = 0; f0 < nfreq; f0 += kMaxBatch) {
        const int F = (int)std::min<unsigned>(kMaxBatch, nfreq - f0);
        DSC_TRY(mixed_batch(*this, F, freqs + f0, tol, max_iters,
                            sigma_host ? sigma_host + (size_t)f0 * 2 * N : nullptr,
                            forces_host ? forces_host + (size_t)f0 * 9 : nullptr,
                            iters ? iters + f0 : nullptr, last_status.data() + f0,
                            last_particles.data() + (size_t)f0 * force.npart * kPartVals));
    }
    return kOk;
}

}  // namespace dsc

namespace dsc {
void destroy_mixed(Session::Mixed *m) { delete m; }
}  // namespace dsc
