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
#include <complex>
#include <vector>

#include "../../include/depsolver_cuda.h"
#include "dsc_blas.cuh"
#include "dsc_common.cuh"
#include "dsc_field.h"
#include "dsc_internal.h"
#include "dsc_session.h"
#include "dsc_singular.cuh"
#include "dsc_tcgemm.h"

namespace dsc {

typedef std::complex<double> cplx;

constexpr int kMaxBatch = 64;   // frequencies per batch
constexpr int kInnerMax = 80;   // Krylov dimension of one inner solve
constexpr int kOuterMax = 6;    // refinement steps
constexpr double kInnerTol = 1e-6;

// ------------------------------------------------------------ GEMM (SIMT)
// C (M x Nc) = A (M x Kd) * B (Kd x Nc), all column-major.  64 x 64 tile,
// 256 threads with 4 x 4 outputs each, k-steps of 16.  TA = element of A,
// TC = accumulation and C type.
template <typename TA, typename TB, typename TC>
__global__ void __launch_bounds__(256) k_gemm_cm(const TA *__restrict__ A, size_t lda,
                                                 const TB *__restrict__ B, size_t ldb,
                                                 TC *__restrict__ C, size_t ldc, int M, int Nc,
                                                 int Kd)
{
    __shared__ TC As[16][64 + 1];
    __shared__ TC Bs[16][64 + 1];
    const int m0 = blockIdx.x * 64, n0 = blockIdx.y * 64;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    TC acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
        for (int v = 0; v < 4; v++) acc[u][v] = 0;
    for (int k0 = 0; k0 < Kd; k0 += 16) {
        for (int t = threadIdx.x; t < 16 * 64; t += 256) {
            int kk = t / 64, mm = t % 64;
            int m = m0 + mm, k = k0 + kk;
            As[kk][mm] = (m < M && k < Kd) ? (TC)A[(size_t)k * lda + m] : (TC)0;
            int nn = t / 16, kb = t % 16;
            int n = n0 + nn, k2 = k0 + kb;
            Bs[kb][nn] = (n < Nc && k2 < Kd) ? (TC)B[(size_t)n * ldb + k2] : (TC)0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; kk++) {
            TC a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                a[u] = As[kk][ty + 16 * u];
                b[u] = Bs[kk][tx + 16 * u];
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int v = 0; v < 4; v++) acc[u][v] += a[u] * b[v];
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
        int m = m0 + ty + 16 * u;
        if (m >= M) continue;
#pragma unroll
        for (int v = 0; v < 4; v++) {
            int n = n0 + tx + 16 * v;
            if (n < Nc) C[(size_t)n * ldc + m] = acc[u][v];
        }
    }
}

__global__ void k_to_float(const double *__restrict__ x, float *__restrict__ y, size_t n)
{
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n;
         t += (size_t)gridDim.x * blockDim.x)
        y[t] = (float)x[t];
}

// K32 = (float) K64, leading dimension kept.
__global__ void k_k_to_float(const double *__restrict__ K, float *__restrict__ K32, size_t n)
{
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n;
         t += (size_t)gridDim.x * blockDim.x)
        K32[t] = (float)K[t];
}

// Vectors of the batch: column 2f = Re, 2f + 1 = Im of system f, stride ld.
// w_f = cs_f o Y_f + cd_f o v_f (complex), Y from the K product.
template <typename TY>
__global__ void k_apply_epilogue(const TY *__restrict__ Y, const double *__restrict__ V,
                                 const double2 *__restrict__ cs, const double2 *__restrict__ cd,
                                 double *__restrict__ W, int N, size_t ld, int F)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (i >= N || f >= F) return;
    const double yr = (double)Y[(size_t)(2 * f) * ld + i], yi = (double)Y[(size_t)(2 * f + 1) * ld + i];
    const double vr = V[(size_t)(2 * f) * ld + i], vi = V[(size_t)(2 * f + 1) * ld + i];
    const double2 s = cs[(size_t)f * N + i], d = cd[(size_t)f * N + i];
    W[(size_t)(2 * f) * ld + i] = s.x * yr - s.y * yi + d.x * vr - d.y * vi;
    W[(size_t)(2 * f + 1) * ld + i] = s.x * yi + s.y * yr + d.x * vi + d.y * vr;
}

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

// Complex dots h[k][f] = <V_k,f, W_f> = sum conj(v) w, for k < nk; one block
// per (f, k), fixed-order block reduction.
__global__ void __launch_bounds__(256) k_cgs_dots(const double *__restrict__ Vb, size_t vstride,
                                                  const double *__restrict__ W, int N, size_t ld,
                                                  int F, const int *__restrict__ active,
                                                  double2 *__restrict__ h)
{
    __shared__ double sh[32];
    const int f = blockIdx.x, k = blockIdx.y;
    if (!active[f]) return;
    const double *vr = Vb + (size_t)k * vstride + (size_t)(2 * f) * ld;
    const double *vi = vr + ld;
    const double *wr = W + (size_t)(2 * f) * ld, *wi = wr + ld;
    double sr = 0.0, si = 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        sr += vr[i] * wr[i] + vi[i] * wi[i];
        si += vr[i] * wi[i] - vi[i] * wr[i];
    }
    double a = block_sum(sr, sh);
    double b = block_sum(si, sh);
    if (threadIdx.x == 0) h[(size_t)k * F + f] = make_double2(a, b);
}

// W_f -= sum_k h[k][f] V_k,f  (and hacc += h)
__global__ void k_cgs_update(const double *__restrict__ Vb, size_t vstride, double *__restrict__ W,
                             int N, size_t ld, int F, int nk, const int *__restrict__ active,
                             const double2 *__restrict__ h, double2 *__restrict__ hacc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (i >= N || !active[f]) return;
    double wr = W[(size_t)(2 * f) * ld + i], wi = W[(size_t)(2 * f + 1) * ld + i];
    for (int k = 0; k < nk; k++) {
        const double2 c = h[(size_t)k * F + f];
        const double vr = Vb[(size_t)k * vstride + (size_t)(2 * f) * ld + i];
        const double vi = Vb[(size_t)k * vstride + (size_t)(2 * f + 1) * ld + i];
        wr -= c.x * vr - c.y * vi;
        wi -= c.x * vi + c.y * vr;
    }
    W[(size_t)(2 * f) * ld + i] = wr;
    W[(size_t)(2 * f + 1) * ld + i] = wi;
    if (hacc && i == 0)
        for (int k = 0; k < nk; k++) {
            double2 a = hacc[(size_t)k * F + f], c = h[(size_t)k * F + f];
            hacc[(size_t)k * F + f] = make_double2(a.x + c.x, a.y + c.y);
        }
}

// nrm[f] = |W_f| (one block per system)
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

// V_f = W_f * scale[f]
__global__ void k_scale_into(const double *__restrict__ W, double *__restrict__ V, int N, size_t ld,
                             int F, const double *__restrict__ scale, const int *__restrict__ active)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (i >= N) return;
    const double s = active[f] ? scale[f] : 0.0;
    V[(size_t)(2 * f) * ld + i] = W[(size_t)(2 * f) * ld + i] * s;
    V[(size_t)(2 * f + 1) * ld + i] = W[(size_t)(2 * f + 1) * ld + i] * s;
}

// X_f += sum_k y[k][f] V_k,f for k < m[f]
__global__ void k_update_solution(double *__restrict__ X, const double *__restrict__ Vb,
                                  size_t vstride, int N, size_t ld, int F,
                                  const double2 *__restrict__ y, const int *__restrict__ m)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (i >= N) return;
    double xr = X[(size_t)(2 * f) * ld + i], xi = X[(size_t)(2 * f + 1) * ld + i];
    for (int k = 0; k < m[f]; k++) {
        const double2 c = y[(size_t)k * F + f];
        const double vr = Vb[(size_t)k * vstride + (size_t)(2 * f) * ld + i];
        const double vi = Vb[(size_t)k * vstride + (size_t)(2 * f + 1) * ld + i];
        xr += c.x * vr - c.y * vi;
        xi += c.x * vi + c.y * vr;
    }
    X[(size_t)(2 * f) * ld + i] = xr;
    X[(size_t)(2 * f + 1) * ld + i] = xi;
}

// ------------------------------------------------------- batched field
// Charge weights of Re(sigma_f) at every quadrature point:
// cf[f][e*7+q] = w_q J_q sum_k N_k(q) Re sigma_f(node k).
template <int NEN>
__global__ void k_charge_batched(const int *__restrict__ elems, int E, const double *__restrict__ qp,
                                 const double *__restrict__ X, size_t ld, int F,
                                 double *__restrict__ cf)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (t >= E * kTriPts) return;
    const int e = t / kTriPts, q = t % kTriPts;
    double N6[NEN];
    shape<NEN>(c_tri7[q][0], c_tri7[q][1], N6);
    const double *xr = X + (size_t)(2 * f) * ld;
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < NEN; k++) s += N6[k] * xr[elems[(size_t)e * NEN + k]];
    cf[(size_t)f * E * kTriPts + t] = qp[(size_t)t * 4 + 3] * s;
}

constexpr int kBF = 16;   // frequencies per thread in the batched field
constexpr int kBChunk = 32;

// part[chunk][f][p][3]: regular contributions of one element chunk.
template <int NEN>
__global__ void __launch_bounds__(128) k_field_batched(const double *__restrict__ px,
                                                       const double *__restrict__ py,
                                                       const double *__restrict__ pz,
                                                       const int4 *__restrict__ coinc, int P,
                                                       const int *__restrict__ elems, int E,
                                                       const double *__restrict__ qp,
                                                       const double *__restrict__ cf, int F,
                                                       double *__restrict__ part)
{
    __shared__ double s_q[kBChunk * kTriPts * 4];
    __shared__ double s_c[kBF][kBChunk * kTriPts];
    __shared__ int s_en[kBChunk * NEN];
    const int chunk = blockIdx.y, fg = blockIdx.z;
    const int e0 = chunk * kBChunk, ne = min(kBChunk, E - e0);
    const int f0 = fg * kBF, nf = min(kBF, F - f0);
    for (int t = threadIdx.x; t < ne * kTriPts * 4; t += blockDim.x)
        s_q[t] = qp[(size_t)e0 * kTriPts * 4 + t];
    for (int t = threadIdx.x; t < kBF * ne * kTriPts; t += blockDim.x) {
        int ff = t / (ne * kTriPts), r = t % (ne * kTriPts);
        s_c[ff][r] = ff < nf ? cf[(size_t)(f0 + ff) * E * kTriPts + (size_t)e0 * kTriPts + r] : 0.0;
    }
    for (int t = threadIdx.x; t < ne * NEN; t += blockDim.x) s_en[t] = elems[(size_t)e0 * NEN + t];
    __syncthreads();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const double x = px[p], y = py[p], z = pz[p];
    const int4 c = coinc[p];
    double acc[kBF][3];
#pragma unroll
    for (int ff = 0; ff < kBF; ff++) acc[ff][0] = acc[ff][1] = acc[ff][2] = 0.0;
    for (int e = 0; e < ne; e++) {
        bool sing = false;
#pragma unroll
        for (int k = 0; k < NEN; k++) {
            int v = s_en[e * NEN + k];
            sing |= (v == c.x) | (v == c.y) | (v == c.z) | (v == c.w);
        }
        if (sing && c.x >= 0) continue;
#pragma unroll
        for (int q = 0; q < kTriPts; q++) {
            const double *Q = s_q + (e * kTriPts + q) * 4;
            double dx = x - Q[0], dy = y - Q[1], dz = z - Q[2];
            double inv = rsqrt(dx * dx + dy * dy + dz * dz);
            double i3 = inv * inv * inv;
            double gx = dx * i3, gy = dy * i3, gz = dz * i3;
#pragma unroll
            for (int ff = 0; ff < kBF; ff++) {
                double cq = s_c[ff][e * kTriPts + q];
                acc[ff][0] += cq * gx;
                acc[ff][1] += cq * gy;
                acc[ff][2] += cq * gz;
            }
        }
    }
    for (int ff = 0; ff < nf; ff++)
        for (int d = 0; d < 3; d++)
            part[(((size_t)chunk * F + f0 + ff) * P + p) * 3 + d] = acc[ff][d];
}

// Singular elements of each point, FP64 subdivision once per (point,
// element), applied to every frequency; lanes = frequencies afterwards.
template <int NEN>
__global__ void __launch_bounds__(128) k_field_batched_singular(
    const double *__restrict__ px, const double *__restrict__ py, const double *__restrict__ pz,
    int P, const int *__restrict__ elems, const double *__restrict__ X, const double *__restrict__ Y,
    const double *__restrict__ Z, const double *__restrict__ normals, const int *__restrict__ sp_ptr,
    const int4 *__restrict__ sp, const double *__restrict__ Xs, size_t ld, int F,
    double *__restrict__ sing)
{
    const int p = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (p >= P) return;
    const double xe[3] = {px[p], py[p], pz[p]};
    const double A = 0.5 / kEps0 / kPi2, B = 0.5 / kEps0;
    double acc[2][3] = {{0, 0, 0}, {0, 0, 0}};  // lanes own f = lane, lane + 32
    for (int t = sp_ptr[p]; t < sp_ptr[p + 1]; t++) {
        const int4 tu = sp[t];
        const int e = tu.x, s = tu.y;
        double Xe[NEN][3];
        int nodes[NEN];
#pragma unroll
        for (int k = 0; k < NEN; k++) {
            int v = elems[(size_t)e * NEN + k];
            nodes[k] = v;
            Xe[k][0] = X[v];
            Xe[k][1] = Y[v];
            Xe[k][2] = Z[v];
        }
        const double n[3] = {normals[3 * (size_t)tu.z], normals[3 * (size_t)tu.z + 1],
                             normals[3 * (size_t)tu.z + 2]};
        double sub[3 * NEN];
        warp_singular_H<NEN, 1>(s, Xe, xe, n, sub);
        for (int r = 0; r < 2; r++) {
            const int f = lane + 32 * r;
            if (f >= F) continue;
            const double *xr = Xs + (size_t)(2 * f) * ld;
#pragma unroll
            for (int k = 0; k < NEN; k++) {
                const double sr = xr[nodes[k]];
#pragma unroll
                for (int c = 0; c < 3; c++) acc[r][c] += A * sub[3 * k + c] * sr;
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
__global__ void k_field_batched_reduce(const double *__restrict__ part, int nchunk, int F, int P,
                                       const double *__restrict__ sing, const int *__restrict__ ids,
                                       int N, double *__restrict__ Enode)
{
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= (size_t)F * P * 3) return;
    const int d = (int)(t % 3), p = (int)((t / 3) % P), f = (int)(t / (3 * (size_t)P));
    const double A = 0.5 / kEps0 / kPi2;
    double s = 0.0;
    for (int c = 0; c < nchunk; c++) s += part[(size_t)c * F * P * 3 + t];
    Enode[((size_t)f * N + ids[p]) * 3 + d] = A * s + sing[t];
}

// Maxwell stress per (particle element, frequency).
template <int NEN>
__global__ void k_mst_batched(const double *__restrict__ X, const double *__restrict__ Y,
                              const double *__restrict__ Z, const int *__restrict__ elems,
                              const int *__restrict__ pel, int npel, const double *__restrict__ Enode,
                              int N, int F, double eps, double *__restrict__ Fce)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (t >= npel) return;
    const int e = pel[t];
    const double *En0 = Enode + (size_t)f * N * 3;
    double Xe[NEN][3], En[NEN][3], N6[NEN], XL[3], n[3];
#pragma unroll
    for (int k = 0; k < NEN; k++) {
        int v = elems[(size_t)e * NEN + k];
        Xe[k][0] = X[v];
        Xe[k][1] = Y[v];
        Xe[k][2] = Z[v];
        En[k][0] = En0[3 * (size_t)v];
        En[k][1] = En0[3 * (size_t)v + 1];
        En[k][2] = En0[3 * (size_t)v + 2];
    }
    double I0 = 0.0, I1 = 0.0, I2 = 0.0;
    for (int q = 0; q < kTriPts; q++) {
        double l1 = c_tri7[q][0], l2 = c_tri7[q][1];
        shape<NEN>(l1, l2, N6);
        double J = map_point<NEN>(Xe, l1, l2, N6, XL);
        local_normal<NEN>(Xe, l1, l2, n);
        double Ex = 0.0, Ey = 0.0, Ez = 0.0;
#pragma unroll
        for (int k = 0; k < NEN; k++) {
            Ex += En[k][0] * N6[k];
            Ey += En[k][1] * N6[k];
            Ez += En[k][2] * N6[k];
        }
        double NE = Ex * n[0] + Ey * n[1] + Ez * n[2];
        double Esq = Ex * Ex + Ey * Ey + Ez * Ez;
        double A = J * c_tri7[q][2];
        I0 += A * (Ex * NE - 0.5 * Esq * n[0]);
        I1 += A * (Ey * NE - 0.5 * Esq * n[1]);
        I2 += A * (Ez * NE - 0.5 * Esq * n[2]);
    }
    const double A = 0.5 * eps;
    double *o = Fce + ((size_t)f * npel + t) * 3;
    o[0] = A * I0;
    o[1] = A * I1;
    o[2] = A * I2;
}

// tot[f][9]: Fcm, Xcm, sum |Fce| (one warp per frequency, fixed order)
__global__ void k_mst_batched_totals(const double *__restrict__ Fce, int npel, int F,
                                     const double *__restrict__ X, const double *__restrict__ Y,
                                     const double *__restrict__ Z, const int *__restrict__ ids, int P,
                                     double *__restrict__ tot)
{
    const int f = blockIdx.x, lane = threadIdx.x;
    const double *Fc = Fce + (size_t)f * npel * 3;
    double s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int t = lane; t < npel; t += 32)
        for (int d = 0; d < 3; d++) {
            s[d] += Fc[3 * (size_t)t + d];
            s[6 + d] += fabs(Fc[3 * (size_t)t + d]);
        }
    for (int q = lane; q < P; q += 32) {
        s[3] += X[ids[q]];
        s[4] += Y[ids[q]];
        s[5] += Z[ids[q]];
    }
    for (int k = 0; k < 9; k++) s[k] = warp_sum(s[k]);
    if (lane == 0)
        for (int k = 0; k < 9; k++) tot[(size_t)f * 9 + k] = (k >= 3 && k < 6) ? s[k] / P : s[k];
}

// ------------------------------------------------------------ workspace

struct Session::Mixed {
    int F = 0, S = 1;
    DevBuf<double> Vb;      // (kInnerMax + 1) blocks of N x 2F (FP64)
    DevBuf<float> Vh, Vl;   // tf32 pair of the current Krylov block
    DevBuf<float> Yp;       // split-K partial products, S blocks
    DevBuf<int> err;        // set by the tensor-core kernel when a wait gives up
    DevBuf<double> W, Xs, R, Y64;
    DevBuf<double2> cs, cd, bt, h, hacc, ycoef;
    DevBuf<double> nrm, scale;
    DevBuf<int> active, mcount;
    // batched field
    DevBuf<double> cf, part, sing, Enode, Fce, tot;
};

int Session::make_k32()
{
    if (k32_ready) return kOk;
    DSC_TRY(assemble64());
    DSC_TRY(Kth.alloc(ld * N));
    DSC_TRY(Ktl.alloc(ld * N));
    DSC_TRY(split_transpose_K(K64.p, ld, N, Kth.p, Ktl.p, ld, st));
    k32_ready = true;
    return kOk;
}

// w_f = cs_f o (sum of the split partials of K v)_f + cd_f o v_f
__global__ void k_apply_epilogue_splits(const float *__restrict__ P, int S, size_t split_stride,
                                        const double *__restrict__ V, const double2 *__restrict__ cs,
                                        const double2 *__restrict__ cd, double *__restrict__ W, int N,
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
    const double vr = V[(size_t)(2 * f) * ld + i], vi = V[(size_t)(2 * f + 1) * ld + i];
    const double2 s = cs[(size_t)f * N + i], d = cd[(size_t)f * N + i];
    W[(size_t)(2 * f) * ld + i] = s.x * yr - s.y * yi + d.x * vr - d.y * vi;
    W[(size_t)(2 * f + 1) * ld + i] = s.x * yi + s.y * yr + d.x * vi + d.y * vr;
}

template <typename TA, typename TB, typename TC>
static int gemm(const TA *A, size_t lda, const TB *B, size_t ldb, TC *C, size_t ldc, int M, int Nc,
                int Kd, cudaStream_t st)
{
    dim3 g((M + 63) / 64, (Nc + 63) / 64);
    DSC_LAUNCH(k_gemm_cm<TA, TB, TC><<<g, 256, 0, st>>>(A, lda, B, ldb, C, ldc, M, Nc, Kd));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

// One batch of F <= kMaxBatch frequencies.
static int mixed_batch(Session &s, int F, const double *freqs, double tol, unsigned max_iters,
                       double *sigma_host, double *tot_host, unsigned *iters)
{
    Session::Mixed &w = *s.mx;
    const int N = s.N;
    const size_t ld = s.ld;
    const size_t blk = ld * 2 * (size_t)F;  // one N x 2F block
    cudaStream_t st = s.st;
    Timer *tm = &s.timer;
    // coefficients, complex Jacobi, scaled right-hand sides
    std::vector<double2> hcs((size_t)F * N), hcd((size_t)F * N), hbt((size_t)F * N);
    std::vector<double> bnorm(F, 0.0);
    for (int f = 0; f < F; f++) {
        std::vector<double> a, b, d;
        s.coeffs(freqs[f], a, b, d);
        for (int i = 0; i < N; i++) {
            cplx sv(a[i], -b[i]);
            cplx diag = sv * s.Kdiag_host[i] + d[i];
            cplx p = 1.0 / diag;
            cplx c1 = p * sv, c2 = p * d[i];
            cplx rhs = p * cplx(s.mbc[3 * (size_t)i], s.mbc[3 * (size_t)(i + N)]);
            hcs[(size_t)f * N + i] = make_double2(c1.real(), c1.imag());
            hcd[(size_t)f * N + i] = make_double2(c2.real(), c2.imag());
            hbt[(size_t)f * N + i] = make_double2(rhs.real(), rhs.imag());
            bnorm[f] += std::norm(rhs);
        }
        bnorm[f] = sqrt(bnorm[f]);
    }
    DSC_TRY(w.cs.upload(hcs, st));
    DSC_TRY(w.cd.upload(hcd, st));
    DSC_TRY(w.bt.upload(hbt, st));
    // x = 0, r = bt
    DSC_CUDA(cudaMemsetAsync(w.Xs.p, 0, blk * sizeof(double), st));
    {
        std::vector<double> r(blk, 0.0);
        for (int f = 0; f < F; f++)
            for (int i = 0; i < N; i++) {
                r[(size_t)(2 * f) * ld + i] = hbt[(size_t)f * N + i].x;
                r[(size_t)(2 * f + 1) * ld + i] = hbt[(size_t)f * N + i].y;
            }
        DSC_CUDA(cudaMemcpyAsync(w.R.p, r.data(), blk * sizeof(double), cudaMemcpyHostToDevice, st));
        DSC_CUDA(cudaStreamSynchronize(st));
    }
    const dim3 vg((N + 255) / 256, F);
    std::vector<int> done(F, 0), total_it(F, 0);
    std::vector<double> rn(F);
    for (int outer = 0; outer <= kOuterMax; outer++) {
        // residual norms
        DSC_LAUNCH(k_norms<<<F, 256, 0, st>>>(w.R.p, N, ld, F, w.nrm.p));
        DSC_CUDA(cudaMemcpyAsync(rn.data(), w.nrm.p, F * sizeof(double), cudaMemcpyDeviceToHost, st));
        DSC_CUDA(cudaStreamSynchronize(st));
        int nact = 0;
        for (int f = 0; f < F; f++) {
            done[f] = rn[f] <= tol * bnorm[f];
            nact += !done[f];
        }
        if (nact == 0) break;
        if (outer == kOuterMax) {
            set_error("mixed solve: residual above tolerance after %d refinement steps", kOuterMax);
            return kErrNoConverge;
        }
        // ---- inner GMRES on M e = r for the active systems
        std::vector<int> act(F), mf(F, 0);
        std::vector<double> beta(F), sc(F);
        for (int f = 0; f < F; f++) {
            act[f] = !done[f];
            beta[f] = rn[f];
            sc[f] = act[f] && beta[f] > 0 ? 1.0 / beta[f] : 0.0;
        }
        DSC_TRY(w.active.upload(act, st));
        DSC_TRY(w.scale.upload(sc, st));
        DSC_LAUNCH(k_scale_into<<<vg, 256, 0, st>>>(w.R.p, w.Vb.p, N, ld, F, w.scale.p, w.active.p));
        std::vector<std::vector<cplx>> H(F), g(F), cs_(F), sn(F);
        for (int f = 0; f < F; f++) {
            H[f].assign((size_t)(kInnerMax + 1) * kInnerMax, 0.0);
            g[f].assign(kInnerMax + 1, 0.0);
            g[f][0] = beta[f];
            cs_[f].assign(kInnerMax, 0.0);
            sn[f].assign(kInnerMax, 0.0);
        }
        std::vector<int> inner_act = act;
        int j = 0;
        std::vector<double2> hh((size_t)(kInnerMax + 1) * F);
        std::vector<double> hn(F);
        for (j = 0; j < kInnerMax; j++) {
            const double *vj = w.Vb.p + (size_t)j * blk;
            double *vn = w.Vb.p + (size_t)(j + 1) * blk;
            {
                TimerScope ts(tm, kTGemmK, st);
                DSC_TRY(split_vec(vj, w.Vh.p, w.Vl.p, blk, st));
                DSC_TRY(tc_gemm_3xtf32(s.Kth.p, s.Ktl.p, ld, w.Vh.p, w.Vl.p, ld, N, 2 * F, N, w.Yp.p, ld,
                                       w.S, w.err.p, st));
            }
            TimerScope ts(tm, kTKrylov, st);
            DSC_LAUNCH(k_apply_epilogue_splits<<<vg, 256, 0, st>>>(w.Yp.p, w.S, ld * 2 * (size_t)F, vj, w.cs.p,
                                                                   w.cd.p, w.W.p, N, ld, F));
            DSC_CUDA(cudaMemsetAsync(w.hacc.p, 0, (size_t)(j + 1) * F * sizeof(double2), st));
            for (int pass = 0; pass < 2; pass++) {
                DSC_LAUNCH(k_cgs_dots<<<dim3(F, j + 1), 256, 0, st>>>(w.Vb.p, blk, w.W.p, N, ld, F, w.active.p, w.h.p));
                DSC_LAUNCH(k_cgs_update<<<vg, 256, 0, st>>>(w.Vb.p, blk, w.W.p, N, ld, F, j + 1, w.active.p, w.h.p,
                                                 w.hacc.p));
            }
            DSC_LAUNCH(k_norms<<<F, 256, 0, st>>>(w.W.p, N, ld, F, w.nrm.p));
            DSC_CUDA(cudaGetLastError());
            DSC_CUDA(cudaMemcpyAsync(hh.data(), w.hacc.p, (size_t)(j + 1) * F * sizeof(double2),
                                     cudaMemcpyDeviceToHost, st));
            DSC_CUDA(cudaMemcpyAsync(hn.data(), w.nrm.p, F * sizeof(double), cudaMemcpyDeviceToHost, st));
            DSC_CUDA(cudaStreamSynchronize(st));
            int still = 0;
            for (int f = 0; f < F; f++) {
                sc[f] = 0.0;
                if (!inner_act[f]) continue;
                std::vector<cplx> col(j + 2);
                for (int k = 0; k <= j; k++) col[k] = cplx(hh[(size_t)k * F + f].x, hh[(size_t)k * F + f].y);
                col[j + 1] = hn[f];
                for (int k = 0; k < j; k++) {
                    cplx t1 = cs_[f][k] * col[k] + sn[f][k] * col[k + 1];
                    cplx t2 = -std::conj(sn[f][k]) * col[k] + cs_[f][k] * col[k + 1];
                    col[k] = t1;
                    col[k + 1] = t2;
                }
                double aa = std::abs(col[j]), bb = std::abs(col[j + 1]);
                double nu = sqrt(aa * aa + bb * bb);
                cplx c, sgn;
                if (aa == 0.0) {
                    c = 0.0;
                    sn[f][j] = 1.0;
                    col[j] = col[j + 1];
                } else {
                    c = aa / nu;
                    sgn = col[j] / aa;
                    sn[f][j] = sgn * std::conj(col[j + 1]) / nu;
                    col[j] = sgn * nu;
                }
                cs_[f][j] = c;
                col[j + 1] = 0.0;
                for (int k = 0; k <= j; k++) H[f][(size_t)k * kInnerMax + j] = col[k];
                g[f][j + 1] = -std::conj(sn[f][j]) * g[f][j];
                g[f][j] = cs_[f][j] * g[f][j];
                mf[f] = j + 1;
                double est = std::abs(g[f][j + 1]);
                if (est <= kInnerTol * beta[f] || hn[f] == 0.0) inner_act[f] = 0;
                else {
                    still++;
                    sc[f] = 1.0 / hn[f];
                }
            }
            if (still == 0 || j + 1 == kInnerMax) break;
            // next basis vector for the systems still iterating
            DSC_TRY(w.scale.upload(sc, st));
            DSC_TRY(w.active.upload(inner_act, st));
            DSC_LAUNCH(k_scale_into<<<vg, 256, 0, st>>>(w.W.p, vn, N, ld, F, w.scale.p, w.active.p));
        }
        // triangular solves and x += V y
        std::vector<double2> yc((size_t)kInnerMax * F, make_double2(0.0, 0.0));
        for (int f = 0; f < F; f++) {
            if (!act[f]) {
                mf[f] = 0;
                continue;
            }
            int m = mf[f];
            std::vector<cplx> yv(m);
            for (int k = m - 1; k >= 0; k--) {
                cplx t = g[f][k];
                for (int q = k + 1; q < m; q++) t -= H[f][(size_t)k * kInnerMax + q] * yv[q];
                yv[k] = t / H[f][(size_t)k * kInnerMax + k];
            }
            for (int k = 0; k < m; k++) yc[(size_t)k * F + f] = make_double2(yv[k].real(), yv[k].imag());
            total_it[f] += m;
        }
        DSC_TRY(w.ycoef.upload(yc, st));
        DSC_TRY(w.mcount.upload(mf, st));
        DSC_LAUNCH(k_update_solution<<<vg, 256, 0, st>>>(w.Xs.p, w.Vb.p, blk, N, ld, F, w.ycoef.p, w.mcount.p));
        // FP64 residual r = bt - M x
        {
            TimerScope ts(tm, kTResidual, st);
            DSC_TRY((gemm<double, double, double>(s.K64.p, ld, w.Xs.p, ld, w.Y64.p, ld, N, 2 * F, N, st)));
            DSC_LAUNCH(k_residual<<<vg, 256, 0, st>>>(w.Y64.p, w.Xs.p, w.cs.p, w.cd.p, w.bt.p, w.R.p, N, ld, F));
        }
        DSC_CUDA(cudaGetLastError());
    }
    if (iters)
        for (int f = 0; f < F; f++) iters[f] = (unsigned)total_it[f];
    (void)max_iters;
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
    ForcePlan &fp = s.force;
    if (fp.P > 0) {
        const int E = s.E, P = fp.P;
        const int nchunk = (E + kBChunk - 1) / kBChunk;
        DSC_TRY(w.cf.alloc((size_t)F * E * kTriPts));
        DSC_TRY(w.part.alloc((size_t)nchunk * F * P * 3));
        DSC_TRY(w.sing.alloc((size_t)F * P * 3));
        DSC_TRY(w.Enode.alloc((size_t)F * N * 3));
        DSC_TRY(w.Fce.alloc((size_t)F * std::max(fp.npel, 1) * 3));
        {
            TimerScope ts(tm, kTField, st);
            dim3 cg((E * kTriPts + 255) / 256, F);
            if (s.nen == 6) DSC_LAUNCH(k_charge_batched<6><<<cg, 256, 0, st>>>(s.dev.elems.p, E, s.dev.qp.p, w.Xs.p, ld, F, w.cf.p));
            else DSC_LAUNCH(k_charge_batched<3><<<cg, 256, 0, st>>>(s.dev.elems.p, E, s.dev.qp.p, w.Xs.p, ld, F, w.cf.p));
            dim3 fg((P + 127) / 128, nchunk, (F + kBF - 1) / kBF);
            if (s.nen == 6)
                DSC_LAUNCH(k_field_batched<6><<<fg, 128, 0, st>>>(fp.ps.px.p, fp.ps.py.p, fp.ps.pz.p, fp.ps.coinc.p, P,
                                                       s.dev.elems.p, E, s.dev.qp.p, w.cf.p, F, w.part.p));
            else
                DSC_LAUNCH(k_field_batched<3><<<fg, 128, 0, st>>>(fp.ps.px.p, fp.ps.py.p, fp.ps.pz.p, fp.ps.coinc.p, P,
                                                       s.dev.elems.p, E, s.dev.qp.p, w.cf.p, F, w.part.p));
            const int sb = (P * 32 + 127) / 128;
            if (s.nen == 6)
                DSC_LAUNCH(k_field_batched_singular<6><<<sb, 128, 0, st>>>(
                    fp.ps.px.p, fp.ps.py.p, fp.ps.pz.p, P, s.dev.elems.p, s.dev.x.p, s.dev.y.p, s.dev.z.p,
                    s.dev.normals.p, fp.ps.sp_ptr.p, fp.ps.sp.p, w.Xs.p, ld, F, w.sing.p));
            else
                DSC_LAUNCH(k_field_batched_singular<3><<<sb, 128, 0, st>>>(
                    fp.ps.px.p, fp.ps.py.p, fp.ps.pz.p, P, s.dev.elems.p, s.dev.x.p, s.dev.y.p, s.dev.z.p,
                    s.dev.normals.p, fp.ps.sp_ptr.p, fp.ps.sp.p, w.Xs.p, ld, F, w.sing.p));
            DSC_CUDA(cudaMemsetAsync(w.Enode.p, 0, (size_t)F * N * 3 * sizeof(double), st));
            const size_t nt = (size_t)F * P * 3;
            DSC_LAUNCH(k_field_batched_reduce<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(
                w.part.p, nchunk, F, P, w.sing.p, fp.ids.p, N, w.Enode.p));
        }
        TimerScope ts(tm, kTMst, st);
        if (fp.npel > 0) {
            dim3 mg((fp.npel + 127) / 128, F);
            if (s.nen == 6)
                DSC_LAUNCH(k_mst_batched<6><<<mg, 128, 0, st>>>(s.dev.x.p, s.dev.y.p, s.dev.z.p, s.dev.elems.p, fp.pel.p,
                                                     fp.npel, w.Enode.p, N, F, s.eps_medium, w.Fce.p));
            else
                DSC_LAUNCH(k_mst_batched<3><<<mg, 128, 0, st>>>(s.dev.x.p, s.dev.y.p, s.dev.z.p, s.dev.elems.p, fp.pel.p,
                                                     fp.npel, w.Enode.p, N, F, s.eps_medium, w.Fce.p));
        }
        DSC_LAUNCH(k_mst_batched_totals<<<F, 32, 0, st>>>(w.Fce.p, fp.npel, F, s.dev.x.p, s.dev.y.p, s.dev.z.p,
                                               fp.ids.p, P, w.tot.p));
        DSC_CUDA(cudaGetLastError());
        if (tot_host)
            DSC_CUDA(cudaMemcpyAsync(tot_host, w.tot.p, (size_t)F * 9 * sizeof(double),
                                     cudaMemcpyDeviceToHost, st));
    } else if (tot_host) {
        memset(tot_host, 0, (size_t)F * 9 * sizeof(double));
    }
    if (sigma_host) {
        // the solution with Re / Im halves, as the reference's vB
        for (int f = 0; f < F; f++) {
            double *o = sigma_host + (size_t)f * 2 * N;
            DSC_CUDA(cudaMemcpyAsync(o, w.Xs.p + (size_t)(2 * f) * ld, N * sizeof(double),
                                     cudaMemcpyDeviceToHost, st));
            DSC_CUDA(cudaMemcpyAsync(o + N, w.Xs.p + (size_t)(2 * f + 1) * ld, N * sizeof(double),
                                     cudaMemcpyDeviceToHost, st));
        }
    }
    DSC_CUDA(cudaStreamSynchronize(st));
    return kOk;
}

int Session::solve_mixed(unsigned nfreq, const double *freqs, double tol, unsigned max_iters,
                         double *sigma_host, double *forces_host, unsigned *iters)
{
    DSC_TRY(make_k32());
    if (!mx) mx = new Mixed();
    Mixed &w = *mx;
    const int Fmax = (int)std::min<unsigned>(nfreq, kMaxBatch);
    if (w.F < Fmax) {
        const size_t blk = ld * 2 * (size_t)Fmax;
        DSC_TRY(w.Vb.alloc(blk * (kInnerMax + 1)));
        w.S = tc_gemm_splits_for(N, N);
        DSC_TRY(w.Vh.alloc(blk));
        DSC_TRY(w.Vl.alloc(blk));
        DSC_TRY(w.Yp.alloc(blk * w.S));
        DSC_TRY(w.err.alloc(1));
        DSC_CUDA(cudaMemsetAsync(w.err.p, 0, sizeof(int), st));
        DSC_TRY(w.W.alloc(blk));
        DSC_TRY(w.Xs.alloc(blk));
        DSC_TRY(w.R.alloc(blk));
        DSC_TRY(w.Y64.alloc(blk));
        DSC_TRY(w.h.alloc((size_t)(kInnerMax + 1) * Fmax));
        DSC_TRY(w.hacc.alloc((size_t)(kInnerMax + 1) * Fmax));
        DSC_TRY(w.ycoef.alloc((size_t)kInnerMax * Fmax));
        DSC_TRY(w.nrm.alloc(Fmax));
        DSC_TRY(w.scale.alloc(Fmax));
        DSC_TRY(w.active.alloc(Fmax));
        DSC_TRY(w.mcount.alloc(Fmax));
        DSC_TRY(w.tot.alloc((size_t)Fmax * 9));
        // the padding rows of the blocks are never read but keep them finite
        DSC_CUDA(cudaMemsetAsync(w.Vb.p, 0, blk * (kInnerMax + 1) * sizeof(double), st));
        w.F = Fmax;
    }
    for (unsigned f0 = 0; f0 < nfreq; f0 += kMaxBatch) {
        const int F = (int)std::min<unsigned>(kMaxBatch, nfreq - f0);
        DSC_TRY(mixed_batch(*this, F, freqs + f0, tol, max_iters,
                            sigma_host ? sigma_host + (size_t)f0 * 2 * N : nullptr,
                            forces_host ? forces_host + (size_t)f0 * 9 : nullptr,
                            iters ? iters + f0 : nullptr));
    }
    return kOk;
}

}  // namespace dsc

namespace dsc {
void destroy_mixed(Session::Mixed *m) { delete m; }
}  // namespace dsc
