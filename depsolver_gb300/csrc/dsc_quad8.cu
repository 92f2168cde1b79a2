// dsc_quad8.cu -- the 8-node quadrilateral (quad8) element family on the
// FP64 path: assembly of K, the field and potential at points, the
// Maxwell-stress force and the node normals.
//
// The reference recognises quad8 (element type 9, src/preProcess.c:142-146)
// but integrates only triangles and its driver rejects quads
// (src/depSolver.c:180-183); this family is an extension, built from the
// same ingredients as the triangle path:
//  * serendipity element on the parent square [-1, 1]^2, nodes 1-4 the
//    corners (-1,-1), (1,-1), (1,1), (-1,1) counter-clockwise (the normal
//    dX/dxi x dX/deta points to the side from which they turn
//    counter-clockwise, as the triangles' does), nodes 5-8 the mid-sides of
//    edges 1-2, 2-3, 3-4, 4-1;
//  * regular pairs: the 3 x 3 Gauss-Legendre product rule;
//  * singular pairs (the collocation node is a node of the element): the
//    parent square cut into triangles with their apex at that node (two for
//    a corner, three for a mid-side node); on each, the triangle path's
//    schemes with the apex as the singular vertex -- the Duffy map with
//    8 x 8 Gauss-Legendre / Gauss-Jacobi points for the weakly singular G
//    (src/kernelIntegrals.c:311-345) and the 8-level subdivision with the
//    7-point rule and the innermost triangle left out for H and for the
//    field's gradient (src/kernelIntegrals.c:472-593);
//  * the field on a node adds the jump (sigma / (2 eps0)) n once, with that
//    node's own sigma and normal (the triangle path keeps the reference's
//    jump per singular element with the element's first node, for parity).
// K has the triangle path's meaning (K[c * ld + i]: C int G N_c on
// conductor rows, -int dG/dn_i N_c on interface rows), so the row forms,
// the solvers and the sessions' FP64 operators take it unchanged.
#include <math.h>

#include <algorithm>
#include <vector>

#include "dsc_common.cuh"
#include "dsc_internal.h"
#include "dsc_quad8.h"

namespace dsc {

// 3-point Gauss-Legendre rule on [-1, 1] (nodes -+sqrt(3/5), 0; weights
// 5/9, 8/9, 5/9).
__constant__ double c_gl3[3][2] = {{-0.7745966692414834, 0.5555555555555556},
                                   {0.0, 0.8888888888888888},
                                   {0.7745966692414834, 0.5555555555555556}};
// parent coordinates of the eight nodes
__constant__ double c_q8n[8][2] = {{-1.0, -1.0}, {1.0, -1.0}, {1.0, 1.0}, {-1.0, 1.0},
                                   {0.0, -1.0},  {1.0, 0.0},  {0.0, 1.0}, {-1.0, 0.0}};
static const double h_q8n[8][2] = {{-1.0, -1.0}, {1.0, -1.0}, {1.0, 1.0}, {-1.0, 1.0},
                                   {0.0, -1.0},  {1.0, 0.0},  {0.0, 1.0}, {-1.0, 0.0}};

// Shape functions and their derivatives at (xi, eta); nodes at parent
// points P (c_q8n or h_q8n).
__host__ __device__ __forceinline__ void q8_shape(const double (*P)[2], double xi, double eta, double *N,
                                                  double *Nx, double *Ne)
{
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const double a = xi * P[k][0], b = eta * P[k][1];
        N[k] = 0.25 * (1.0 + a) * (1.0 + b) * (a + b - 1.0);
        Nx[k] = 0.25 * P[k][0] * (1.0 + b) * (2.0 * a + b);
        Ne[k] = 0.25 * P[k][1] * (1.0 + a) * (a + 2.0 * b);
    }
#pragma unroll
    for (int k = 4; k < 8; k++) {
        if (P[k][0] == 0.0) {  // edges 1-2 and 3-4
            const double b = eta * P[k][1];
            N[k] = 0.5 * (1.0 - xi * xi) * (1.0 + b);
            Nx[k] = -xi * (1.0 + b);
            Ne[k] = 0.5 * P[k][1] * (1.0 - xi * xi);
        } else {  // edges 2-3 and 4-1
            const double a = xi * P[k][0];
            N[k] = 0.5 * (1.0 + a) * (1.0 - eta * eta);
            Nx[k] = 0.5 * P[k][0] * (1.0 - eta * eta);
            Ne[k] = -eta * (1.0 + a);
        }
    }
}

// X(xi, eta), its surface Jacobian |dX/dxi x dX/deta| (returned) and, when
// nrm is not null, the unit normal; N receives the shape values.
__host__ __device__ __forceinline__ double q8_map(const double (*P)[2], const double (*X)[3], double xi, double eta,
                                                  double *XL, double *N, double *nrm)
{
    double Nx[8], Ne[8], t1[3] = {0, 0, 0}, t2[3] = {0, 0, 0};
    q8_shape(P, xi, eta, N, Nx, Ne);
#pragma unroll
    for (int d = 0; d < 3; d++) {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            s += N[k] * X[k][d];
            t1[d] += Nx[k] * X[k][d];
            t2[d] += Ne[k] * X[k][d];
        }
        XL[d] = s;
    }
    const double n0 = t1[1] * t2[2] - t2[1] * t1[2];
    const double n1 = t2[0] * t1[2] - t1[0] * t2[2];
    const double n2 = t1[0] * t2[1] - t2[0] * t1[1];
    const double J = sqrt(n0 * n0 + n1 * n1 + n2 * n2);
    if (nrm) {
        nrm[0] = n0 / J;
        nrm[1] = n1 / J;
        nrm[2] = n2 / J;
    }
    return J;
}

// The triangles of the parent square with their apex at node s (0-based):
// tri[t] = (apex, P1, P2) counter-clockwise; returns their number.
__host__ __device__ __forceinline__ int q8_apex_tris(const double (*P)[2], int s, double (*tri)[3][2])
{
    const int c = s < 4 ? s : s - 4;  // corner index, or the first corner of the edge
    int nt = 0;
    const int count = s < 4 ? 2 : 3;
    for (int t = 0; t < count; t++) {
        const int a = (c + 1 + t) & 3, b = (c + 2 + t) & 3;
        tri[nt][0][0] = P[s][0];
        tri[nt][0][1] = P[s][1];
        tri[nt][1][0] = P[a][0];
        tri[nt][1][1] = P[a][1];
        tri[nt][2][0] = P[b][0];
        tri[nt][2][1] = P[b][1];
        nt++;
    }
    return nt;
}

// Weakly singular G of node s: out[k] = int N_k / r dS over the element
// (xe = X at node s), warp-cooperative, every lane holds the sums.
__device__ void q8_warp_singular_G(int s, const double (*X)[3], const double *xe, double *out)
{
    const int lane = threadIdx.x & 31;
    double tri[3][3][2];
    const int nt = q8_apex_tris(c_q8n, s, tri);
    double acc[8];
#pragma unroll
    for (int k = 0; k < 8; k++) acc[k] = 0.0;
    for (int p = lane; p < 64 * nt; p += 32) {
        const int t = p / 64, i = (p / 8) % 8, j = p % 8;
        const double u1 = c_gl8[i][0], w1 = c_gl8[i][1], u2 = c_gj8[j][0], w2 = c_gj8[j][1];
        const double l1 = 0.25 * (1.0 + u1) * (1.0 + u2), l2 = 0.25 * (1.0 - u1) * (1.0 + u2);
        const double a1 = tri[t][1][0] - tri[t][0][0], a2 = tri[t][1][1] - tri[t][0][1];
        const double b1 = tri[t][2][0] - tri[t][0][0], b2 = tri[t][2][1] - tri[t][0][1];
        const double det = a1 * b2 - a2 * b1;
        const double xi = tri[t][0][0] + l1 * a1 + l2 * b1, eta = tri[t][0][1] + l1 * a2 + l2 * b2;
        double XL[3], N[8];
        const double J = q8_map(c_q8n, X, xi, eta, XL, N, nullptr);
        const double dx = xe[0] - XL[0], dy = xe[1] - XL[1], dz = xe[2] - XL[2];
        const double A = w1 * w2 * 0.125 * det * J / sqrt(dx * dx + dy * dy + dz * dz);
#pragma unroll
        for (int k = 0; k < 8; k++) acc[k] += A * N[k];
    }
#pragma unroll
    for (int k = 0; k < 8; k++) out[k] = warp_sum(acc[k]);
}

// Strongly singular H of node s (FLAG 0: out[k] = -int (d . n) / r^3 N_k dS
// with the node normal n, d = xe - X; FLAG 1: out[3k + c] = int d_c / r^3
// N_k dS), warp-cooperative: per apex triangle 8 levels x 3 sub-triangles x
// 7 points towards the apex, the innermost triangle left out.
template <int FLAG>
__device__ void q8_warp_singular_H(int s, const double (*X)[3], const double *xe, const double *n, double *out)
{
    constexpr int NOUT = FLAG ? 24 : 8;
    const int lane = threadIdx.x & 31;
    double tri[3][3][2];
    const int nt = q8_apex_tris(c_q8n, s, tri);
    // sub-triangles of the unit triangle away from its vertex (0, 0)
    const double xs0[3][3][2] = {{{1.0, 0.0}, {0.5, 0.5}, {0.5, 0.0}},
                                 {{0.5, 0.0}, {0.5, 0.5}, {0.0, 0.5}},
                                 {{0.5, 0.5}, {0.0, 1.0}, {0.0, 0.5}}};
    double acc[NOUT];
#pragma unroll
    for (int k = 0; k < NOUT; k++) acc[k] = 0.0;
    for (int p = lane; p < nt * kSubdiv * 3 * kTriPts; p += 32) {
        const int t = p / (kSubdiv * 3 * kTriPts), r = p % (kSubdiv * 3 * kTriPts);
        const int m = r / (3 * kTriPts), i = (r / kTriPts) % 3, q = r % kTriPts;
        const double scale = ldexp(1.0, -m), Jsub = ldexp(1.0, -2 * (m + 1));
        const double M1 = c_tri7[q][0], M2 = c_tri7[q][1], M3 = 1.0 - M1 - M2, W = c_tri7[q][2];
        const double l1 = (xs0[i][0][0] * M1 + xs0[i][1][0] * M2 + xs0[i][2][0] * M3) * scale;
        const double l2 = (xs0[i][0][1] * M1 + xs0[i][1][1] * M2 + xs0[i][2][1] * M3) * scale;
        const double a1 = tri[t][1][0] - tri[t][0][0], a2 = tri[t][1][1] - tri[t][0][1];
        const double b1 = tri[t][2][0] - tri[t][0][0], b2 = tri[t][2][1] - tri[t][0][1];
        const double det = a1 * b2 - a2 * b1;
        const double xi = tri[t][0][0] + l1 * a1 + l2 * b1, eta = tri[t][0][1] + l1 * a2 + l2 * b2;
        double XL[3], N[8];
        const double J = q8_map(c_q8n, X, xi, eta, XL, N, nullptr);
        const double dx = xe[0] - XL[0], dy = xe[1] - XL[1], dz = xe[2] - XL[2];
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double A = Jsub * W * det * J / (r2 * sqrt(r2));
        if (FLAG == 0) {
            const double An = A * (dx * n[0] + dy * n[1] + dz * n[2]);
#pragma unroll
            for (int k = 0; k < 8; k++) acc[k] -= An * N[k];
        } else {
#pragma unroll
            for (int k = 0; k < 8; k++) {
                acc[3 * k + 0] += A * dx * N[k];
                acc[3 * k + 1] += A * dy * N[k];
                acc[3 * k + 2] += A * dz * N[k];
            }
        }
    }
#pragma unroll
    for (int k = 0; k < NOUT; k++) out[k] = warp_sum(acc[k]);
}

__device__ __forceinline__ void q8_load(const double *__restrict__ X, const double *__restrict__ Y,
                                        const double *__restrict__ Z, const int *__restrict__ en, double (*Xe)[3])
{
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int v = en[k];
        Xe[k][0] = X[v];
        Xe[k][1] = Y[v];
        Xe[k][2] = Z[v];
    }
}

// ------------------------------------------------------------ assembly
// Pass 1, regular pairs: T[(i - r0) * E + e][k] = fac_i * sum over the
// 3 x 3 points of w J N_k * (1/r on conductor rows, (d . n_i)/r^3 on
// interface rows, fac -1 there); 0 where node i belongs to element e.
__global__ void k_q8_pairs(const double *__restrict__ X, const double *__restrict__ Y, const double *__restrict__ Z,
                           const double *__restrict__ normals, const int *__restrict__ row_kind,
                           const double *__restrict__ row_fac, const int *__restrict__ elems, int E, int r0, int r1,
                           double *__restrict__ T)
{
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t npair = (size_t)(r1 - r0) * E;
    if (t >= npair) return;
    const int i = r0 + (int)(t / E), e = (int)(t % E);
    const int *en = elems + (size_t)e * 8;
    double *o = T + t * 8;
    bool sing = false;
#pragma unroll
    for (int k = 0; k < 8; k++) sing |= en[k] == i;
    double acc[8];
#pragma unroll
    for (int k = 0; k < 8; k++) acc[k] = 0.0;
    if (!sing) {
        double Xe[8][3];
        q8_load(X, Y, Z, en, Xe);
        const double xi_[3] = {X[i], Y[i], Z[i]};
        const double n[3] = {normals[3 * (size_t)i], normals[3 * (size_t)i + 1], normals[3 * (size_t)i + 2]};
        const bool isH = row_kind[i] == 1;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                double XL[3], N[8];
                const double J = q8_map(c_q8n, Xe, c_gl3[a][0], c_gl3[b][0], XL, N, nullptr);
                const double dx = xi_[0] - XL[0], dy = xi_[1] - XL[1], dz = xi_[2] - XL[2];
                const double r2 = dx * dx + dy * dy + dz * dz, ri = 1.0 / sqrt(r2);
                const double w = c_gl3[a][1] * c_gl3[b][1] * J;
                const double g = isH ? w * ri * ri * ri * (dx * n[0] + dy * n[1] + dz * n[2]) : w * ri;
#pragma unroll
                for (int k = 0; k < 8; k++) acc[k] += g * N[k];
            }
        const double fac = row_fac[i];
#pragma unroll
        for (int k = 0; k < 8; k++) acc[k] *= fac;
    }
#pragma unroll
    for (int k = 0; k < 8; k++) o[k] = acc[k];
}

// Pass 1, singular pairs: warp per (row i, element e) with i a node of e,
// rows [r0, r1) only; conductor rows C * G, interface rows H (which carries
// its minus sign).
__global__ void k_q8_singular_pairs(const double *__restrict__ X, const double *__restrict__ Y,
                                    const double *__restrict__ Z, const double *__restrict__ normals,
                                    const int *__restrict__ row_kind, const double *__restrict__ row_fac,
                                    const int *__restrict__ elems, const int *__restrict__ sp_row,
                                    const int *__restrict__ sp_elem, const int *__restrict__ sp_pos, int nsp, int E,
                                    int r0, int r1, double *__restrict__ T)
{
    const int w = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (w >= nsp) return;
    const int i = sp_row[w];
    if (i < r0 || i >= r1) return;
    const int e = sp_elem[w], s = sp_pos[w];
    double Xe[8][3], out[8];
    q8_load(X, Y, Z, elems + (size_t)e * 8, Xe);
    const double xe[3] = {X[i], Y[i], Z[i]};
    if (row_kind[i] == 0) {
        q8_warp_singular_G(s, Xe, xe, out);
        const double fac = row_fac[i];
#pragma unroll
        for (int k = 0; k < 8; k++) out[k] *= fac;
    } else {
        const double n[3] = {normals[3 * (size_t)i], normals[3 * (size_t)i + 1], normals[3 * (size_t)i + 2]};
        q8_warp_singular_H<0>(s, Xe, xe, n, out);
    }
    if (lane == 0) {
        double *o = T + ((size_t)(i - r0) * E + e) * 8;
#pragma unroll
        for (int k = 0; k < 8; k++) o[k] = out[k];
    }
}

// Pass 2: K[c * ld + i] = sum over the (element, position) pairs of node c,
// in element order, of T[(i - r0) * E + e][pos].
__global__ void k_q8_gather(const double *__restrict__ T, const int *__restrict__ ne_ptr,
                            const int *__restrict__ ne_elem, const int *__restrict__ ne_pos, int N, int E, int r0,
                            int r1, double *__restrict__ K, size_t ld)
{
    // block b: node c = b / nrb, rows r0 + (b % nrb) * blockDim.x + thread
    const int nrb = (r1 - r0 + blockDim.x - 1) / blockDim.x;
    const int c = (int)(blockIdx.x / nrb), i = r0 + (int)(blockIdx.x % nrb) * blockDim.x + threadIdx.x;
    if (c >= N || i >= r1) return;
    double s = 0.0;
    for (int t = ne_ptr[c]; t < ne_ptr[c + 1]; t++)
        s += T[((size_t)(i - r0) * E + ne_elem[t]) * 8 + ne_pos[t]];
    K[(size_t)c * ld + i] = s;
}

// ------------------------------------------------------------ points
// Regular parts of the field (FIELD 1: sum of sigma w J d / r^3, 6 values)
// or potential (sum of sigma w J / r, 2 values) at point p from the
// elements of chunk blockIdx.y, skipping the point's singular elements;
// block reduction into part[(p * nchunk + chunk) * NV + v].
template <int FIELD>
__global__ void __launch_bounds__(128) k_q8_points_regular(
    const double *__restrict__ X, const double *__restrict__ Y, const double *__restrict__ Z,
    const int *__restrict__ elems, int E, int N, const double *__restrict__ sigma, const double *__restrict__ pts,
    const int4 *__restrict__ coinc, int nchunk, double *__restrict__ part)
{
    constexpr int NV = FIELD ? 6 : 2;
    __shared__ double sh[4][NV];
    const int p = blockIdx.x, chunk = blockIdx.y;
    const int e = chunk * blockDim.x + threadIdx.x;
    double acc[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) acc[v] = 0.0;
    if (e < E) {
        const int *en = elems + (size_t)e * 8;
        const int4 c = coinc[p];
        bool sing = false;
#pragma unroll
        for (int k = 0; k < 8; k++) sing |= en[k] == c.x || en[k] == c.y || en[k] == c.z || en[k] == c.w;
        if (!sing) {
            double Xe[8][3];
            q8_load(X, Y, Z, en, Xe);
            const double x = pts[3 * (size_t)p], y = pts[3 * (size_t)p + 1], z = pts[3 * (size_t)p + 2];
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) {
                    double XL[3], Nq[8];
                    const double J = q8_map(c_q8n, Xe, c_gl3[a][0], c_gl3[b][0], XL, Nq, nullptr);
                    double sr = 0.0, si = 0.0;
#pragma unroll
                    for (int k = 0; k < 8; k++) {
                        sr += Nq[k] * sigma[en[k]];
                        si += Nq[k] * sigma[en[k] + N];
                    }
                    const double w = c_gl3[a][1] * c_gl3[b][1] * J;
                    const double dx = x - XL[0], dy = y - XL[1], dz = z - XL[2];
                    const double ri = 1.0 / sqrt(dx * dx + dy * dy + dz * dz);
                    if (FIELD) {
                        const double g = w * ri * ri * ri;
                        acc[0] += g * sr * dx;
                        acc[1] += g * si * dx;
                        acc[2] += g * sr * dy;
                        acc[3] += g * si * dy;
                        acc[4] += g * sr * dz;
                        acc[5] += g * si * dz;
                    } else {
                        acc[0] += w * ri * sr;
                        acc[1] += w * ri * si;
                    }
                }
        }
    }
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
    for (int v = 0; v < NV; v++) {
        const double s = warp_sum(acc[v]);
        if (lane == 0) sh[wp][v] = s;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double t = 0.0;
        for (int u = 0; u < 4; u++) t += sh[u][threadIdx.x];
        part[((size_t)p * nchunk + chunk) * NV + threadIdx.x] = t;
    }
}

// Singular parts at point p (warp per point): the point's singular tuples
// (element, position, node) in element order, FIELD: the gradient sums
// (src/field.c:164-186's scheme on the apex triangles) times sigma, then
// the jump (sigma / (2 eps0)) n of the point's first coincident node once;
// potential: the weakly singular G sums times sigma.  out[p * NV + v] in
// the units of the regular sums (the caller scales by 1/(4 pi eps0)).
template <int FIELD>
__global__ void __launch_bounds__(128) k_q8_points_singular(
    const double *__restrict__ X, const double *__restrict__ Y, const double *__restrict__ Z,
    const double *__restrict__ normals, const int *__restrict__ elems, int N, const double *__restrict__ sigma,
    const double *__restrict__ pts, const int4 *__restrict__ coinc, const int *__restrict__ sp_ptr,
    const int4 *__restrict__ sp, int P, double *__restrict__ out)
{
    constexpr int NV = FIELD ? 6 : 2;
    const int p = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (p >= P) return;
    const double xe[3] = {pts[3 * (size_t)p], pts[3 * (size_t)p + 1], pts[3 * (size_t)p + 2]};
    double acc[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) acc[v] = 0.0;
    for (int t = sp_ptr[p]; t < sp_ptr[p + 1]; t++) {
        const int4 tu = sp[t];  // x element, y position (0-based), z node
        const int *en = elems + (size_t)tu.x * 8;
        double Xe[8][3];
        q8_load(X, Y, Z, en, Xe);
        if (FIELD) {
            double sub[24];
            const double n0[3] = {0.0, 0.0, 0.0};
            q8_warp_singular_H<1>(tu.y, Xe, xe, n0, sub);
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const double sr = sigma[en[k]], si = sigma[en[k] + N];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    acc[2 * c] += sub[3 * k + c] * sr;
                    acc[2 * c + 1] += sub[3 * k + c] * si;
                }
            }
        } else {
            double sub[8];
            q8_warp_singular_G(tu.y, Xe, xe, sub);
#pragma unroll
            for (int k = 0; k < 8; k++) {
                acc[0] += sub[k] * sigma[en[k]];
                acc[1] += sub[k] * sigma[en[k] + N];
            }
        }
    }
    if (lane == 0) {
        if (FIELD && coinc[p].x >= 0) {
            // the jump in units of the regular sums: (1 / (2 eps0)) / (1 / (4 pi eps0)) = 2 pi
            const int v = coinc[p].x;
            const double n[3] = {normals[3 * (size_t)v], normals[3 * (size_t)v + 1], normals[3 * (size_t)v + 2]};
#pragma unroll
            for (int c = 0; c < 3; c++) {
                acc[2 * c] += kPi2 * sigma[v] * n[c];
                acc[2 * c + 1] += kPi2 * sigma[v + N] * n[c];
            }
        }
#pragma unroll
        for (int v = 0; v < NV; v++) out[(size_t)p * NV + v] = acc[v];
    }
}

// out[p][v] = (sum of the chunks, in order, + the singular part) / (4 pi eps0).
__global__ void k_q8_points_reduce(const double *__restrict__ part, const double *__restrict__ sing, int P,
                                   int nchunk, int NV, double *__restrict__ out)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P * NV) return;
    const int p = t / NV, v = t % NV;
    double s = 0.0;
    for (int c = 0; c < nchunk; c++) s += part[((size_t)p * nchunk + c) * NV + v];
    out[t] = (s + sing[t]) / (kPi4 * kEps0);
}

// ------------------------------------------------------------ MST force
// Per particle element (first node of type 6): Fce = eps / 2 * int [E (E.n)
// - |E|^2 n / 2] dS over the 3 x 3 rule, Re(E) interpolated from the nodes,
// n the element's unit normal; Xce = X(0, 0).
__global__ void k_q8_mst(const double *__restrict__ X, const double *__restrict__ Y, const double *__restrict__ Z,
                         const int *__restrict__ elems, const int *__restrict__ pel, int npel,
                         const double *__restrict__ Enode, double eps, double *__restrict__ Fce,
                         double *__restrict__ Xce)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npel) return;
    const int *en = elems + (size_t)pel[t] * 8;
    double Xe[8][3], En[8][3];
    q8_load(X, Y, Z, en, Xe);
#pragma unroll
    for (int k = 0; k < 8; k++)
#pragma unroll
        for (int d = 0; d < 3; d++) En[k][d] = Enode[3 * (size_t)en[k] + d];
    double I[3] = {0.0, 0.0, 0.0};
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            double XL[3], N[8], n[3];
            const double J = q8_map(c_q8n, Xe, c_gl3[a][0], c_gl3[b][0], XL, N, n);
            double Ev[3] = {0.0, 0.0, 0.0};
#pragma unroll
            for (int k = 0; k < 8; k++)
#pragma unroll
                for (int d = 0; d < 3; d++) Ev[d] += En[k][d] * N[k];
            const double NE = Ev[0] * n[0] + Ev[1] * n[1] + Ev[2] * n[2];
            const double Esq = Ev[0] * Ev[0] + Ev[1] * Ev[1] + Ev[2] * Ev[2];
            const double A = c_gl3[a][1] * c_gl3[b][1] * J;
#pragma unroll
            for (int d = 0; d < 3; d++) I[d] += A * (Ev[d] * NE - 0.5 * Esq * n[d]);
        }
    double XL[3], N[8];
    q8_map(c_q8n, Xe, 0.0, 0.0, XL, N, nullptr);
#pragma unroll
    for (int d = 0; d < 3; d++) {
        Fce[3 * (size_t)t + d] = 0.5 * eps * I[d];
        Xce[3 * (size_t)t + d] = XL[d];
    }
}

// ------------------------------------------------------------ host

void q8_node_normals(int N, int E, const double *nodes, const int *elems0, double *out)
{
    std::vector<double> acc((size_t)N * 3, 0.0);
    double X[8][3], XL[3], Nv[8], n[3];
    for (int e = 0; e < E; e++) {
        const int *en = elems0 + (size_t)e * 8;
        for (int k = 0; k < 8; k++)
            for (int d = 0; d < 3; d++) X[k][d] = nodes[3 * (size_t)en[k] + d];
        for (int k = 0; k < 8; k++) {
            bool first = true;
            for (int j = 0; j < k; j++)
                if (en[j] == en[k]) first = false;
            if (!first) continue;
            q8_map(h_q8n, X, h_q8n[k][0], h_q8n[k][1], XL, Nv, n);
            for (int d = 0; d < 3; d++) acc[3 * (size_t)en[k] + d] += n[d];
        }
    }
    for (int i = 0; i < N; i++) {
        const double *a = &acc[3 * (size_t)i];
        const double inv = 1.0 / sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        for (int d = 0; d < 3; d++) out[3 * (size_t)i + d] = a[d] * inv;
    }
}

int Q8Mesh::build(int N_, int E_, const double *nodes, const int *elems0, cudaStream_t st)
{
    if (N_ <= 0 || E_ <= 0) {
        set_error("quad8: empty mesh");
        return kErrArg;
    }
    for (size_t t = 0; t < (size_t)E_ * 8; t++)
        if (elems0[t] < 0 || elems0[t] >= N_) {
            set_error("quad8: element %zu names node %d outside 1..%d", t / 8 + 1, elems0[t] + 1, N_);
            return kErrArg;
        }
    N = N_;
    E = E_;
    hnodes.assign(nodes, nodes + 3 * (size_t)N);
    helems.assign(elems0, elems0 + 8 * (size_t)E);
    hnormals.resize(3 * (size_t)N);
    q8_node_normals(N, E, nodes, elems0, hnormals.data());
    // node -> (element, position), element order
    ne_ptr.assign(N + 1, 0);
    for (int e = 0; e < E; e++)
        for (int k = 0; k < 8; k++) ne_ptr[helems[(size_t)e * 8 + k] + 1]++;
    for (int i = 0; i < N; i++) ne_ptr[i + 1] += ne_ptr[i];
    ne_elem.assign(ne_ptr[N], 0);
    ne_pos.assign(ne_ptr[N], 0);
    std::vector<int> fill(ne_ptr.begin(), ne_ptr.end() - 1);
    for (int e = 0; e < E; e++)
        for (int k = 0; k < 8; k++) {
            const int v = helems[(size_t)e * 8 + k];
            ne_elem[fill[v]] = e;
            ne_pos[fill[v]++] = k;
        }
    // nodes sorted by coordinates (coincident nodes of the points)
    order.resize(N);
    for (int i = 0; i < N; i++) order[i] = i;
    std::sort(order.begin(), order.end(), [&](int a, int b) {
        const double *u = &hnodes[3 * (size_t)a], *v = &hnodes[3 * (size_t)b];
        if (u[0] != v[0]) return u[0] < v[0];
        if (u[1] != v[1]) return u[1] < v[1];
        if (u[2] != v[2]) return u[2] < v[2];
        return a < b;
    });
    std::vector<double> xs(N), ys(N), zs(N);
    for (int i = 0; i < N; i++) {
        xs[i] = nodes[3 * (size_t)i];
        ys[i] = nodes[3 * (size_t)i + 1];
        zs[i] = nodes[3 * (size_t)i + 2];
    }
    DSC_TRY(x.upload(xs, st));
    DSC_TRY(y.upload(ys, st));
    DSC_TRY(z.upload(zs, st));
    DSC_TRY(elems.upload(helems, st));
    DSC_TRY(normals.upload(hnormals, st));
    DSC_TRY(d_ne_ptr.upload(ne_ptr, st));
    DSC_TRY(d_ne_elem.upload(ne_elem, st));
    DSC_TRY(d_ne_pos.upload(ne_pos, st));
    DSC_CUDA(cudaStreamSynchronize(st));
    return kOk;
}

int q8_assemble_K(const Q8Mesh &m, const unsigned *bctype, double *K, size_t ld, cudaStream_t st)
{
    const double C = 1.0 / (kPi4 * kEps0);
    std::vector<int> kind(m.N);
    std::vector<double> fac(m.N);
    for (int i = 0; i < m.N; i++) {
        const unsigned t = bctype[i];
        if (t == 1) {
            kind[i] = 0;
            fac[i] = C;
        } else if (t == 0 || t == 6) {
            kind[i] = 1;
            fac[i] = -1.0;
        } else {
            set_error("node %d has boundary type %u; the assembly defines only 0, 1 and 6", i + 1, t);
            return kErrBcType;
        }
    }
    // singular pairs: (node, element containing it, its position)
    std::vector<int> sr, se, sp;
    for (int i = 0; i < m.N; i++)
        for (int t = m.ne_ptr[i]; t < m.ne_ptr[i + 1]; t++) {
            sr.push_back(i);
            se.push_back(m.ne_elem[t]);
            sp.push_back(m.ne_pos[t]);
        }
    DevBuf<int> dkind, dsr, dse, dsp;
    DevBuf<double> dfac, T;
    DSC_TRY(dkind.upload(kind, st));
    DSC_TRY(dfac.upload(fac, st));
    DSC_TRY(dsr.upload(sr, st));
    DSC_TRY(dse.upload(se, st));
    DSC_TRY(dsp.upload(sp, st));
    // rows in chunks whose pair values take at most 512 MB
    const int rows = (int)std::max<size_t>(1, std::min<size_t>(m.N, ((size_t)512 << 20) / ((size_t)m.E * 64)));
    DSC_TRY(T.alloc((size_t)rows * m.E * 8));
    for (int r0 = 0; r0 < m.N; r0 += rows) {
        const int r1 = std::min(m.N, r0 + rows);
        const size_t npair = (size_t)(r1 - r0) * m.E;
        DSC_LAUNCH(k_q8_pairs<<<(unsigned)((npair + 127) / 128), 128, 0, st>>>(
            m.x.p, m.y.p, m.z.p, m.normals.p, dkind.p, dfac.p, m.elems.p, m.E, r0, r1, T.p));
        const int nsp = (int)sr.size();
        DSC_LAUNCH(k_q8_singular_pairs<<<(nsp * 32 + 127) / 128, 128, 0, st>>>(
            m.x.p, m.y.p, m.z.p, m.normals.p, dkind.p, dfac.p, m.elems.p, dsr.p, dse.p, dsp.p, nsp, m.E, r0, r1,
            T.p));
        DSC_LAUNCH(k_q8_gather<<<(unsigned)((size_t)m.N * ((r1 - r0 + 127) / 128)), 128, 0, st>>>(
            T.p, m.d_ne_ptr.p, m.d_ne_elem.p, m.d_ne_pos.p, m.N, m.E, r0, r1, K, ld));
        DSC_CUDA(cudaGetLastError());
    }
    DSC_CUDA(cudaStreamSynchronize(st));
    return kOk;
}

// Points: coincident nodes (up to four, by exact coordinates) and the
// singular tuples (element, first position matching the point, node).
static int q8_classify(const Q8Mesh &m, int P, const double *pts, std::vector<int4> &co, std::vector<int> &ptr,
                       std::vector<int4> &tup)
{
    co.assign(P, make_int4(-1, -1, -1, -1));
    ptr.assign(1, 0);
    tup.clear();
    for (int p = 0; p < P; p++) {
        const double x = pts[3 * (size_t)p], y = pts[3 * (size_t)p + 1], z = pts[3 * (size_t)p + 2];
        auto less = [&](int a, const double *key) {
            const double *u = &m.hnodes[3 * (size_t)a];
            if (u[0] != key[0]) return u[0] < key[0];
            if (u[1] != key[1]) return u[1] < key[1];
            return u[2] < key[2];
        };
        const double key[3] = {x, y, z};
        auto it = std::lower_bound(m.order.begin(), m.order.end(), key, less);
        std::vector<int> found;
        for (; it != m.order.end(); ++it) {
            const double *u = &m.hnodes[3 * (size_t)*it];
            if (u[0] == x && u[1] == y && u[2] == z) found.push_back(*it);
            else break;
        }
        std::sort(found.begin(), found.end());
        if (found.size() > 4) {
            set_error("more than 4 mesh nodes share the coordinates of point %d", p);
            return kErrArg;
        }
        int ids[4] = {-1, -1, -1, -1};
        for (size_t u = 0; u < found.size(); u++) ids[u] = found[u];
        co[p] = make_int4(ids[0], ids[1], ids[2], ids[3]);
        std::vector<int> cand;
        for (int v : found)
            for (int t = m.ne_ptr[v]; t < m.ne_ptr[v + 1]; t++) cand.push_back(m.ne_elem[t]);
        std::sort(cand.begin(), cand.end());
        cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
        for (int e : cand)
            for (int k = 0; k < 8; k++) {
                const int v = m.helems[(size_t)e * 8 + k];
                if (m.hnodes[3 * (size_t)v] == x && m.hnodes[3 * (size_t)v + 1] == y &&
                    m.hnodes[3 * (size_t)v + 2] == z) {
                    tup.push_back(make_int4(e, k, v, 0));
                    break;
                }
            }
        ptr.push_back((int)tup.size());
    }
    return kOk;
}

int q8_points(const Q8Mesh &m, const double *dsigma, int P, const double *pts_host, int field, double *dout,
              cudaStream_t st)
{
    std::vector<int4> co, tup;
    std::vector<int> ptr;
    DSC_TRY(q8_classify(m, P, pts_host, co, ptr, tup));
    if (tup.empty()) tup.push_back(make_int4(0, 0, 0, 0));
    DevBuf<double> dpts, part, sing;
    DevBuf<int4> dco, dtup;
    DevBuf<int> dptr;
    DSC_TRY(dpts.upload(pts_host, 3 * (size_t)P, st));
    DSC_TRY(dco.upload(co, st));
    DSC_TRY(dptr.upload(ptr, st));
    DSC_TRY(dtup.upload(tup, st));
    const int NV = field ? 6 : 2, nchunk = (m.E + 127) / 128;
    DSC_TRY(part.alloc((size_t)P * nchunk * NV));
    DSC_TRY(sing.alloc((size_t)P * NV));
    const dim3 g(P, nchunk);
    if (field) {
        DSC_LAUNCH(k_q8_points_regular<1><<<g, 128, 0, st>>>(m.x.p, m.y.p, m.z.p, m.elems.p, m.E, m.N, dsigma,
                                                             dpts.p, dco.p, nchunk, part.p));
        DSC_LAUNCH(k_q8_points_singular<1><<<(P * 32 + 127) / 128, 128, 0, st>>>(
            m.x.p, m.y.p, m.z.p, m.normals.p, m.elems.p, m.N, dsigma, dpts.p, dco.p, dptr.p, dtup.p, P, sing.p));
    } else {
        DSC_LAUNCH(k_q8_points_regular<0><<<g, 128, 0, st>>>(m.x.p, m.y.p, m.z.p, m.elems.p, m.E, m.N, dsigma,
                                                             dpts.p, dco.p, nchunk, part.p));
        DSC_LAUNCH(k_q8_points_singular<0><<<(P * 32 + 127) / 128, 128, 0, st>>>(
            m.x.p, m.y.p, m.z.p, m.normals.p, m.elems.p, m.N, dsigma, dpts.p, dco.p, dptr.p, dtup.p, P, sing.p));
    }
    DSC_LAUNCH(k_q8_points_reduce<<<(P * NV + 255) / 256, 256, 0, st>>>(part.p, sing.p, P, nchunk, NV, dout));
    DSC_CUDA(cudaGetLastError());
    DSC_CUDA(cudaStreamSynchronize(st));
    return kOk;
}

int q8_force_mst(const Q8Mesh &m, const unsigned *bctype, const double *dsigma, double eps, double *Fce_host,
                 double *Xce_host, double *Fcm, double *Xcm, cudaStream_t st)
{
    std::vector<int> ids, pel;
    std::vector<double> pts;
    for (int i = 0; i < m.N; i++)
        if (bctype[i] == 6) {
            ids.push_back(i);
            for (int d = 0; d < 3; d++) pts.push_back(m.hnodes[3 * (size_t)i + d]);
        }
    for (int e = 0; e < m.E; e++)
        if (bctype[m.helems[(size_t)e * 8]] == 6) pel.push_back(e);
    for (int d = 0; d < 3; d++) Fcm[d] = Xcm[d] = 0.0;
    if (ids.empty()) return kOk;  // no particle (the reference divides by zero here)
    const int P = (int)ids.size(), npel = (int)pel.size();
    DevBuf<double> Ept, Enode, Fce, Xce;
    DSC_TRY(Ept.alloc((size_t)P * 6));
    DSC_TRY(q8_points(m, dsigma, P, pts.data(), 1, Ept.p, st));
    std::vector<double> eh((size_t)P * 6), en((size_t)m.N * 3, 0.0);
    DSC_CUDA(cudaMemcpyAsync(eh.data(), Ept.p, eh.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    DSC_CUDA(cudaStreamSynchronize(st));
    for (int p = 0; p < P; p++)
        for (int d = 0; d < 3; d++) en[3 * (size_t)ids[p] + d] = eh[6 * (size_t)p + 2 * d];
    DSC_TRY(Enode.upload(en, st));
    std::vector<double> f((size_t)npel * 3), x((size_t)npel * 3);
    if (npel > 0) {
        DevBuf<int> dpel;
        DSC_TRY(dpel.upload(pel, st));
        DSC_TRY(Fce.alloc((size_t)npel * 3));
        DSC_TRY(Xce.alloc((size_t)npel * 3));
        DSC_LAUNCH(k_q8_mst<<<(npel + 127) / 128, 128, 0, st>>>(m.x.p, m.y.p, m.z.p, m.elems.p, dpel.p, npel,
                                                                Enode.p, eps, Fce.p, Xce.p));
        DSC_CUDA(cudaMemcpyAsync(f.data(), Fce.p, f.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
        DSC_CUDA(cudaMemcpyAsync(x.data(), Xce.p, x.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
        DSC_CUDA(cudaStreamSynchronize(st));
    }
    // totals in element and node order (the reference's loops)
    for (int t = 0; t < npel; t++)
        for (int d = 0; d < 3; d++) {
            Fcm[d] += f[3 * (size_t)t + d];
            if (Fce_host) Fce_host[3 * (size_t)pel[t] + d] = f[3 * (size_t)t + d];
            if (Xce_host) Xce_host[3 * (size_t)pel[t] + d] = x[3 * (size_t)t + d];
        }
    for (int p = 0; p < P; p++)
        for (int d = 0; d < 3; d++) Xcm[d] += m.hnodes[3 * (size_t)ids[p] + d];
    for (int d = 0; d < 3; d++) Xcm[d] /= P;
    return kOk;
}

}  // namespace dsc
