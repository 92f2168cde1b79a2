// dsc_field.cu -- potential, field and Maxwell-stress force from the nodal
// surface charge (field_tria*, potential_tria* src/field.c:57-200,
// src/potential.c:55-179; forceMST_tria* src/force.c:348-552 with intF_*
// src/forceIntegrals.c:632-723).
//
// Regular pairs: the 7 quadrature points of every element carry their
// charge weights c_q = w_q J_q sum_k N_k(q) sigma_k (Re and Im), so a
// (point, element) pair costs 7 kernel evaluations and no shape functions.
// Two layouts: thread per point over a chunk of elements staged in shared
// memory (many points), or thread per element with a block reduction (a
// handful of points).  Partial sums per element chunk are reduced in chunk
// order, so results do not depend on scheduling.
// Singular pairs (the point coincides with a node of the element, by exact
// coordinate equality as the reference tests it) use the FP64 subdivision
// rule, one warp per point, plus the reference's jump term: once per such
// element, sigma/(2 eps0) of the element's FIRST node times the averaged
// normal of the coincident node (src/field.c:171-195), kept for parity.
#include <math.h>

#include <algorithm>
#include <numeric>
#include <thread>

#include "dsc_common.cuh"
#include "dsc_field.h"
#include "dsc_internal.h"
#include "dsc_singular.cuh"

namespace dsc {

constexpr int kFieldChunk = 64;  // elements per chunk

// Charge-weighted quadrature points: cq[(e*7+q)*5 + {x,y,z,re,im}].
template <int NEN>
__global__ void k_charge_qp(const double *__restrict__ X, const double *__restrict__ Y,
                            const double *__restrict__ Z, const int *__restrict__ elems, int E, int N,
                            const double *__restrict__ sigma, double *__restrict__ cq)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= E * kTriPts) return;
    int e = t / kTriPts, q = t % kTriPts;
    double Xe[NEN][3], N6[NEN], XL[3];
    double sr = 0.0, si = 0.0;
    double l1 = c_tri7[q][0], l2 = c_tri7[q][1];
    shape<NEN>(l1, l2, N6);
#pragma unroll
    for (int k = 0; k < NEN; k++) {
        int v = elems[(size_t)e * NEN + k];
        Xe[k][0] = X[v];
        Xe[k][1] = Y[v];
        Xe[k][2] = Z[v];
        sr += N6[k] * sigma[v];
        si += N6[k] * sigma[v + N];
    }
    double J = map_point<NEN>(Xe, l1, l2, N6, XL);
    double w = c_tri7[q][2] * J;
    double *o = cq + (size_t)t * 5;
    o[0] = XL[0];
    o[1] = XL[1];
    o[2] = XL[2];
    o[3] = w * sr;
    o[4] = w * si;
}

struct PointArgs {
    const double *px, *py, *pz;   // points
    const int4 *coinc;            // up to 4 coincident node ids per point (-1 pad)
    int P;
    const int *elems;
    const double *cq;
    int E;
};

template <int NEN>
__device__ __forceinline__ bool is_singular(const int *en, int4 c)
{
    bool s = false;
#pragma unroll
    for (int k = 0; k < NEN; k++)
        s |= (en[k] == c.x) | (en[k] == c.y) | (en[k] == c.z) | (en[k] == c.w);
    return s && c.x >= 0;
}

// FIELD = 1: out has 6 values per point (Re/Im of E x, y, z without the
// 1/(4 pi eps0) factor); FIELD = 0: 2 values (Re/Im potential).
template <int NEN, int FIELD>
__global__ void __launch_bounds__(128) k_point_regular(PointArgs a, double *__restrict__ part)
{
    constexpr int NV = FIELD ? 6 : 2;
    __shared__ double s_cq[kFieldChunk * kTriPts * 5];
    __shared__ int s_en[kFieldChunk * NEN];
    const int chunk = blockIdx.y;
    const int e0 = chunk * kFieldChunk;
    const int ne = min(kFieldChunk, a.E - e0);
    for (int t = threadIdx.x; t < ne * kTriPts * 5; t += blockDim.x)
        s_cq[t] = a.cq[(size_t)e0 * kTriPts * 5 + t];
    for (int t = threadIdx.x; t < ne * NEN; t += blockDim.x) s_en[t] = a.elems[(size_t)e0 * NEN + t];
    __syncthreads();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.P) return;
    const double x = a.px[p], y = a.py[p], z = a.pz[p];
    const int4 c = a.coinc[p];
    double acc[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) acc[v] = 0.0;
    for (int e = 0; e < ne; e++) {
        if (is_singular<NEN>(s_en + e * NEN, c)) continue;
        const double *Q = s_cq + e * kTriPts * 5;
#pragma unroll
        for (int q = 0; q < kTriPts; q++) {
            double dx = x - Q[q * 5], dy = y - Q[q * 5 + 1], dz = z - Q[q * 5 + 2];
            double inv = rsqrt(dx * dx + dy * dy + dz * dz);
            if (FIELD) {
                double i3 = inv * inv * inv;
                double gr = Q[q * 5 + 3] * i3, gi = Q[q * 5 + 4] * i3;
                acc[0] += gr * dx; acc[1] += gi * dx;
                acc[2] += gr * dy; acc[3] += gi * dy;
                acc[4] += gr * dz; acc[5] += gi * dz;
            } else {
                acc[0] += Q[q * 5 + 3] * inv;
                acc[1] += Q[q * 5 + 4] * inv;
            }
        }
    }
    double *o = part + ((size_t)chunk * a.P + p) * NV;
#pragma unroll
    for (int v = 0; v < NV; v++) o[v] = acc[v];
}

// Few points: thread per element of chunk `chunk` (blockDim.x elements),
// block reduction per point.
template <int NEN, int FIELD>
__device__ __forceinline__ void point_regular_few(const PointArgs &a, int chunk, double *__restrict__ part)
{
    constexpr int NV = FIELD ? 6 : 2;
    __shared__ double sh[32];
    const int e = chunk * blockDim.x + threadIdx.x;
    for (int p = 0; p < a.P; p++) {
        double acc[NV];
#pragma unroll
        for (int v = 0; v < NV; v++) acc[v] = 0.0;
        if (e < a.E && !is_singular<NEN>(a.elems + (size_t)e * NEN, a.coinc[p])) {
            const double x = a.px[p], y = a.py[p], z = a.pz[p];
            const double *Q = a.cq + (size_t)e * kTriPts * 5;
#pragma unroll
            for (int q = 0; q < kTriPts; q++) {
                double dx = x - Q[q * 5], dy = y - Q[q * 5 + 1], dz = z - Q[q * 5 + 2];
                double inv = rsqrt(dx * dx + dy * dy + dz * dz);
                if (FIELD) {
                    double i3 = inv * inv * inv;
                    double gr = Q[q * 5 + 3] * i3, gi = Q[q * 5 + 4] * i3;
                    acc[0] += gr * dx; acc[1] += gi * dx;
                    acc[2] += gr * dy; acc[3] += gi * dy;
                    acc[4] += gr * dz; acc[5] += gi * dz;
                } else {
                    acc[0] += Q[q * 5 + 3] * inv;
                    acc[1] += Q[q * 5 + 4] * inv;
                }
            }
        }
#pragma unroll
        for (int v = 0; v < NV; v++) {
            double s = warp_sum(acc[v]);
            const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
            if (lane == 0) sh[w] = s;
            __syncthreads();
            if (threadIdx.x == 0) {
                double t = 0.0;
                for (int u = 0; u < (int)(blockDim.x >> 5); u++) t += sh[u];
                part[((size_t)chunk * a.P + p) * NV + v] = t;
            }
            __syncthreads();
        }
    }
}

template <int NEN, int FIELD>
__global__ void __launch_bounds__(128) k_point_regular_few(PointArgs a, double *__restrict__ part)
{
    point_regular_few<NEN, FIELD>(a, blockIdx.x, part);
}

// Singular pairs of each point: tuples (element, local position s of the
// coincident node, node whose averaged normal is used), in element order;
// warp p of the grid (block b of blockDim.x threads) takes point p.
template <int NEN, int FIELD>
__device__ __forceinline__ void point_singular(const PointArgs &a, int b, const double *__restrict__ X,
                                               const double *__restrict__ Y, const double *__restrict__ Z,
                                               const double *__restrict__ normals, int N,
                                               const double *__restrict__ sigma, const int *__restrict__ sp_ptr,
                                               const int4 *__restrict__ sp, double *__restrict__ out)
{
    constexpr int NV = FIELD ? 6 : 2;
    const int p = (int)((b * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (p >= a.P) return;
    const double xe[3] = {a.px[p], a.py[p], a.pz[p]};
    // field: (0.5/eps0)/(2 pi) as src/field.c:149-150; potential:
    // 1/(4 pi eps0) as src/potential.c:138
    const double A = FIELD ? 0.5 / kEps0 / kPi2 : 1.0 / (kPi4 * kEps0), B = 0.5 / kEps0;
    double acc[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) acc[v] = 0.0;
    for (int t = sp_ptr[p]; t < sp_ptr[p + 1]; t++) {
        const int4 tu = sp[t];  // x: element, y: position (1-based), z: normal node
        const int e = tu.x, s = tu.y;
        double Xe[NEN][3];
        int nodes[NEN];
#pragma unroll
        for (int k = 0; k < NEN; k++) {
            int v = a.elems[(size_t)e * NEN + k];
            nodes[k] = v;
            Xe[k][0] = X[v];
            Xe[k][1] = Y[v];
            Xe[k][2] = Z[v];
        }
        if (FIELD) {
            double n[3] = {normals[3 * (size_t)tu.z], normals[3 * (size_t)tu.z + 1],
                           normals[3 * (size_t)tu.z + 2]};
            double sub[3 * NEN];
            warp_singular_H<NEN, 1>(s, Xe, xe, n, sub);
#pragma unroll
            for (int k = 0; k < NEN; k++) {
                const double sr = sigma[nodes[k]], si = sigma[nodes[k] + N];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    acc[2 * c] += A * sub[3 * k + c] * sr;
                    acc[2 * c + 1] += A * sub[3 * k + c] * si;
                }
            }
            const double sr0 = sigma[nodes[0]], si0 = sigma[nodes[0] + N];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                acc[2 * c] += B * sr0 * n[c];
                acc[2 * c + 1] += B * si0 * n[c];
            }
        } else {
            double sub[NEN];
            warp_singular_G<NEN>(s, Xe, xe, sub);
#pragma unroll
            for (int k = 0; k < NEN; k++) {
                acc[0] += A * sub[k] * sigma[nodes[k]];
                acc[1] += A * sub[k] * sigma[nodes[k] + N];
            }
        }
    }
    if (lane == 0) {
#pragma unroll
        for (int v = 0; v < NV; v++) out[(size_t)p * NV + v] = acc[v];
    }
}

template <int NEN, int FIELD>
__global__ void __launch_bounds__(128) k_point_singular(
    PointArgs a, const double *__restrict__ X, const double *__restrict__ Y,
    const double *__restrict__ Z, const double *__restrict__ normals, int N,
    const double *__restrict__ sigma, const int *__restrict__ sp_ptr, const int4 *__restrict__ sp,
    double *__restrict__ out)
{
    point_singular<NEN, FIELD>(a, blockIdx.x, X, Y, Z, normals, N, sigma, sp_ptr, sp, out);
}

// result[p] = 1/(4 pi eps0) * sum_chunks part + singular part.
template <int NV>
__global__ void k_point_reduce(const double *__restrict__ part, int nchunk, int P,
                               const double *__restrict__ sing, double *__restrict__ out)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P * NV) return;
    const double A = NV == 6 ? 0.5 / kEps0 / kPi2 : 1.0 / (kPi4 * kEps0);
    double s = 0.0;
    for (int c = 0; c < nchunk; c++) s += part[(size_t)c * P * NV + t];
    out[t] = A * s + sing[t];
}

// The few-point pass in one launch: blocks [0, nchunk) the regular parts
// (point_regular_few), the blocks after them the singular parts (a warp per
// point); the last block to finish (a ticket taken after each block's
// results are visible) sums the chunks as k_point_reduce does and returns
// the ticket to zero for the next launch.
template <int NEN, int FIELD>
__global__ void __launch_bounds__(128) k_point_few(PointArgs a, int nchunk, const double *__restrict__ X,
                                                   const double *__restrict__ Y, const double *__restrict__ Z,
                                                   const double *__restrict__ normals, int N,
                                                   const double *__restrict__ sigma, const int *__restrict__ sp_ptr,
                                                   const int4 *__restrict__ sp, double *__restrict__ part,
                                                   double *__restrict__ sing, unsigned *ticket,
                                                   double *__restrict__ out)
{
    constexpr int NV = FIELD ? 6 : 2;
    if ((int)blockIdx.x < nchunk) point_regular_few<NEN, FIELD>(a, blockIdx.x, part);
    else point_singular<NEN, FIELD>(a, blockIdx.x - nchunk, X, Y, Z, normals, N, sigma, sp_ptr, sp, sing);
    __shared__ bool last;
    __threadfence();  // every thread's partial results, before the ticket
    __syncthreads();
    if (threadIdx.x == 0) {
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    const double A = FIELD ? 0.5 / kEps0 / kPi2 : 1.0 / (kPi4 * kEps0);
    for (int t = threadIdx.x; t < a.P * NV; t += blockDim.x) {
        double s = 0.0;
        for (int c = 0; c < nchunk; c++) s += ((volatile const double *)part)[(size_t)c * a.P * NV + t];
        out[t] = A * s + ((volatile const double *)sing)[t];
    }
    if (threadIdx.x == 0) *ticket = 0u;
}

// Maxwell stress on the particle elements (first node of type 6):
// Fce = eps/2 * int [E (E.n) - |E|^2 n / 2] dS with Re(E) interpolated from
// the nodes, Xce = X(1/4, 1/4).
template <int NEN>
__global__ void k_mst(const double *__restrict__ X, const double *__restrict__ Y,
                      const double *__restrict__ Z, const int *__restrict__ elems,
                      const int *__restrict__ pel, int npel, const double *__restrict__ Enode,
                      double eps, double *__restrict__ Fce, double *__restrict__ Xce)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npel) return;
    const int e = pel[t];
    double Xe[NEN][3], En[NEN][3], N6[NEN], XL[3], n[3];
#pragma unroll
    for (int k = 0; k < NEN; k++) {
        int v = elems[(size_t)e * NEN + k];
        Xe[k][0] = X[v];
        Xe[k][1] = Y[v];
        Xe[k][2] = Z[v];
        En[k][0] = Enode[3 * (size_t)v];
        En[k][1] = Enode[3 * (size_t)v + 1];
        En[k][2] = Enode[3 * (size_t)v + 2];
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
    Fce[3 * (size_t)t] = A * I0;
    Fce[3 * (size_t)t + 1] = A * I1;
    Fce[3 * (size_t)t + 2] = A * I2;
    shape<NEN>(0.25, 0.25, N6);
    map_point<NEN>(Xe, 0.25, 0.25, N6, XL);
    Xce[3 * (size_t)t] = XL[0];
    Xce[3 * (size_t)t + 1] = XL[1];
    Xce[3 * (size_t)t + 2] = XL[2];
}

// Scatter Re(E) of each particle node into a node-indexed array.
__global__ void k_scatter_re(const double *__restrict__ Ept, const int *__restrict__ ids, int P,
                             double *__restrict__ Enode)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const int v = ids[p];
    Enode[3 * (size_t)v] = Ept[6 * (size_t)p];
    Enode[3 * (size_t)v + 1] = Ept[6 * (size_t)p + 2];
    Enode[3 * (size_t)v + 2] = Ept[6 * (size_t)p + 4];
}

// Totals: Fcm = sum Fce, Xcm = mean of the particle nodes (one warp,
// lane-strided sums and a tree reduction: a fixed order).
__global__ void k_mst_totals(const double *__restrict__ Fce, int npel, const double *__restrict__ X,
                             const double *__restrict__ Y, const double *__restrict__ Z,
                             const int *__restrict__ ids, int P, double *__restrict__ tot)
{
    const int lane = threadIdx.x;
    double f[3] = {0, 0, 0}, x[3] = {0, 0, 0};
    for (int t = lane; t < npel; t += 32)
        for (int d = 0; d < 3; d++) f[d] += Fce[3 * (size_t)t + d];
    for (int p = lane; p < P; p += 32) {
        x[0] += X[ids[p]];
        x[1] += Y[ids[p]];
        x[2] += Z[ids[p]];
    }
    for (int d = 0; d < 3; d++) {
        f[d] = warp_sum(f[d]);
        x[d] = warp_sum(x[d]);
    }
    double fa[3] = {0, 0, 0};
    for (int t = lane; t < npel; t += 32)
        for (int d = 0; d < 3; d++) fa[d] += fabs(Fce[3 * (size_t)t + d]);
    for (int d = 0; d < 3; d++) fa[d] = warp_sum(fa[d]);
    if (lane == 0) {
        for (int d = 0; d < 3; d++) {
            tot[d] = f[d];
            tot[3 + d] = x[d] / P;
            tot[6 + d] = fa[d];
        }
    }
}

// Per-particle results (see mst_particles): block per (particle, system),
// thread-strided sums in a fixed order, then warp sums and the warps' sums
// in order.
constexpr int kPartThreads = 256;
__device__ __forceinline__ void part_block_sum(double *v, int n, double (*sh)[kPartThreads / 32])
{
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    for (int k = 0; k < n; k++) v[k] = warp_sum(v[k]);
    __syncthreads();
    if (lane == 0)
        for (int k = 0; k < n; k++) sh[k][wp] = v[k];
    __syncthreads();
    for (int k = 0; k < n; k++) {
        double t = 0.0;
        for (int w = 0; w < kPartThreads / 32; w++) t += sh[k][w];
        v[k] = t;
    }
}

__global__ void __launch_bounds__(kPartThreads) k_mst_particles(
    const double *__restrict__ Fce, size_t fstride, const double *__restrict__ Xce, int npel,
    const int *__restrict__ pel_part, const double *__restrict__ X, const double *__restrict__ Y,
    const double *__restrict__ Z, const int *__restrict__ ids, const int *__restrict__ ids_part, int P, int npart,
    double *__restrict__ out)
{
    __shared__ double sh[9][kPartThreads / 32];
    const int p = blockIdx.x, f = blockIdx.y;
    double c[4] = {0, 0, 0, 0};
    for (int q = threadIdx.x; q < P; q += kPartThreads)
        if (ids_part[q] == p) {
            const int v = ids[q];
            c[0] += X[v];
            c[1] += Y[v];
            c[2] += Z[v];
            c[3] += 1.0;
        }
    part_block_sum(c, 4, sh);
    const double cx = c[0] / c[3], cy = c[1] / c[3], cz = c[2] / c[3];
    const double *Fc = Fce + (size_t)f * fstride;
    double s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int t = threadIdx.x; t < npel; t += kPartThreads)
        if (pel_part[t] == p) {
            const double fx = Fc[3 * (size_t)t], fy = Fc[3 * (size_t)t + 1], fz = Fc[3 * (size_t)t + 2];
            const double rx = Xce[3 * (size_t)t] - cx, ry = Xce[3 * (size_t)t + 1] - cy,
                         rz = Xce[3 * (size_t)t + 2] - cz;
            s[0] += fx;
            s[1] += fy;
            s[2] += fz;
            s[3] += fabs(fx);
            s[4] += fabs(fy);
            s[5] += fabs(fz);
            s[6] += ry * fz - rz * fy;
            s[7] += rz * fx - rx * fz;
            s[8] += rx * fy - ry * fx;
        }
    part_block_sum(s, 9, sh);
    if (threadIdx.x == 0) {
        double *o = out + ((size_t)f * npart + p) * kPartVals;
        o[0] = s[0];
        o[1] = s[1];
        o[2] = s[2];
        o[3] = cx;
        o[4] = cy;
        o[5] = cz;
        o[6] = s[3];
        o[7] = s[4];
        o[8] = s[5];
        o[9] = s[6];
        o[10] = s[7];
        o[11] = s[8];
    }
}

template <int NEN>
__global__ void k_mst_centres(const double *__restrict__ X, const double *__restrict__ Y,
                              const double *__restrict__ Z, const int *__restrict__ elems,
                              const int *__restrict__ pel, int npel, double *__restrict__ Xce)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npel) return;
    const int e = pel[t];
    double Xe[NEN][3], N6[NEN], XL[3];
#pragma unroll
    for (int k = 0; k < NEN; k++) {
        const int v = elems[(size_t)e * NEN + k];
        Xe[k][0] = X[v];
        Xe[k][1] = Y[v];
        Xe[k][2] = Z[v];
    }
    shape<NEN>(0.25, 0.25, N6);
    map_point<NEN>(Xe, 0.25, 0.25, N6, XL);
    Xce[3 * (size_t)t] = XL[0];
    Xce[3 * (size_t)t + 1] = XL[1];
    Xce[3 * (size_t)t + 2] = XL[2];
}

int mst_particles(const ForcePlan &fp, const double *X, const double *Y, const double *Z, const double *Fce,
                  size_t fstride, const double *Xce, int nsys, double *out, cudaStream_t st)
{
    if (fp.npart == 0 || nsys == 0) return kOk;
    DSC_LAUNCH(k_mst_particles<<<dim3(fp.npart, nsys), kPartThreads, 0, st>>>(
        Fce, fstride, Xce, fp.npel, fp.pel_part.p, X, Y, Z, fp.ids.p, fp.ids_part.p, fp.P, fp.npart, out));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

int mst_centres(const DeviceMesh &m, const ForcePlan &fp, double *Xce, cudaStream_t st)
{
    if (fp.npel == 0) return kOk;
    const int g = (fp.npel + 127) / 128;
    if (m.nen == 6)
        DSC_LAUNCH(k_mst_centres<6><<<g, 128, 0, st>>>(m.x.p, m.y.p, m.z.p, m.elems.p, fp.pel.p, fp.npel, Xce));
    else
        DSC_LAUNCH(k_mst_centres<3><<<g, 128, 0, st>>>(m.x.p, m.y.p, m.z.p, m.elems.p, fp.pel.p, fp.npel, Xce));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

// ------------------------------------------------------------------ host

// Host classification of P points: coordinates, up to four coincident
// mesh nodes each (-1 padded) and the singular tuples (element, local
// position, node) in point order, ptr their offsets.
static int classify_points(const HostPlan &plan, int P, const double *pts, const int *node_ids,
                           std::vector<double> &xs, std::vector<double> &ys, std::vector<double> &zs,
                           std::vector<int4> &co, std::vector<int> &ptr, std::vector<int4> &tup)
{
    xs.assign(P, 0.0);
    ys.assign(P, 0.0);
    zs.assign(P, 0.0);
    co.assign(P, make_int4(-1, -1, -1, -1));
    ptr.assign(1, 0);
    tup.clear();
    const int nen = plan.nen;
    // points that are mesh nodes: each node's group of nodes with identical
    // coordinates (a run of the coordinate order), found in one pass
    std::vector<int> grp_lo, grp_hi;
    if (node_ids) {
        grp_lo.resize(plan.N);
        grp_hi.resize(plan.N);
        for (int a = 0; a < plan.N;) {
            const double *u = &plan.nodes[3 * (size_t)plan.coord_order[a]];
            int b = a + 1;
            while (b < plan.N) {
                const double *w = &plan.nodes[3 * (size_t)plan.coord_order[b]];
                if (w[0] != u[0] || w[1] != u[1] || w[2] != u[2]) break;
                b++;
            }
            for (int t = a; t < b; t++) {
                grp_lo[plan.coord_order[t]] = a;
                grp_hi[plan.coord_order[t]] = b;
            }
            a = b;
        }
    }
    // points split over host threads in contiguous ranges (tuples
    // concatenated in point order afterwards)
    const int nth = P >= 2048 ? std::min(8, (P + 1023) / 1024) : 1;
    std::vector<std::vector<int4>> tups(nth);
    std::vector<int> cnt(P, 0), bad(nth, -1);
    auto work = [&](int th) {
        std::vector<int> found, cand;
        const int p0 = (int)((long long)P * th / nth), p1 = (int)((long long)P * (th + 1) / nth);
        std::vector<int4> &tu = tups[th];
        for (int p = p0; p < p1; p++) {
            xs[p] = pts[3 * p];
            ys[p] = pts[3 * p + 1];
            zs[p] = pts[3 * p + 2];
            // exact-coordinate lookup of mesh nodes
            if (node_ids) {
                const int v = node_ids[p];
                found.assign(plan.coord_order.begin() + grp_lo[v], plan.coord_order.begin() + grp_hi[v]);
                std::sort(found.begin(), found.end());
            } else {
                found = plan_coords_find(plan, xs[p], ys[p], zs[p]);
            }
            if (found.size() > 4) {
                bad[th] = p;
                return;
            }
            int ids[4] = {-1, -1, -1, -1};
            const int nco = (int)found.size();
            for (int u = 0; u < nco; u++) ids[u] = found[u];
            co[p] = make_int4(ids[0], ids[1], ids[2], ids[3]);
            // singular elements of this point, element order, first matching
            // position within the element (src/field.c:164-173)
            const size_t before = tu.size();
            if (nco > 0) {
                cand.clear();
                for (int u = 0; u < nco; u++)
                    for (int t = plan.ne_ptr[ids[u]]; t < plan.ne_ptr[ids[u] + 1]; t++)
                        cand.push_back(plan.ne_elem[t]);
                std::sort(cand.begin(), cand.end());
                cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
                for (int e : cand) {
                    for (int k = 0; k < nen; k++) {
                        int v = plan.elems[(size_t)e * nen + k];
                        if (plan.nodes[3 * (size_t)v] == xs[p] && plan.nodes[3 * (size_t)v + 1] == ys[p] &&
                            plan.nodes[3 * (size_t)v + 2] == zs[p]) {
                            tu.push_back(make_int4(e, k + 1, v, 0));
                            break;
                        }
                    }
                }
            }
            cnt[p] = (int)(tu.size() - before);
        }
    };
    {
        std::vector<std::thread> th;
        for (int t = 1; t < nth; t++) th.emplace_back(work, t);
        work(0);
        for (auto &t : th) t.join();
    }
    for (int t = 0; t < nth; t++)
        if (bad[t] >= 0) {
            set_error("more than 4 mesh nodes share the coordinates of point %d", bad[t]);
            return kErrArg;
        }
    for (int p = 0; p < P; p++) ptr.push_back(ptr.back() + cnt[p]);
    for (int t = 0; t < nth; t++) tup.insert(tup.end(), tups[t].begin(), tups[t].end());
    return kOk;
}

int PointSet::build(const HostPlan &plan, int P, const double *pts, const int *node_ids)
{
    this->P = P;
    std::vector<double> xs, ys, zs;
    std::vector<int4> co, tup;
    std::vector<int> ptr;
    DSC_TRY(classify_points(plan, P, pts, node_ids, xs, ys, zs, co, ptr, tup));
    cudaStream_t st = 0;
    DSC_TRY(px.upload(xs, st));
    DSC_TRY(py.upload(ys, st));
    DSC_TRY(pz.upload(zs, st));
    DSC_TRY(coinc.upload(co, st));
    DSC_TRY(sp_ptr.upload(ptr, st));
    sp_ptr_h = ptr;
    sp_h = tup;
    if (tup.empty()) tup.push_back(make_int4(0, 0, 0, 0));
    DSC_TRY(sp.upload(tup, st));
    DSC_CUDA(cudaStreamSynchronize(st));
    return kOk;
}

template <int NEN>
static int eval_points_impl(const DeviceMesh &m, PointSet &ps, const double *dsigma, int field,
                            double *dout, cudaStream_t st, bool sync)
{
    const int NV = field ? 6 : 2;
    DevBuf<double> &cq = ps.cq, &part = ps.part, &sing = ps.sing;
    DSC_TRY(cq.alloc((size_t)m.E * kTriPts * 5));
    DSC_LAUNCH(k_charge_qp<NEN><<<(m.E * kTriPts + 255) / 256, 256, 0, st>>>(m.x.p, m.y.p, m.z.p, m.elems.p, m.E,
                                                                    m.N, dsigma, cq.p));
    PointArgs a{ps.px.p, ps.py.p, ps.pz.p, ps.coinc.p, ps.P, m.elems.p, cq.p, m.E};
    int nchunk;
    if (ps.P >= 64) {
        nchunk = (m.E + kFieldChunk - 1) / kFieldChunk;
        DSC_TRY(part.alloc((size_t)nchunk * ps.P * NV));
        dim3 g((ps.P + 127) / 128, nchunk);
        if (field) DSC_LAUNCH(k_point_regular<NEN, 1><<<g, 128, 0, st>>>(a, part.p));
        else DSC_LAUNCH(k_point_regular<NEN, 0><<<g, 128, 0, st>>>(a, part.p));
    } else {
        nchunk = (m.E + 127) / 128;
        DSC_TRY(part.alloc((size_t)nchunk * ps.P * NV));
        if (field) DSC_LAUNCH(k_point_regular_few<NEN, 1><<<nchunk, 128, 0, st>>>(a, part.p));
        else DSC_LAUNCH(k_point_regular_few<NEN, 0><<<nchunk, 128, 0, st>>>(a, part.p));
    }
    DSC_CUDA(cudaGetLastError());
    DSC_TRY(sing.alloc((size_t)ps.P * NV));
    const int sblocks = (ps.P * 32 + 127) / 128;
    if (field)
        DSC_LAUNCH(k_point_singular<NEN, 1><<<sblocks, 128, 0, st>>>(a, m.x.p, m.y.p, m.z.p, m.normals.p, m.N,
                                                          dsigma, ps.sp_ptr.p, ps.sp.p, sing.p));
    else
        DSC_LAUNCH(k_point_singular<NEN, 0><<<sblocks, 128, 0, st>>>(a, m.x.p, m.y.p, m.z.p, m.normals.p, m.N,
                                                          dsigma, ps.sp_ptr.p, ps.sp.p, sing.p));
    DSC_CUDA(cudaGetLastError());
    if (field) DSC_LAUNCH(k_point_reduce<6><<<(ps.P * 6 + 255) / 256, 256, 0, st>>>(part.p, nchunk, ps.P, sing.p, dout));
    else DSC_LAUNCH(k_point_reduce<2><<<(ps.P * 2 + 255) / 256, 256, 0, st>>>(part.p, nchunk, ps.P, sing.p, dout));
    DSC_CUDA(cudaGetLastError());
    if (sync) DSC_CUDA(cudaStreamSynchronize(st));
    return kOk;
}

FewPointWork::~FewPointWork()
{
    if (host) cudaFreeHost(host);
}

int point_charges(const DeviceMesh &m, const double *dsigma, DevBuf<double> &cq, cudaStream_t st)
{
    DSC_TRY(cq.alloc((size_t)m.E * kTriPts * 5));
    if (m.nen == 6)
        DSC_LAUNCH(k_charge_qp<6><<<(m.E * kTriPts + 255) / 256, 256, 0, st>>>(m.x.p, m.y.p, m.z.p, m.elems.p, m.E,
                                                                            m.N, dsigma, cq.p));
    else
        DSC_LAUNCH(k_charge_qp<3><<<(m.E * kTriPts + 255) / 256, 256, 0, st>>>(m.x.p, m.y.p, m.z.p, m.elems.p, m.E,
                                                                            m.N, dsigma, cq.p));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

template <int NEN, int FIELD>
static int few_kernels(const DeviceMesh &m, const PointArgs &a, const double *dsigma, const int *sp_ptr,
                       const int4 *sp, FewPointWork &w, cudaStream_t st)
{
    constexpr int NV = FIELD ? 6 : 2;
    const int nchunk = (m.E + 127) / 128, nsing = (a.P * 32 + 127) / 128;
    DSC_TRY(w.part.alloc((size_t)nchunk * a.P * NV));
    DSC_TRY(w.sing.alloc((size_t)a.P * NV));
    DSC_TRY(w.out.alloc((size_t)a.P * NV));
    if (!w.ticket.p) {
        DSC_TRY(w.ticket.alloc(1));
        DSC_CUDA(cudaMemsetAsync(w.ticket.p, 0, sizeof(unsigned), st));
    }
    DSC_LAUNCH(k_point_few<NEN, FIELD><<<nchunk + nsing, 128, 0, st>>>(a, nchunk, m.x.p, m.y.p, m.z.p, m.normals.p,
                                                                      m.N, dsigma, sp_ptr, sp, w.part.p, w.sing.p,
                                                                      w.ticket.p, w.out.p));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

int eval_few_points(const DeviceMesh &m, const HostPlan &plan, const double *cq, const double *dsigma, int P,
                    const double *pts, int field, double *out, FewPointWork &w, cudaStream_t st)
{
    if (P < 1 || P > kFewPoints) {
        set_error("eval_few_points: %d points (1 .. %d)", P, kFewPoints);
        return kErrArg;
    }
    std::vector<double> xs, ys, zs;
    std::vector<int4> co, tup;
    std::vector<int> ptr;
    DSC_TRY(classify_points(plan, P, pts, nullptr, xs, ys, zs, co, ptr, tup));
    if (tup.empty()) tup.push_back(make_int4(0, 0, 0, 0));
    // one packed upload: x, y, z (P doubles each), coincident nodes (P int4),
    // tuple offsets (P + 1 ints), tuples; 16-byte aligned parts
    auto al = [](size_t b) { return (b + 15) & ~(size_t)15; };
    const size_t o_co = al(24 * (size_t)P), o_ptr = o_co + 16 * (size_t)P, o_sp = al(o_ptr + 4 * ((size_t)P + 1));
    const size_t up = o_sp + 16 * tup.size(), o_out = al(up);
    const int NV = field ? 6 : 2;
    const size_t need = o_out + sizeof(double) * P * NV;
    if (w.host_bytes < need) {
        if (w.host) cudaFreeHost(w.host);
        w.host = nullptr;
        w.host_bytes = 0;
        const size_t cap = std::max(need, (size_t)64 << 10);
        DSC_CUDA(cudaHostAlloc((void **)&w.host, cap, cudaHostAllocDefault));
        w.host_bytes = cap;
    }
    unsigned char *h = w.host;
    memcpy(h, xs.data(), 8 * (size_t)P);
    memcpy(h + 8 * (size_t)P, ys.data(), 8 * (size_t)P);
    memcpy(h + 16 * (size_t)P, zs.data(), 8 * (size_t)P);
    memcpy(h + o_co, co.data(), 16 * (size_t)P);
    memcpy(h + o_ptr, ptr.data(), 4 * ((size_t)P + 1));
    memcpy(h + o_sp, tup.data(), 16 * tup.size());
    DSC_TRY(w.pack.alloc(up));
    DSC_CUDA(cudaMemcpyAsync(w.pack.p, h, up, cudaMemcpyHostToDevice, st));
    const unsigned char *d = w.pack.p;
    const PointArgs a{(const double *)d, (const double *)(d + 8 * (size_t)P), (const double *)(d + 16 * (size_t)P),
                      (const int4 *)(d + o_co), P, m.elems.p, cq, m.E};
    const int *sp_ptr = (const int *)(d + o_ptr);
    const int4 *sp = (const int4 *)(d + o_sp);
    if (m.nen == 6) {
        if (field) DSC_TRY((few_kernels<6, 1>(m, a, dsigma, sp_ptr, sp, w, st)));
        else DSC_TRY((few_kernels<6, 0>(m, a, dsigma, sp_ptr, sp, w, st)));
    } else {
        if (field) DSC_TRY((few_kernels<3, 1>(m, a, dsigma, sp_ptr, sp, w, st)));
        else DSC_TRY((few_kernels<3, 0>(m, a, dsigma, sp_ptr, sp, w, st)));
    }
    DSC_CUDA(cudaMemcpyAsync(h + o_out, w.out.p, sizeof(double) * P * NV, cudaMemcpyDeviceToHost, st));
    DSC_CUDA(cudaStreamSynchronize(st));
    memcpy(out, h + o_out, sizeof(double) * P * NV);
    return kOk;
}

int eval_points(const DeviceMesh &m, PointSet &ps, const double *dsigma, int field, double *dout,
                cudaStream_t st, bool sync)
{
    return m.nen == 6 ? eval_points_impl<6>(m, ps, dsigma, field, dout, st, sync)
                      : eval_points_impl<3>(m, ps, dsigma, field, dout, st, sync);
}

int force_mst(const DeviceMesh &m, const HostPlan &plan, const unsigned *bctype,
              const double *dsigma, double eps, double *Fce_host /*E x 3, may be null*/,
              double *Xce_host, double *Fcm, double *Xcm, cudaStream_t st)
{
    std::vector<int> ids, pel;
    std::vector<double> pts;
    for (int i = 0; i < m.N; i++)
        if (bctype[i] == 6) {
            ids.push_back(i);
            pts.push_back(plan.nodes[3 * (size_t)i]);
            pts.push_back(plan.nodes[3 * (size_t)i + 1]);
            pts.push_back(plan.nodes[3 * (size_t)i + 2]);
        }
    for (int e = 0; e < m.E; e++)
        if (bctype[plan.elems[(size_t)e * m.nen]] == 6) pel.push_back(e);
    (void)pts;
    ForcePlan fp;
    DSC_TRY(fp.build(plan, bctype, st));
    if (fp.P == 0) {
        // the reference divides by a zero count here; report zeros
        for (int d = 0; d < 3; d++) Fcm[d] = Xcm[d] = 0.0;
        return kOk;
    }
    DevBuf<double> tot;
    DSC_TRY(tot.alloc(9));
    DSC_TRY(force_mst_dev(m, fp, dsigma, eps, tot.p, st));
    double h[9];
    DSC_CUDA(cudaMemcpyAsync(h, tot.p, sizeof h, cudaMemcpyDeviceToHost, st));
    const int npel = fp.npel;
    std::vector<double> f((size_t)npel * 3), x((size_t)npel * 3);
    if (npel > 0 && (Fce_host || Xce_host)) {
        DSC_CUDA(cudaMemcpyAsync(f.data(), fp.Fce.p, f.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
        DSC_CUDA(cudaMemcpyAsync(x.data(), fp.Xce.p, x.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    DSC_CUDA(cudaStreamSynchronize(st));
    for (int d = 0; d < 3; d++) {
        Fcm[d] = h[d];
        Xcm[d] = h[3 + d];
    }
    for (int t = 0; t < npel; t++)
        for (int d = 0; d < 3; d++) {
            if (Fce_host) Fce_host[3 * (size_t)fp.pel_host[t] + d] = f[3 * (size_t)t + d];
            if (Xce_host) Xce_host[3 * (size_t)fp.pel_host[t] + d] = x[3 * (size_t)t + d];
        }
    return kOk;
}

int ForcePlan::build(const HostPlan &plan, const unsigned *bctype, cudaStream_t st)
{
    std::vector<int> idv;
    for (int i = 0; i < plan.N; i++)
        if (bctype[i] == 6) idv.push_back(i);
    {
        // points in Morton order of their coordinates (10 bits per axis
        // over the points' bounding box): a warp of consecutive points is
        // one patch of the surface, whose near elements it shares
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int i : idv)
            for (int d = 0; d < 3; d++) {
                lo[d] = std::min(lo[d], plan.nodes[3 * (size_t)i + d]);
                hi[d] = std::max(hi[d], plan.nodes[3 * (size_t)i + d]);
            }
        auto spread = [](unsigned v) {  // 10 bits to every third of 30
            v &= 0x3FFu;
            v = (v | (v << 16)) & 0x030000FFu;
            v = (v | (v << 8)) & 0x0300F00Fu;
            v = (v | (v << 4)) & 0x030C30C3u;
            v = (v | (v << 2)) & 0x09249249u;
            return v;
        };
        std::vector<std::pair<unsigned, int>> key;
        key.reserve(idv.size());
        for (int i : idv) {
            unsigned c = 0;
            for (int d = 0; d < 3; d++) {
                const double w = hi[d] > lo[d] ? (plan.nodes[3 * (size_t)i + d] - lo[d]) / (hi[d] - lo[d]) : 0.0;
                c |= spread((unsigned)std::min(1023.0, w * 1024.0)) << d;
            }
            key.push_back({c, i});
        }
        std::stable_sort(key.begin(), key.end(),
                         [](const std::pair<unsigned, int> &a, const std::pair<unsigned, int> &b) {
                             return a.first < b.first;
                         });
        for (size_t t = 0; t < key.size(); t++) idv[t] = key[t].second;
    }
    std::vector<double> pts;
    for (int i : idv)
        for (int d = 0; d < 3; d++) pts.push_back(plan.nodes[3 * (size_t)i + d]);
    pel_host.clear();
    for (int e = 0; e < plan.E; e++)
        if (bctype[plan.elems[(size_t)e * plan.nen]] == 6) pel_host.push_back(e);
    P = (int)idv.size();
    npel = (int)pel_host.size();
    if (P == 0) return kOk;
    DSC_TRY(ps.build(plan, P, pts.data(), idv.data()));
    {
        // tuple (e, s, v) of the field = tuple (row v, element e, position
        // s - 1) of the assembly's singular pass, which takes it at v's
        // coordinates, the point's
        std::vector<int> tm(std::max<size_t>(ps.sp_h.size(), 1), 0), rg(plan.N, 0);
        for (size_t t = 0; t < ps.sp_h.size(); t++) {
            const int4 u = ps.sp_h[t];
            int found = -1;
            for (int a = plan.ne_ptr[u.z]; a < plan.ne_ptr[u.z + 1]; a++)
                if (plan.ne_elem[a] == u.x && plan.ne_pos[a] == u.y - 1) found = a;
            if (found < 0) {
                set_error("field tuple of element %d has no singular pair in the assembly", u.x);
                return kErrArg;
            }
            tm[t] = found;
            rg[u.z] = 1;
        }
        DSC_TRY(tmap.upload(tm, st));
        DSC_TRY(row_grad.upload(rg, st));
    }
    {
        // particles: union of the nodes of every particle element
        std::vector<int> par(plan.N);
        std::iota(par.begin(), par.end(), 0);
        auto find = [&](int a) {
            while (par[a] != a) {
                par[a] = par[par[a]];
                a = par[a];
            }
            return a;
        };
        for (int e : pel_host)
            for (int k = 1; k < plan.nen; k++) {
                const int a = find(plan.elems[(size_t)e * plan.nen]), b = find(plan.elems[(size_t)e * plan.nen + k]);
                if (a != b) par[std::max(a, b)] = std::min(a, b);
            }
        std::vector<int> pid(plan.N, -1), ip(P), ep(std::max(npel, 1), 0);
        npart = 0;
        for (int i = 0; i < plan.N; i++)  // numbered by their lowest node
            if (bctype[i] == 6 && pid[find(i)] < 0) pid[find(i)] = npart++;
        for (int e : pel_host) {  // a first node of type 6 whose element has no type-6 peers
            const int r = find(plan.elems[(size_t)e * plan.nen]);
            if (pid[r] < 0) pid[r] = npart++;
        }
        for (int t = 0; t < P; t++) ip[t] = pid[find(idv[t])];
        for (int t = 0; t < npel; t++) ep[t] = pid[find(plan.elems[(size_t)pel_host[t] * plan.nen])];
        DSC_TRY(ids_part.upload(ip, st));
        DSC_TRY(pel_part.upload(ep, st));
        DSC_CUDA(cudaStreamSynchronize(st));  // ip, ep go out of scope
    }
    DSC_TRY(ids.upload(idv, st));
    DSC_TRY(pel.upload(pel_host.empty() ? std::vector<int>{0} : pel_host, st));
    DSC_TRY(Ept.alloc((size_t)P * 6));
    DSC_TRY(Enode.alloc((size_t)plan.N * 3));
    DSC_TRY(Fce.alloc((size_t)std::max(npel, 1) * 3));
    DSC_TRY(Xce.alloc((size_t)std::max(npel, 1) * 3));
    DSC_CUDA(cudaMemsetAsync(Enode.p, 0, (size_t)plan.N * 3 * sizeof(double), st));
    DSC_CUDA(cudaStreamSynchronize(st));
    return kOk;
}

int force_mst_dev(const DeviceMesh &m, ForcePlan &fp, const double *dsigma, double eps,
                  double *d_tot, cudaStream_t st, Timer *tm)
{
    if (fp.P == 0) {
        DSC_CUDA(cudaMemsetAsync(d_tot, 0, 9 * sizeof(double), st));
        return kOk;
    }
    {
        TimerScope ts(tm, kTField, st);
        DSC_TRY(eval_points(m, fp.ps, dsigma, 1, fp.Ept.p, st, false));
    }
    TimerScope ts(tm, kTMst, st);
    DSC_LAUNCH(k_scatter_re<<<(fp.P + 255) / 256, 256, 0, st>>>(fp.Ept.p, fp.ids.p, fp.P, fp.Enode.p));
    if (fp.npel > 0) {
        if (m.nen == 6)
            DSC_LAUNCH(k_mst<6><<<(fp.npel + 127) / 128, 128, 0, st>>>(m.x.p, m.y.p, m.z.p, m.elems.p, fp.pel.p,
                                                            fp.npel, fp.Enode.p, eps, fp.Fce.p, fp.Xce.p));
        else
            DSC_LAUNCH(k_mst<3><<<(fp.npel + 127) / 128, 128, 0, st>>>(m.x.p, m.y.p, m.z.p, m.elems.p, fp.pel.p,
                                                            fp.npel, fp.Enode.p, eps, fp.Fce.p, fp.Xce.p));
    }
    DSC_LAUNCH(k_mst_totals<<<1, 32, 0, st>>>(fp.Fce.p, fp.npel, m.x.p, m.y.p, m.z.p, fp.ids.p, fp.P, d_tot));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

}  // namespace dsc

// ------------------------------------------------------------ derivatives
namespace dsc {

// T[deriv_index(a)] = d^a (1/|d|) / dx^a for |a| <= kDerivOrder, by the
// recurrence that follows from |d|^2 d_i(1/r) = -d_i / r differentiated
// d^b times (a = b + e_i, i the first axis of a with a_i > 0):
//   |d|^2 T_a = -d_i T_b - b_i T_{b - e_i}
//               - sum_j [2 b_j d_j T_{b + e_i - e_j} + b_j (b_j - 1) T_{b + e_i - 2 e_j}].
// The loops unroll completely, so every index is a constant.
__device__ __forceinline__ void inv_r_derivs(const double d[3], double (&T)[kDerivCount])
{
    const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2], ir2 = 1.0 / r2;
    T[0] = sqrt(ir2);
#pragma unroll
    for (int n = 1; n <= kDerivOrder; n++)
#pragma unroll
        for (int p = n; p >= 0; p--)
#pragma unroll
            for (int q = n - p; q >= 0; q--) {
                const int a[3] = {p, q, n - p - q};
                const int i = p > 0 ? 0 : (q > 0 ? 1 : 2);
                int b[3] = {a[0], a[1], a[2]};
                b[i]--;
                double v = -d[i] * T[deriv_index(b[0], b[1], b[2])];
                if (b[i] > 0) {
                    int c[3] = {b[0], b[1], b[2]};
                    c[i]--;
                    v -= b[i] * T[deriv_index(c[0], c[1], c[2])];
                }
#pragma unroll
                for (int j = 0; j < 3; j++) {
                    if (b[j] > 0) {
                        int c[3] = {b[0], b[1], b[2]};
                        c[i]++;
                        c[j]--;
                        v -= 2.0 * b[j] * d[j] * T[deriv_index(c[0], c[1], c[2])];
                    }
                    if (b[j] > 1) {
                        int c[3] = {b[0], b[1], b[2]};
                        c[i]++;
                        c[j] -= 2;
                        v -= (double)(b[j] * (b[j] - 1)) * T[deriv_index(c[0], c[1], c[2])];
                    }
                }
                T[deriv_index(a[0], a[1], a[2])] = v * ir2;
            }
}

// part[(pt * nchunk + chunk) * kDerivCount + a] = sum over the chunk's
// quadrature points (charge c = w J Re sigma, cq layout of k_charge_qp) of
// c T_a(x_pt - y_q); block per (point, chunk), fixed-order reduction.
constexpr int kDerivThreads = 128;
__global__ void __launch_bounds__(kDerivThreads) k_point_derivs(const double *__restrict__ pts, int npts,
                                                                const double *__restrict__ cq, int nq, int per,
                                                                double *__restrict__ part)
{
    __shared__ double sh[kDerivThreads / 32][kDerivCount];
    const int pt = blockIdx.x, chunk = blockIdx.y, nchunk = gridDim.y;
    const double x = pts[3 * pt], y = pts[3 * pt + 1], z = pts[3 * pt + 2];
    double S[kDerivCount];
#pragma unroll
    for (int a = 0; a < kDerivCount; a++) S[a] = 0.0;
    const int q0 = chunk * per, q1 = min(nq, q0 + per);
    for (int q = q0 + threadIdx.x; q < q1; q += kDerivThreads) {
        const double *c = cq + (size_t)q * 5;
        const double d[3] = {x - c[0], y - c[1], z - c[2]};
        double T[kDerivCount];
        inv_r_derivs(d, T);
        const double w = c[3];
#pragma unroll
        for (int a = 0; a < kDerivCount; a++) S[a] = fma(w, T[a], S[a]);
    }
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
    for (int a = 0; a < kDerivCount; a++) {
        const double v = warp_sum(S[a]);
        if (lane == 0) sh[wp][a] = v;
    }
    __syncthreads();
    for (int a = threadIdx.x; a < kDerivCount; a += kDerivThreads) {
        double t = 0.0;
        for (int w2 = 0; w2 < kDerivThreads / 32; w2++) t += sh[w2][a];
        part[((size_t)pt * nchunk + chunk) * kDerivCount + a] = t;
    }
    (void)npts;
}

// E[pt][a] = -scale * sum over the chunks (in order) of part: the field
// (|a| = 1) and its derivatives (|a| > 1) at the point, E = -grad phi.
__global__ void k_point_derivs_sum(const double *__restrict__ part, int npts, int nchunk, double scale,
                                   double *__restrict__ E)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npts * kDerivCount) return;
    const int pt = t / kDerivCount, a = t % kDerivCount;
    double s = 0.0;
    for (int c = 0; c < nchunk; c++) s += part[((size_t)pt * nchunk + c) * kDerivCount + a];
    E[t] = -scale * s;
}

int point_derivatives(const DeviceMesh &m, const double *dsigma, int npts, const double *dpts, DerivWork &w,
                      double *E_host, cudaStream_t st)
{
    const int nq = m.E * kTriPts;
    DSC_TRY(w.cq.alloc((size_t)nq * 5));
    if (m.nen == 6)
        DSC_LAUNCH(k_charge_qp<6><<<(nq + 255) / 256, 256, 0, st>>>(m.x.p, m.y.p, m.z.p, m.elems.p, m.E, m.N, dsigma,
                                                                    w.cq.p));
    else
        DSC_LAUNCH(k_charge_qp<3><<<(nq + 255) / 256, 256, 0, st>>>(m.x.p, m.y.p, m.z.p, m.elems.p, m.E, m.N, dsigma,
                                                                    w.cq.p));
    // about 4 blocks per SM over all points
    int nsm = 0;
    DSC_TRY(current_sm_count(&nsm));
    const int nchunk = std::max(1, std::min((4 * nsm + npts - 1) / npts, (nq + kDerivThreads - 1) / kDerivThreads));
    const int per = (nq + nchunk - 1) / nchunk;
    DSC_TRY(w.part.alloc((size_t)npts * nchunk * kDerivCount));
    DSC_TRY(w.E.alloc((size_t)npts * kDerivCount));
    DSC_LAUNCH(k_point_derivs<<<dim3(npts, nchunk), kDerivThreads, 0, st>>>(dpts, npts, w.cq.p, nq, per, w.part.p));
    const double B = 1.0 / (kPi4 * kEps0);  // src/force.c:232
    DSC_LAUNCH(k_point_derivs_sum<<<(npts * kDerivCount + 255) / 256, 256, 0, st>>>(w.part.p, npts, nchunk, B, w.E.p));
    DSC_CUDA(cudaGetLastError());
    DSC_CUDA(cudaMemcpyAsync(E_host, w.E.p, (size_t)npts * kDerivCount * sizeof(double), cudaMemcpyDeviceToHost,
                             st));
    DSC_CUDA(cudaStreamSynchronize(st));
    return kOk;
}

}  // namespace dsc
