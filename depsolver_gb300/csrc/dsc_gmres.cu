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
                                 const double *__restrict__ x, double *__restrict__ y, const int *skip)
{
    if (skip && *skip) return;  // the GMRES has stopped: nothing to do
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

// ---- one Arnoldi column in one launch: a cluster of kMgsCta CTAs holds
// the new vector w in shared memory (a contiguous slice per CTA) and runs
// the whole modified Gram-Schmidt sequence of the reference's column i
// (src/gmres_el.c:190-200): h_j = v_j . w then w -= h_j v_j for j = 0..i in
// that order, then |w| and w / |w| (written to V[i + 1]).  Each dot product
// is a block sum per CTA and the CTAs' sums added in rank order through
// distributed shared memory between cluster barriers (hardware barriers: no
// polling); the partial-sum slots alternate by parity, so one barrier per
// dot product suffices.  ww (the reference's |w|^2 before the
// orthogonalisation, its zero test) and h[0..i+1] go to global memory.
constexpr int kMgsCta = 8;         // CTAs per cluster (the portable maximum)
constexpr int kMgsThreads = 1024;
constexpr size_t kMgsMaxSlice = 26 * 1024;  // doubles of w per CTA (208 KB of shared memory)

__device__ __forceinline__ void cluster_sync_all()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ unsigned cluster_rank()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// The cluster-wide sum of every thread's v, identical in all threads of all
// CTAs (fixed order: a shuffle tree within each warp, one over the warps'
// sums, one over the CTAs' sums by rank).  slot[p] holds this CTA's partial
// of parity p (read by every CTA of the cluster through distributed shared
// memory), sum[p] the cluster's sum for this CTA's threads.
__device__ __forceinline__ double cluster_sum(double v, double *wsum, double *slot, double *sum, int p)
{
    static_assert(kMgsThreads / 32 == 32 && kMgsCta <= 32, "one warp reduces the warps' and the CTAs' sums");
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    if (lane == 0) wsum[wp] = v;
    __syncthreads();
    if (wp == 0) {
        const double t = warp_sum(wsum[lane]);
        if (lane == 0) slot[p] = t;
    }
    cluster_sync_all();  // every CTA's partial of this parity is written
    if (wp == 0) {
        double x = 0.0;
        if (lane < kMgsCta) {
            const unsigned local = (unsigned)__cvta_generic_to_shared(&slot[p]);
            unsigned remote;
            asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(local), "r"(lane));
            asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(x) : "r"(remote) : "memory");
        }
        x = warp_sum(x);
        if (lane == 0) sum[p] = x;
    }
    __syncthreads();
    return sum[p];
}

__global__ void __launch_bounds__(kMgsThreads, 1) k_mgs_cluster(double *__restrict__ V, int n, int i,
                                                                 double *__restrict__ h, double *__restrict__ ww,
                                                                 const int *__restrict__ done)
{
    extern __shared__ double ws[];                    // this CTA's slice of w
    __shared__ double wsum[kMgsThreads / 32], slot[2], csum[2];
    if (*done) return;  // the whole cluster reads the same flag
    const unsigned rank = cluster_rank();
    const int L = (n + kMgsCta - 1) / kMgsCta;
    const int lo = (int)rank * L, hi = min(n, lo + L);
    double *w = V + (size_t)(i + 1) * n;
    double s = 0.0;
    for (int t = lo + threadIdx.x; t < hi; t += kMgsThreads) {
        const double x = w[t];
        ws[t - lo] = x;
        s += x * x;
    }
    int p = 0;
    const double w2 = cluster_sum(s, wsum, slot, csum, p);
    if (rank == 0 && threadIdx.x == 0) *ww = w2;
    for (int j = 0; j <= i + 1; j++) {
        const double *v = V + (size_t)j * n;
        double d = 0.0;
        if (j <= i)
            for (int t = lo + threadIdx.x; t < hi; t += kMgsThreads) d += v[t] * ws[t - lo];
        else
            for (int t = lo + threadIdx.x; t < hi; t += kMgsThreads) d += ws[t - lo] * ws[t - lo];
        p ^= 1;
        const double hj = cluster_sum(d, wsum, slot, csum, p);
        if (j <= i) {
            for (int t = lo + threadIdx.x; t < hi; t += kMgsThreads) ws[t - lo] = ws[t - lo] - hj * v[t];
            if (rank == 0 && threadIdx.x == 0) h[j] = hj;
        } else {
            const double nr = sqrt(hj);
            if (rank == 0 && threadIdx.x == 0) h[i + 1] = nr;
            for (int t = lo + threadIdx.x; t < hi; t += kMgsThreads) w[t] = nr != 0.0 ? ws[t - lo] / nr : ws[t - lo];
        }
    }
    cluster_sync_all();  // no CTA leaves while another may still read its slots
}

// ---- the reference's Givens step for column i on the device (one thread;
// src/gmres_el.c:202-237), in its operation order without fused
// multiply-adds; the iteration's residual estimate goes to err[i + 1], the
// outcome to st[0] (0 running, 1 converged, 2 "CONVERGENCE RATE TOO SLOW")
// and st[1] = iterations done.
struct GivensDev {
    double *H;     // (M + 2) x (M + 2), row-major
    double *c, *s, *res, *err;
    int *st;       // [0] status, [1] iterations
    double *e0;    // err0
    int M;
};

__global__ void k_givens64(GivensDev g, const double *__restrict__ hcol, const double *__restrict__ ww, int i,
                           double tolerance)
{
    if (g.st[0] != 0) return;
    const int ld = g.M + 2;
    double *H = g.H;
    for (int j = 0; j <= i + 1; j++) H[(size_t)j * ld + i] = hcol[j];
    for (int j = 0; j + 1 <= i; j++) {
        const double a = H[(size_t)j * ld + i], b = H[(size_t)(j + 1) * ld + i];
        const double h1 = __dadd_rn(__dmul_rn(g.c[j], a), __dmul_rn(g.s[j], b));
        const double h2 = __dadd_rn(__dmul_rn(-g.s[j], a), __dmul_rn(g.c[j], b));
        H[(size_t)j * ld + i] = h1;
        H[(size_t)(j + 1) * ld + i] = h2;
    }
    const double htmp = H[(size_t)(i + 1) * ld + i] / H[(size_t)i * ld + i];
    if (sqrt(*ww) != 0.0) {
        const double ci = 1.0 / sqrt(__dadd_rn(1.0, __dmul_rn(htmp, htmp)));
        const double si = __dmul_rn(ci, htmp);
        g.c[i] = ci;
        g.s[i] = si;
        H[(size_t)i * ld + i] = __dadd_rn(__dmul_rn(ci, H[(size_t)i * ld + i]), __dmul_rn(si, H[(size_t)(i + 1) * ld + i]));
        H[(size_t)(i + 1) * ld + i] = 0.0;
        g.res[i + 1] = __dmul_rn(-si, g.res[i]);
        g.res[i] = __dmul_rn(ci, g.res[i]);
    }
    const double err1 = fabs(g.res[i + 1]);
    g.err[i + 1] = err1;
    g.st[1] = i + 1;
    if (err1 < tolerance) g.st[0] = 1;
    else if (fabs(__ddiv_rn(__dsub_rn(err1, *g.e0), *g.e0)) < 1.0e-6 * tolerance) g.st[0] = 2;
    *g.e0 = err1;
}

// The compact N x 2N matrix as an operator.
struct CompactOp : RealOp {
    const double *A;
    size_t lda;
    int N;
    int apply(const double *x, double *y, cudaStream_t st) override
    {
        DSC_LAUNCH(k_matvec_compact<<<(N * 32 + 255) / 256, 256, 0, st>>>(A, lda, N, x, y, skip));
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
    const size_t mgs_slice = ((size_t)n + kMgsCta - 1) / kMgsCta;
    if (err0 < tolerance) {
        status = 0;
    } else if (mgs_slice <= kMgsMaxSlice) {
        // Arnoldi columns in one cluster launch each and the Givens step on
        // the device; the host only looks at the outcome every kPoll
        // iterations (iterations queued after the stop return at once)
        constexpr unsigned kPoll = 4;
        DevBuf<double> dH, dcs, derr, de0;
        DevBuf<int> dst;
        DSC_TRY(dH.alloc((size_t)(M + 2) * (M + 2)));
        DSC_TRY(dcs.alloc(3 * (size_t)(M + 2)));
        DSC_TRY(derr.alloc(M + 2));
        DSC_TRY(de0.alloc(1));
        DSC_TRY(dst.alloc(2));
        DSC_CUDA(cudaMemsetAsync(dH.p, 0, (size_t)(M + 2) * (M + 2) * sizeof(double), st));
        DSC_CUDA(cudaMemsetAsync(dcs.p, 0, 3 * (size_t)(M + 2) * sizeof(double), st));
        DSC_CUDA(cudaMemsetAsync(dst.p, 0, 2 * sizeof(int), st));
        DSC_CUDA(cudaMemcpyAsync(dcs.p + 2 * (M + 2), &r0, sizeof(double), cudaMemcpyHostToDevice, st));
        DSC_CUDA(cudaMemcpyAsync(de0.p, &r0, sizeof(double), cudaMemcpyHostToDevice, st));
        GivensDev gd{dH.p, dcs.p, dcs.p + (M + 2), dcs.p + 2 * (M + 2), derr.p, dst.p, de0.p, (int)M};
        const size_t smem = mgs_slice * sizeof(double);
        DSC_TRY(raise_smem_limit((const void *)k_mgs_cluster, (int)smem));
        op.skip = dst.p;  // status != 0: the operator's kernels return at once
        int hst[2] = {0, 0};
        for (unsigned i0 = 0; i0 < M && hst[0] == 0; i0 += kPoll) {
            for (unsigned i = i0; i < std::min(M, i0 + kPoll); i++) {
                double *vi = V.p + (size_t)i * n, *w = V.p + (size_t)(i + 1) * n;
                DSC_TRY(op.apply(vi, w, st));
                cudaLaunchConfig_t cfg = {};
                cfg.gridDim = dim3(kMgsCta);
                cfg.blockDim = dim3(kMgsThreads);
                cfg.dynamicSmemBytes = smem;
                cfg.stream = st;
                cudaLaunchAttribute at[1];
                at[0].id = cudaLaunchAttributeClusterDimension;
                at[0].val.clusterDim.x = kMgsCta;
                at[0].val.clusterDim.y = 1;
                at[0].val.clusterDim.z = 1;
                cfg.attrs = at;
                cfg.numAttrs = 1;
                note_launch();
                DSC_CUDA(cudaLaunchKernelEx(&cfg, k_mgs_cluster, V.p, n, (int)i, hcol, aux, (const int *)dst.p));
                DSC_LAUNCH(k_givens64<<<1, 1, 0, st>>>(gd, hcol, aux, (int)i, tolerance));
                DSC_CUDA(cudaGetLastError());
            }
            DSC_CUDA(cudaMemcpyAsync(hst, dst.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
            DSC_CUDA(cudaStreamSynchronize(st));
        }
        op.skip = nullptr;
        it = (unsigned)hst[1];
        status = hst[0] == 1 ? 0 : hst[0] == 2 ? 2 : 1;
        // the log lines and what the back substitution needs
        std::vector<double> errs(M + 2);
        DSC_CUDA(cudaMemcpyAsync(errs.data(), derr.p, (M + 2) * sizeof(double), cudaMemcpyDeviceToHost, st));
        DSC_CUDA(cudaMemcpyAsync(h.data(), dH.p, (size_t)(it + 1) * (M + 2) * sizeof(double), cudaMemcpyDeviceToHost,
                                 st));
        DSC_CUDA(cudaMemcpyAsync(res.data(), dcs.p + 2 * (M + 2), (it + 1) * sizeof(double), cudaMemcpyDeviceToHost,
                                 st));
        DSC_CUDA(cudaStreamSynchronize(st));
        if (log)
            for (unsigned q = 1; q <= it; q++) fprintf(log, "%8d%25.4e\n", (int)q, errs[q]);
        if (log) fflush(log);
        if (status != 2) {
            for (int i = (int)it - 1; i >= 0; i--) {
                for (unsigned j = (unsigned)i + 1; j <= it; j++) res[i] -= H(i, j) * res[j];
                res[i] = res[i] / H(i, i);
            }
            DSC_CUDA(cudaMemcpyAsync(resd.p, res.data(), it * sizeof(double), cudaMemcpyHostToDevice, st));
            DSC_LAUNCH(k_update_x<<<vblocks, 256, 0, st>>>(x.p, V.p, n, resd.p, (int)it, n));
            DSC_CUDA(cudaGetLastError());
        }
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
