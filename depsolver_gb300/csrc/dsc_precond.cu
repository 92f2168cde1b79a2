// dsc_precond.cu -- conductor-block right preconditioner of the mixed sweep:
// blocks from the mesh, their inverses by blocked Gauss-Jordan on the
// device, and the application to Krylov blocks and corrections on the
// tensor cores (see dsc_precond.h).
#include <algorithm>
#include <numeric>

#include "dsc_common.cuh"
#include "dsc_df32.cuh"
#include "dsc_gjtile.cuh"
#include "dsc_precond.h"
#include "dsc_session.h"
#include "dsc_tcgemm.h"

namespace dsc {

constexpr int kPreMaxBlocks = 16;     // preconditioner blocks per Gauss-Jordan launch
constexpr int kPreOneStream = 1024;   // blocks up to this size applied on one stream
constexpr int kPreMinRows = 32;       // smaller electrodes keep the Jacobi scaling only
constexpr int kPreMaxRows = 6144;     // larger ones are cut into pieces of at most this
constexpr float kPreVScale = 16384.0f;  // 2^14: fp16 scale of unit Krylov vectors

// ------------------------------------------------------------------ plan

static int uf_find(std::vector<int> &p, int a)
{
    while (p[a] != a) {
        p[a] = p[p[a]];
        a = p[a];
    }
    return a;
}

int precond_plan(Session &s)
{
    Precond &pc = *s.pre;
    const int N = s.N, nen = s.nen;
    std::vector<int> par(N);
    std::iota(par.begin(), par.end(), 0);
    // conductor nodes sharing an element belong to one electrode
    for (int e = 0; e < s.E; e++) {
        int first = -1;
        for (int k = 0; k < nen; k++) {
            const int v = s.plan.elems[(size_t)e * nen + k];
            if (s.iface_of_row[v] >= 0) continue;
            if (first < 0) first = v;
            else {
                const int a = uf_find(par, first), b = uf_find(par, v);
                if (a != b) par[std::max(a, b)] = std::min(a, b);
            }
        }
    }
    std::vector<std::vector<int>> comp;
    std::vector<int> id(N, -1);
    for (int i = 0; i < N; i++) {
        if (s.iface_of_row[i] >= 0) continue;
        const int r = uf_find(par, i);
        if (id[r] < 0) {
            id[r] = (int)comp.size();
            comp.emplace_back();
        }
        comp[id[r]].push_back(i);  // ascending node order
    }
    std::vector<std::vector<int>> blocks;
    for (auto &c : comp) {
        if ((int)c.size() < kPreMinRows) continue;
        const int pieces = ((int)c.size() + kPreMaxRows - 1) / kPreMaxRows;
        const int per = ((int)c.size() + pieces - 1) / pieces;
        for (size_t o = 0; o < c.size(); o += per)
            blocks.emplace_back(c.begin() + o, c.begin() + std::min(c.size(), o + per));
    }
    pc.nb = (int)blocks.size();
    pc.n.clear();
    pc.ldx.clear();
    pc.nbk.clear();
    pc.xoff.clear();
    pc.noff.clear();
    pc.toff.clear();
    if (!pc.nb) return kOk;
    std::vector<int> all, rblk(N, -1), rpos(N, 0);
    size_t xo = 0, no = 0, to = 0;
    for (int b = 0; b < pc.nb; b++) {
        const int n = (int)blocks[b].size(), ldx = (n + kPB - 1) / kPB * kPB;
        pc.n.push_back(n);
        pc.ldx.push_back(ldx);
        pc.nbk.push_back(ldx / kPB);
        pc.xoff.push_back(xo);
        pc.noff.push_back(no);
        pc.toff.push_back(to);
        for (int r = 0; r < n; r++) {
            rblk[blocks[b][r]] = b;
            rpos[blocks[b][r]] = r;
        }
        all.insert(all.end(), blocks[b].begin(), blocks[b].end());
        xo += (size_t)ldx * ldx;
        no += n;
        to += (size_t)kPB * ldx;
    }
    pc.nodes_h = all;
    DSC_TRY(pc.nodes.upload(all, s.st));
    DSC_TRY(pc.rblk.upload(rblk, s.st));
    DSC_TRY(pc.rpos.upload(rpos, s.st));
    DSC_CUDA(cudaStreamSynchronize(s.st));  // the host vectors go out of scope
    return kOk;
}

// ----------------------------------------------------------- Gauss-Jordan
//
// Blocked Gauss-Jordan without pivoting on the padded, Jacobi-scaled block
// (column-major FP32, ldx a multiple of 128; the padding is the identity).
// Step k: P = inverse of the diagonal block (one CTA in shared memory);
// R_J = P X_kJ becomes row block k (X_kk = P); every other tile takes
// X_IJ -= X_Ik R_J and X_Ik = -X_Ik P -- the update runs on the tensor
// cores (3xFP16 on scaled fp16 pairs of the old column block and of R^T,
// tc_gj_update_f16), everything else on the FP32 pipes.

struct GJArgs {
    float *X[kPreMaxBlocks];
    float *tP[kPreMaxBlocks];
    __half *Ah[kPreMaxBlocks], *Al[kPreMaxBlocks];  // ldx x 128: old column block, rows scaled
    __half *Bh[kPreMaxBlocks], *Bl[kPreMaxBlocks];  // ldx x 128: R^T (P^T in tile k), rows scaled
    float *ra[kPreMaxBlocks], *rb[kPreMaxBlocks];   // their row factors
    int ldx[kPreMaxBlocks];
    int nbk[kPreMaxBlocks];
};

// X[c * ldx + a] = K(E[a], E[c]) / K(E[a], E[a]) for a, c < n (K
// column-major FP64, rounded to FP32), the identity on the padding.
__global__ void k_pre_init(const double *__restrict__ K, size_t ld, const double *__restrict__ Kdiag,
                           const int *__restrict__ nodes, int n, float *__restrict__ X, int ldx)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
    if (a >= ldx) return;
    float v;
    if (a < n && c < n) v = (float)K[(size_t)nodes[c] * ld + nodes[a]] * (1.0f / (float)Kdiag[nodes[a]]);
    else v = (a == c) ? 1.0f : 0.0f;
    X[(size_t)c * ldx + a] = v;
}

// tP = the transposed inverse of the 128 x 128 diagonal block k of each
// matrix (blocked Gauss-Jordan without pivoting, one CTA of kGjThreads
// threads per matrix; see gj_invert_tile).
__global__ void __launch_bounds__(kGjThreads) k_gj_pivot(GJArgs g, int nb, int k)
{
    grid_dep_wait();  // a programmatic dependent of the previous step's update
    const int b = blockIdx.x;
    if (b >= nb || k >= g.nbk[b]) return;
    gj_invert_tile(g.X[b] + (size_t)k * kPB * g.ldx[b] + k * kPB, g.ldx[b], nullptr, g.tP[b], 0.0f, nullptr, 0);
}

// Step k, per matrix (blockIdx.z), tile J = blockIdx.x: blockIdx.y < 4:
// columns 32 y .. 32 y + 31 of R_J = P X_kJ (P itself for J = k) written
// into row block k of X and, transposed, as the update's B rows;
// blockIdx.y = 4: tile I = J of the old column block as the update's A
// rows (zero rows for I = k).  256 threads.
__global__ void __launch_bounds__(256) k_gj_row(GJArgs g, int nb, int k)
{
    grid_dep_wait();  // a programmatic dependent of the pivot inversion
    const int b = blockIdx.z, J = blockIdx.x;
    if (b >= nb || k >= g.nbk[b] || J >= g.nbk[b]) return;
    float *X = g.X[b];
    const int ldx = g.ldx[b];
    extern __shared__ __align__(16) float sm[];
    const int warp = threadIdx.x >> 5;
    if (blockIdx.y == 4) {
        // A rows: row i of tile J of column block k, A[i][kk] = X(J*128 + i, k*128 + kk)
        __half *Ah = g.Ah[b] + (size_t)J * kPB * kPB, *Al = g.Al[b] + (size_t)J * kPB * kPB;
        if (J == k) {
            for (int t = threadIdx.x; t < kPB * kPB; t += blockDim.x) {
                Ah[t] = __float2half_rn(0.0f);
                Al[t] = __float2half_rn(0.0f);
            }
            if (threadIdx.x < kPB) g.ra[b][J * kPB + threadIdx.x] = 1.0f;
            return;
        }
        gj_load_rows(X + (size_t)k * kPB * ldx + J * kPB, (size_t)ldx, sm);
        for (int i = warp; i < kPB; i += 8)
            pre_row_pair(&sm[i * 129], Ah + (size_t)i * kPB, Al + (size_t)i * kPB, &g.ra[b][J * kPB + i]);
        return;
    }
    const int j0 = 32 * blockIdx.y;
    const float *PT = g.tP[b];
    const float *T;
    if (J == k) {
        // R_k = P: T[jj][kk] = P(kk, j0 + jj) = PT[(j0 + jj) * 128 + kk]
        for (int t = threadIdx.x; t < 32 * kPB; t += blockDim.x) {
            const int jj = t >> 7, kk = t & 127;
            sm[jj * 129 + kk] = PT[(size_t)(j0 + jj) * kPB + kk];
        }
        __syncthreads();
        T = sm;
    } else {
        T = gj_row_product(PT, X + (size_t)J * kPB * ldx + k * kPB, (size_t)ldx, j0, sm);
    }
    // row block k of X takes R_J: X(k*128 + kk, J*128 + j)
    for (int t = threadIdx.x; t < 32 * kPB; t += blockDim.x) {
        const int jj = t >> 7, kk = t & 127;
        X[(size_t)(J * kPB + j0 + jj) * ldx + k * kPB + kk] = T[jj * 129 + kk];
    }
    __half *Bh = g.Bh[b] + (size_t)J * kPB * kPB, *Bl = g.Bl[b] + (size_t)J * kPB * kPB;
    for (int jj = warp; jj < 32; jj += 8)
        pre_row_pair(&T[jj * 129], Bh + (size_t)(j0 + jj) * kPB, Bl + (size_t)(j0 + jj) * kPB,
                     &g.rb[b][J * kPB + j0 + jj]);
}

// *bound = max(*bound, largest row sum of |Xt| over the first n rows and
// columns) as FP32 bits (non-negative floats order as their bits); one warp
// per row.
__global__ void k_pre_rowsum_max(const float *__restrict__ Xt, int ldx, int n, unsigned *bound)
{
    const int r = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (r >= n) return;
    float t = 0.0f;
    for (int c = lane; c < n; c += 32) t += fabsf(Xt[(size_t)r * ldx + c]);
    t = warp_sum(t);
    if (lane == 0) atomicMax(bound, __float_as_uint(t * 1.001f));  // margin for the rounding of the sum
}

// Xt[r * ldx + c] = X[c * ldx + r] (32 x 32 tiles).
__global__ void k_pre_transpose(const float *__restrict__ X, int ldx, float *__restrict__ Xt)
{
    __shared__ float t[32][33];
    const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) t[y][threadIdx.x] = X[(size_t)(c0 + y) * ldx + r0 + threadIdx.x];
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) Xt[(size_t)(r0 + y) * ldx + c0 + threadIdx.x] = t[threadIdx.x][y];
}

int precond_build(Session &s, cudaStream_t main, cudaStream_t aux)
{
    Precond &pc = *s.pre;
    if (!pc.nb || pc.ready) return kOk;
    cudaStream_t st = main ? main : s.st;
    cudaStream_t side = main ? aux : s.side;
    TimerScope ts(&s.timer, kTPreBuild, st);
    const size_t xtot = pc.xoff.back() + (size_t)pc.ldx.back() * pc.ldx.back();
    const size_t ttot = pc.toff.back() + (size_t)kPB * pc.ldx.back();
    DSC_TRY(pc.X.alloc(xtot));
    DSC_TRY(pc.Xt.alloc(xtot));
    DSC_TRY(pc.Xh.alloc(xtot));
    DSC_TRY(pc.Xl.alloc(xtot));
    DSC_TRY(pc.rs.alloc(pc.noff.back() + pc.n.back()));
    DSC_TRY(pc.tP.alloc((size_t)kPreMaxBlocks * kPB * kPB));
    DSC_TRY(pc.gAh.alloc(2 * ttot));  // two halves: see the step loop
    DSC_TRY(pc.gAl.alloc(2 * ttot));
    DSC_TRY(pc.gBh.alloc(2 * ttot));
    DSC_TRY(pc.gBl.alloc(2 * ttot));
    DSC_TRY(pc.gra.alloc(2 * ttot / kPB));
    DSC_TRY(pc.grb.alloc(2 * ttot / kPB));
    DSC_TRY(pc.err.alloc(1));
    DSC_CUDA(cudaMemsetAsync(pc.err.p, 0, sizeof(int), st));
    double flops = 0.0;
    for (int b = 0; b < pc.nb; b++) {
        const dim3 g((pc.ldx[b] + 255) / 256, pc.ldx[b]);
        DSC_LAUNCH(k_pre_init<<<g, 256, 0, st>>>(s.K64.p, s.ld, s.Kdiag.p, pc.nodes.p + pc.noff[b], pc.n[b],
                                                 pc.X.p + pc.xoff[b], pc.ldx[b]));
        flops += 2.0 * pc.ldx[b] * (double)pc.ldx[b] * pc.ldx[b];
    }
    const size_t rsmem = std::max(kGjRowSmem, sizeof(float) * kPB * 129);
    DSC_CUDA(cudaFuncSetAttribute(k_gj_row, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsmem));
    for (int b0 = 0; b0 < pc.nb; b0 += kPreMaxBlocks) {
        const int nb = std::min(kPreMaxBlocks, pc.nb - b0);
        GJArgs ga{};
        for (int q = 0; q < nb; q++) {
            const int b = b0 + q;
            ga.X[q] = pc.X.p + pc.xoff[b];
            ga.tP[q] = pc.tP.p + (size_t)q * kPB * kPB;
            ga.Ah[q] = pc.gAh.p + pc.toff[b];
            ga.Al[q] = pc.gAl.p + pc.toff[b];
            ga.Bh[q] = pc.gBh.p + pc.toff[b];
            ga.Bl[q] = pc.gBl.p + pc.toff[b];
            ga.ra[q] = pc.gra.p + pc.toff[b] / kPB;
            ga.rb[q] = pc.grb.p + pc.toff[b] / kPB;
            ga.ldx[q] = pc.ldx[b];
            ga.nbk[q] = pc.nbk[b];
        }
        // the update operands alternate between two halves of the buffers
        // by the parity of the step (the rest of step k is still reading
        // its half while step k + 1's row blocks are formed)
        GJArgs gp[2] = {ga, ga};
        for (int q = 0; q < nb; q++) {
            const size_t o = ttot;
            gp[1].Ah[q] += o;
            gp[1].Al[q] += o;
            gp[1].Bh[q] += o;
            gp[1].Bl[q] += o;
            gp[1].ra[q] += o / kPB;
            gp[1].rb[q] += o / kPB;
        }
        int nbk_max = 0;
        for (int q = 0; q < nb; q++) nbk_max = std::max(nbk_max, ga.nbk[q]);
        std::vector<TcGjPlan> plans(2 * (size_t)nb);
        for (int h = 0; h < 2; h++)
            for (int q = 0; q < nb; q++)
                DSC_TRY(tc_gj_plan(plans[2 * q + h], gp[h].Ah[q], gp[h].Al[q], kPB, gp[h].Bh[q], gp[h].Bl[q], kPB,
                                   ga.ldx[q], ga.ldx[q], ga.X[q], (size_t)ga.ldx[q], pc.err.p, gp[h].ra[q],
                                   gp[h].rb[q]));
        // Step k on st: the pivot inverses and row blocks of every block,
        // then (after the rest of step k - 1) the cross of tile k + 1 of the
        // update -- the next pivot tile, row block and column block -- on
        // every SM, and after it, on the side stream, the rest of the update
        // on all but kGjReserveSms SMs, which step k + 1's pivots and row
        // blocks have to themselves.  A block's last step updates
        // everything on st.  Without a side stream every update is whole.
        const bool la = side != nullptr;
        EventPair ev;  // a: step k's cross is done; b: the rest of the last step is
        if (la) DSC_TRY(ev.create());
        int nsm = 0;
        DSC_TRY(current_sm_count(&nsm));
        const int rest_ctas = std::max(1, nsm - kGjReserveSms);
        bool rest_pending = false;
        for (int k = 0; k < nbk_max; k++) {
            const GJArgs &g = gp[k & 1];
            DSC_TRY(launch_dependent(k_gj_pivot, dim3(nb), dim3(kGjThreads), 0, st, g, nb, k));
            DSC_TRY(launch_dependent(k_gj_row, dim3(nbk_max, 5, nb), dim3(256), rsmem, st, g, nb, k));
            if (rest_pending) DSC_CUDA(cudaStreamWaitEvent(st, ev.b, 0));
            // the blocks' updates in one launch per kind: split into cross
            // and rest, or (a block's last step) whole
            const TcGjPlan *sp[kPreMaxBlocks], *wp[kPreMaxBlocks];
            int ns = 0, nw = 0;
            for (int q = 0; q < nb; q++) {
                if (k >= ga.nbk[q]) continue;
                const TcGjPlan *pl = &plans[2 * q + (k & 1)];
                if (la && k + 1 < ga.nbk[q]) sp[ns++] = pl;
                else wp[nw++] = pl;
            }
            constexpr int G = kTcGjMaxProblems;
            for (int i = 0; i < ns; i += G) DSC_TRY(tc_gj_run_batch(sp + i, std::min(G, ns - i), k, st, 1, k + 1));
            for (int i = 0; i < nw; i += G) DSC_TRY(tc_gj_run_batch(wp + i, std::min(G, nw - i), k, st));
            const bool any_rest = ns > 0;
            if (any_rest) {
                DSC_CUDA(cudaEventRecord(ev.a, st));
                DSC_CUDA(cudaStreamWaitEvent(side, ev.a, 0));
                for (int i = 0; i < ns; i += G)
                    DSC_TRY(tc_gj_run_batch(sp + i, std::min(G, ns - i), k, side, 2, k + 1, rest_ctas));
                DSC_CUDA(cudaEventRecord(ev.b, side));
            }
            rest_pending = any_rest;
        }
        if (rest_pending) DSC_CUDA(cudaStreamWaitEvent(st, ev.b, 0));
    }
    // the inverses as row-scaled fp16 pairs for the products (X is
    // column-major: its transpose's rows are X's columns; the products take
    // X^T's rows as their A rows, so the transposed copy goes first), and
    // the bound on |P^-1 v| for unit vectors v
    DSC_TRY(pc.zbound.alloc(1));
    {
        const unsigned one = 0x3F800000u;  // 1.0f: the interface rows keep v
        DSC_CUDA(cudaMemcpyAsync(pc.zbound.p, &one, sizeof(unsigned), cudaMemcpyHostToDevice, st));
    }
    for (int b = 0; b < pc.nb; b++) {
        const int ldx = pc.ldx[b];
        DSC_LAUNCH(k_pre_transpose<<<dim3(ldx / 32, ldx / 32), dim3(32, 8), 0, st>>>(pc.X.p + pc.xoff[b], ldx,
                                                                                     pc.Xt.p + pc.xoff[b]));
        DSC_TRY(split_cols_f16(pc.Xt.p + pc.xoff[b], (size_t)ldx, pc.n[b], pc.n[b], pc.Xh.p + pc.xoff[b],
                               pc.Xl.p + pc.xoff[b], (size_t)ldx, pc.rs.p + pc.noff[b], st));
        DSC_LAUNCH(k_pre_rowsum_max<<<(pc.n[b] * 32 + 255) / 256, 256, 0, st>>>(pc.Xt.p + pc.xoff[b], ldx,
                                                                                pc.n[b], pc.zbound.p));
    }
    s.timer.add_work(kTPreBuild, flops);
    DSC_CUDA(cudaGetLastError());
    int herr = 0;
    DSC_CUDA(cudaMemcpyAsync(&herr, pc.err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    DSC_CUDA(cudaStreamSynchronize(st));
    if (herr) {
        set_error("conductor-block inverse: a pipeline wait of the tensor-core update gave up (code %d)", herr);
        return kErrCuda;
    }
    pc.ready = true;
    return kOk;
}

int precond_export(Session &s, PrecondShare &sh)
{
    Precond &pc = *s.pre;
    if (!pc.ready) {
        set_error("precond_export: the session's inverses are not built");
        return kErrArg;
    }
    AllocStreamScope plain(nullptr);  // the share outlives the session's stream
    sh.nb = pc.nb;
    sh.n = pc.n;
    sh.nodes_h = pc.nodes_h;
    if (!pc.nb) return kOk;
    sh.xtot = pc.xoff.back() + (size_t)pc.ldx.back() * pc.ldx.back();
    sh.rtot = pc.noff.back() + pc.n.back();
    DSC_TRY(sh.Xh.alloc(sh.xtot));
    DSC_TRY(sh.Xl.alloc(sh.xtot));
    DSC_TRY(sh.rs.alloc(sh.rtot));
    DSC_TRY(sh.zbound.alloc(1));
    DSC_CUDA(cudaMemcpyAsync(sh.Xh.p, pc.Xh.p, sh.xtot * sizeof(__half), cudaMemcpyDeviceToDevice, s.st));
    DSC_CUDA(cudaMemcpyAsync(sh.Xl.p, pc.Xl.p, sh.xtot * sizeof(__half), cudaMemcpyDeviceToDevice, s.st));
    DSC_CUDA(cudaMemcpyAsync(sh.rs.p, pc.rs.p, sh.rtot * sizeof(float), cudaMemcpyDeviceToDevice, s.st));
    DSC_CUDA(cudaMemcpyAsync(sh.zbound.p, pc.zbound.p, sizeof(unsigned), cudaMemcpyDeviceToDevice, s.st));
    DSC_CUDA(cudaStreamSynchronize(s.st));
    return kOk;
}

int precond_adopt(Session &s, const PrecondShare &sh)
{
    Precond &pc = *s.pre;
    if (sh.nb != pc.nb || sh.n != pc.n || sh.nodes_h != pc.nodes_h) {
        set_error("precond_adopt: the session's conductor blocks differ from the shared ones");
        return kErrArg;
    }
    if (pc.nb) {
        DSC_TRY(pc.Xh.alloc(sh.xtot));
        DSC_TRY(pc.Xl.alloc(sh.xtot));
        DSC_TRY(pc.rs.alloc(sh.rtot));
        DSC_TRY(pc.zbound.alloc(1));
        DSC_CUDA(cudaMemcpyAsync(pc.Xh.p, sh.Xh.p, sh.xtot * sizeof(__half), cudaMemcpyDeviceToDevice, s.st));
        DSC_CUDA(cudaMemcpyAsync(pc.Xl.p, sh.Xl.p, sh.xtot * sizeof(__half), cudaMemcpyDeviceToDevice, s.st));
        DSC_CUDA(cudaMemcpyAsync(pc.rs.p, sh.rs.p, sh.rtot * sizeof(float), cudaMemcpyDeviceToDevice, s.st));
        DSC_CUDA(cudaMemcpyAsync(pc.zbound.p, sh.zbound.p, sizeof(unsigned), cudaMemcpyDeviceToDevice, s.st));
    }
    pc.ready = true;
    pc.adopted = true;
    return kOk;
}

// ------------------------------------------------------------------ apply

int precond_reserve(Session &s, int F)
{
    Precond &pc = *s.pre;
    // the partial tiles' layout follows F (split stride ldx x 2F), so it is
    // laid out again whenever a batch has another size than the last one;
    // the buffers only grow
    if (!pc.nb || pc.F == F) return kOk;
    pc.S.clear();
    pc.yoff.clear();
    pc.boff.clear();
    size_t yo = 0, bo = 0;
    std::vector<long long> info;
    // splits: about two waves of units over all blocks' products (more
    // splits cost partial tiles written and summed; fewer leave SMs idle)
    int nsm = 0;
    DSC_TRY(current_sm_count(&nsm));
    int tiles = 0;
    for (int b = 0; b < pc.nb; b++) tiles += (pc.n[b] + kPB - 1) / kPB;
    for (int b = 0; b < pc.nb; b++) {
        const int nkb = (pc.n[b] + 63) / 64;  // fp16 k-blocks
        const int S = tc_gemm_f16_splits_norm(pc.n[b], std::max(1, std::min(2 * nsm / tiles, nkb / 4)));
        pc.S.push_back(S);
        pc.yoff.push_back(yo);
        pc.boff.push_back(bo);
        const size_t sstride = (size_t)pc.ldx[b] * 2 * F;
        info.push_back((long long)yo);
        info.push_back((long long)sstride);
        info.push_back(S);
        info.push_back(pc.ldx[b]);
        yo += sstride * S;
        bo += sstride;
    }
    DSC_TRY(pc.Y.alloc(yo));
    DSC_TRY(pc.Bh.alloc(bo));
    DSC_TRY(pc.Bl.alloc(bo));
    DSC_TRY(pc.G.alloc(bo));
    DSC_TRY(pc.csc.alloc((size_t)2 * F * pc.nb));
    DSC_TRY(pc.cz.alloc((size_t)2 * F));
    DSC_TRY(pc.yinfo.upload(info, s.st));
    DSC_CUDA(cudaStreamSynchronize(s.st));
    pc.F = F;
    return kOk;
}

// fp16 pair of 2^14 v (v = V[c][E[r]] in double-FP32, |v| <= 1) at
// B[c * ldb + r], for the rows of one block.
__global__ void k_pre_gather_v(const float2 *__restrict__ V, size_t ld, const int *__restrict__ nodes, int n,
                               __half *__restrict__ Bh, __half *__restrict__ Bl, int ldb)
{
    grid_dep_wait();
    const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
    if (r >= n) return;
    const float2 v = V[(size_t)c * ld + nodes[r]];
    const float x = v.x * kPreVScale;
    const __half h = __float2half_rn(x);
    Bh[(size_t)c * ldb + r] = h;
    Bl[(size_t)c * ldb + r] = __float2half_rn(__fadd_rn(__fsub_rn(x, __half2float(h)), v.y * kPreVScale));
}

// z = P^-1 v for column c: the block products' partial tiles summed in
// split order on preconditioned rows, v (hi + lo, rounded) elsewhere;
// written as the fp16 pair of 2^t z (Zh, Zl) for the product with K, t
// fixed by zbound (the FP32 bits of a bound on |z|: max(1, the largest row
// sum of |X_b|)); cz[c] = 2^-t.
__global__ void k_pre_combine(const float2 *__restrict__ V, size_t ld, int N, const int *__restrict__ rblk,
                              const int *__restrict__ rpos, const float *__restrict__ Y,
                              const long long *__restrict__ yinfo, const unsigned *__restrict__ zbound,
                              __half *__restrict__ Zh, __half *__restrict__ Zl, float *__restrict__ cz)
{
    grid_dep_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
    const int sh = max(-100, min(100, 14 - ((int)(*zbound >> 23) - 127)));
    if (i == 0) cz[c] = pre_pow2(-sh);
    if (i >= N) return;
    const int b = rblk[i];
    float z;
    if (b < 0) {
        const float2 v = V[(size_t)c * ld + i];
        z = v.x + v.y;
    } else {
        const long long *inf = yinfo + 4 * b;
        const float *y = Y + inf[0] + (size_t)c * inf[3] + rpos[i];
        float2 acc = make_float2(0.f, 0.f);
        for (long long sp = 0; sp < inf[2]; sp++) {
            const float2 t = df_two_sum(acc.x, y[sp * inf[1]]);
            acc = make_float2(t.x, acc.y + t.y);
        }
        z = acc.x + acc.y;
    }
    const float x = z * pre_pow2(sh);
    const __half h = __float2half_rn(x);
    Zh[(size_t)c * ld + i] = h;
    Zl[(size_t)c * ld + i] = __float2half_rn(x - __half2float(h));
}


// G[c * ldg + r] = D[c][E[r]] for the rows of one block.
__global__ void k_pre_gather_d(const double *__restrict__ D, size_t ld, const int *__restrict__ nodes, int n,
                               double *__restrict__ G, int ldg)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
    if (r < n) G[(size_t)c * ldg + r] = D[(size_t)c * ld + nodes[r]];
}

// D[c][E[r]] = the block product's partial tiles summed in split order (FP64).
__global__ void k_pre_scatter_d(double *__restrict__ D, size_t ld, const int *__restrict__ nodes, int n,
                                const float *__restrict__ Y, int S, size_t sstride, int ldy)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
    if (r >= n) return;
    const float *y = Y + (size_t)c * ldy + r;
    double t = 0.0;
    for (int sp = 0; sp < S; sp++) t += (double)y[(size_t)sp * sstride];
    D[(size_t)c * ld + nodes[r]] = t;
}

int precond_apply_v(Session &s, const float2 *V, int F, __half *Zh, __half *Zl, const float *cscK, int *d_err,
                    const float **cz)
{
    Precond &pc = *s.pre;
    cudaStream_t st = s.st;
    TimerScope ts(&s.timer, kTPreApply, st);
    const int F2 = 2 * F;
    // odd blocks on the side stream: each block's product is a small GEMM
    // (tens of CTAs), two of them fill more of the GPU; blocks of at most
    // kPreOneStream rows stay on st (the products take microseconds, less
    // than the streams' fork and join)
    SideJoin sj;
    int nmax = 0;
    for (int b = 0; b < pc.nb; b++) nmax = std::max(nmax, pc.n[b]);
    const bool two = pc.nb >= 2 && s.side && nmax > kPreOneStream;
    if (two) DSC_TRY(sj.fork(st, s.side));
    for (int b = 0; b < pc.nb; b++) {
        const int n = pc.n[b], ldx = pc.ldx[b];
        cudaStream_t sb = two && (b & 1) ? s.side : st;
        DSC_TRY(launch_dependent(k_pre_gather_v, dim3((n + 255) / 256, F2), dim3(256), 0, sb, V, s.ld,
                                 pc.nodes.p + pc.noff[b], n, pc.Bh.p + pc.boff[b], pc.Bl.p + pc.boff[b], ldx));
        DSC_TRY(tc_gemm_3xf16(pc.Xh.p + pc.xoff[b], pc.Xl.p + pc.xoff[b], ldx, pc.Bh.p + pc.boff[b],
                              pc.Bl.p + pc.boff[b], ldx, n, F2, n, pc.Y.p + pc.yoff[b], ldx, pc.S[b], d_err, sb,
                              pc.rs.p + pc.noff[b], cscK));
        s.timer.add_work(kTPreApply, 6.0 * n * (double)n * F2);
    }
    if (two) {
        DSC_TRY(sj.done(s.side));
        DSC_TRY(sj.join());
    }
    DSC_TRY(launch_dependent(k_pre_combine, dim3((s.N + 255) / 256, F2), dim3(256), 0, st, V, s.ld, s.N,
                             pc.rblk.p, pc.rpos.p, pc.Y.p, pc.yinfo.p, pc.zbound.p, Zh, Zl, pc.cz.p));
    DSC_CUDA(cudaGetLastError());
    *cz = pc.cz.p;
    return kOk;
}

int precond_apply_d(Session &s, double *D, int F, int *d_err)
{
    Precond &pc = *s.pre;
    cudaStream_t st = s.st;
    TimerScope ts(&s.timer, kTPreApply, st);
    const int F2 = 2 * F;
    // blocks' rows are disjoint: odd blocks on the side stream (large
    // blocks only, as above)
    SideJoin sj;
    int nmax = 0;
    for (int b = 0; b < pc.nb; b++) nmax = std::max(nmax, pc.n[b]);
    const bool two = pc.nb >= 2 && s.side && nmax > kPreOneStream;
    if (two) DSC_TRY(sj.fork(st, s.side));
    for (int b = 0; b < pc.nb; b++) {
        const int n = pc.n[b], ldx = pc.ldx[b];
        const dim3 g((n + 255) / 256, F2);
        cudaStream_t sb = two && (b & 1) ? s.side : st;
        DSC_LAUNCH(k_pre_gather_d<<<g, 256, 0, sb>>>(D, s.ld, pc.nodes.p + pc.noff[b], n, pc.G.p + pc.boff[b], ldx));
        float *csc = pc.csc.p + (size_t)F2 * b;
        DSC_TRY(split_cols_f16(pc.G.p + pc.boff[b], (size_t)ldx, n, F2, pc.Bh.p + pc.boff[b], pc.Bl.p + pc.boff[b],
                               (size_t)ldx, csc, sb));
        DSC_TRY(tc_gemm_3xf16(pc.Xh.p + pc.xoff[b], pc.Xl.p + pc.xoff[b], ldx, pc.Bh.p + pc.boff[b],
                              pc.Bl.p + pc.boff[b], ldx, n, F2, n, pc.Y.p + pc.yoff[b], ldx, pc.S[b], d_err, sb,
                              pc.rs.p + pc.noff[b], csc));
        DSC_LAUNCH(k_pre_scatter_d<<<g, 256, 0, sb>>>(D, s.ld, pc.nodes.p + pc.noff[b], n, pc.Y.p + pc.yoff[b],
                                                      pc.S[b], (size_t)ldx * F2, ldx));
        s.timer.add_work(kTPreApply, 6.0 * n * (double)n * F2);
    }
    if (two) {
        DSC_TRY(sj.done(s.side));
        DSC_TRY(sj.join());
    }
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

void destroy_precond(Precond *p) { delete p; }

}  // namespace dsc
