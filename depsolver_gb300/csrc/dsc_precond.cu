// dsc_precond.cu -- conductor-block right preconditioner of the mixed sweep:
// blocks from the mesh, their inverses by blocked Gauss-Jordan on the
// device, and the application to Krylov blocks and corrections on the
// tensor cores (see dsc_precond.h).
#include <algorithm>
#include <numeric>

#include "dsc_df32.cuh"
#include "dsc_precond.h"
#include "dsc_session.h"
#include "dsc_tcgemm.h"

namespace dsc {

constexpr int kPB = 128;              // Gauss-Jordan block
constexpr int kPreMaxBlocks = 16;     // preconditioner blocks per Gauss-Jordan launch
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
    DSC_TRY(pc.nodes.upload(all, s.st));
    DSC_TRY(pc.rblk.upload(rblk, s.st));
    DSC_TRY(pc.rpos.upload(rpos, s.st));
    DSC_CUDA(cudaStreamSynchronize(s.st));  // the host vectors go out of scope
    return kOk;
}

// ----------------------------------------------------------- Gauss-Jordan

struct GJArgs {
    float *X[kPreMaxBlocks];
    float *tP[kPreMaxBlocks];
    float *tR[kPreMaxBlocks];
    float *tC[kPreMaxBlocks];
    int ldx[kPreMaxBlocks];
    int nbk[kPreMaxBlocks];
};

// X[a][c] (row-major, ldx) = K(E[a], E[c]) / K(E[a], E[a]) for a, c < n (K
// column-major FP64, rounded to FP32), the identity on the padding; 32 x 32
// tiles through shared memory.
__global__ void k_pre_init(const double *__restrict__ K, size_t ld, const double *__restrict__ Kdiag,
                           const int *__restrict__ nodes, int n, float *__restrict__ X, int ldx)
{
    __shared__ float t[32][33];
    const int a0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
    {
        const int a = a0 + threadIdx.x;
        const float rd = a < n ? 1.0f / (float)Kdiag[nodes[a]] : 0.0f;
        for (int y = threadIdx.y; y < 32; y += blockDim.y) {
            const int c = c0 + y;
            float v;
            if (a < n && c < n) v = (float)K[(size_t)nodes[c] * ld + nodes[a]] * rd;
            else v = (a == c) ? 1.0f : 0.0f;
            t[y][threadIdx.x] = v;  // t[c - c0][a - a0]
        }
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int a = a0 + y, c = c0 + threadIdx.x;
        X[(size_t)a * ldx + c] = t[threadIdx.x][y];
    }
}

// tP = inverse of the 128 x 128 diagonal block k of each matrix
// (Gauss-Jordan without pivoting in shared memory, one CTA per matrix).
__global__ void __launch_bounds__(1024) k_gj_pivot(GJArgs g, int nb, int k)
{
    const int b = blockIdx.x;
    if (b >= nb || k >= g.nbk[b]) return;
    const float *X = g.X[b];
    const int ldx = g.ldx[b];
    extern __shared__ float sm[];
    float *a = sm;                // 128 x 129
    float *col = sm + kPB * 129;  // 128
    for (int t = threadIdx.x; t < kPB * kPB; t += blockDim.x) {
        const int r = t >> 7, c = t & 127;
        a[r * 129 + c] = X[(size_t)(k * kPB + r) * ldx + k * kPB + c];
    }
    __syncthreads();
    for (int j = 0; j < kPB; j++) {
        if (threadIdx.x < kPB) col[threadIdx.x] = a[threadIdx.x * 129 + j];
        __syncthreads();
        const float piv = 1.0f / col[j];
        if (threadIdx.x < kPB) {
            const int c = threadIdx.x;
            a[j * 129 + c] = (c == j) ? piv : a[j * 129 + c] * piv;
        }
        __syncthreads();
        for (int t = threadIdx.x; t < kPB * kPB; t += blockDim.x) {
            const int r = t >> 7, c = t & 127;
            if (r == j) continue;
            const float f = col[r];
            a[r * 129 + c] = (c == j) ? -f * piv : a[r * 129 + c] - f * a[j * 129 + c];
        }
        __syncthreads();
    }
    float *P = g.tP[b];
    for (int t = threadIdx.x; t < kPB * kPB; t += blockDim.x) P[t] = a[(t >> 7) * 129 + (t & 127)];
}

// acc (8 x 8 per thread: rows 8 ty + u, columns 8 tx + v of a 128 x 128
// tile; 256 threads) = A (128 x 128, row-major, lda) * B (128 x 128,
// row-major, ldb), k in chunks of 32 through shared memory.
__device__ __forceinline__ void tile_gemm128(const float *__restrict__ A, int lda, const float *__restrict__ B,
                                             int ldb, float (*As)[129], float (*Bs)[128], float acc[8][8])
{
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
#pragma unroll
    for (int u = 0; u < 8; u++)
#pragma unroll
        for (int v = 0; v < 8; v++) acc[u][v] = 0.0f;
    for (int k0 = 0; k0 < kPB; k0 += 32) {
        // A chunk: 128 rows x 32 k, stored transposed As[kk][row]
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const int t = tid + 256 * q, kk = t & 31, row = t >> 5;
            As[kk][row] = A[(size_t)row * lda + k0 + kk];
        }
        // B chunk: 32 k x 128 columns
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int t = tid + 256 * q, kk = t >> 5, c4 = t & 31;
            *(float4 *)&Bs[kk][4 * c4] = *(const float4 *)(B + (size_t)(k0 + kk) * ldb + 4 * c4);
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < 32; kk++) {
            float a[8], bv[8];
#pragma unroll
            for (int u = 0; u < 8; u++) a[u] = As[kk][8 * ty + u];
            const float4 b0 = *(const float4 *)&Bs[kk][8 * tx], b1 = *(const float4 *)&Bs[kk][8 * tx + 4];
            bv[0] = b0.x; bv[1] = b0.y; bv[2] = b0.z; bv[3] = b0.w;
            bv[4] = b1.x; bv[5] = b1.y; bv[6] = b1.z; bv[7] = b1.w;
#pragma unroll
            for (int u = 0; u < 8; u++)
#pragma unroll
                for (int v = 0; v < 8; v++) acc[u][v] = fmaf(a[u], bv[v], acc[u][v]);
        }
        __syncthreads();
    }
}

constexpr size_t kTileSmem = sizeof(float) * (32 * 129 + 32 * 128);

// Step k, per matrix: tR[:, J] = tP * X[row block k][column block J] (J != k)
// for blockIdx.y = 0, tC[row block J][:] = X[row block J][column block k]
// for blockIdx.y = 1.
__global__ void __launch_bounds__(256) k_gj_row(GJArgs g, int nb, int k)
{
    const int b = blockIdx.z, J = blockIdx.x;
    if (b >= nb || k >= g.nbk[b] || J >= g.nbk[b]) return;
    const float *X = g.X[b];
    const int ldx = g.ldx[b];
    if (blockIdx.y == 1) {
        float *C = g.tC[b] + (size_t)J * kPB * kPB;
        for (int t = threadIdx.x; t < kPB * kPB / 4; t += blockDim.x) {
            const int r = t >> 5, c4 = t & 31;
            *(float4 *)(C + (size_t)r * kPB + 4 * c4) =
                *(const float4 *)(X + (size_t)(J * kPB + r) * ldx + k * kPB + 4 * c4);
        }
        return;
    }
    if (J == k) return;
    extern __shared__ float sm[];
    float(*As)[129] = (float(*)[129])sm;
    float(*Bs)[128] = (float(*)[128])(sm + 32 * 129);
    float acc[8][8];
    tile_gemm128(g.tP[b], kPB, X + (size_t)k * kPB * ldx + J * kPB, ldx, As, Bs, acc);
    const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
    float *R = g.tR[b] + J * kPB;
#pragma unroll
    for (int u = 0; u < 8; u++) {
        float *o = R + (size_t)(8 * ty + u) * ldx + 8 * tx;
        *(float4 *)o = make_float4(acc[u][0], acc[u][1], acc[u][2], acc[u][3]);
        *(float4 *)(o + 4) = make_float4(acc[u][4], acc[u][5], acc[u][6], acc[u][7]);
    }
}

// Step k, per matrix and tile (I, J): row block k takes tR (and tP on the
// diagonal); other rows X_IJ -= tC_I tR_J, and X_Ik = -tC_I tP.
__global__ void __launch_bounds__(256) k_gj_update(GJArgs g, int nb, int k)
{
    const int b = blockIdx.z, I = blockIdx.y, J = blockIdx.x;
    if (b >= nb || k >= g.nbk[b] || I >= g.nbk[b] || J >= g.nbk[b]) return;
    float *X = g.X[b];
    const int ldx = g.ldx[b];
    float *T = X + (size_t)I * kPB * ldx + J * kPB;
    if (I == k) {
        const float *src = J == k ? g.tP[b] : g.tR[b] + J * kPB;
        const int lds = J == k ? kPB : ldx;
        for (int t = threadIdx.x; t < kPB * kPB / 4; t += blockDim.x) {
            const int r = t >> 5, c4 = t & 31;
            *(float4 *)(T + (size_t)r * ldx + 4 * c4) = *(const float4 *)(src + (size_t)r * lds + 4 * c4);
        }
        return;
    }
    extern __shared__ float sm[];
    float(*As)[129] = (float(*)[129])sm;
    float(*Bs)[128] = (float(*)[128])(sm + 32 * 129);
    float acc[8][8];
    const bool diag = J == k;
    tile_gemm128(g.tC[b] + (size_t)I * kPB * kPB, kPB, diag ? g.tP[b] : g.tR[b] + J * kPB, diag ? kPB : ldx, As,
                 Bs, acc);
    const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
#pragma unroll
    for (int u = 0; u < 8; u++) {
        float *o = T + (size_t)(8 * ty + u) * ldx + 8 * tx;
        float4 p = *(const float4 *)o, q = *(const float4 *)(o + 4);
        if (diag) {
            p = make_float4(-acc[u][0], -acc[u][1], -acc[u][2], -acc[u][3]);
            q = make_float4(-acc[u][4], -acc[u][5], -acc[u][6], -acc[u][7]);
        } else {
            p.x -= acc[u][0]; p.y -= acc[u][1]; p.z -= acc[u][2]; p.w -= acc[u][3];
            q.x -= acc[u][4]; q.y -= acc[u][5]; q.z -= acc[u][6]; q.w -= acc[u][7];
        }
        *(float4 *)o = p;
        *(float4 *)(o + 4) = q;
    }
}

int precond_build(Session &s)
{
    Precond &pc = *s.pre;
    if (!pc.nb || pc.ready) return kOk;
    cudaStream_t st = s.st;
    TimerScope ts(&s.timer, kTPreBuild, st);
    const size_t xtot = pc.xoff.back() + (size_t)pc.ldx.back() * pc.ldx.back();
    const size_t ttot = pc.toff.back() + (size_t)kPB * pc.ldx.back();
    DSC_TRY(pc.X.alloc(xtot));
    DSC_TRY(pc.Xh.alloc(xtot));
    DSC_TRY(pc.Xl.alloc(xtot));
    DSC_TRY(pc.rs.alloc(pc.noff.back() + pc.n.back()));
    DSC_TRY(pc.tP.alloc((size_t)kPreMaxBlocks * kPB * kPB));
    DSC_TRY(pc.tR.alloc(ttot));
    DSC_TRY(pc.tC.alloc(ttot));
    double flops = 0.0;
    for (int b = 0; b < pc.nb; b++) {
        const dim3 g(pc.ldx[b] / 32, pc.ldx[b] / 32);
        DSC_LAUNCH(k_pre_init<<<g, dim3(32, 8), 0, st>>>(s.K64.p, s.ld, s.Kdiag.p, pc.nodes.p + pc.noff[b], pc.n[b],
                                                         pc.X.p + pc.xoff[b], pc.ldx[b]));
        flops += 2.0 * pc.ldx[b] * (double)pc.ldx[b] * pc.ldx[b];
    }
    const size_t psmem = sizeof(float) * (kPB * 129 + kPB);
    DSC_CUDA(cudaFuncSetAttribute(k_gj_pivot, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem));
    DSC_CUDA(cudaFuncSetAttribute(k_gj_row, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTileSmem));
    DSC_CUDA(cudaFuncSetAttribute(k_gj_update, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTileSmem));
    for (int b0 = 0; b0 < pc.nb; b0 += kPreMaxBlocks) {
        const int nb = std::min(kPreMaxBlocks, pc.nb - b0);
        GJArgs ga{};
        int nbk_max = 0;
        for (int q = 0; q < nb; q++) {
            const int b = b0 + q;
            ga.X[q] = pc.X.p + pc.xoff[b];
            ga.tP[q] = pc.tP.p + (size_t)q * kPB * kPB;
            ga.tR[q] = pc.tR.p + pc.toff[b];
            ga.tC[q] = pc.tC.p + pc.toff[b];
            ga.ldx[q] = pc.ldx[b];
            ga.nbk[q] = pc.nbk[b];
            nbk_max = std::max(nbk_max, pc.nbk[b]);
        }
        for (int k = 0; k < nbk_max; k++) {
            DSC_LAUNCH(k_gj_pivot<<<nb, 1024, psmem, st>>>(ga, nb, k));
            DSC_LAUNCH(k_gj_row<<<dim3(nbk_max, 2, nb), 256, kTileSmem, st>>>(ga, nb, k));
            DSC_LAUNCH(k_gj_update<<<dim3(nbk_max, nbk_max, nb), 256, kTileSmem, st>>>(ga, nb, k));
        }
    }
    // the inverses as row-scaled fp16 pairs (rows of X are the K-major rows
    // of the product's A operand; their factors are the epilogue's)
    for (int b = 0; b < pc.nb; b++)
        DSC_TRY(split_cols_f16(pc.X.p + pc.xoff[b], (size_t)pc.ldx[b], pc.n[b], pc.n[b], pc.Xh.p + pc.xoff[b],
                               pc.Xl.p + pc.xoff[b], (size_t)pc.ldx[b], pc.rs.p + pc.noff[b], st));
    s.timer.add_work(kTPreBuild, flops);
    DSC_CUDA(cudaGetLastError());
    pc.ready = true;
    return kOk;
}

// ------------------------------------------------------------------ apply

int precond_reserve(Session &s, int F)
{
    Precond &pc = *s.pre;
    if (!pc.nb || pc.F >= F) return kOk;
    pc.S.clear();
    pc.yoff.clear();
    pc.boff.clear();
    size_t yo = 0, bo = 0;
    std::vector<long long> info;
    for (int b = 0; b < pc.nb; b++) {
        const int S = tc_gemm_f16_splits_for(pc.n[b], pc.n[b]);
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
    const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
    if (r >= n) return;
    const float2 v = V[(size_t)c * ld + nodes[r]];
    const float x = v.x * kPreVScale;
    const __half h = __float2half_rn(x);
    Bh[(size_t)c * ldb + r] = h;
    Bl[(size_t)c * ldb + r] = __float2half_rn(__fadd_rn(__fsub_rn(x, __half2float(h)), v.y * kPreVScale));
}

// Z[c][i] = P^-1 v: the block products' partial tiles summed in split order
// on preconditioned rows, v (hi + lo, rounded) elsewhere.
__global__ void k_pre_combine(const float2 *__restrict__ V, size_t ld, int N, const int *__restrict__ rblk,
                              const int *__restrict__ rpos, const float *__restrict__ Y,
                              const long long *__restrict__ yinfo, float *__restrict__ Z)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
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
    Z[(size_t)c * ld + i] = z;
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

int precond_apply_v(Session &s, const float2 *V, int F, float *Z, const float *cscK, int *d_err)
{
    Precond &pc = *s.pre;
    cudaStream_t st = s.st;
    TimerScope ts(&s.timer, kTPreApply, st);
    const int F2 = 2 * F;
    for (int b = 0; b < pc.nb; b++) {
        const int n = pc.n[b], ldx = pc.ldx[b];
        DSC_LAUNCH(k_pre_gather_v<<<dim3((n + 255) / 256, F2), 256, 0, st>>>(
            V, s.ld, pc.nodes.p + pc.noff[b], n, pc.Bh.p + pc.boff[b], pc.Bl.p + pc.boff[b], ldx));
        DSC_TRY(tc_gemm_3xf16(pc.Xh.p + pc.xoff[b], pc.Xl.p + pc.xoff[b], ldx, pc.Bh.p + pc.boff[b],
                              pc.Bl.p + pc.boff[b], ldx, n, F2, n, pc.Y.p + pc.yoff[b], ldx, pc.S[b], d_err, st,
                              pc.rs.p + pc.noff[b], cscK));
        s.timer.add_work(kTPreApply, 6.0 * n * (double)n * F2);
    }
    DSC_LAUNCH(k_pre_combine<<<dim3((s.N + 255) / 256, F2), 256, 0, st>>>(V, s.ld, s.N, pc.rblk.p, pc.rpos.p,
                                                                         pc.Y.p, pc.yinfo.p, Z));
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

int precond_apply_d(Session &s, double *D, int F, int *d_err)
{
    Precond &pc = *s.pre;
    cudaStream_t st = s.st;
    TimerScope ts(&s.timer, kTPreApply, st);
    const int F2 = 2 * F;
    for (int b = 0; b < pc.nb; b++) {
        const int n = pc.n[b], ldx = pc.ldx[b];
        const dim3 g((n + 255) / 256, F2);
        DSC_LAUNCH(k_pre_gather_d<<<g, 256, 0, st>>>(D, s.ld, pc.nodes.p + pc.noff[b], n, pc.G.p + pc.boff[b], ldx));
        float *csc = pc.csc.p + (size_t)F2 * b;
        DSC_TRY(split_cols_f16(pc.G.p + pc.boff[b], (size_t)ldx, n, F2, pc.Bh.p + pc.boff[b], pc.Bl.p + pc.boff[b],
                               (size_t)ldx, csc, st));
        DSC_TRY(tc_gemm_3xf16(pc.Xh.p + pc.xoff[b], pc.Xl.p + pc.xoff[b], ldx, pc.Bh.p + pc.boff[b],
                              pc.Bl.p + pc.boff[b], ldx, n, F2, n, pc.Y.p + pc.yoff[b], ldx, pc.S[b], d_err, st,
                              pc.rs.p + pc.noff[b], csc));
        DSC_LAUNCH(k_pre_scatter_d<<<g, 256, 0, st>>>(D, s.ld, pc.nodes.p + pc.noff[b], n, pc.Y.p + pc.yoff[b],
                                                      pc.S[b], (size_t)ldx * F2, ldx));
        s.timer.add_work(kTPreApply, 6.0 * n * (double)n * F2);
    }
    DSC_CUDA(cudaGetLastError());
    return kOk;
}

void destroy_precond(Precond *p) { delete p; }

}  // namespace dsc
