// dsc_capi.cu -- the exported C ABI (include/depsolver_cuda.h).
//
// Drop-in entry points keep the reference's names, signatures, globals and
// error behaviour; dsc_* entry points take flat arrays and return status
// codes.  Both run the same device code.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/depsolver_cuda.h"
#include "dsc_common.cuh"
#include "dsc_field.h"
#include "dsc_quad8.h"
#include "dsc_gmres.h"
#include "dsc_internal.h"

// Globals read by the drop-in entry points (the reference defines them in
// src/depSolver.c:46-50; a host program's definitions take precedence).
unsigned int nNodes, nElems, nInterfaces;
FILE *file_log;

namespace dsc {

// ---------------------------------------------------------------- context
struct MeshEntry {
    uint64_t key = 0;
    HostPlan plan;
    DeviceMesh dev;
};

struct Context {
    std::mutex mu;
    cudaStream_t st = nullptr;
    std::unique_ptr<MeshEntry> mesh;
    uint64_t sigma_key = 0;
    DevBuf<double> sigma;
    std::vector<double> sigma_host;  // host copy of the solution on the device
    // point evaluations: one point set and output buffer kept between calls
    // (the reference's post-processing evaluates one point per call); for
    // few points the quadrature charges of the current solution (cq, for
    // solution upload cq_gen of mesh cq_key) and the packed staging
    PointSet pts;
    DevBuf<double> pout;
    uint64_t sigma_gen = 0, cq_gen = ~(uint64_t)0, cq_key = 0;
    DevBuf<double> cq;
    FewPointWork few;
    // the quad8 family: its mesh (rebuilt when the content changes), the
    // solution and the point results on the device
    std::unique_ptr<Q8Mesh> q8;
    uint64_t q8_key = 0;
    DevBuf<double> q8_sigma, q8_out;
    // multipole / ellipsoid force points: their coordinates and workspace
    DevBuf<double> dpts;
    DerivWork deriv;
    double *pinned = nullptr;
    size_t pinned_bytes = 0;
    // direct solve: the tensor-core block LU with FP64 refinement (default)
    // or the FP64 LU; the last solve's refinement steps, relative residual
    // and whether it fell back to the FP64 LU
    int gauss_mode = DSC_GAUSS_MIXED;
    LuMixedInfo gauss_info;
    int gauss_fell_back = 0;
};

static Context &ctx()
{
    static Context c;
    return c;
}

static int ensure_stream()
{
    Context &c = ctx();
    if (!c.st) {
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
            cudaGetLastError();
            set_error("no CUDA device available");
            return kErrCuda;
        }
        DSC_CUDA(cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking));
    }
    return kOk;
}

static int ensure_pinned(size_t bytes)
{
    Context &c = ctx();
    if (c.pinned_bytes >= bytes) return kOk;
    if (c.pinned) cudaFreeHost(c.pinned);
    c.pinned = nullptr;
    c.pinned_bytes = 0;
    DSC_CUDA(cudaHostAlloc((void **)&c.pinned, bytes, cudaHostAllocDefault));
    c.pinned_bytes = bytes;
    return kOk;
}

// ---------------------------------------------------------------- row movers
// The drop-ins' matrices are the reference's row-pointer arrays (or strided
// flat rows), gigabytes at the 12k-node scene.  They move in chunks of rows
// through two halves of one pinned buffer: host threads fill (or drain) one
// half while the copy engine moves the other.
constexpr size_t kMoverChunkBytes = (size_t)128 << 20;

static int mover_threads()
{
    const unsigned h = std::thread::hardware_concurrency();
    return (int)std::max(1u, std::min(16u, h ? h : 1u));
}

// fn(r) for r in [r0, r1) on the host threads (contiguous ranges).
template <typename Fn>
static void host_parallel_rows(size_t r0, size_t r1, Fn fn)
{
    const int T = mover_threads();
    const size_t n = r1 - r0;
    if (T == 1 || n < 64) {
        for (size_t r = r0; r < r1; r++) fn(r);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < T; t++) {
        const size_t a = r0 + n * t / T, b = r0 + n * (t + 1) / T;
        th.emplace_back([=] {
            for (size_t r = a; r < b; r++) fn(r);
        });
    }
    for (auto &x : th) x.join();
}

// dst (device, row r at dst + r * ldd) row r = fill(r, host row of ldd
// doubles) for r < nrows.
template <typename Fill>
static int rows_to_device(size_t nrows, size_t ldd, double *dst, Fill fill, cudaStream_t st)
{
    const size_t per = std::max<size_t>(1, kMoverChunkBytes / (ldd * sizeof(double)));
    DSC_TRY(ensure_pinned(2 * per * ldd * sizeof(double)));
    double *half[2] = {ctx().pinned, ctx().pinned + per * ldd};
    cudaEvent_t ev[2];
    DSC_CUDA(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
    DSC_CUDA(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
    int rc = kOk;
    size_t q = 0;
    for (size_t r0 = 0; r0 < nrows && rc == kOk; r0 += per, q++) {
        const size_t r1 = std::min(nrows, r0 + per);
        double *h = half[q & 1];
        if (q >= 2 && cudaEventSynchronize(ev[q & 1]) != cudaSuccess) rc = kErrCuda;  // its last copy is done
        if (rc != kOk) break;
        host_parallel_rows(r0, r1, [&](size_t r) { fill(r, h + (r - r0) * ldd); });
        if (cudaMemcpyAsync(dst + r0 * ldd, h, (r1 - r0) * ldd * sizeof(double), cudaMemcpyHostToDevice, st) !=
                cudaSuccess ||
            cudaEventRecord(ev[q & 1], st) != cudaSuccess)
            rc = kErrCuda;
    }
    if (rc == kOk && cudaStreamSynchronize(st) != cudaSuccess) rc = kErrCuda;
    if (rc != kOk) set_error("row upload: %s", cudaGetErrorString(cudaGetLastError()));
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    return rc;
}

// ---------------------------------------------------------------- host rows read by the device
// On a device that reads pageable host memory through the host's page
// tables (Grace-Blackwell over NVLink-C2C), the drop-ins' row-pointer
// matrices go to the device in one gather kernel that reads the caller's
// rows where they are, instead of host threads copying them into pinned
// halves first (mode 1, the default).  Mode 2 also adds the assembled rows
// into the caller's rows from the device; on the 12k-node scene that took
// 0.12 to 0.59 s from one box and run to the next for 5 GB of rows (the
// device's first writes to the caller's pages), the staged copy a steady
// 0.18 s, so it is not the default.  Mode 0: staged both ways.
static int g_host_direct = 1;

static bool host_direct(bool write)
{
    if (g_host_direct < (write ? 2 : 1)) return false;
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return v != 0;
}

// dst row r (stride ldd) = the caller's row r (rows[r], or flat + r * lda)
// for r in [r0, r1), and dst[r][ncopy] = extra[r] when extra is not null;
// a block per row.
__global__ void k_rows_from_host(const double *const *rows, const double *flat, size_t lda, size_t ncopy,
                                 const double *extra, double *__restrict__ dst, size_t ldd, size_t r0)
{
    const size_t r = r0 + blockIdx.x;
    const double *src = rows ? rows[r] : flat + r * lda;
    double *d = dst + r * ldd;
    for (size_t c = threadIdx.x; c < ncopy; c += blockDim.x) d[c] = src[c];
    if (extra && threadIdx.x == 0) d[ncopy] = extra[r];
}

static int rows_from_host(size_t nrows, size_t ncopy, const double *const *rows, const double *flat, size_t lda,
                          const double *extra, double *dst, size_t ldd, cudaStream_t st)
{
    constexpr size_t kChunk = 65535;  // rows per launch (grid limit kept small)
    for (size_t r0 = 0; r0 < nrows; r0 += kChunk) {
        const size_t m = std::min(kChunk, nrows - r0);
        DSC_LAUNCH(k_rows_from_host<<<(unsigned)m, 256, 0, st>>>(rows, flat, lda, ncopy, extra, dst, ldd, r0));
    }
    DSC_CUDA(cudaGetLastError());
    DSC_CUDA(cudaStreamSynchronize(st));
    return kOk;
}

static uint64_t mix(uint64_t h, uint64_t v)
{
    h ^= v + 0x9e3779b97f4a7c15ULL + (h << 6) + (h >> 2);
    return h * 0xff51afd7ed558ccdULL;
}

static uint64_t hash_bytes(uint64_t h, const void *p, size_t n)
{
    const unsigned char *b = (const unsigned char *)p;
    size_t w = n / 8;
    for (size_t i = 0; i < w; i++) {
        uint64_t v;
        memcpy(&v, b + 8 * i, 8);
        h = mix(h, v);
    }
    for (size_t i = 8 * w; i < n; i++) h = mix(h, b[i]);
    return mix(h, n);
}

// Geometry (and its device copy) for these nodes and 0-based elements,
// rebuilt only when the content changes.
static int get_mesh(int nen, int N, int E, const double *nodes, const int *elems0,
                    MeshEntry **out)
{
    DSC_TRY(ensure_stream());
    Context &c = ctx();
    uint64_t key = mix(mix(mix(0x243f6a8885a308d3ULL, nen), N), E);
    key = hash_bytes(key, nodes, (size_t)N * 3 * sizeof(double));
    key = hash_bytes(key, elems0, (size_t)E * nen * sizeof(int));
    if (!c.mesh || c.mesh->key != key) {
        auto m = std::make_unique<MeshEntry>();
        DSC_TRY(build_plan(nen, N, E, nodes, elems0, nullptr, m->plan));
        DSC_TRY(m->dev.upload(m->plan, c.st));
        m->key = key;
        c.mesh = std::move(m);
        c.sigma_key = 0;
    }
    *out = c.mesh.get();
    return kOk;
}

static int get_q8_mesh(int N, int E, const double *nodes, const int *elems0, Q8Mesh **out)
{
    DSC_TRY(ensure_stream());
    Context &c = ctx();
    uint64_t key = mix(mix(mix(0x243f6a8885a308d3ULL, 8), N), E);
    key = hash_bytes(key, nodes, (size_t)N * 3 * sizeof(double));
    key = hash_bytes(key, elems0, (size_t)E * 8 * sizeof(int));
    if (!c.q8 || c.q8_key != key) {
        auto m = std::make_unique<Q8Mesh>();
        DSC_TRY(m->build(N, E, nodes, elems0, c.st));
        c.q8 = std::move(m);
        c.q8_key = key;
    }
    *out = c.q8.get();
    return kOk;
}

static int get_sigma(int N, const double *vB, const double **dsig)
{
    // the solution goes up again only when it differs from the copy on the
    // device (compared value by value with its host copy)
    Context &c = ctx();
    const size_t n2 = 2 * (size_t)N;
    if (c.sigma_key != c.mesh->key || c.sigma_host.size() != n2 ||
        memcmp(c.sigma_host.data(), vB, n2 * sizeof(double)) != 0) {
        c.sigma_host.assign(vB, vB + n2);
        DSC_TRY(c.sigma.upload(c.sigma_host.data(), n2, c.st));
        DSC_CUDA(cudaStreamSynchronize(c.st));
        c.sigma_key = c.mesh->key;
        c.sigma_gen++;
    }
    *dsig = c.sigma.p;
    return kOk;
}

// The cached mesh when it holds exactly these row-pointer inputs (checked
// value by value against its flattened copy, without allocating), else
// null: the reference's post-processing calls field_* once per point with
// the same mesh, which then needs neither a new flat copy nor a hash.
static MeshEntry *cached_rows(int nen, int N, int E, double **mNodes, unsigned **mElems)
{
    MeshEntry *m = ctx().mesh.get();
    if (!m || m->plan.nen != nen || m->plan.N != N || m->plan.E != E) return nullptr;
    // bit patterns, compared inline (a call per 24-byte row costs more than
    // the comparison)
    const double *x = m->plan.nodes.data();
    for (int i = 0; i < N; i++) {
        const double *r = mNodes[i];
        uint64_t a[3], b[3];
        memcpy(a, r, sizeof a);
        memcpy(b, x + 3 * (size_t)i, sizeof b);
        if ((a[0] ^ b[0]) | (a[1] ^ b[1]) | (a[2] ^ b[2])) return nullptr;
    }
    const int *el = m->plan.elems.data();
    for (int e = 0; e < E; e++) {
        const unsigned *r = mElems[e];
        const int *q = el + (size_t)e * nen;
        unsigned diff = 0;
        for (int k = 0; k < nen; k++) diff |= (r[k] - 1u) ^ (unsigned)q[k];
        if (diff) return nullptr;
    }
    return m;
}

// Flattened copies of the reference's row-pointer inputs.
struct FlatMesh {
    std::vector<double> nodes;
    std::vector<int> elems0;
};

static void flatten(int nen, int N, int E, double **mNodes, unsigned **mElems, FlatMesh &f)
{
    f.nodes.resize((size_t)N * 3);
    f.elems0.resize((size_t)E * nen);
    for (int i = 0; i < N; i++)
        for (int d = 0; d < 3; d++) f.nodes[3 * (size_t)i + d] = mNodes[i][d];
    for (int e = 0; e < E; e++)
        for (int k = 0; k < nen; k++) f.elems0[(size_t)e * nen + k] = (int)mElems[e][k] - 1;
}

static int elems_to0(int nen, int E, const unsigned *elems1, std::vector<int> &out)
{
    out.resize((size_t)E * nen);
    for (size_t t = 0; t < out.size(); t++) out[t] = (int)elems1[t] - 1;
    return kOk;
}

// ---------------------------------------------------------------- assembly
// Rows [r0, r1) of the compact (full = 0) or full (full = 1) system from K:
// top rows i:    [a_i K_i + d_i e_i | b_i K_i]
// bottom rows N+i (full only): [-b_i K_i | a_i K_i + d_i e_(N+i)]
// K is column-major; a 32 x 32 shared tile turns its columns into rows.
// out: the staging block (rows from r0); or, with hrows or hflat not null,
// the caller's host rows themselves (rows[r] or hflat + r * hlda), added
// to in place (a device that reads and writes pageable host memory).
__global__ void k_form_rows(const double *__restrict__ K, size_t ld, int N, int full, int r0,
                            int r1, const double *__restrict__ ca, const double *__restrict__ cb,
                            const double *__restrict__ cd, double *__restrict__ out,
                            double *const *hrows = nullptr, double *hflat = nullptr, size_t hlda = 0)
{
    __shared__ double t[32][33];
    const int c0 = blockIdx.x * 32, rr0 = r0 + blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
    for (int k = ty; k < 32; k += 8) {
        int c = c0 + k, r = rr0 + tx;
        int i = r < N ? r : r - N;
        t[k][tx] = (c < N && r < r1) ? K[(size_t)c * ld + i] : 0.0;
    }
    __syncthreads();
    const size_t ncol = 2 * (size_t)N;
    for (int k = ty; k < 32; k += 8) {
        int r = rr0 + k, c = c0 + tx;
        if (r >= r1 || c >= N) continue;
        const bool top = r < N;
        const int i = top ? r : r - N;
        const double kv = t[tx][k];
        const double a = ca[i], b = cb[i], d = cd[i];
        double left, right;
        if (top) {
            left = a * kv + (c == i ? d : 0.0);
            right = b * kv;
        } else {
            left = -b * kv;
            right = a * kv + (c == i ? d : 0.0);
        }
        if (hrows || hflat) {
            double *o = hrows ? hrows[r] : hflat + (size_t)r * hlda;
            o[c] += left;
            o[c + N] += right;
        } else {
            double *o = out + (size_t)(r - r0) * ncol;
            o[c] = left;
            o[c + N] = right;
        }
    }
}

typedef void (*RowSinkFn)(void *user, int row, const double *vals, size_t n);

// Assembles K in FP64 and streams the requested form out row-chunk by
// row-chunk: device transpose into a staging block, copy to pinned host
// memory, then sink(row, values) for every row.
static int assemble_impl(int nen, int full, unsigned N, unsigned E, unsigned nIf,
                         const double *nodes, const int *elems0, const unsigned *bctype,
                         const unsigned *ifaces, const double *mat, double freq, const double *mbc,
                         RowSinkFn sink, void *user, double *const *drows, double *dflat, size_t dlda)
{
    cudaStream_t st = ctx().st;
    const size_t ld = ((size_t)N + 31) / 32 * 32;
    DevBuf<double> K;
    std::vector<int> row_kind(N);
    if (nen == 8) {
        Q8Mesh *q;
        DSC_TRY(get_q8_mesh((int)N, (int)E, nodes, elems0, &q));
        DSC_TRY(K.alloc(ld * N));
        DSC_TRY(q8_assemble_K(*q, bctype, K.p, ld, st));
        for (unsigned i = 0; i < N; i++) row_kind[i] = bctype[i] == 1 ? 0 : 1;
    } else {
        MeshEntry *m;
        DSC_TRY(get_mesh(nen, (int)N, (int)E, nodes, elems0, &m));
        DSC_TRY(set_rows(m->plan, bctype));
        DSC_TRY(m->dev.upload_rows(m->plan, st));
        DSC_TRY(K.alloc(ld * N));
        DSC_TRY(assemble_K_fp64(m->dev, K.p, ld, st));
        row_kind = m->plan.row_kind;
    }
    // Per-row coefficients: conductor rows a = 1 (K holds C int G N);
    // interface rows a = A_k, b = B_k, d = -1/(2 eps0) with k the row's
    // interface id mBC[i][1] (src/assembly_el.c:245-256).
    std::vector<double> Ak(nIf ? nIf : 1), Bk(nIf ? nIf : 1);
    if (nIf) interface_coeffs(nIf, ifaces, mat, freq, Ak.data(), Bk.data());
    std::vector<double> ca(N), cb(N), cd(N);
    for (unsigned i = 0; i < N; i++) {
        if (row_kind[i] == 0) {
            ca[i] = 1.0;
            cb[i] = 0.0;
            cd[i] = 0.0;
        } else {
            unsigned k = (unsigned)mbc[3 * (size_t)i + 1] - 1;
            if (k >= nIf) {
                set_error("node %u: interface id %g outside 1..%u", i + 1, mbc[3 * (size_t)i + 1], nIf);
                return kErrArg;
            }
            ca[i] = Ak[k];
            cb[i] = Bk[k];
            cd[i] = -0.5 / kEps0;
        }
    }
    DevBuf<double> dca, dcb, dcd, stage;
    DSC_TRY(dca.upload(ca, st));
    DSC_TRY(dcb.upload(cb, st));
    DSC_TRY(dcd.upload(cd, st));

    const size_t ncol = 2 * (size_t)N;
    const int nrows = full ? 2 * (int)N : (int)N;
    if ((drows || dflat) && host_direct(true)) {
        // the caller's rows take the form in place, read and written by the device
        dim3 grid(((int)N + 31) / 32, (nrows + 31) / 32), blk(32, 8);
        DSC_LAUNCH(k_form_rows<<<grid, blk, 0, st>>>(K.p, ld, (int)N, full, 0, nrows, dca.p, dcb.p, dcd.p, nullptr,
                                                     drows, dflat, dlda));
        DSC_CUDA(cudaGetLastError());
        DSC_CUDA(cudaStreamSynchronize(st));
        return kOk;
    }
    // chunks of rows formed on the device into one of two staging blocks,
    // copied into one of two pinned halves; the host threads add chunk q - 1
    // into the caller's rows while chunk q is formed and copied
    int rows_per = (int)std::max<size_t>(32, kMoverChunkBytes / (ncol * sizeof(double)) / 32 * 32);
    rows_per = std::min(rows_per, (nrows + 31) / 32 * 32);
    const size_t cb_ = (size_t)rows_per * ncol;
    DSC_TRY(stage.alloc(2 * cb_));
    DSC_TRY(ensure_pinned(2 * cb_ * sizeof(double)));
    double *half[2] = {ctx().pinned, ctx().pinned + cb_};
    cudaEvent_t ev[2];
    DSC_CUDA(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
    DSC_CUDA(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
    int rc = kOk;
    const int nq = (nrows + rows_per - 1) / rows_per;
    for (int q = 0; q <= nq && rc == kOk; q++) {
        if (q < nq) {
            const int r0 = q * rows_per, r1 = std::min(nrows, r0 + rows_per);
            double *sq = stage.p + (size_t)(q & 1) * cb_;
            dim3 grid(((int)N + 31) / 32, (r1 - r0 + 31) / 32), blk(32, 8);
            note_launch();
            k_form_rows<<<grid, blk, 0, st>>>(K.p, ld, (int)N, full, r0, r1, dca.p, dcb.p, dcd.p, sq);
            if (cudaGetLastError() != cudaSuccess ||
                cudaMemcpyAsync(half[q & 1], sq, (size_t)(r1 - r0) * ncol * sizeof(double), cudaMemcpyDeviceToHost,
                                st) != cudaSuccess ||
                cudaEventRecord(ev[q & 1], st) != cudaSuccess)
                rc = kErrCuda;
        }
        if (q >= 1 && rc == kOk) {
            const int p = q - 1, r0 = p * rows_per, r1 = std::min(nrows, r0 + rows_per);
            if (cudaEventSynchronize(ev[p & 1]) != cudaSuccess) {
                rc = kErrCuda;
                break;
            }
            const double *hp = half[p & 1];
            host_parallel_rows((size_t)r0, (size_t)r1,
                               [&](size_t r) { sink(user, (int)r, hp + (r - r0) * ncol, ncol); });
        }
    }
    if (rc != kOk) set_error("assembly rows to the host: %s", cudaGetErrorString(cudaGetLastError()));
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    return rc;
}

struct RowPtrSink {
    double **rows;
};

static void add_to_rowptr(void *u, int r, const double *v, size_t n)
{
    double *row = ((RowPtrSink *)u)->rows[r];
    for (size_t c = 0; c < n; c++) row[c] += v[c];
}

struct FlatSink {
    double *A;
    size_t lda;
};

static void add_to_flat(void *u, int r, const double *v, size_t n)
{
    FlatSink *f = (FlatSink *)u;
    double *row = f->A + (size_t)r * f->lda;
    for (size_t c = 0; c < n; c++) row[c] += v[c];
}

// ---------------------------------------------------------------- solvers
static int gauss_impl(unsigned n, const double *const *rows, const double *flat, size_t lda,
                      double *B, int *bad_row)
{
    DSC_TRY(ensure_stream());
    cudaStream_t st = ctx().st;
    const size_t ldd = ((size_t)n + 1 + 31) / 32 * 32;
    DevBuf<double> A;
    DSC_TRY(A.alloc(ldd * n));
    // the rows, with B as column n
    if (host_direct(false)) {
        DSC_TRY(rows_from_host(n, n, rows, flat, lda, B, A.p, ldd, st));
    } else {
        DSC_TRY(rows_to_device((size_t)n, ldd, A.p,
                               [&](size_t r, double *dst) {
                                   memcpy(dst, rows ? rows[r] : flat + r * lda, n * sizeof(double));
                                   dst[n] = B[r];
                               },
                               st));
    }
    DevBuf<double> x;
    DSC_TRY(x.alloc(n));
    Context &c = ctx();
    c.gauss_info = LuMixedInfo();
    c.gauss_fell_back = 0;
    bool done = false;
    if (c.gauss_mode == DSC_GAUSS_MIXED) {
        const int rc = lu_solve_mixed((int)n, A.p, ldd, x.p, 1e-15, &c.gauss_info, bad_row, st);
        if (rc == kOk) done = true;
        else if (rc == kErrStagnation) c.gauss_fell_back = 1;  // the matrix needs the FP64 factors
        else return rc;
    }
    if (!done) {
        DSC_TRY(lu_solve_augmented_fp64((int)n, A.p, ldd, bad_row, st));
        DSC_TRY(lu_extract_solution((int)n, A.p, ldd, x.p, st));
    }
    DSC_CUDA(cudaMemcpyAsync(B, x.p, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    DSC_CUDA(cudaStreamSynchronize(st));
    return kOk;
}

static int gmres_impl(unsigned N, unsigned preCond, double tol, unsigned maxit,
                      const double *const *rows, const double *flat, size_t lda, double *B,
                      const double *x0, FILE *log, unsigned *iters)
{
    DSC_TRY(ensure_stream());
    cudaStream_t st = ctx().st;
    const size_t ncol = 2 * (size_t)N;
    const size_t ldd = (ncol + 31) / 32 * 32;
    DevBuf<double> A, dB, dx0;
    DSC_TRY(A.alloc(ldd * N));
    if (host_direct(false)) {
        DSC_TRY(rows_from_host(N, ncol, rows, flat, lda, nullptr, A.p, ldd, st));
    } else {
        DSC_TRY(rows_to_device((size_t)N, ldd, A.p,
                               [&](size_t r, double *dst) {
                                   memcpy(dst, rows ? rows[r] : flat + r * lda, ncol * sizeof(double));
                               },
                               st));
    }
    DSC_TRY(dB.upload(B, ncol, st));
    if (x0) DSC_TRY(dx0.upload(x0, ncol, st));
    int rc = gmres_compact_fp64((int)N, A.p, ldd, dB.p, x0 ? dx0.p : nullptr, preCond, tol, maxit,
                                log, iters, st);
    if (rc == kOk) {
        DSC_CUDA(cudaMemcpyAsync(B, dB.p, ncol * sizeof(double), cudaMemcpyDeviceToHost, st));
        DSC_CUDA(cudaStreamSynchronize(st));
    }
    return rc;
}

// Points on a mesh already on the device; the point set and the output
// buffer are the context's, reused (grown only) from call to call.
static int points_on(MeshEntry *m, const double *vB, unsigned npts, const double *pts, int field, double *out)
{
    Context &c = ctx();
    const double *dsig;
    DSC_TRY(get_sigma(m->plan.N, vB, &dsig));
    cudaStream_t st = c.st;
    if (npts <= (unsigned)kFewPoints) {
        if (c.cq_gen != c.sigma_gen || c.cq_key != m->key) {
            DSC_TRY(point_charges(m->dev, dsig, c.cq, st));
            c.cq_gen = c.sigma_gen;
            c.cq_key = m->key;
        }
        return eval_few_points(m->dev, m->plan, c.cq.p, dsig, (int)npts, pts, field, out, c.few, st);
    }
    DSC_TRY(c.pts.build(m->plan, (int)npts, pts));
    const int nv = field ? 6 : 2;
    DSC_TRY(c.pout.alloc((size_t)npts * nv));
    DSC_TRY(eval_points(m->dev, c.pts, dsig, field, c.pout.p, st));
    DSC_CUDA(cudaMemcpyAsync(out, c.pout.p, (size_t)npts * nv * sizeof(double), cudaMemcpyDeviceToHost, st));
    DSC_CUDA(cudaStreamSynchronize(st));
    return kOk;
}

static int points_impl(int nen, unsigned N, unsigned E, const double *nodes, const int *elems0,
                       const double *vB, unsigned npts, const double *pts, int field, double *out)
{
    MeshEntry *m;
    DSC_TRY(get_mesh(nen, (int)N, (int)E, nodes, elems0, &m));
    return points_on(m, vB, npts, pts, field, out);
}

static int force_impl(int nen, unsigned N, unsigned E, const double *nodes, const int *elems0,
                      const unsigned *bctype, const double *vB, double eps, double *Fce,
                      double *Xce, double *Fcm, double *Xcm)
{
    MeshEntry *m;
    DSC_TRY(get_mesh(nen, (int)N, (int)E, nodes, elems0, &m));
    const double *dsig;
    DSC_TRY(get_sigma((int)N, vB, &dsig));
    return force_mst(m->dev, m->plan, bctype, dsig, eps, Fce, Xce, Fcm, Xcm, ctx().st);
}

// ---------------------------------------------------------------- fatal
// The reference's errorHandler (src/errorHandler.c:42-52): message on
// stderr and in bem.log, then exit(1).
static void fatal(const char *msg)
{
    fprintf(stderr, "\nERROR: %s\n", msg);
    fprintf(stderr, "*** PROGRAM TERMINATED ***\n\n");
    if (file_log) {
        fprintf(file_log, "\nERROR: %s\n", msg);
        fprintf(file_log, "*** PROGRAM TERMINATED ***\n\n");
        fclose(file_log);
    }
    exit(1);
}

static void check_or_die(int rc)
{
    if (rc != kOk) fatal(last_error());
}

// Material table size implied by the interfaces (ids are 1-based).
static unsigned n_materials(unsigned nIf, unsigned **vInterfaces)
{
    unsigned m = 0;
    for (unsigned i = 0; i < nIf; i++) m = std::max(m, std::max(vInterfaces[i][0], vInterfaces[i][1]));
    return m;
}

static int electric_form(int nen, int full, double **mNodes, unsigned **mElems, unsigned *vBCType,
                         unsigned **vInterfaces, double **vMatParam, double *vProbParam, double **mA,
                         double **mBC, double *vB)
{
    std::lock_guard<std::mutex> lk(ctx().mu);
    const unsigned N = nNodes, E = nElems, nIf = nInterfaces;
    FlatMesh f;
    flatten(nen, (int)N, (int)E, mNodes, mElems, f);
    std::vector<unsigned> ifc((size_t)nIf * 2);
    for (unsigned i = 0; i < nIf; i++) {
        ifc[2 * i] = vInterfaces[i][0];
        ifc[2 * i + 1] = vInterfaces[i][1];
    }
    unsigned nm = n_materials(nIf, vInterfaces);
    std::vector<double> mat((size_t)std::max(nm, 1u) * 2, 0.0);
    for (unsigned i = 0; i < nm; i++) {
        mat[2 * i] = vMatParam[i][0];
        mat[2 * i + 1] = vMatParam[i][1];
    }
    std::vector<double> mbc((size_t)2 * N * 3);
    for (size_t j = 0; j < 2 * (size_t)N; j++)
        for (int d = 0; d < 3; d++) mbc[3 * j + d] = mBC[j][d];
    RowPtrSink sink{mA};
    check_or_die(assemble_impl(nen, full, N, E, nIf, f.nodes.data(), f.elems0.data(), vBCType,
                               ifc.data(), mat.data(), vProbParam[0], mbc.data(), add_to_rowptr,
                               &sink, mA, nullptr, 0));
    // right-hand side (src/assembly_el.c:296-298)
    for (unsigned i = 0; i < N; i++) {
        vB[i] = mBC[i][0];
        vB[i + N] = mBC[i + N][0];
    }
    return 0;
}

}  // namespace dsc

using namespace dsc;

// ================================================================ drop-in

extern "C" int electricFormA_tria3(double **mNodes, unsigned int **mElems, unsigned int *vBCType,
                                   unsigned int **vInterfaces, double **vMatParam,
                                   double *vProbParam, double **mA, double **mBC, double *vB)
{
    return electric_form(3, 0, mNodes, mElems, vBCType, vInterfaces, vMatParam, vProbParam, mA, mBC, vB);
}

extern "C" int electricFormA_tria6(double **mNodes, unsigned int **mElems, unsigned int *vBCType,
                                   unsigned int **vInterfaces, double **vMatParam,
                                   double *vProbParam, double **mA, double **mBC, double *vB)
{
    return electric_form(6, 0, mNodes, mElems, vBCType, vInterfaces, vMatParam, vProbParam, mA, mBC, vB);
}

extern "C" int electricFormFullA_tria3(double **mNodes, unsigned int **mElems,
                                       unsigned int *vBCType, unsigned int **vInterfaces,
                                       double **vMatParam, double *vProbParam, double **mA,
                                       double **mBC, double *vB)
{
    return electric_form(3, 1, mNodes, mElems, vBCType, vInterfaces, vMatParam, vProbParam, mA, mBC, vB);
}

extern "C" int electricFormFullA_tria6(double **mNodes, unsigned int **mElems,
                                       unsigned int *vBCType, unsigned int **vInterfaces,
                                       double **vMatParam, double *vProbParam, double **mA,
                                       double **mBC, double *vB)
{
    return electric_form(6, 1, mNodes, mElems, vBCType, vInterfaces, vMatParam, vProbParam, mA, mBC, vB);
}

extern "C" int gaussBksb(unsigned int N, double **A, double *B)
{
    std::lock_guard<std::mutex> lk(ctx().mu);
    int bad = -1;
    int rc = gauss_impl(N, A, nullptr, 0, B, &bad);
    if (rc == kErrSingular) {
        // the reference's message and exit (src/gaussBksb.c:68-69)
        printf("\nSingularity in row %d in system matrix", bad);
        exit(1);
    }
    check_or_die(rc);
    return 0;
}

extern "C" void solverGMRES_el(unsigned int preCond, unsigned int nInit, double **A, double *B)
{
    std::lock_guard<std::mutex> lk(ctx().mu);
    const unsigned N = nNodes;
    std::vector<double> x0;
    if (nInit != 0) {
        // initial guess (src/gmres_el.c:80-84)
        x0.assign(2 * (size_t)N, 0.0);
        FILE *fin = fopen("solution.init", "r");
        if (!fin) fatal("Can't open solution.init");
        for (unsigned i = 0; i < nInit && i < 2 * N; i++)
            if (fscanf(fin, "%le", &x0[i]) != 1) break;
        fclose(fin);
    }
    FILE *fg = fopen("gmres.log", "w");
    unsigned iters = 0;
    int rc = gmres_impl(N, preCond, 1.0E-6, 600, A, nullptr, 0, B, x0.empty() ? nullptr : x0.data(),
                        fg, &iters);
    if (rc == kErrNoConverge) {
        if (fg) fclose(fg);
        fatal("Linear system may be ill-conditioned");
    }
    if (rc == kErrStagnation) {
        if (fg) fclose(fg);
        fatal("CONVERGENCE RATE TOO SLOW");
    }
    check_or_die(rc);
    if (fg) fclose(fg);
}

static int field_dropin(int nen, int field, double *Xin, double **mNodes, unsigned **mElems,
                        double *vB, double *out)
{
    std::lock_guard<std::mutex> lk(ctx().mu);
    check_or_die(ensure_stream());
    if (MeshEntry *m = cached_rows(nen, (int)nNodes, (int)nElems, mNodes, mElems)) {
        check_or_die(points_on(m, vB, 1, Xin, field, out));
        return 0;
    }
    FlatMesh f;
    flatten(nen, (int)nNodes, (int)nElems, mNodes, mElems, f);
    check_or_die(points_impl(nen, nNodes, nElems, f.nodes.data(), f.elems0.data(), vB, 1, Xin, field, out));
    return 0;
}

extern "C" int field_tria3(double *Xin, double **mNodes, unsigned int **mElems, double *vB, double *mE)
{
    return field_dropin(3, 1, Xin, mNodes, mElems, vB, mE);
}

extern "C" int field_tria6(double *Xin, double **mNodes, unsigned int **mElems, double *vB, double *mE)
{
    return field_dropin(6, 1, Xin, mNodes, mElems, vB, mE);
}

extern "C" int potential_tria3(double *Xin, double **mNodes, unsigned int **mElems, double *vB,
                               double *mPot)
{
    return field_dropin(3, 0, Xin, mNodes, mElems, vB, mPot);
}

extern "C" int potential_tria6(double *Xin, double **mNodes, unsigned int **mElems, double *vB,
                               double *mPot)
{
    return field_dropin(6, 0, Xin, mNodes, mElems, vB, mPot);
}

// ---------------------------------------------------------- multipole forces
// The multipole and ellipsoid DEP forces (src/force.c:65-322,572-825) from
// the field and its derivatives at the evaluation point.  E_a is the
// derivative tensor of point_derivatives (E_(1,0,0) = Re Ex, E_(2,0,0) =
// dEx/dx, ...).  Sphere of radius R, order n <= 3 of the expansion:
//   F_i = sum_n C_n sum_{|a| = n} (n! / a!) E_a E_{a + e_i},
//   C_1 = 2 pi eps_m R^3 CM_1,  C_n = C_{n-1} R^2 / ((n - 1)(2n - 1)) with
//   CM_n = Re[(e_p - e_m) / (n e_p + (n + 1) e_m)] in place of CM_{n-1},
// e = eps + sigma / (i omega) (the reference's EpsDif / EpsPlus / SigDif /
// SigPlus form).  The reference computes the order 4 and 5 coefficients but
// adds only the terms up to n = 3 (src/force.c:814-826): orders 4 and 5 give
// the order-3 force here too.  The tria6 form multiplies by 0.333...33 and
// 0.1 where the tria3 form divides by 3 and 10 (src/force.c:636-642,773-779);
// both are kept.
static double deriv_E(const double *E, int p, int q, int r) { return E[deriv_index(p, q, r)]; }

static double cm_factor(const double *mat, double freq, int n)
{
    const double w = freq * kPi2 * kEps0;
    const double ed = w * (mat[3] - mat[1]), sd = mat[2] - mat[0];
    const double ep = w * (n * mat[3] + (n + 1) * mat[1]), sp = n * mat[2] + (n + 1) * mat[0];
    return (ed * ep + sd * sp) / (ep * ep + sp * sp);
}

static void multipole_from_derivs(int nen, const double *E, unsigned nOrder, double R, const double *mat,
                                  double freq, double *F)
{
    const double Eps = mat[1] * kEps0;
    double C[4];
    C[1] = kPi2 * Eps * R * R * R;
    C[2] = nen == 6 ? C[1] * R * R * 0.333333333333333333 : C[1] * R * R / 3.0;
    C[3] = nen == 6 ? C[2] * R * R * 0.1 : C[2] * R * R / 10.0;
    const int top = (int)std::min(3u, std::max(1u, nOrder));
    for (int n = 1; n <= top; n++) C[n] *= cm_factor(mat, freq, n);
    F[0] = F[1] = F[2] = 0.0;
    for (int n = 1; n <= top; n++) {
        double f[3] = {0.0, 0.0, 0.0};
        for (int p = n; p >= 0; p--)
            for (int q = n - p; q >= 0; q--) {
                const int r = n - p - q;
                double fact = 1.0;
                for (int k = 2; k <= n; k++) fact *= k;
                for (int k = 2; k <= p; k++) fact /= k;
                for (int k = 2; k <= q; k++) fact /= k;
                for (int k = 2; k <= r; k++) fact /= k;
                const double ea = deriv_E(E, p, q, r);
                f[0] += fact * ea * deriv_E(E, p + 1, q, r);
                f[1] += fact * ea * deriv_E(E, p, q + 1, r);
                f[2] += fact * ea * deriv_E(E, p, q, r + 1);
            }
        for (int i = 0; i < 3; i++) F[i] += C[n] * f[i];
    }
}

// 64-point Gauss-Legendre rule on [-1, 1], ascending (Newton on P_64 from
// the usual cosine guesses), for the depolarisation integrals.
static const double (*gauss_legendre64())[2]
{
    static double rule[64][2];
    static std::once_flag once;
    std::call_once(once, [] {
        const int n = 64;
        for (int i = 0; i < n; i++) {
            double x = cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 1.0;
            for (int it = 0; it < 100; it++) {
                double p0 = 1.0, p1 = x;
                for (int k = 2; k <= n; k++) {
                    const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
                    p0 = p1;
                    p1 = p2;
                }
                dp = n * (x * p1 - p0) / (x * x - 1.0);
                const double dx = p1 / dp;
                x -= dx;
                if (fabs(dx) < 1e-17) break;
            }
            rule[n - 1 - i][0] = x;  // ascending
            rule[n - 1 - i][1] = 2.0 / ((1.0 - x * x) * dp * dp);
        }
    });
    return rule;
}

// Depolarisation factors of an ellipsoid of semi-axes `axis`
// (src/depolarization.c:44-115): L_k = (abc / 2) int_0^inf ds /
// ((s + a_k^2) sqrt((s + a^2)(s + b^2)(s + c^2))), the range cut at
// 100 a_k^2 and integrated with the 64-point rule.  Returns false when a
// factor comes out negative (the reference's fatal error); *warn is set when
// they do not add up to 1 within 0.05 (the reference's warning).
static bool depolarization_factors(const double *axis, double *Ld, bool *warn)
{
    const double(*g)[2] = gauss_legendre64();
    const double A = 0.5 * axis[0] * axis[1] * axis[2];
    const double a2 = axis[0] * axis[0], b2 = axis[1] * axis[1], c2 = axis[2] * axis[2];
    const double s2[3] = {a2, b2, c2};
    for (int k = 0; k < 3; k++) {
        const double X1 = 100 * s2[k], J = 0.5 * X1;
        double acc = 0.0;
        for (int i = 0; i < 64; i++) {
            const double x = 0.5 * (1.0 + g[i][0]) * X1;  // the line from 0 to X1 at the rule's point
            const double R = J * g[i][1] / sqrt((x + a2) * (x + b2) * (x + c2));
            acc += R / (x + s2[k]);
        }
        Ld[k] = A * acc;
    }
    *warn = fabs(1.0 - Ld[0] - Ld[1] - Ld[2]) > 0.05;
    return Ld[0] >= 0.0 && Ld[1] >= 0.0 && Ld[2] >= 0.0;
}

// The ellipsoid's dipole force (analysis 10: homogeneous; 11: single-shell
// oblate, the particle's sigma and eps scaled by a c / (2 c + a) and divided
// by each L_k), src/force.c:260-318.
static void ellipsoid_from_derivs(const double *E, unsigned analysis, const double *axis, const double *Ld,
                                  const double *mat, double freq, double *F)
{
    const double w = freq * kPi2 * kEps0, Eps = mat[1] * kEps0;
    const double A = kPi2 * Eps * axis[0] * axis[1] * axis[2] / 3.0;
    double K[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < 3; d++) {
        double ep = mat[3], sp = mat[2];
        if (analysis == 11) {
            const double Cs = axis[0] * axis[2] / (2.0 * axis[2] + axis[0]);
            ep = mat[3] * Cs / Ld[d];
            sp = mat[2] * Cs / Ld[d];
        } else if (analysis != 10) {
            break;
        }
        const double ed = w * (ep - mat[1]), sd = sp - mat[0];
        const double epl = w * (mat[1] + (ep - mat[1]) * Ld[d]), spl = mat[0] + (sp - mat[0]) * Ld[d];
        K[d] = (ed * epl + sd * spl) / (epl * epl + spl * spl);
    }
    const double Ex = deriv_E(E, 1, 0, 0), Ey = deriv_E(E, 0, 1, 0), Ez = deriv_E(E, 0, 0, 1);
    F[0] = A * (K[0] * Ex * deriv_E(E, 2, 0, 0) + K[1] * Ey * deriv_E(E, 1, 1, 0) + K[2] * Ez * deriv_E(E, 1, 0, 1));
    F[1] = A * (K[0] * Ex * deriv_E(E, 1, 1, 0) + K[1] * Ey * deriv_E(E, 0, 2, 0) + K[2] * Ez * deriv_E(E, 0, 1, 1));
    F[2] = A * (K[0] * Ex * deriv_E(E, 1, 0, 1) + K[1] * Ey * deriv_E(E, 0, 1, 1) + K[2] * Ez * deriv_E(E, 0, 0, 2));
}

// E tensors at npts points on mesh m from the nodal solution vB.
static int derivs_on(MeshEntry *m, const double *vB, unsigned npts, const double *pts, std::vector<double> &E)
{
    Context &c = ctx();
    const double *dsig;
    DSC_TRY(get_sigma(m->plan.N, vB, &dsig));
    DSC_TRY(c.dpts.upload(pts, 3 * (size_t)npts, c.st));
    E.assign((size_t)npts * kDerivCount, 0.0);
    return point_derivatives(m->dev, dsig, (int)npts, c.dpts.p, c.deriv, E.data(), c.st);
}

static MeshEntry *mesh_of_rows(int nen, double **mNodes, unsigned **mElems)
{
    check_or_die(ensure_stream());
    MeshEntry *m = cached_rows(nen, (int)nNodes, (int)nElems, mNodes, mElems);
    if (m) return m;
    FlatMesh f;
    flatten(nen, (int)nNodes, (int)nElems, mNodes, mElems, f);
    check_or_die(get_mesh(nen, (int)nNodes, (int)nElems, f.nodes.data(), f.elems0.data(), &m));
    return m;
}

static int multipole_dropin(int nen, unsigned nOrder, double R, double *Xeval, double **mNodes, unsigned **mElems,
                            double *vB, double **vMatParam, double *vProbParam, double *F)
{
    std::lock_guard<std::mutex> lk(ctx().mu);
    MeshEntry *m = mesh_of_rows(nen, mNodes, mElems);
    std::vector<double> E;
    check_or_die(derivs_on(m, vB, 1, Xeval, E));
    const double mat[4] = {vMatParam[0][0], vMatParam[0][1], vMatParam[1][0], vMatParam[1][1]};
    multipole_from_derivs(nen, E.data(), nOrder, R, mat, vProbParam[0], F);
    return 0;
}

static int ellipsoid_dropin(int nen, unsigned ANALYSIS, double *axis, double *Xeval, double **mNodes,
                            unsigned **mElems, double *vB, double **vMatParam, double *vProbParam, double *F)
{
    std::lock_guard<std::mutex> lk(ctx().mu);
    MeshEntry *m = mesh_of_rows(nen, mNodes, mElems);
    std::vector<double> E;
    check_or_die(derivs_on(m, vB, 1, Xeval, E));
    double Ld[3];
    bool warn = false;
    if (!depolarization_factors(axis, Ld, &warn)) fatal("Error: depolarization() - factors must be positive!");
    if (warn) printf("Warning: depolarization() - error is larger than 0.05");
    const double mat[4] = {vMatParam[0][0], vMatParam[0][1], vMatParam[1][0], vMatParam[1][1]};
    ellipsoid_from_derivs(E.data(), ANALYSIS, axis, Ld, mat, vProbParam[0], F);
    if (ANALYSIS == 11) {
        // the reference scales the particle's row of vMatParam in place
        // (src/force.c:286-292), and its later calls see the scaled values
        const double Cs = axis[0] * axis[2] / (2.0 * axis[2] + axis[0]);
        vMatParam[1][1] *= Cs;
        vMatParam[1][0] *= Cs;
    }
    return 0;
}

extern "C" int forceMultipole_tria3(unsigned int nOrder, double R, double *Xeval, double **mNodes,
                                    unsigned int **mElems, double *vB, double **vMatParam, double *vProbParam,
                                    double *F)
{
    return multipole_dropin(3, nOrder, R, Xeval, mNodes, mElems, vB, vMatParam, vProbParam, F);
}

extern "C" int forceMultipole_tria6(unsigned int nOrder, double R, double *Xeval, double **mNodes,
                                    unsigned int **mElems, double *vB, double **vMatParam, double *vProbParam,
                                    double *F)
{
    return multipole_dropin(6, nOrder, R, Xeval, mNodes, mElems, vB, vMatParam, vProbParam, F);
}

extern "C" int forceEllipsoid_tria3(unsigned int ANALYSIS, unsigned int nOrder, double *axis, double *Xeval,
                                    double **mNodes, unsigned int **mElems, double *vB, double **vMatParam,
                                    double *vProbParam, double *F)
{
    (void)nOrder;
    return ellipsoid_dropin(3, ANALYSIS, axis, Xeval, mNodes, mElems, vB, vMatParam, vProbParam, F);
}

extern "C" int forceEllipsoid_tria6(unsigned int ANALYSIS, unsigned int nOrder, double *axis, double *Xeval,
                                    double **mNodes, unsigned int **mElems, double *vB, double **vMatParam,
                                    double *vProbParam, double *F)
{
    (void)nOrder;
    return ellipsoid_dropin(6, ANALYSIS, axis, Xeval, mNodes, mElems, vB, vMatParam, vProbParam, F);
}

static int force_dropin(int nen, double **mNodes, unsigned **mElems, unsigned *vBCType, double *vB,
                        double Eps, double **Fce, double **Xce, double *Fcm, double *Xcm)
{
    std::lock_guard<std::mutex> lk(ctx().mu);
    const unsigned N = nNodes, E = nElems;
    FlatMesh f;
    flatten(nen, (int)N, (int)E, mNodes, mElems, f);
    std::vector<double> fce((size_t)E * 3, NAN), xce((size_t)E * 3, NAN);
    check_or_die(force_impl(nen, N, E, f.nodes.data(), f.elems0.data(), vBCType, vB, Eps, fce.data(),
                            xce.data(), Fcm, Xcm));
    for (unsigned e = 0; e < E; e++) {
        if (vBCType[mElems[e][0] - 1] != 6) continue;
        for (int d = 0; d < 3; d++) {
            Fce[e][d] = fce[3 * (size_t)e + d];
            Xce[e][d] = xce[3 * (size_t)e + d];
        }
    }
    return 0;
}

extern "C" int forceMST_tria3(double **mNodes, unsigned int **mElems, unsigned int *vBCType,
                              double *vB, double Eps, double **Fce, double **Xce, double *Fcm,
                              double *Xcm)
{
    return force_dropin(3, mNodes, mElems, vBCType, vB, Eps, Fce, Xce, Fcm, Xcm);
}

extern "C" int forceMST_tria6(double **mNodes, unsigned int **mElems, unsigned int *vBCType,
                              double *vB, double Eps, double **Fce, double **Xce, double *Fcm,
                              double *Xcm)
{
    return force_dropin(6, mNodes, mElems, vBCType, vB, Eps, Fce, Xce, Fcm, Xcm);
}

// ================================================================ dsc_ API

extern "C" const char *dsc_last_error(void) { return last_error(); }

extern "C" int dsc_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

// Element families of the flat calls: tria3, tria6 and the quad8 extension.
static bool family_ok(int nen) { return nen == 3 || nen == 6 || nen == 8; }

extern "C" int dsc_assemble(int nen, int full, unsigned N, unsigned E, unsigned nIf,
                            const double *nodes, const unsigned *elems, const unsigned *bctype,
                            const unsigned *ifaces, const double *mat, double freq,
                            const double *mbc, double *A, size_t lda, double *B)
{
    std::lock_guard<std::mutex> lk(ctx().mu);
    if (!family_ok(nen) || !nodes || !elems || !bctype || !mbc || !A || !B || lda < 2 * (size_t)N) {
        set_error("dsc_assemble: bad arguments");
        return kErrArg;
    }
    std::vector<int> e0;
    elems_to0(nen, (int)E, elems, e0);
    FlatSink sink{A, lda};
    DSC_TRY(assemble_impl(nen, full, N, E, nIf, nodes, e0.data(), bctype, ifaces, mat, freq, mbc,
                          add_to_flat, &sink, nullptr, A, lda));
    for (unsigned i = 0; i < N; i++) {
        B[i] = mbc[3 * (size_t)i];
        B[i + N] = mbc[3 * (size_t)(i + N)];
    }
    return kOk;
}

extern "C" int dsc_gauss(unsigned n, const double *A, size_t lda, double *B)
{
    std::lock_guard<std::mutex> lk(ctx().mu);
    if (!A || !B || lda < n || n == 0) {
        set_error("dsc_gauss: bad arguments");
        return kErrArg;
    }
    int bad = -1;
    return gauss_impl(n, nullptr, A, lda, B, &bad);
}

extern "C" int dsc_set_host_direct(int mode)
{
    if (mode < 0 || mode > 2) {
        set_error("dsc_set_host_direct: mode %d (0, 1 or 2)", mode);
        return kErrArg;
    }
    std::lock_guard<std::mutex> lk(ctx().mu);
    g_host_direct = mode;
    return kOk;
}

extern "C" int dsc_set_gauss_mode(int mode)
{
    if (mode != DSC_GAUSS_MIXED && mode != DSC_GAUSS_FP64) {
        set_error("dsc_set_gauss_mode: unknown mode %d", mode);
        return kErrArg;
    }
    std::lock_guard<std::mutex> lk(ctx().mu);
    ctx().gauss_mode = mode;
    return kOk;
}

extern "C" int dsc_gauss_info(int *refinements, double *rel_residual, int *fell_back, double *ms)
{
    std::lock_guard<std::mutex> lk(ctx().mu);
    const Context &c = ctx();
    if (refinements) *refinements = c.gauss_info.refinements;
    if (rel_residual) *rel_residual = c.gauss_info.rel_residual;
    if (fell_back) *fell_back = c.gauss_fell_back;
    if (ms) {
        ms[0] = c.gauss_info.factor_ms;
        ms[1] = c.gauss_info.refine_ms;
    }
    return c.gauss_mode;
}

extern "C" int dsc_gmres(unsigned N, unsigned preCond, double tol, unsigned max_iters,
                         const double *A, size_t lda, double *B, const double *x0,
                         const char *log_path, unsigned *iters)
{
    std::lock_guard<std::mutex> lk(ctx().mu);
    if (!A || !B || lda < 2 * (size_t)N || N == 0 || max_iters == 0) {
        set_error("dsc_gmres: bad arguments");
        return kErrArg;
    }
    FILE *log = log_path ? fopen(log_path, "w") : nullptr;
    int rc = gmres_impl(N, preCond, tol, max_iters, nullptr, A, lda, B, x0, log, iters);
    if (log) fclose(log);
    return rc;
}

// Field or potential of a quad8 mesh at host points (out: npts x 6 or 2).
static int q8_points_host(unsigned N, unsigned E, const double *nodes, const int *elems0, const double *vB,
                          unsigned npts, const double *pts, int field, double *out)
{
    Context &c = ctx();
    Q8Mesh *q;
    DSC_TRY(get_q8_mesh((int)N, (int)E, nodes, elems0, &q));
    if (npts == 0) return kOk;
    const int NV = field ? 6 : 2;
    DSC_TRY(c.q8_sigma.upload(vB, 2 * (size_t)N, c.st));
    DSC_TRY(c.q8_out.alloc((size_t)npts * NV));
    DSC_TRY(q8_points(*q, c.q8_sigma.p, (int)npts, pts, field, c.q8_out.p, c.st));
    DSC_CUDA(cudaMemcpyAsync(out, c.q8_out.p, (size_t)npts * NV * sizeof(double), cudaMemcpyDeviceToHost, c.st));
    DSC_CUDA(cudaStreamSynchronize(c.st));
    return kOk;
}

extern "C" int dsc_field_points(int nen, unsigned N, unsigned E, const double *nodes,
                                const unsigned *elems, const double *vB, unsigned npts,
                                const double *pts, double *mE)
{
    std::lock_guard<std::mutex> lk(ctx().mu);
    if (!family_ok(nen) || !nodes || !elems || !vB || (npts && (!pts || !mE))) {
        set_error("dsc_field_points: bad arguments");
        return kErrArg;
    }
    std::vector<int> e0;
    elems_to0(nen, (int)E, elems, e0);
    if (nen == 8) return q8_points_host(N, E, nodes, e0.data(), vB, npts, pts, 1, mE);
    return points_impl(nen, N, E, nodes, e0.data(), vB, npts, pts, 1, mE);
}

extern "C" int dsc_potential_points(int nen, unsigned N, unsigned E, const double *nodes,
                                    const unsigned *elems, const double *vB, unsigned npts,
                                    const double *pts, double *mPot)
{
    std::lock_guard<std::mutex> lk(ctx().mu);
    if (!family_ok(nen) || !nodes || !elems || !vB || (npts && (!pts || !mPot))) {
        set_error("dsc_potential_points: bad arguments");
        return kErrArg;
    }
    std::vector<int> e0;
    elems_to0(nen, (int)E, elems, e0);
    if (nen == 8) return q8_points_host(N, E, nodes, e0.data(), vB, npts, pts, 0, mPot);
    return points_impl(nen, N, E, nodes, e0.data(), vB, npts, pts, 0, mPot);
}

extern "C" int dsc_force_multipole(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
                                   const double *vB, unsigned npts, const double *pts, unsigned order, double R,
                                   const double *mat, double freq, double *F)
{
    std::lock_guard<std::mutex> lk(ctx().mu);
    if ((nen != 3 && nen != 6) || !nodes || !elems || !vB || !pts || !mat || !F || order < 1) {
        set_error("dsc_force_multipole: bad arguments");
        return kErrArg;
    }
    std::vector<int> e0;
    elems_to0(nen, (int)E, elems, e0);
    MeshEntry *m;
    DSC_TRY(get_mesh(nen, (int)N, (int)E, nodes, e0.data(), &m));
    std::vector<double> Ed;
    DSC_TRY(derivs_on(m, vB, npts, pts, Ed));
    for (unsigned q = 0; q < npts; q++)
        multipole_from_derivs(nen, Ed.data() + (size_t)q * kDerivCount, order, R, mat, freq, F + 3 * (size_t)q);
    return kOk;
}

extern "C" int dsc_force_ellipsoid(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
                                   const double *vB, unsigned npts, const double *pts, unsigned analysis,
                                   const double *axis, const double *mat, double freq, double *F)
{
    std::lock_guard<std::mutex> lk(ctx().mu);
    if ((nen != 3 && nen != 6) || !nodes || !elems || !vB || !pts || !mat || !F || !axis ||
        (analysis != 10 && analysis != 11)) {
        set_error("dsc_force_ellipsoid: bad arguments");
        return kErrArg;
    }
    double Ld[3];
    bool warn = false;
    if (!depolarization_factors(axis, Ld, &warn)) {
        set_error("dsc_force_ellipsoid: negative depolarisation factors (%g %g %g)", Ld[0], Ld[1], Ld[2]);
        return kErrArg;
    }
    std::vector<int> e0;
    elems_to0(nen, (int)E, elems, e0);
    MeshEntry *m;
    DSC_TRY(get_mesh(nen, (int)N, (int)E, nodes, e0.data(), &m));
    std::vector<double> Ed;
    DSC_TRY(derivs_on(m, vB, npts, pts, Ed));
    for (unsigned q = 0; q < npts; q++)
        ellipsoid_from_derivs(Ed.data() + (size_t)q * kDerivCount, analysis, axis, Ld, mat, freq,
                              F + 3 * (size_t)q);
    return kOk;
}

extern "C" int dsc_depolarization(const double *axis, double *Ld)
{
    bool warn = false;
    if (!axis || !Ld) {
        set_error("dsc_depolarization: bad arguments");
        return kErrArg;
    }
    if (!depolarization_factors(axis, Ld, &warn)) {
        set_error("negative depolarisation factors");
        return kErrArg;
    }
    return kOk;
}

extern "C" int dsc_force_mst(int nen, unsigned N, unsigned E, const double *nodes,
                             const unsigned *elems, const unsigned *bctype, const double *vB,
                             double eps, double *Fce, double *Xce, double *Fcm, double *Xcm)
{
    std::lock_guard<std::mutex> lk(ctx().mu);
    if (!family_ok(nen) || !nodes || !elems || !bctype || !vB || !Fcm || !Xcm) {
        set_error("dsc_force_mst: bad arguments");
        return kErrArg;
    }
    std::vector<int> e0;
    elems_to0(nen, (int)E, elems, e0);
    if (nen == 8) {
        Context &c = ctx();
        Q8Mesh *q;
        DSC_TRY(get_q8_mesh((int)N, (int)E, nodes, e0.data(), &q));
        DSC_TRY(c.q8_sigma.upload(vB, 2 * (size_t)N, c.st));
        return q8_force_mst(*q, bctype, c.q8_sigma.p, eps, Fce, Xce, Fcm, Xcm, c.st);
    }
    return force_impl(nen, N, E, nodes, e0.data(), bctype, vB, eps, Fce, Xce, Fcm, Xcm);
}
