// dsc_session.cu -- device-resident scenes and frequency sweeps.
//
// A session keeps one geometry in HBM: the mesh plan, the geometric matrix
// K (assembled once, frequency independent) and the force plan.  Each
// frequency f only changes per-row coefficients (src/assembly_el.c:223-256):
//   M_f = diag(a - i b) K + diag(d),   a, b = A_k, B_k on interface rows,
//   a = 1, b = 0 on conductor rows, d = -1/(2 eps0) on interface rows,
// so a sweep assembles once and solves many systems.
//
// Plain FP64 path (DSC_MODE_FP64): per frequency, the reference's GMRES
// (real 2N form, Jacobi row scaling with the real diagonal, MGS, Givens;
// src/gmres_el.c:66-260) on the K-form operator
//   y_re = a (K x_re) + d x_re + b (K x_im),  y_im = a (K x_im) + d x_im - b (K x_re)
// whose K products are one FP64 GEMV with two right-hand sides, then the
// FP64 field at the type-6 nodes and the Maxwell-stress force.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <complex>
#include <limits>
#include <memory>
#include <vector>

#include "../../include/depsolver_cuda.h"
#include "dsc_blas.cuh"
#include "dsc_common.cuh"
#include "dsc_field.h"
#include "dsc_gmres.h"
#include "dsc_internal.h"
#include "dsc_session.h"

namespace dsc {

// ---------------------------------------------------------------- kernels

// y = K-form operator applied to x (real 2N layout), from the split sums.
__global__ void k_kform_epilogue(const double *__restrict__ part, int S, int N,
                                 const double *__restrict__ ca, const double *__restrict__ cb,
                                 const double *__restrict__ cd, const double *__restrict__ x,
                                 double *__restrict__ y, const int *skip)
{
    if (skip && *skip) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    double tr = 0.0, ti = 0.0;
    for (int s = 0; s < S; s++) {
        tr += part[((size_t)s * 2) * N + i];
        ti += part[((size_t)s * 2 + 1) * N + i];
    }
    const double a = ca[i], b = cb[i], d = cd[i];
    y[i] = a * tr + d * x[i] + b * ti;
    y[i + N] = a * ti + d * x[i + N] - b * tr;
}

__global__ void k_diag(const double *__restrict__ K, size_t ld, int N, double *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) out[i] = K[(size_t)i * ld + i];
}

// ---------------------------------------------------------------- operator

struct KFormOp : RealOp {
    const double *K = nullptr;
    size_t ld = 0;
    int N = 0, S = 1, cols = 0;
    const double *ca = nullptr, *cb = nullptr, *cd = nullptr;
    double *part = nullptr;
    Timer *tm = nullptr;
    int apply(const double *x, double *y, cudaStream_t st) override
    {
        {
            TimerScope ts(tm, kTGemvK, st);
            dim3 g((N + 255) / 256, S);
            DSC_LAUNCH(k_gemv_K2<double><<<g, 256, 0, st>>>(K, ld, N, x, x + N, cols, part, skip));
            if (tm) tm->add_work(kTGemvK, 8.0 * N * N);  // bytes of K read
        }
        DSC_LAUNCH(k_kform_epilogue<<<(N + 255) / 256, 256, 0, st>>>(part, S, N, ca, cb, cd, x, y, skip));
        DSC_CUDA(cudaGetLastError());
        return kOk;
    }
};

// ---------------------------------------------------------------- session

int Session::create(int nen_, unsigned N_, unsigned E_, const double *nodes, const unsigned *elems,
                    const unsigned *bctype_, const double *mbc_, unsigned nIf_,
                    const unsigned *ifaces_, unsigned nMat, const double *mat_)
{
    nen = nen_;
    N = (int)N_;
    E = (int)E_;
    nIf = nIf_;
    DSC_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    {
        // side2 runs the conductor-block inverses' chain of small dependent
        // kernels and side the rest of their updates, beside K's conversion
        // on st: they go first whenever SMs free up
        int least = 0, greatest = 0;
        DSC_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        DSC_CUDA(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, greatest));
        DSC_CUDA(cudaStreamCreateWithPriority(&side2, cudaStreamNonBlocking, greatest));
    }
    AllocStreamScope as(st);
    std::vector<int> e0((size_t)E * nen);
    for (size_t t = 0; t < e0.size(); t++) e0[t] = (int)elems[t] - 1;
    DSC_TRY(build_plan(nen, N, E, nodes, e0.data(), bctype_, plan));
    bctype.assign(bctype_, bctype_ + 2 * (size_t)N);
    mbc.assign(mbc_, mbc_ + 6 * (size_t)N);
    ifaces.assign(ifaces_, ifaces_ + 2 * (size_t)nIf);
    mat.assign(mat_, mat_ + 2 * (size_t)nMat);
    for (unsigned i = 0; i < nIf; i++)
        if (ifaces[2 * i] < 1 || ifaces[2 * i] > nMat || ifaces[2 * i + 1] < 1 || ifaces[2 * i + 1] > nMat) {
            set_error("interface %u references a material outside 1..%u", i + 1, nMat);
            return kErrArg;
        }
    iface_of_row.assign(N, -1);
    for (int i = 0; i < N; i++)
        if (plan.row_kind[i] == 1) {
            unsigned k = (unsigned)mbc[3 * (size_t)i + 1] - 1;
            if (k >= nIf) {
                set_error("node %d: interface id %g outside 1..%u", i + 1, mbc[3 * (size_t)i + 1], nIf);
                return kErrArg;
            }
            iface_of_row[i] = (int)k;
        }
    eps_medium = mat[1] * kEps0;
    {
        // per-row data of the systems: interface of the row, boundary value
        std::vector<double> re(N), im(N);
        for (int i = 0; i < N; i++) {
            re[i] = mbc[3 * (size_t)i];
            im[i] = mbc[3 * (size_t)(i + N)];
        }
        DSC_TRY(rows.upload(iface_of_row, st));
        DSC_TRY(bre.upload(re, st));
        DSC_TRY(bim.upload(im, st));
        DSC_CUDA(cudaStreamSynchronize(st));
    }
    DSC_TRY(dev.upload(plan, st));
    force_job = std::thread([this] {
        AllocStreamScope fs(side);
        force_rc = force.build(plan, bctype.data(), side);
        if (force_rc != (int)kOk) force_err = last_error();
    });
    ld = ((size_t)N + 31) / 32 * 32;
    pre = new Precond();
    DSC_TRY(precond_plan(*this));
    return kOk;
}

void destroy_mixed(Session::Mixed *m);
void destroy_precond(Precond *p);

int Session::force_wait()
{
    if (force_job.joinable()) force_job.join();
    if (force_rc != kOk) set_error("%s", force_err.c_str());
    return force_rc;
}

Session::~Session()
{
    if (force_job.joinable()) force_job.join();
    if (st) cudaStreamSynchronize(st);  // nothing on st still reads a buffer freed on side
    // the stream itself goes last (StreamGuard)
    if (mx) destroy_mixed(mx);
    if (pre) destroy_precond(pre);
}

int Session::assemble64(bool need_fp64)
{
    // a K assembled in FP64 serves both modes; one assembled in
    // double-FP32 serves the mixed mode only
    const int want = need_fp64 ? kAsmF64 : mixed_asm;
    if (k64_ready && k64_prec <= want) return kOk;
    k16_ready = false;  // the fp16 copies and the preconditioner follow K
    if (pre && !pre->adopted) pre->ready = false;
    DSC_TRY(K64.alloc(ld * N));
    // the force plan is joined only before the singular pairs, which store
    // the gradients its points take
    const std::function<int(const int **, double **)> late = [this](const int **row_grad, double **Wg) -> int {
        DSC_TRY(force_wait());
        *row_grad = force.row_grad.p;
        *Wg = nullptr;
        if (force.P > 0) {
            DSC_TRY(Wsing.alloc((size_t)std::max(dev.ne_total, 1) * 3 * nen));
            *Wg = Wsing.p;
        }
        return kOk;
    };
    DSC_TRY(assemble_K_fp64(dev, K64.p, ld, st, &timer, want, &asm_ws, nullptr, nullptr, &late));
    k64_prec = want;
    DSC_TRY(Kdiag.alloc(N));
    DSC_LAUNCH(k_diag<<<(N + 255) / 256, 256, 0, st>>>(K64.p, ld, N, Kdiag.p));
    DSC_CUDA(cudaGetLastError());
    Kdiag_host.resize(N);
    DSC_CUDA(cudaMemcpyAsync(Kdiag_host.data(), Kdiag.p, N * sizeof(double), cudaMemcpyDeviceToHost, st));
    DSC_CUDA(cudaStreamSynchronize(st));
    k64_ready = true;
    return kOk;
}

// Row coefficients at frequency f: a, b, d as above.
void Session::coeffs(double f, std::vector<double> &a, std::vector<double> &b,
                     std::vector<double> &d) const
{
    std::vector<double> Ak(nIf ? nIf : 1), Bk(nIf ? nIf : 1);
    if (nIf) interface_coeffs(nIf, ifaces.data(), mat.data(), f, Ak.data(), Bk.data());
    a.resize(N);
    b.resize(N);
    d.resize(N);
    for (int i = 0; i < N; i++) {
        if (iface_of_row[i] < 0) {
            a[i] = 1.0;
            b[i] = 0.0;
            d[i] = 0.0;
        } else {
            a[i] = Ak[iface_of_row[i]];
            b[i] = Bk[iface_of_row[i]];
            d[i] = -0.5 / kEps0;
        }
    }
}

// One frequency on the plain FP64 path.  sigma_dev (2N) receives the
// solution; d_tot (9) the force totals.
int Session::solve_fp64(double f, double tol, unsigned max_iters, double *sigma_dev,
                        double *d_tot, unsigned *iters)
{
    DSC_TRY(assemble64(true));
    std::vector<double> a, b, d;
    coeffs(f, a, b, d);
    std::vector<double> B(2 * (size_t)N);
    for (int i = 0; i < N; i++) {
        B[i] = mbc[3 * (size_t)i];
        B[i + N] = mbc[3 * (size_t)(i + N)];
    }
    // Jacobi scaling of the reference: row i (both halves) and B[i] (real
    // part only) times 1 / A1[i][i] (src/gmres_el.c:87-93).  The imaginary
    // right-hand side B[N + i] stays unscaled there, so with a complex
    // boundary value (a phase-shifted electrode) the reference solves for an
    // imaginary part off by the factor A1[i][i]; jacobi_full scales it too
    // (the system the mixed mode solves)
    for (int i = 0; i < N; i++) {
        double p = 1.0 / (a[i] * Kdiag_host[i] + d[i]);
        a[i] *= p;
        b[i] *= p;
        d[i] *= p;
        B[i] *= p;
        if (jacobi_full) B[i + N] *= p;
    }
    DSC_TRY(ca.upload(a, st));
    DSC_TRY(cb.upload(b, st));
    DSC_TRY(cd.upload(d, st));
    DSC_CUDA(cudaMemcpyAsync(sigma_dev, B.data(), B.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    KFormOp op;
    op.K = K64.p;
    op.ld = ld;
    op.N = N;
    int rowblocks = (N + 255) / 256;
    op.S = std::max(1, std::min(64, 4 * 152 / rowblocks));
    op.cols = (N + op.S - 1) / op.S;
    op.ca = ca.p;
    op.cb = cb.p;
    op.cd = cd.p;
    DSC_TRY(gemv_part.alloc((size_t)op.S * 2 * N));
    op.part = gemv_part.p;
    op.tm = &timer;
    DSC_TRY(gmres_real_fp64(2 * N, op, sigma_dev, nullptr, tol, max_iters, nullptr, iters, st));
    DSC_TRY(force_wait());
    DSC_TRY(force_mst_dev(dev, force, sigma_dev, eps_medium, d_tot, st, &timer));
    return kOk;
}

}  // namespace dsc

// ================================================================ C ABI
using namespace dsc;

struct dsc_session {
    Session s;
};

extern "C" int dsc_session_create(int nen, unsigned N, unsigned E, const double *nodes,
                                  const unsigned *elems, const unsigned *bctype, const double *mbc,
                                  unsigned nIf, const unsigned *ifaces, unsigned nMat,
                                  const double *mat, dsc_session **out)
{
    *out = nullptr;
    if ((nen != 3 && nen != 6) || !nodes || !elems || !bctype || !mbc || !mat || nMat == 0 ||
        (nIf && !ifaces)) {
        set_error("dsc_session_create: bad arguments");
        return kErrArg;
    }
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        set_error("no CUDA device available");
        return kErrCuda;
    }
    auto s = std::make_unique<dsc_session>();
    DSC_TRY(s->s.create(nen, N, E, nodes, elems, bctype, mbc, nIf, ifaces, nMat, mat));
    *out = s.release();
    return kOk;
}

extern "C" void dsc_session_destroy(dsc_session *s) { delete s; }

extern "C" void *dsc_session_stream(dsc_session *s) { return (void *)s->s.st; }

extern "C" int dsc_session_set_timing(dsc_session *s, int on)
{
    s->s.timer.on = on != 0;
    return kOk;
}

extern "C" int dsc_session_set_preconditioner(dsc_session *s, int on)
{
    s->s.pre_on = on != 0;
    return kOk;
}

extern "C" int dsc_set_autotune(int on) { return autotune_set(on); }

extern "C" int dsc_autotune_table(int *rows, int n) { return autotune_table(rows, n); }

extern "C" int dsc_session_set_fp64_jacobi(dsc_session *s, int full)
{
    s->s.jacobi_full = full != 0;
    return kOk;
}

extern "C" int dsc_session_set_residual(dsc_session *s, int how)
{
    if (how != DSC_RESIDUAL_AUTO && how != DSC_RESIDUAL_DIGITS && how != DSC_RESIDUAL_FP64) {
        set_error("dsc_session_set_residual: unknown choice %d", how);
        return kErrArg;
    }
    if (how != s->s.residual_mode) s->s.k16_ready = false;  // the digits follow the choice
    s->s.residual_mode = how;
    return kOk;
}

extern "C" int dsc_session_set_field_tensor(dsc_session *s, int on)
{
    s->s.field_tc = on != 0;
    return kOk;
}

extern "C" int dsc_session_set_mixed_assembly(dsc_session *s, int prec)
{
    if (prec != DSC_ASM_FP32 && prec != DSC_ASM_DF32) {
        set_error("dsc_session_set_mixed_assembly: unknown arithmetic %d", prec);
        return kErrArg;
    }
    s->s.mixed_asm = prec == DSC_ASM_FP32 ? kAsmF32 : kAsmDf32;
    return kOk;
}

extern "C" int dsc_session_preconditioner_blocks(dsc_session *s, int *rows, int n)
{
    const Precond *p = s->s.pre;
    const int nb = p ? p->nb : 0;
    for (int b = 0; b < nb && b < n && rows; b++) rows[b] = p->n[b];
    return nb;
}

extern "C" int dsc_session_timing(dsc_session *s, double *ms, int *count, double *work, int n)
{
    double t[kTCount], wk[kTCount];
    int c[kTCount];
    DSC_TRY(s->s.collect_timing(t, c, wk));
    for (int k = 0; k < n && k < kTCount; k++) {
        if (ms) ms[k] = t[k];
        if (count) count[k] = c[k];
        if (work) work[k] = wk[k];
    }
    return kOk;
}

extern "C" int dsc_session_assemble(dsc_session *s, int mode)
{
    AllocStreamScope as(s->s.st);
    if (mode != DSC_MODE_FP64 && mode != DSC_MODE_MIXED) {
        set_error("dsc_session_assemble: unknown mode %d", mode);
        return kErrArg;
    }
    // always re-assemble: the caller asks for the work to be done now
    s->s.k64_ready = false;
    s->s.k16_ready = false;
    DSC_TRY(s->s.assemble64(mode == DSC_MODE_FP64));
    return mode == DSC_MODE_MIXED ? s->s.make_k16() : kOk;
}

extern "C" int dsc_session_geometric_matrix(dsc_session *s, int mode, double *K, size_t ldk)
{
    AllocStreamScope as(s->s.st);
    Session &S = s->s;
    if ((mode != DSC_MODE_FP64 && mode != DSC_MODE_MIXED) || !K || ldk < (size_t)S.N) {
        set_error("dsc_session_geometric_matrix: bad arguments");
        return kErrArg;
    }
    DSC_TRY(S.assemble64(mode == DSC_MODE_FP64));
    DSC_CUDA(cudaMemcpy2DAsync(K, ldk * sizeof(double), S.K64.p, S.ld * sizeof(double),
                               (size_t)S.N * sizeof(double), S.N, cudaMemcpyDeviceToHost, S.st));
    DSC_CUDA(cudaStreamSynchronize(S.st));
    return kOk;
}

// DSC_OK when every system of the sweep converged, else DSC_ERR_NOCONVERGE
// naming how many did not (their outcomes: dsc_session_status).
static int sweep_status(const std::vector<int> &st)
{
    int capped = 0, stag = 0;
    for (int v : st) {
        capped += v == kSysCapped;
        stag += v == kSysStagnated;
    }
    if (capped + stag == 0) return kOk;
    set_error("%d of %zu systems did not converge (%d reached max_iters, %d stagnated); their results are NaN",
              capped + stag, st.size(), capped, stag);
    return kErrNoConverge;
}

extern "C" int dsc_session_solve(dsc_session *sess, int mode, unsigned nfreq, const double *freqs,
                                 double tol, unsigned max_iters, double *sigma, double *forces,
                                 unsigned *iters)
{
    Session &s = sess->s;
    AllocStreamScope as(s.st);
    if (mode != DSC_MODE_FP64 && mode != DSC_MODE_MIXED) {
        set_error("dsc_session_solve: unknown mode %d", mode);
        return kErrArg;
    }
    if (nfreq && !freqs) {
        set_error("dsc_session_solve: freqs is NULL");
        return kErrArg;
    }
    if (mode == DSC_MODE_MIXED) {
        DSC_TRY(s.solve_mixed(nfreq, freqs, tol, max_iters, sigma, forces, iters));
        return sweep_status(s.last_status);
    }
    const size_t n2 = 2 * (size_t)s.N;
    s.last_status.assign(nfreq, kSysStagnated);
    s.last_particles.clear();
    DevBuf<double> sig, tot, ptot;
    DSC_TRY(sig.alloc(n2));
    DSC_TRY(tot.alloc(9 * (size_t)std::max(1u, nfreq)));
    const double nan = std::numeric_limits<double>::quiet_NaN();
    size_t pv = 0;
    for (unsigned k = 0; k < nfreq; k++) {
        unsigned it = 0;
        // a frequency whose GMRES stops short (cap or stagnation) gets NaN
        // results and a status; the sweep goes on with the next one
        int rc = s.solve_fp64(freqs[k], tol, max_iters, sig.p, tot.p + 9 * (size_t)k, &it);
        if (iters) iters[k] = it;
        if (k == 0) {
            // the force plan (its particles) is joined by the first assembly
            DSC_TRY(s.force_wait());
            pv = (size_t)s.force.npart * kPartVals;
            DSC_TRY(ptot.alloc(std::max<size_t>(1, pv * nfreq)));
            s.last_particles.assign(pv * nfreq, nan);
        }
        if (rc == kErrNoConverge || rc == kErrStagnation) {
            s.last_status[k] = rc == kErrNoConverge ? kSysCapped : kSysStagnated;
            DSC_CUDA(cudaStreamSynchronize(s.st));
            if (sigma) std::fill(sigma + n2 * k, sigma + n2 * (k + 1), nan);
            std::vector<double> t9(9, nan);
            DSC_CUDA(cudaMemcpyAsync(tot.p + 9 * (size_t)k, t9.data(), 9 * sizeof(double),
                                     cudaMemcpyHostToDevice, s.st));
            DSC_CUDA(cudaStreamSynchronize(s.st));
            continue;
        }
        if (rc != kOk) return rc;
        s.last_status[k] = kSysConverged;
        DSC_TRY(mst_particles(s.force, s.dev.x.p, s.dev.y.p, s.dev.z.p, s.force.Fce.p, 0, s.force.Xce.p, 1,
                              ptot.p + pv * k, s.st));
        if (sigma)
            DSC_CUDA(cudaMemcpyAsync(sigma + n2 * k, sig.p, n2 * sizeof(double), cudaMemcpyDeviceToHost,
                                     s.st));
    }
    if (forces)
        DSC_CUDA(cudaMemcpyAsync(forces, tot.p, 9 * (size_t)nfreq * sizeof(double),
                                 cudaMemcpyDeviceToHost, s.st));
    std::vector<double> ph(pv * nfreq);
    if (pv) DSC_CUDA(cudaMemcpyAsync(ph.data(), ptot.p, ph.size() * sizeof(double), cudaMemcpyDeviceToHost, s.st));
    DSC_CUDA(cudaStreamSynchronize(s.st));
    for (unsigned k = 0; k < nfreq; k++)
        if (s.last_status[k] == kSysConverged)
            std::copy(ph.begin() + pv * k, ph.begin() + pv * (k + 1), s.last_particles.begin() + pv * k);
    return sweep_status(s.last_status);
}

extern "C" int dsc_session_particles(dsc_session *sess, double *out, unsigned n)
{
    const Session &s = sess->s;
    const size_t pv = (size_t)s.force.npart * kPartVals;
    if (out && pv) {
        const size_t nf = pv ? s.last_particles.size() / pv : 0;
        std::copy(s.last_particles.begin(), s.last_particles.begin() + pv * std::min<size_t>(n, nf), out);
    }
    return s.force.npart;
}

extern "C" int dsc_session_status(dsc_session *sess, int *status, unsigned n)
{
    const std::vector<int> &st = sess->s.last_status;
    for (unsigned k = 0; k < n && k < st.size() && status; k++) status[k] = st[k];
    return (int)st.size();
}

extern "C" int dsc_sweep(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
                         const unsigned *bctype, const double *mbc, unsigned nIf,
                         const unsigned *ifaces, unsigned nMat, const double *mat, int mode,
                         unsigned nfreq, const double *freqs, double tol, unsigned max_iters,
                         double *sigma, double *forces, unsigned *iters)
{
    dsc_session *s = nullptr;
    DSC_TRY(dsc_session_create(nen, N, E, nodes, elems, bctype, mbc, nIf, ifaces, nMat, mat, &s));
    int rc = dsc_session_solve(s, mode, nfreq, freqs, tol, max_iters, sigma, forces, iters);
    dsc_session_destroy(s);
    return rc;
}
