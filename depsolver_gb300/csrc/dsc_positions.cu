// dsc_positions.cu -- particle-position sweeps with uneven mesh sizes.
//
// The reference solves one particle position per process run of
// depSolver-sft: nodes pNodes..nNodes-1 (the particle) are shifted rigidly
// by the REPOSITION vector and the whole system is assembled and solved
// again (src/depSolver-shift.c:129-133,212-217).  Here a sweep takes a fixed
// part (electrodes, in the reference's input model) and particle meshes
// ("templates", each with its own node count), and solves every (position,
// frequency) system of a list of (template, centre) positions in one call:
//
//  * every position is a scene of its own (fixed nodes first, then the
//    template's nodes plus the centre -- exactly the reference's shifted
//    coordinates) and runs as a device-resident mixed sweep over all
//    frequencies at once (dsc_session_solve's DSC_MODE_MIXED);
//  * the conductor-block inverses depend only on the fixed electrodes (their
//    rows and columns of K are integrals over the electrodes alone), so they
//    are computed once, by the first position to get there, and every other
//    position takes a device-to-device copy instead of a Gauss-Jordan
//    inversion;
//  * positions are taken from a work queue, largest first, by a pool of
//    host workers, each driving its own CUDA stream, so that several
//    positions' kernels share the GPU: a small system (1.5k nodes) fills a
//    few dozen SMs per kernel, and the streams fill the rest of the 152.
//    Each worker's host work (mesh plan, force plan) overlaps the other
//    workers' kernels.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <limits>
#include <memory>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

#include "../../include/depsolver_cuda.h"
#include "dsc_internal.h"
#include "dsc_precond.h"
#include "dsc_session.h"

namespace dsc {

struct Positions {
    int nen = 6;
    // fixed part, in the reference's input model (elems 1-based)
    int Nf = 0, Ef = 0;
    std::vector<double> nodes, mbc;
    std::vector<unsigned> elems, bctype;
    unsigned nIf = 0, nMat = 0;
    std::vector<unsigned> ifaces;
    std::vector<double> mat;
    struct Template {
        int N = 0, E = 0;
        std::vector<double> nodes;     // N x 3, about the template's origin
        std::vector<unsigned> elems;   // E x nen, 1-based within the template
        unsigned iface = 1;
    };
    std::vector<Template> tmpl;
    int workers = 4;
    int asm_prec = kAsmF32;
    bool timing = false;
    // conductor-block inverses of the fixed part (from the first position
    // that built them)
    std::mutex share_mu;
    bool share_ready = false;
    PrecondShare share;
    int share_builds = 0;  // positions that inverted the blocks themselves
    // timing sums over the positions' sessions
    std::mutex tm_mu;
    double ms[kTCount] = {}, work[kTCount] = {};
    int count[kTCount] = {};
};

// Projection of Fcm(f) on the direction of the lowest frequency's force;
// the crossover is where it first changes sign, interpolated linearly in
// log f between the two frequencies around the change (NaN: none).
static double crossover(const double *forces, const double *freqs, int F, const int *status)
{
    const double nan = std::numeric_limits<double>::quiet_NaN();
    if (F < 2 || (status && status[0] != kSysConverged)) return nan;
    const double *f0 = forces;
    const double n0 = sqrt(f0[0] * f0[0] + f0[1] * f0[1] + f0[2] * f0[2]);
    if (!(n0 > 0.0)) return nan;
    auto proj = [&](int k) {
        const double *q = forces + (size_t)k * 9;
        return (q[0] * f0[0] + q[1] * f0[1] + q[2] * f0[2]) / n0;
    };
    double p0 = proj(0);
    for (int k = 1; k < F; k++) {
        if (status && status[k] != kSysConverged) return nan;
        const double p1 = proj(k);
        if ((p0 > 0.0) != (p1 > 0.0)) {
            const double t = p0 / (p0 - p1);
            return exp(log(freqs[k - 1]) + t * (log(freqs[k]) - log(freqs[k - 1])));
        }
        p0 = p1;
    }
    return nan;
}

// One position: its scene, a session, the inverses shared or built, the
// mixed sweep.  forces (F x 9), iters, status (F) for this position.
static int solve_position(Positions &P, int t, const double *c, unsigned F, const double *freqs, double tol,
                          unsigned max_iters, double *forces, unsigned *iters, int *status, double *sigma)
{
    const Positions::Template &T = P.tmpl[t];
    const int Nf = P.Nf, N = Nf + T.N, E = P.Ef + T.E, nen = P.nen;
    std::vector<double> nodes((size_t)3 * N), mbc((size_t)6 * N);
    std::vector<unsigned> elems((size_t)nen * E), bct((size_t)2 * N);
    std::copy(P.nodes.begin(), P.nodes.end(), nodes.begin());
    for (int i = 0; i < T.N; i++)
        for (int d = 0; d < 3; d++) nodes[(size_t)3 * (Nf + i) + d] = T.nodes[(size_t)3 * i + d] + c[d];
    std::copy(P.elems.begin(), P.elems.end(), elems.begin());
    for (size_t q = 0; q < T.elems.size(); q++) elems[(size_t)nen * P.Ef + q] = T.elems[q] + (unsigned)Nf;
    // rows of the real equations, then of the imaginary ones
    for (int h = 0; h < 2; h++) {
        for (int i = 0; i < Nf; i++) {
            bct[(size_t)h * N + i] = P.bctype[(size_t)h * Nf + i];
            for (int d = 0; d < 3; d++) mbc[((size_t)h * N + i) * 3 + d] = P.mbc[((size_t)h * Nf + i) * 3 + d];
        }
        for (int i = 0; i < T.N; i++) {
            bct[(size_t)h * N + Nf + i] = 6;
            double *m = &mbc[((size_t)h * N + Nf + i) * 3];
            m[0] = 0.0;
            m[1] = (double)T.iface;
            m[2] = 0.0;
        }
    }
    auto sess = std::make_unique<Session>();
    Session &s = *sess;
    DSC_TRY(s.create(nen, N, E, nodes.data(), elems.data(), bct.data(), mbc.data(), P.nIf, P.ifaces.data(), P.nMat,
                     P.mat.data()));
    AllocStreamScope as(s.st);
    s.mixed_asm = P.asm_prec;
    s.timer.on = P.timing;
    DSC_TRY(s.assemble64(false));
    bool adopted = false;
    {
        std::lock_guard<std::mutex> lk(P.share_mu);
        if (P.share_ready) {
            DSC_TRY(precond_adopt(s, P.share));
            adopted = true;
        }
    }
    DSC_TRY(s.make_k16());  // builds the inverses unless they were adopted
    if (!adopted && s.pre && s.pre->ready) {
        std::lock_guard<std::mutex> lk(P.share_mu);
        P.share_builds++;
        if (!P.share_ready) {
            DSC_TRY(precond_export(s, P.share));
            P.share_ready = true;
        }
    }
    DSC_TRY(s.solve_mixed(F, freqs, tol, max_iters, sigma, forces, iters));
    for (unsigned k = 0; k < F; k++) status[k] = s.last_status[k];
    if (P.timing) {
        double m[kTCount], w[kTCount];
        int n[kTCount];
        DSC_TRY(s.collect_timing(m, n, w));
        std::lock_guard<std::mutex> lk(P.tm_mu);
        for (int k = 0; k < kTCount; k++) {
            P.ms[k] += m[k];
            P.count[k] += n[k];
            P.work[k] += w[k];
        }
    }
    return kOk;
}

}  // namespace dsc

// ================================================================ C ABI
using namespace dsc;

struct dsc_positions {
    Positions p;
};

extern "C" double dsc_force_crossover(unsigned nfreq, const double *freqs, const double *forces,
                                      const int *status)
{
    if (!freqs || !forces) return std::numeric_limits<double>::quiet_NaN();
    return crossover(forces, freqs, (int)nfreq, status);
}

extern "C" int dsc_positions_create(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
                                    const unsigned *bctype, const double *mbc, unsigned nIf, const unsigned *ifaces,
                                    unsigned nMat, const double *mat, dsc_positions **out)
{
    *out = nullptr;
    if ((nen != 3 && nen != 6) || !mat || nMat == 0 || (nIf && !ifaces) || (N && (!nodes || !bctype || !mbc)) ||
        (E && !elems)) {
        set_error("dsc_positions_create: bad arguments");
        return kErrArg;
    }
    for (size_t q = 0; q < (size_t)E * nen; q++)
        if (elems[q] < 1 || elems[q] > N) {
            set_error("dsc_positions_create: element node id %u outside 1..%u", elems[q], N);
            return kErrArg;
        }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        set_error("no CUDA device available");
        return kErrCuda;
    }
    auto o = std::make_unique<dsc_positions>();
    Positions &P = o->p;
    P.nen = nen;
    P.Nf = (int)N;
    P.Ef = (int)E;
    P.nodes.assign(nodes, nodes + 3 * (size_t)N);
    P.elems.assign(elems, elems + (size_t)nen * E);
    P.bctype.assign(bctype, bctype + 2 * (size_t)N);
    P.mbc.assign(mbc, mbc + 6 * (size_t)N);
    P.nIf = nIf;
    P.nMat = nMat;
    P.ifaces.assign(ifaces, ifaces + 2 * (size_t)nIf);
    P.mat.assign(mat, mat + 2 * (size_t)nMat);
    *out = o.release();
    return kOk;
}

extern "C" void dsc_positions_destroy(dsc_positions *p) { delete p; }

extern "C" int dsc_positions_add_particle(dsc_positions *o, unsigned N, unsigned E, const double *nodes,
                                          const unsigned *elems, unsigned iface)
{
    Positions &P = o->p;
    if (!N || !E || !nodes || !elems || iface < 1 || iface > P.nIf) {
        set_error("dsc_positions_add_particle: bad arguments (interface %u of %u)", iface, P.nIf);
        return -kErrArg;
    }
    for (size_t q = 0; q < (size_t)E * P.nen; q++)
        if (elems[q] < 1 || elems[q] > N) {
            set_error("dsc_positions_add_particle: element node id %u outside 1..%u", elems[q], N);
            return -kErrArg;
        }
    Positions::Template T;
    T.N = (int)N;
    T.E = (int)E;
    T.nodes.assign(nodes, nodes + 3 * (size_t)N);
    T.elems.assign(elems, elems + (size_t)P.nen * E);
    T.iface = iface;
    P.tmpl.push_back(std::move(T));
    return (int)P.tmpl.size() - 1;
}

extern "C" int dsc_positions_set_workers(dsc_positions *o, int workers)
{
    if (workers < 1 || workers > 64) {
        set_error("dsc_positions_set_workers: %d workers (1..64)", workers);
        return kErrArg;
    }
    o->p.workers = workers;
    return kOk;
}

extern "C" int dsc_positions_set_mixed_assembly(dsc_positions *o, int prec)
{
    if (prec != DSC_ASM_FP32 && prec != DSC_ASM_DF32) {
        set_error("dsc_positions_set_mixed_assembly: unknown arithmetic %d", prec);
        return kErrArg;
    }
    o->p.asm_prec = prec == DSC_ASM_FP32 ? kAsmF32 : kAsmDf32;
    return kOk;
}

extern "C" int dsc_positions_set_timing(dsc_positions *o, int on)
{
    o->p.timing = on != 0;
    return kOk;
}

extern "C" int dsc_positions_timing(dsc_positions *o, double *ms, int *count, double *work, int n)
{
    Positions &P = o->p;
    std::lock_guard<std::mutex> lk(P.tm_mu);
    for (int k = 0; k < n && k < kTCount; k++) {
        if (ms) ms[k] = P.ms[k];
        if (count) count[k] = P.count[k];
        if (work) work[k] = P.work[k];
        P.ms[k] = P.work[k] = 0.0;
        P.count[k] = 0;
    }
    return kOk;
}

extern "C" int dsc_positions_inversions(dsc_positions *o)
{
    std::lock_guard<std::mutex> lk(o->p.share_mu);
    return o->p.share_builds;
}

extern "C" int dsc_positions_solve(dsc_positions *o, unsigned npos, const unsigned *tmpl, const double *centres,
                                   unsigned nfreq, const double *freqs, double tol, unsigned max_iters,
                                   double *forces, unsigned *iters, int *status, double *crossover_hz,
                                   double *sigma)
{
    Positions &P = o->p;
    if (!npos) return kOk;
    if (!tmpl || !centres || !nfreq || !freqs || !forces || !status || max_iters == 0) {
        set_error("dsc_positions_solve: bad arguments");
        return kErrArg;
    }
    for (unsigned q = 0; q < npos; q++)
        if (tmpl[q] >= P.tmpl.size()) {
            set_error("dsc_positions_solve: position %u names particle %u of %zu", q, tmpl[q], P.tmpl.size());
            return kErrArg;
        }
    int dev = 0;
    DSC_CUDA(cudaGetDevice(&dev));
    // largest systems first (the longest jobs start first)
    std::vector<unsigned> order(npos);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(),
                     [&](unsigned a, unsigned b) { return P.tmpl[tmpl[a]].N > P.tmpl[tmpl[b]].N; });
    // sigma rows of position q start at the sum of the earlier positions' 2N x F
    std::vector<size_t> soff(npos + 1, 0);
    for (unsigned q = 0; q < npos; q++) soff[q + 1] = soff[q] + (size_t)2 * (P.Nf + P.tmpl[tmpl[q]].N) * nfreq;
    std::vector<unsigned> it_local(iters ? 0 : (size_t)npos * nfreq);
    unsigned *it_out = iters ? iters : it_local.data();
    std::atomic<unsigned> next{0};
    std::atomic<int> failed{0};
    std::mutex err_mu;
    std::string first_err;
    int first_rc = kOk;
    auto work = [&]() {
        if (cudaSetDevice(dev) != cudaSuccess) {
            cudaGetLastError();
            std::lock_guard<std::mutex> lk(err_mu);
            if (first_rc == kOk) {
                first_rc = kErrCuda;
                first_err = "dsc_positions_solve: cudaSetDevice failed on a worker";
            }
            failed = 1;
            return;
        }
        for (;;) {
            if (failed.load()) return;
            const unsigned k = next.fetch_add(1);
            if (k >= npos) return;
            const unsigned q = order[k];
            const int rc = solve_position(P, (int)tmpl[q], centres + 3 * (size_t)q, nfreq, freqs, tol, max_iters,
                                          forces + (size_t)q * nfreq * 9, it_out + (size_t)q * nfreq,
                                          status + (size_t)q * nfreq, sigma ? sigma + soff[q] : nullptr);
            if (rc != kOk) {
                std::lock_guard<std::mutex> lk(err_mu);
                if (first_rc == kOk) {
                    first_rc = rc;
                    first_err = last_error();
                }
                failed = 1;
                return;
            }
        }
    };
    const int W = std::max(1, std::min<int>(P.workers, (int)npos));
    std::vector<std::thread> pool;
    for (int t = 1; t < W; t++) pool.emplace_back(work);
    work();
    for (auto &th : pool) th.join();
    if (first_rc != kOk) {
        set_error("%s", first_err.c_str());
        return first_rc;
    }
    int bad = 0;
    for (unsigned q = 0; q < npos; q++) {
        if (crossover_hz)
            crossover_hz[q] = crossover(forces + (size_t)q * nfreq * 9, freqs, (int)nfreq, status + (size_t)q * nfreq);
        for (unsigned k = 0; k < nfreq; k++) bad += status[(size_t)q * nfreq + k] != kSysConverged;
    }
    if (bad) {
        set_error("%d of %zu systems did not converge; their results are NaN", bad, (size_t)npos * nfreq);
        return kErrNoConverge;
    }
    return kOk;
}
