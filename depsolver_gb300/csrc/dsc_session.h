// dsc_session.h -- device-resident scene of libdepsolver_cuda (not exported).
#pragma once

#include <cuda_fp16.h>

#include <functional>
#include <string>
#include <thread>
#include <vector>

#include "dsc_field.h"
#include "dsc_internal.h"
#include "dsc_precond.h"

namespace dsc {

// Destroys the session's stream after every other member (members go in
// reverse order of declaration): buffers of stream-ordered allocations are
// freed on the stream first, then the stream is drained and destroyed.
struct StreamGuard {
    cudaStream_t *st;
    explicit StreamGuard(cudaStream_t *s) : st(s) {}
    ~StreamGuard()
    {
        if (*st) {
            cudaStreamSynchronize(*st);
            cudaStreamDestroy(*st);
        }
    }
};

struct Session {
    int nen = 6, N = 0, E = 0;
    unsigned nIf = 0;
    cudaStream_t st = nullptr;
    StreamGuard st_guard{&st};  // declared before every device buffer
    // a second stream for independent work beside st (the conductor blocks'
    // Gauss-Jordan sequences), joined back by events
    cudaStream_t side = nullptr;
    StreamGuard side_guard{&side};
    // a third stream: the conductor-block inverses run on it (and on side)
    // while K's conversion runs on st
    cudaStream_t side2 = nullptr;
    StreamGuard side2_guard{&side2};
    HostPlan plan;
    DeviceMesh dev;
    ForcePlan force;
    // the force plan's host part (field points, their near lists, the
    // singular tuples they share with the assembly) is built on a thread
    // from create() on, beside the first assembly's regular pairs, with its
    // uploads on the side stream; force_wait() joins it (the destructor too)
    std::thread force_job;
    int force_rc = 0;
    std::string force_err;
    int force_wait();
    Timer timer;
    std::vector<unsigned> bctype, ifaces;
    std::vector<double> mbc, mat;
    std::vector<int> iface_of_row;
    DevBuf<int> rows;          // iface_of_row on the device (-1: conductor row)
    DevBuf<double> bre, bim;   // boundary value of each row, Re and Im
    double eps_medium = 0.0;
    size_t ld = 0;

    // FP64 geometric matrix and its diagonal
    bool k64_ready = false;
    int k64_prec = kAsmF64;   // arithmetic K64's regular pairs were integrated in
    int mixed_asm = kAsmF32;  // the mixed mode's choice (kAsmF32 or kAsmDf32)
    AsmWorkspace asm_ws;    // kept between assemblies
    // the gradient integrals of the force points' singular elements, left
    // by each assembly (3 nen per singular tuple; see assemble_K_fp64)
    DevBuf<double> Wsing;
    DevBuf<double> K64, Kdiag;
    std::vector<double> Kdiag_host;
    // plain FP64 path workspace; jacobi_full: its Jacobi scaling also
    // scales the imaginary right-hand side (the reference scales B[i] only)
    DevBuf<double> ca, cb, cd, gemv_part;
    bool jacobi_full = false;

    // mixed path: K as row-major scaled fp16 pairs (2^s_i fl32(K) per row i)
    // for the tensor-core products, K's fixed-point row digits (kKDigits
    // fp16 matrices) for the first FP64-accurate residual, the epilogue's
    // row factors, and the batched-solver workspace
    bool k16_ready = false;
    // the first residual's K x: from K's digits on the tensor cores, or by
    // an FP64 GEMV over K64 (residual_mode: kResidAuto decides by size)
    enum { kResidAuto = 0, kResidDigits = 1, kResidFp64 = 2 };
    int residual_mode = kResidAuto;
    bool digits = true;
    DevBuf<__half> Kh16, Kl16, Kdig;
    DevBuf<int> rowE;           // biased FP64 exponent of each row's largest entry
    DevBuf<float> rsK;          // 2^-s_i
    struct Mixed;
    Mixed *mx = nullptr;
    // conductor-block right preconditioner of the mixed sweep (pre_on: used
    // by mixed solves)
    Precond *pre = nullptr;
    bool pre_on = true;
    // mixed solves: the batched field's far pairs on the tensor cores (else
    // all pairs on the FP32 pipes)
    bool field_tc = true;

    int create(int nen, unsigned N, unsigned E, const double *nodes, const unsigned *elems,
               const unsigned *bctype, const double *mbc, unsigned nIf, const unsigned *ifaces,
               unsigned nMat, const double *mat);
    ~Session();
    // K64 (and Kdiag) if not there yet; need_fp64: the regular pairs in FP64
    // (else in mixed_asm's arithmetic; a more accurate K64 is kept)
    int assemble64(bool need_fp64);
    int make_k16();
    void coeffs(double f, std::vector<double> &a, std::vector<double> &b,
                std::vector<double> &d) const;
    int solve_fp64(double f, double tol, unsigned max_iters, double *sigma_dev, double *d_tot,
                   unsigned *iters);
    // timer sums, scope counts and algorithmic work per class; resets
    int collect_timing(double *ms, int *count, double *work);
    int solve_mixed(unsigned nfreq, const double *freqs, double tol, unsigned max_iters,
                    double *sigma_host, double *forces_host, unsigned *iters);
    // outcome of each system of the last solve (SysStatus), and the
    // per-particle results of its systems (nfreq x force.npart x kPartVals)
    std::vector<int> last_status;
    std::vector<double> last_particles;
};

// The split-count autotuner of the mixed sweep's tensor-core product
// (dsc_mixed.cu): on/off, and its table of tuned sizes.
int autotune_set(int on);
int autotune_table(int *rows, int n);

}  // namespace dsc
