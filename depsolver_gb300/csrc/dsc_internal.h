// dsc_internal.h -- host-side structures of libdepsolver_cuda (not exported).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>
#include <string>
#include <utility>
#include <vector>

namespace dsc {

// ---------------------------------------------------------------- errors
enum Status {
    kOk = 0,
    kErrCuda = 1,
    kErrArg = 2,
    kErrBcType = 3,      // boundary type the assembly does not define
    kErrSingular = 4,    // pivot within 1e-9 of zero
    kErrNoConverge = 5,  // GMRES hit its iteration cap
    kErrStagnation = 6,  // "CONVERGENCE RATE TOO SLOW"
    kErrMemory = 7,
};

// Outcome of one system of a sweep (dsc_session_status).
enum SysStatus { kSysConverged = 0, kSysCapped = 1, kSysStagnated = 2 };

void set_error(const char *fmt, ...);
const char *last_error();

// Every kernel launch of the library goes through DSC_LAUNCH, which counts
// it (dsc_kernel_launches() in the C ABI reports the running total).
void note_launch();
#define DSC_LAUNCH(...)         \
    do {                        \
        ::dsc::note_launch();   \
        __VA_ARGS__;            \
    } while (0)

#define DSC_CUDA(call)                                                                       \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            ::dsc::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
            return ::dsc::kErrCuda;                                                          \
        }                                                                                    \
    } while (0)

#define DSC_TRY(call)                     \
    do {                                  \
        int s_ = (call);                  \
        if (s_ != ::dsc::kOk) return s_;  \
    } while (0)

// Programmatic dependent launch: the kernel may be scheduled while the
// stream's previous kernel drains (its launch latency hidden behind that
// kernel's tail).  The kernel must call grid_dep_wait() before it reads
// anything the previous kernels wrote (the wait returns once they have
// completed and their writes are visible).
template <typename... KArgs, typename... Args>
int launch_dependent(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args &&...args)
{
    note_launch();
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    DSC_CUDA(cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...));
    return kOk;
}

#ifdef __CUDACC__
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
#endif

// ---------------------------------------------------------------- buffers
// Stream-ordered allocation.  While an AllocStreamScope is active on a
// thread (a session's calls set one with the session's stream), DevBuf
// takes memory with cudaMallocAsync on that stream from the device's
// default pool, which keeps freed memory for the next allocation (a new
// session reuses the previous one's blocks instead of mapping new memory),
// and gives it back with cudaFreeAsync on the same stream.  Outside a scope
// it uses cudaMalloc / cudaFree.
cudaStream_t &alloc_stream();
int alloc_pool_setup();  // once per device: the default pool keeps freed memory

// Per-device facts cached for every thread (safe to call from several
// threads at once, each on its own device or stream): the current device's
// SM count, and raising a kernel's dynamic shared-memory limit on the
// current device to at least `bytes` (set once per device and size).
int current_sm_count(int *nsm);
int raise_smem_limit(const void *kern, int bytes);

struct AllocStreamScope {
    cudaStream_t prev;
    explicit AllocStreamScope(cudaStream_t s) : prev(alloc_stream()) { alloc_stream() = s; }
    ~AllocStreamScope() { alloc_stream() = prev; }
    AllocStreamScope(const AllocStreamScope &) = delete;
    AllocStreamScope &operator=(const AllocStreamScope &) = delete;
};

template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaStream_t s = nullptr;  // the stream of a stream-ordered allocation
    bool async = false;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (p) {
            if (async) cudaFreeAsync(p, s);
            else cudaFree(p);
        }
        p = nullptr;
        n = 0;
        async = false;
    }
    int alloc(size_t count)
    {
        if (count <= n && p) return kOk;
        release();
        if (count == 0) count = 1;
        const cudaStream_t as = alloc_stream();
        cudaError_t e;
        if (as) {
            DSC_TRY(alloc_pool_setup());
            e = cudaMallocAsync((void **)&p, count * sizeof(T), as);
        } else {
            e = cudaMalloc(&p, count * sizeof(T));
        }
        if (e != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            set_error("device allocation of %zu bytes failed", count * sizeof(T));
            return kErrMemory;
        }
        async = as != nullptr;
        s = as;
        n = count;
        return kOk;
    }
    int upload(const T *h, size_t count, cudaStream_t st)
    {
        DSC_TRY(alloc(count));
        DSC_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, st));
        return kOk;
    }
    int upload(const std::vector<T> &v, cudaStream_t st) { return upload(v.data(), v.size(), st); }
};

// ---------------------------------------------------------------- timing
// CUDA-event timing of kernel classes on the launching stream (enabled by
// the caller; off by default so that the plain entry points pay nothing).
enum TimerId {
    kTAsmRegular = 0, kTAsmFixup, kTAsmSingular, kTGemvK, kTGemmK, kTField, kTMst, kTResidual,
    kTKrylov, kTCgs, kTConvertK, kTPreBuild, kTPreApply, kTCount
};

struct Timer {
    bool on = false;
    struct Rec {
        int id;
        cudaEvent_t a, b;
    };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> pool;
    // scopes begun and not yet ended, innermost last (scopes nest)
    std::vector<std::pair<int, cudaEvent_t>> open;
    // algorithmic work per id since the last collect (units per id in the
    // C ABI's dsc_session_timing)
    double work[kTCount] = {};
    cudaEvent_t take();
    void begin(int id, cudaStream_t st);
    void end(cudaStream_t st);
    void add_work(int id, double w)
    {
        if (on) work[id] += w;
    }
    // sums (ms), scope counts and work per id since the last collect; resets
    int collect(double *ms, int *count, double *wk);
    ~Timer();
};

// Two events without timing (the look-ahead sequences of the blocked
// Gauss-Jordan and block LU: one stream signals the other).
struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    int create()
    {
        DSC_CUDA(cudaEventCreateWithFlags(&a, cudaEventDisableTiming));
        DSC_CUDA(cudaEventCreateWithFlags(&b, cudaEventDisableTiming));
        return kOk;
    }
    ~EventPair()
    {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

// Work on a second stream between fork() and done(), joined back into the
// main stream by join() -- or by the destructor, on every early return, so
// that nothing queued on the main stream later (a free of a buffer the side
// work uses) overtakes it.
struct SideJoin {
    cudaStream_t main = nullptr;
    cudaEvent_t ev = nullptr;
    int fork(cudaStream_t m, cudaStream_t side)
    {
        main = m;
        cudaEvent_t e0;
        DSC_CUDA(cudaEventCreateWithFlags(&e0, cudaEventDisableTiming));
        cudaError_t r = cudaEventRecord(e0, m);
        if (r == cudaSuccess) r = cudaStreamWaitEvent(side, e0, 0);
        cudaEventDestroy(e0);
        DSC_CUDA(r);
        return kOk;
    }
    int done(cudaStream_t side)
    {
        DSC_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        DSC_CUDA(cudaEventRecord(ev, side));
        return kOk;
    }
    int join()
    {
        if (!ev) return kOk;
        const cudaError_t r = cudaStreamWaitEvent(main, ev, 0);
        cudaEventDestroy(ev);
        ev = nullptr;
        DSC_CUDA(r);
        return kOk;
    }
    ~SideJoin() { join(); }
};

struct TimerScope {
    Timer *t;
    cudaStream_t st;
    TimerScope(Timer *t_, int id, cudaStream_t s) : t(t_ && t_->on ? t_ : nullptr), st(s)
    {
        if (t) t->begin(id, st);
    }
    ~TimerScope()
    {
        if (t) t->end(st);
    }
};

// ---------------------------------------------------------------- mesh plan
// Element groups: elements in Morton order of their centroids, cut into
// groups of kGroup.  A group's footprint is the set of nodes its elements
// touch; a footprint node that no other group touches is written straight
// into K, the others go to partial-sum slots that a fix-up pass adds in
// group order.
constexpr int kGroup = 32;   // elements per group
constexpr int kRowTile = 32; // collocation rows per assembly CTA

struct HostPlan {
    int nen = 6, N = 0, E = 0;
    std::vector<double> nodes;    // N x 3
    std::vector<int> elems;       // E x nen, 0-based
    std::vector<int> row_kind;    // N: 0 conductor (G), 1 interface (H)
    std::vector<double> row_fac;  // N: C for G rows, -1 for H rows
    std::vector<double> normals;  // N x 3 averaged node normals
    int G = 0;
    std::vector<int> grp_elem;    // G x kGroup, -1 padded
    std::vector<int> fp_ptr;      // G + 1
    std::vector<int> fp_dest;     // >= 0: K column; < 0: -(slot + 1)
    std::vector<int> fp_sl_ptr;   // entries + 1
    std::vector<uint16_t> fp_sl;  // local slot e * nen + k
    int n_slots = 0;
    int max_fp = 0;
    std::vector<int> fix_ptr, fix_slot, fix_col;  // boundary nodes
    std::vector<int> ne_ptr, ne_elem, ne_pos;     // node -> (element, position)
    std::vector<int> coord_order;                 // node ids sorted by (x, y, z)
};

// Builds everything above from 0-based connectivity; bctype (may be null)
// has N entries (the real-equation rows).  Fails on boundary types other
// than 0, 1, 6.
int build_plan(int nen, int N, int E, const double *nodes, const int *elems0,
               const unsigned *bctype, HostPlan &plan);
int set_rows(HostPlan &plan, const unsigned *bctype);

// Averaged node normals in element order (reference src/normals.c:120-319).
void node_normals(int nen, int N, int E, const double *nodes, const int *elems0, double *out);

// Interface coefficients (reference src/assembly_el.c:223-239).
void interface_coeffs(unsigned nIf, const unsigned *ifaces, const double *mat, double freq,
                      double *Ak, double *Bk);

// Device copy of a plan plus the element quadrature data.
struct DeviceMesh {
    int nen = 6, N = 0, E = 0, G = 0, n_slots = 0, n_fix = 0;
    int ne_total = 0;              // (node, element containing it) tuples
    DevBuf<double> x, y, z;        // node coordinates (SoA)
    DevBuf<int> elems;             // E x nen
    DevBuf<int> row_kind;
    DevBuf<double> row_fac, normals;
    DevBuf<int> grp_elem, fp_ptr, fp_dest, fp_sl_ptr;
    DevBuf<uint16_t> fp_sl;
    DevBuf<int> fix_ptr, fix_slot, fix_col;
    DevBuf<int> ne_ptr, ne_elem, ne_pos;
    DevBuf<double> qp;             // E x 7 x 4: x, y, z, w * J
    int upload(const HostPlan &p, cudaStream_t st);
    int upload_rows(const HostPlan &p, cudaStream_t st);
};

// K (N x N, column-major, leading dimension ld): K[c * ld + i] is the
// geometric integral of row i against node c: C * int G N_c for conductor
// rows, int H N_c (normal derivative, sign as the reference) for interface
// rows.  The frequency enters only through per-row coefficients.
// Device workspace of an assembly (partial slots, double-FP32 quadrature
// points, FP32 centroid-relative points); a caller that assembles
// repeatedly keeps one to avoid allocating every time.
struct AsmWorkspace {
    DevBuf<double> P;
    DevBuf<float> P32;  // the FP32 assembly's partial slots
    DevBuf<float2> qpd;
    DevBuf<float2> cen;
    DevBuf<float4> qloc;
    DevBuf<unsigned char> rows;  // per-row FP32 data of the FP32 assembly
    DevBuf<float2> nodes_df;     // node coordinates, then normals, in double-FP32 (singular pairs)
};

// Arithmetic of the regular pairs, most accurate first: FP64 (the
// reference's), double-FP32 on the FP32 pipes (about 2^-46 per operation),
// FP32 (about 1e-7 per entry: the mixed mode's far-field assembly).
enum { kAsmF64 = 0, kAsmDf32 = 1, kAsmF32 = 2 };

// prec: one of the above for the regular pairs.  Singular pairs are FP64
// (the reference's sums) with kAsmF64, else double-FP32; K is FP64.  ws (may be null: a local one, freed before
// returning) holds the scratch.  With Wg not null, the rows flagged in
// row_grad (N flags) also leave the gradient integrals of their singular
// elements there: 3 nen doubles per (node, element) tuple of the plan's
// ne_ptr numbering.  late (may be null) is called once, after the regular
// pairs are queued and before the singular ones, to give row_grad and Wg
// in place of the arguments (so that their producer may still be running
// while the regular pairs are launched).
int assemble_K_fp64(const DeviceMesh &m, double *K, size_t ld, cudaStream_t st, Timer *tm = nullptr,
                    int prec = kAsmF64, AsmWorkspace *ws = nullptr, const int *row_grad = nullptr,
                    double *Wg = nullptr, const std::function<int(const int **, double **)> *late = nullptr);

}  // namespace dsc
