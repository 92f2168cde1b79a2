// dsc_plan.cu -- host-side mesh planning for the assembly kernels.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <numeric>
#include <set>
#include <thread>
#include <utility>

#include "dsc_common.cuh"
#include "dsc_field.h"
#include "dsc_internal.h"

namespace dsc {

static thread_local char g_err[512];
static std::atomic<unsigned long long> g_launches{0};

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

}  // namespace dsc

extern "C" unsigned long long dsc_kernel_launches(void)
{
    return dsc::g_launches.load(std::memory_order_relaxed);
}

namespace dsc {

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

const char *last_error() { return g_err; }

// Local coordinates of node position p of a tria6 (src/normals.c:240-264);
// a tria3 normal is constant over the element.
static const double kTria6NodeL[6][2] = {{1.0, 0.0}, {0.5, 0.5}, {0.0, 1.0},
                                         {0.0, 0.5}, {0.0, 0.0}, {0.5, 0.0}};

// One pass over the elements in order adds each element's unit normal at
// the node's local position to the node's sum -- the same additions, in the
// same order, as the reference's per-node scan (getNormal_tria6
// src/normals.c:207-319) -- then normalises.
void node_normals(int nen, int N, int E, const double *nodes, const int *el, double *out)
{
    std::vector<double> acc((size_t)N * 3, 0.0);
    double X[6][3], n[3];
    for (int e = 0; e < E; e++) {
        const int *en = el + (size_t)e * nen;
        for (int k = 0; k < nen; k++)
            for (int d = 0; d < 3; d++) X[k][d] = nodes[3 * (size_t)en[k] + d];
        for (int k = 0; k < nen; k++) {
            bool first = true;
            for (int j = 0; j < k; j++)
                if (en[j] == en[k]) first = false;
            if (!first) continue;
            if (nen == 6) local_normal<6>(X, kTria6NodeL[k][0], kTria6NodeL[k][1], n);
            else local_normal<3>(X, 0.0, 0.0, n);
            double *a = &acc[3 * (size_t)en[k]];
            a[0] += n[0];
            a[1] += n[1];
            a[2] += n[2];
        }
    }
    for (int i = 0; i < N; i++) {
        const double *a = &acc[3 * (size_t)i];
        double inv = 1.0 / sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        out[3 * (size_t)i + 0] = a[0] * inv;
        out[3 * (size_t)i + 1] = a[1] * inv;
        out[3 * (size_t)i + 2] = a[2] * inv;
    }
}

void interface_coeffs(unsigned nIf, const unsigned *ifaces, const double *mat, double freq,
                      double *Ak, double *Bk)
{
    const double C = 1.0 / (kPi4 * kEps0);
    const double W = freq * kPi2 * kEps0;
    for (unsigned i = 0; i < nIf; i++) {
        unsigned m1 = ifaces[2 * i] - 1, m2 = ifaces[2 * i + 1] - 1;
        double sigTot = mat[2 * m1] + mat[2 * m2];
        double sigDif = mat[2 * m1] - mat[2 * m2];
        double epsTot = W * (mat[2 * m1 + 1] + mat[2 * m2 + 1]);
        double epsDif = W * (mat[2 * m1 + 1] - mat[2 * m2 + 1]);
        double D = C / (sigTot * sigTot + epsTot * epsTot);
        Ak[i] = D * (sigTot * sigDif + epsTot * epsDif);
        Bk[i] = D * (sigDif * epsTot - sigTot * epsDif);
    }
}

static uint64_t spread3(uint64_t v)
{
    v &= 0x1fffff;
    v = (v | v << 32) & 0x1f00000000ffffULL;
    v = (v | v << 16) & 0x1f0000ff0000ffULL;
    v = (v | v << 8) & 0x100f00f00f00f00fULL;
    v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
    v = (v | v << 2) & 0x1249249249249249ULL;
    return v;
}

int set_rows(HostPlan &p, const unsigned *bctype)
{
    const double C = 1.0 / (kPi4 * kEps0);
    p.row_kind.resize(p.N);
    p.row_fac.resize(p.N);
    for (int i = 0; i < p.N; i++) {
        unsigned t = bctype[i];
        if (t == 1) { p.row_kind[i] = 0; p.row_fac[i] = C; }
        else if (t == 0 || t == 6) { p.row_kind[i] = 1; p.row_fac[i] = -1.0; }
        else {
            set_error("node %d has boundary type %u; the assembly defines only 0, 1 and 6", i + 1, t);
            return kErrBcType;
        }
    }
    return kOk;
}

// node -> elements containing it (element order, first position in the
// element) and the nodes sorted by (x, y, z).
static void plan_adjacency_and_coords(HostPlan &p, int nen, int N, int E, const int *el)
{
    // node -> elements containing it, element order, first position
    std::vector<int> cnt(N + 1, 0);
    for (int e = 0; e < E; e++)
        for (int k = 0; k < nen; k++) {
            int v = el[(size_t)e * nen + k];
            bool first = true;
            for (int j = 0; j < k; j++)
                if (el[(size_t)e * nen + j] == v) first = false;
            if (first) cnt[v + 1]++;
        }
    for (int i = 0; i < N; i++) cnt[i + 1] += cnt[i];
    p.ne_ptr = cnt;
    p.ne_elem.assign(cnt[N], 0);
    p.ne_pos.assign(cnt[N], 0);
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (int e = 0; e < E; e++)
        for (int k = 0; k < nen; k++) {
            int v = el[(size_t)e * nen + k];
            bool first = true;
            for (int j = 0; j < k; j++)
                if (el[(size_t)e * nen + j] == v) first = false;
            if (!first) continue;
            p.ne_elem[fill[v]] = e;
            p.ne_pos[fill[v]] = k;
            fill[v]++;
        }
    // (x, y, z, node) records sorted directly (no indirection through the
    // node array); ties in the coordinates keep node order
    struct Rec {
        double x, y, z;
        int i;
    };
    std::vector<Rec> r(N);
    for (int i = 0; i < N; i++) r[i] = {p.nodes[3 * (size_t)i], p.nodes[3 * (size_t)i + 1], p.nodes[3 * (size_t)i + 2], i};
    std::sort(r.begin(), r.end(), [](const Rec &a, const Rec &b) {
        if (a.x != b.x) return a.x < b.x;
        if (a.y != b.y) return a.y < b.y;
        if (a.z != b.z) return a.z < b.z;
        return a.i < b.i;
    });
    p.coord_order.resize(N);
    for (int t = 0; t < N; t++) p.coord_order[t] = r[t].i;
}

int build_plan(int nen, int N, int E, const double *nodes, const int *el,
               const unsigned *bctype, HostPlan &p)
{
    if ((nen != 3 && nen != 6) || N <= 0 || E <= 0) {
        set_error("bad mesh sizes (nen %d, N %d, E %d)", nen, N, E);
        return kErrArg;
    }
    for (size_t t = 0; t < (size_t)E * nen; t++)
        if (el[t] < 0 || el[t] >= N) {
            set_error("element %zu references node %d outside 1..%d", t / nen, el[t] + 1, N);
            return kErrArg;
        }
    p.nen = nen;
    p.N = N;
    p.E = E;
    p.nodes.assign(nodes, nodes + (size_t)N * 3);
    p.elems.assign(el, el + (size_t)E * nen);
    p.row_kind.assign(N, 1);
    p.row_fac.assign(N, -1.0);
    if (bctype) DSC_TRY(set_rows(p, bctype));
    // node normals, node -> element adjacency and the coordinate order
    // are independent of the groups below: two host threads build them
    // meanwhile
    p.normals.resize((size_t)N * 3);
    std::thread t_normals([&] { node_normals(nen, N, E, nodes, el, p.normals.data()); });
    std::thread t_side([&] { plan_adjacency_and_coords(p, nen, N, E, el); });

    // Morton order of element centroids.
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int i = 0; i < N; i++)
        for (int d = 0; d < 3; d++) {
            lo[d] = std::min(lo[d], nodes[3 * (size_t)i + d]);
            hi[d] = std::max(hi[d], nodes[3 * (size_t)i + d]);
        }
    std::vector<uint64_t> code(E);
    for (int e = 0; e < E; e++) {
        uint64_t c = 0;
        for (int d = 0; d < 3; d++) {
            double s = 0.0;
            for (int k = 0; k < nen; k++) s += nodes[3 * (size_t)el[(size_t)e * nen + k] + d];
            s /= nen;
            double span = hi[d] - lo[d];
            double f = span > 0 ? (s - lo[d]) / span : 0.0;
            uint64_t q = (uint64_t)std::min(2097151.0, std::max(0.0, f * 2097151.0));
            c |= spread3(q) << d;
        }
        code[e] = c;
    }
    // (code, element) pairs sorted directly; equal codes keep element order
    std::vector<std::pair<uint64_t, int>> ce(E);
    for (int e = 0; e < E; e++) ce[e] = {code[e], e};
    std::sort(ce.begin(), ce.end());
    std::vector<int> order(E);
    for (int t = 0; t < E; t++) order[t] = ce[t].second;

    p.G = (E + kGroup - 1) / kGroup;
    p.grp_elem.assign((size_t)p.G * kGroup, -1);
    for (int t = 0; t < E; t++) p.grp_elem[t] = order[t];

    // Footprints: (node, slot) pairs of each group sorted by node, in one
    // flat array (group g at [g * kGroup * nen, ...)).
    const size_t per = (size_t)kGroup * nen;
    std::vector<std::pair<int, int>> fpa((size_t)p.G * per);
    std::vector<int> fpn(p.G, 0);
    std::vector<int> ngroups(N, 0), lastg(N, -1);
    {
        // each group's (node, slot) pairs sorted, groups split over host threads
        const int nt = std::max(1, std::min(8, (p.G + 31) / 32));
        auto work = [&](int t0) {
            for (int g = t0; g < p.G; g += nt) {
                std::pair<int, int> *f = fpa.data() + (size_t)g * per;
                int n = 0;
                for (int j = 0; j < kGroup; j++) {
                    int e = p.grp_elem[(size_t)g * kGroup + j];
                    if (e < 0) continue;
                    for (int k = 0; k < nen; k++) f[n++] = {el[(size_t)e * nen + k], j * nen + k};
                }
                std::sort(f, f + n);
                fpn[g] = n;
            }
        };
        std::vector<std::thread> th;
        for (int t = 1; t < nt; t++) th.emplace_back(work, t);
        work(0);
        for (auto &t : th) t.join();
    }
    for (int g = 0; g < p.G; g++) {
        const std::pair<int, int> *f = fpa.data() + (size_t)g * per;
        const int n = fpn[g];
        for (int t = 0; t < n; t++) {
            int v = f[t].first;
            if (lastg[v] != g) {
                lastg[v] = g;
                ngroups[v]++;
            }
        }
    }
    // a node in more than one footprint gets one partial slot per group
    // (numbered in group order); fix_* list them per node in node order
    p.fix_ptr.assign(1, 0);
    p.fix_col.clear();
    std::vector<int> fix_at(N, -1);
    for (int v = 0; v < N; v++) {
        if (ngroups[v] == 1) continue;
        fix_at[v] = p.fix_ptr.back();
        p.fix_col.push_back(v);
        p.fix_ptr.push_back(p.fix_ptr.back() + ngroups[v]);
    }
    p.fix_slot.assign(p.fix_ptr.back(), 0);
    p.fp_ptr.assign(1, 0);
    p.fp_dest.clear();
    p.fp_dest.reserve((size_t)E * nen);
    p.fp_sl_ptr.assign(1, 0);
    p.fp_sl_ptr.reserve((size_t)E * nen + 1);
    p.fp_sl.clear();
    p.fp_sl.reserve((size_t)E * nen);
    p.n_slots = 0;
    p.max_fp = 0;
    for (int g = 0; g < p.G; g++) {
        const std::pair<int, int> *f = fpa.data() + (size_t)g * per;
        const int n = fpn[g];
        int nfp = 0;
        for (int t = 0; t < n;) {
            int v = f[t].first;
            int u = t;
            while (u < n && f[u].first == v) p.fp_sl.push_back((uint16_t)f[u++].second);
            if (ngroups[v] == 1) p.fp_dest.push_back(v);
            else {
                p.fix_slot[fix_at[v]++] = p.n_slots;
                p.fp_dest.push_back(-(p.n_slots + 1));
                p.n_slots++;
            }
            p.fp_sl_ptr.push_back((int)p.fp_sl.size());
            nfp++;
            t = u;
        }
        p.max_fp = std::max(p.max_fp, nfp);
        p.fp_ptr.push_back((int)p.fp_dest.size());
    }
    t_normals.join();
    t_side.join();
    return kOk;
}

std::vector<int> plan_coords_find(const HostPlan &p, double x, double y, double z)
{
    const double key[3] = {x, y, z};
    auto less = [&](const double *u, const double *v) {
        if (u[0] != v[0]) return u[0] < v[0];
        if (u[1] != v[1]) return u[1] < v[1];
        return u[2] < v[2];
    };
    auto lo = std::lower_bound(p.coord_order.begin(), p.coord_order.end(), 0,
                               [&](int a, int) { return less(&p.nodes[3 * (size_t)a], key); });
    std::vector<int> out;
    for (auto it = lo; it != p.coord_order.end(); ++it) {
        const double *u = &p.nodes[3 * (size_t)*it];
        if (u[0] == x && u[1] == y && u[2] == z) out.push_back(*it);
        else break;
    }
    std::sort(out.begin(), out.end());
    return out;
}

cudaStream_t &alloc_stream()
{
    static thread_local cudaStream_t s = nullptr;
    return s;
}

namespace {
std::mutex g_dev_mu;  // guards the per-device caches below
std::map<int, int> g_nsm;
std::map<std::pair<int, const void *>, int> g_smem;
std::set<int> g_pool_done;
}  // namespace

int alloc_pool_setup()
{
    int dev = 0;
    DSC_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_dev_mu);
    if (g_pool_done.count(dev)) return kOk;
    cudaMemPool_t pool;
    DSC_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
    uint64_t keep = ~(uint64_t)0;
    DSC_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    g_pool_done.insert(dev);
    return kOk;
}

int current_sm_count(int *nsm)
{
    int dev = 0;
    DSC_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_dev_mu);
    auto it = g_nsm.find(dev);
    if (it == g_nsm.end()) {
        int n = 0;
        DSC_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
        it = g_nsm.emplace(dev, n).first;
    }
    *nsm = it->second;
    return kOk;
}

int raise_smem_limit(const void *kern, int bytes)
{
    int dev = 0;
    DSC_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_dev_mu);
    int &cur = g_smem[{dev, kern}];
    if (cur < bytes) {
        DSC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        cur = bytes;
    }
    return kOk;
}

cudaEvent_t Timer::take()
{
    if (!pool.empty()) {
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void Timer::begin(int id, cudaStream_t st)
{
    cudaEvent_t a = take();
    cudaEventRecord(a, st);
    open.emplace_back(id, a);
}

void Timer::end(cudaStream_t st)
{
    if (open.empty()) return;
    cudaEvent_t b = take();
    cudaEventRecord(b, st);
    recs.push_back({open.back().first, open.back().second, b});
    open.pop_back();
}

int Timer::collect(double *ms, int *count, double *wk)
{
    for (int k = 0; k < kTCount; k++) {
        ms[k] = 0.0;
        count[k] = 0;
        wk[k] = work[k];
        work[k] = 0.0;
    }
    for (auto &r : recs) {
        DSC_CUDA(cudaEventSynchronize(r.b));
        float t = 0.0f;
        DSC_CUDA(cudaEventElapsedTime(&t, r.a, r.b));
        if (r.id >= 0 && r.id < kTCount) {
            ms[r.id] += t;
            count[r.id] += 1;
        }
        pool.push_back(r.a);
        pool.push_back(r.b);
    }
    recs.clear();
    return kOk;
}

Timer::~Timer()
{
    for (auto &o : open) pool.push_back(o.second);
    for (auto &r : recs) {
        pool.push_back(r.a);
        pool.push_back(r.b);
    }
    for (auto e : pool) cudaEventDestroy(e);
}

int DeviceMesh::upload_rows(const HostPlan &p, cudaStream_t st)
{
    DSC_TRY(row_kind.upload(p.row_kind, st));
    DSC_TRY(row_fac.upload(p.row_fac, st));
    DSC_CUDA(cudaStreamSynchronize(st));
    return kOk;
}

int DeviceMesh::upload(const HostPlan &p, cudaStream_t st)
{
    nen = p.nen;
    N = p.N;
    E = p.E;
    G = p.G;
    n_slots = p.n_slots;
    n_fix = (int)p.fix_col.size();
    std::vector<double> xs(N), ys(N), zs(N);
    for (int i = 0; i < N; i++) {
        xs[i] = p.nodes[3 * (size_t)i];
        ys[i] = p.nodes[3 * (size_t)i + 1];
        zs[i] = p.nodes[3 * (size_t)i + 2];
    }
    DSC_TRY(x.upload(xs, st));
    DSC_TRY(y.upload(ys, st));
    DSC_TRY(z.upload(zs, st));
    DSC_TRY(elems.upload(p.elems, st));
    DSC_TRY(upload_rows(p, st));
    DSC_TRY(normals.upload(p.normals, st));
    DSC_TRY(grp_elem.upload(p.grp_elem, st));
    DSC_TRY(fp_ptr.upload(p.fp_ptr, st));
    DSC_TRY(fp_dest.upload(p.fp_dest, st));
    DSC_TRY(fp_sl_ptr.upload(p.fp_sl_ptr, st));
    DSC_TRY(fp_sl.upload(p.fp_sl, st));
    DSC_TRY(fix_ptr.upload(p.fix_ptr, st));
    DSC_TRY(fix_slot.upload(p.fix_slot.empty() ? std::vector<int>{0} : p.fix_slot, st));
    DSC_TRY(fix_col.upload(p.fix_col.empty() ? std::vector<int>{0} : p.fix_col, st));
    DSC_TRY(ne_ptr.upload(p.ne_ptr, st));
    ne_total = (int)p.ne_elem.size();
    DSC_TRY(ne_elem.upload(p.ne_elem, st));
    DSC_TRY(ne_pos.upload(p.ne_pos, st));
    DSC_TRY(qp.alloc((size_t)E * kTriPts * 4));
    // host vectors go out of scope: wait for the copies
    DSC_CUDA(cudaStreamSynchronize(st));
    return kOk;
}

}  // namespace dsc
