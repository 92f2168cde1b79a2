// dsc_field.h -- point evaluation and force inside libdepsolver_cuda (not exported).
#pragma once

#include <vector>

#include "dsc_internal.h"

namespace dsc {

// Nodes whose coordinates equal (x, y, z) exactly.
std::vector<int> plan_coords_find(const HostPlan &plan, double x, double y, double z);

// Evaluation points on the device with, for each point, the mesh nodes it
// coincides with and its singular (point, element) tuples.
struct PointSet {
    int P = 0;
    DevBuf<double> px, py, pz;
    DevBuf<int4> coinc;
    DevBuf<int> sp_ptr;
    DevBuf<int4> sp;
    std::vector<int> sp_ptr_h;  // host copies of the singular tuples
    std::vector<int4> sp_h;
    // workspace of eval_points (charge-weighted points, chunk partials,
    // singular parts), kept between calls
    DevBuf<double> cq, part, sing;
    // node_ids (may be null): point p is mesh node node_ids[p] (its
    // coincident nodes then come from one pass over the coordinate order
    // instead of a search per point)
    int build(const HostPlan &plan, int P, const double *pts, const int *node_ids = nullptr);
};

// Few points at a time (the reference's post-processing evaluates one point
// per call): the quadrature points' charges stay on the device while the
// solution does not change (point_charges), and each call moves its points,
// coincident nodes and singular tuples up in one copy and its results down
// in one, through a pinned staging buffer.
constexpr int kFewPoints = 64;
struct FewPointWork {
    DevBuf<unsigned char> pack;
    DevBuf<double> part, sing, out;
    DevBuf<unsigned> ticket;  // k_point_few's count of finished blocks (zero between launches)
    unsigned char *host = nullptr;  // pinned
    size_t host_bytes = 0;
    FewPointWork() = default;
    FewPointWork(const FewPointWork &) = delete;
    FewPointWork &operator=(const FewPointWork &) = delete;
    ~FewPointWork();
};
// cq (E x 7 x 5: the point and both charges of every quadrature point).
int point_charges(const DeviceMesh &m, const double *dsigma, DevBuf<double> &cq, cudaStream_t st);
// Field (field = 1: P x 6) or potential (P x 2) at P <= kFewPoints points,
// into host memory, with cq from point_charges for dsigma.
int eval_few_points(const DeviceMesh &m, const HostPlan &plan, const double *cq, const double *dsigma, int P,
                    const double *pts, int field, double *out, FewPointWork &w, cudaStream_t st);

// field = 1: dout = P x 6 (Re Ex, Im Ex, Re Ey, Im Ey, Re Ez, Im Ez);
// field = 0: dout = P x 2 (Re, Im potential).  dsigma: device, 2N.
// sync = false leaves the work queued on st.
int eval_points(const DeviceMesh &m, PointSet &ps, const double *dsigma, int field, double *dout,
                cudaStream_t st, bool sync = true);

// What the force step needs, built once per scene: the type-6 nodes as
// evaluation points and the elements whose first node has type 6.
struct ForcePlan {
    int P = 0, npel = 0;
    PointSet ps;
    DevBuf<int> ids, pel;
    // the field's singular tuples (ps.sp) as tuples of the assembly's
    // singular pass (node, element: the plan's ne_ptr numbering), whose
    // gradient integrals it leaves for the rows flagged in row_grad
    DevBuf<int> tmap, row_grad;
    std::vector<int> pel_host;
    DevBuf<double> Ept, Enode, Fce, Xce;
    // particles: the connected sets of particle elements (elements sharing
    // a node belong to one particle), numbered by their lowest node; the
    // particle of each force point (ids order) and of each particle element
    int npart = 0;
    DevBuf<int> ids_part, pel_part;
    int build(const HostPlan &plan, const unsigned *bctype, cudaStream_t st);
};

// Derivatives of the field at points (the reference's intDE_* tensors
// summed over the mesh, src/forceIntegrals.c:61-619): for every multi-index
// a with 1 <= |a| <= kDerivOrder, E_a = -d^a phi at the point with
// phi = (1 / 4 pi eps0) sum over the elements of int Re(sigma) / r (so
// E_(1,0,0) = Re Ex, E_(2,0,0) = dEx/dx, E_(1,1,0) = dEx/dy, ...), from the
// 7-point rule of every element (the points are away from the surface).
// Entries in the order of deriv_index (index 0, the potential's order 0, is
// left at zero).
constexpr int kDerivOrder = 4;
constexpr int kDerivCount = (kDerivOrder + 1) * (kDerivOrder + 2) * (kDerivOrder + 3) / 6;
// Index of the multi-index (p, q, r), p + q + r = n <= kDerivOrder, in the
// flat derivative arrays: orders in turn, within an order p descending,
// then q descending.
__host__ __device__ constexpr int deriv_index(int p, int q, int r)
{
    const int n = p + q + r;
    const int start = n * (n + 1) * (n + 2) / 6;
    // entries of order n before (p, q): those with a larger p, then larger q
    int before = 0;
    for (int pp = n; pp > p; pp--) before += n - pp + 1;
    return start + before + (n - p - q);
}

struct DerivWork {
    DevBuf<double> cq, part, E;
};
int point_derivatives(const DeviceMesh &m, const double *dsigma, int npts, const double *dpts, DerivWork &w,
                      double *E_host, cudaStream_t st);

// Values per particle and system of the per-particle Maxwell-stress results.
constexpr int kPartVals = 12;
// out[(f * npart + p) * kPartVals + ...] for the nsys systems whose element
// forces are Fce + f * fstride (npel x 3 each; Xce npel x 3 shared):
//   [0..2] the particle's force (sum of its elements' Fce), [3..5] its
//   centre (mean of its force points), [6..8] sum of |Fce| per component,
//   [9..11] torque about the centre, sum over its elements of
//   (Xce - centre) x Fce.
int mst_particles(const ForcePlan &fp, const double *X, const double *Y, const double *Z, const double *Fce,
                  size_t fstride, const double *Xce, int nsys, double *out, cudaStream_t st);
// Xce (npel x 3) = X(1/4, 1/4) of each particle element, where the reference
// reports an element's force (src/force.c:486-487,531-541).
int mst_centres(const DeviceMesh &m, const ForcePlan &fp, double *Xce, cudaStream_t st);

// Force for one nodal solution dsigma (device, 2N); d_tot (device, 9):
// Fcm[3], Xcm[3], sum over elements of |Fce| per component[3].  Fce/Xce
// of the particle elements stay in fp.Fce / fp.Xce (npel x 3).
int force_mst_dev(const DeviceMesh &m, ForcePlan &fp, const double *dsigma, double eps,
                  double *d_tot, cudaStream_t st, Timer *tm = nullptr);

// Maxwell-stress force on the type-6 surface; Fce/Xce (host, E x 3, may be
// null) receive the rows of particle elements only.
int force_mst(const DeviceMesh &m, const HostPlan &plan, const unsigned *bctype,
              const double *dsigma, double eps, double *Fce, double *Xce, double *Fcm,
              double *Xcm, cudaStream_t st);

}  // namespace dsc
