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
    int build(const HostPlan &plan, int P, const double *pts);
};

// field = 1: dout = P x 6 (Re Ex, Im Ex, Re Ey, Im Ey, Re Ez, Im Ez);
// field = 0: dout = P x 2 (Re, Im potential).  dsigma: device, 2N.
int eval_points(const DeviceMesh &m, const PointSet &ps, const double *dsigma, int field,
                double *dout, cudaStream_t st);

// Maxwell-stress force on the type-6 surface; Fce/Xce (host, E x 3, may be
// null) receive the rows of particle elements only.
int force_mst(const DeviceMesh &m, const HostPlan &plan, const unsigned *bctype,
              const double *dsigma, double eps, double *Fce, double *Xce, double *Fcm,
              double *Xcm, cudaStream_t st);

}  // namespace dsc
