// dsc_quad8.h -- the quad8 element family on the FP64 path (dsc_quad8.cu).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "dsc_internal.h"

namespace dsc {

// A quad8 mesh on the device: coordinates (SoA), 0-based connectivity
// (E x 8), averaged node normals, node -> (element, position) in element
// order, and on the host the same plus the nodes sorted by coordinates.
struct Q8Mesh {
    int N = 0, E = 0;
    std::vector<double> hnodes, hnormals;
    std::vector<int> helems, ne_ptr, ne_elem, ne_pos, order;
    DevBuf<double> x, y, z, normals;
    DevBuf<int> elems, d_ne_ptr, d_ne_elem, d_ne_pos;
    int build(int N, int E, const double *nodes, const int *elems0, cudaStream_t st);
};

// Averaged unit node normals (normals: N x 3): per node the sum over the
// elements containing it of the unit normal at its parent point.
void q8_node_normals(int N, int E, const double *nodes, const int *elems0, double *normals);

// K (column-major FP64, K[c * ld + i], N x N) of the mesh: C int G N_c on
// conductor rows (bctype 1), -int dG/dn_i N_c on interface rows (0, 6).
int q8_assemble_K(const Q8Mesh &m, const unsigned *bctype, double *K, size_t ld, cudaStream_t st);

// Field (field = 1: P x 6, Re/Im of x, y, z) or potential (P x 2) at P
// host points into device memory dout, from the device solution dsigma (2N).
int q8_points(const Q8Mesh &m, const double *dsigma, int P, const double *pts_host, int field, double *dout,
              cudaStream_t st);

// Maxwell-stress force on the type-6 elements (Fce, Xce E x 3 on the host,
// may be null; totals Fcm, Xcm).
int q8_force_mst(const Q8Mesh &m, const unsigned *bctype, const double *dsigma, double eps, double *Fce_host,
                 double *Xce_host, double *Fcm, double *Xcm, cudaStream_t st);

}  // namespace dsc
