// dsc_field_tc.h -- far-field part of the batched field on the tensor cores
// (not exported).
#pragma once

#include <cuda_fp16.h>

#include "dsc_internal.h"

namespace dsc {

struct FieldTcWork {
    DevBuf<__half> Ch, Cl;  // the charges' fp16 pairs, 64 rows of 8 slots per element
    DevBuf<float4> q8;      // the quadrature points' offsets, 8 slots per element
    DevBuf<float> csc, gsc;
    DevBuf<int> emax;
};

// part[s][f][p][3] (s < *nsplit_out <= nsplit_max) = the far pairs' field
// sums (without the 1/(4 pi eps0) factor) at the P points (phl: hi, lo
// coordinates) from the charges cT (FP32, [f / 32][q][f % 32], rows of E7p)
// of F <= 64 systems, for the pairs outside the near radius of ecent
// (centroid hi, lo, squared near radius per element; qoff the quadrature
// points relative to their centroid, as the FP32 pass takes them).
int field_far_tc(const float *phl, int P, const float *ecent, const float *qoff, int E, const float *cT, int E7p,
                 int F, FieldTcWork &w, float *part, int nsplit_max, int *d_err, cudaStream_t st, int *nsplit_out);

}  // namespace dsc
