// dsc_blas.cuh -- small deterministic vector kernels shared by the solvers.
#pragma once

#include "dsc_common.cuh"

namespace dsc {

// Fixed grid so that every reduction adds the same partials in the same
// order on every run and every device.
constexpr int kRedBlocks = 256;
constexpr int kRedThreads = 256;

// Workspace of one reduction: kRedBlocks partials and a completion counter.
struct RedWork {
    double *partials;  // kRedBlocks
    unsigned *counter; // 1, zero between uses
};

__device__ __forceinline__ double block_sum(double v, double *sh)
{
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
        r = warp_sum(r);
    }
    __syncthreads();
    return r;  // valid in warp 0
}

// The last block to finish adds the partials (in block order) and writes
// *out; the counter is reset for the next reduction.
__device__ __forceinline__ void finish_reduction(double v, RedWork rw, double *out, double *sh)
{
    double b = block_sum(v, sh);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        rw.partials[blockIdx.x] = b;
        __threadfence();
        unsigned done = atomicAdd(rw.counter, 1u);
        last = done == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x < 32) {
        __threadfence();
        double s = 0.0;
        for (int t = threadIdx.x; t < (int)gridDim.x; t += 32) s += ((volatile double *)rw.partials)[t];
        s = warp_sum(s);
        if (threadIdx.x == 0) {
            *out = s;
            *rw.counter = 0;
        }
    }
}

// part[s][0/1][i] = sum over the column split s of K[c][i] * x{re,im}[c];
// K column-major; thread per row, x chunks staged in shared memory.
template <typename T>
__global__ void __launch_bounds__(256) k_gemv_K2(const T *__restrict__ K, size_t ld, int N,
                                                 const double *__restrict__ xr,
                                                 const double *__restrict__ xi, int cols,
                                                 double *__restrict__ part, const int *skip = nullptr)
{
    if (skip && *skip) return;
    __shared__ double sxr[256], sxi[256];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int s = blockIdx.y;
    const int c0 = s * cols, c1 = min(N, c0 + cols);
    double ar = 0.0, ai = 0.0;
    for (int cb = c0; cb < c1; cb += 256) {
        __syncthreads();
        if (cb + (int)threadIdx.x < c1) {
            sxr[threadIdx.x] = xr[cb + threadIdx.x];
            sxi[threadIdx.x] = xi[cb + threadIdx.x];
        }
        __syncthreads();
        const int cn = min(256, c1 - cb);
        if (i < N) {
            const T *kp = K + (size_t)cb * ld + i;
#pragma unroll 8
            for (int c = 0; c < cn; c++) {
                double k = (double)kp[(size_t)c * ld];
                ar += k * sxr[c];
                ai += k * sxi[c];
            }
        }
    }
    if (i < N) {
        part[((size_t)s * 2) * N + i] = ar;
        part[((size_t)s * 2 + 1) * N + i] = ai;
    }
}

}  // namespace dsc
