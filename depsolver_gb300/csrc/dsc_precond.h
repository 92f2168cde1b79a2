// dsc_precond.h -- conductor-block right preconditioner of the mixed sweep
// (not exported).
//
// Conductor rows (boundary type 1: a fixed potential) carry the first-kind
// single-layer equations of the electrodes; their part of every system's
// matrix is the same at every frequency (s = 1, d = 0) and, after the
// Jacobi scaling, is the real block D_E^-1 K_EE.  That block is what makes
// GMRES slow (its condition number grows with the mesh), while the
// interface rows form a second-kind equation.  The preconditioner is
// P^-1 = blockdiag(X_1, ..., X_m, I): X_b the inverse of the scaled block
// of one connected electrode (Gauss-Jordan in FP32 on the device, once per
// assembly of K), I on the interface rows.  It is applied on the right:
// GMRES runs on M P^-1 and the correction is P^-1 (V y), so the solution
// stays that of M; the inverse only needs to be good enough to cluster the
// spectrum (an fp16-accurate one already does).
#pragma once

#include <cuda_fp16.h>

#include <vector>

#include "dsc_internal.h"

namespace dsc {

struct Session;

struct Precond {
    int nb = 0;                       // blocks (connected electrodes)
    std::vector<int> n, ldx, nbk;     // rows, padded size (multiple of 128), 128-blocks
    std::vector<size_t> xoff;         // block b's ldx^2 matrix in X, Xh, Xl
    std::vector<size_t> noff;         // block b's rows in `nodes`, `rs`
    std::vector<size_t> toff;         // block b's ldx x 128 Gauss-Jordan operands
    std::vector<int> S;               // split count of block b's product
    std::vector<size_t> yoff;         // block b's partial tiles in Y
    std::vector<size_t> boff;         // block b's operand pairs in Bh, Bl, G
    int F = 0;                        // systems the apply workspace is laid out for
    DevBuf<int> nodes;                // rows of each block, ascending
    DevBuf<int> rblk, rpos;           // per row: its block (-1: none) and position
    DevBuf<float> X;                  // scaled blocks (column-major), inverted in place
    DevBuf<float> Xt;                 // the inverses transposed (row-major)
    DevBuf<__half> Xh, Xl;            // the inverses as row-scaled fp16 pairs
    DevBuf<float> rs;                 // their row factors
    DevBuf<float> tP;                 // Gauss-Jordan pivot-block inverses
    DevBuf<__half> gAh, gAl, gBh, gBl;  // Gauss-Jordan update operands (fp16 pairs)
    DevBuf<float> gra, grb;           // their row factors
    DevBuf<int> err;                  // set when a wait of the update kernel gives up
    DevBuf<__half> Bh, Bl;            // gathered operands (2F x ldx per block)
    DevBuf<double> G;                 // gathered corrections (FP64)
    DevBuf<float> csc;                // column factors of gathered corrections
    DevBuf<float> Y;                  // split partials of the block products
    DevBuf<long long> yinfo;          // per block: Y offset, split stride, S (device copy)
    DevBuf<unsigned> zbound;          // FP32 bits of a bound on |P^-1 v| for |v| <= 1
    DevBuf<float> cz;                 // the K product's column factors of z's pair
    std::vector<int> nodes_h;         // host copy of `nodes`
    bool ready = false;               // the inverses match the current K
    // the inverses were copied from a PrecondShare (blocks of a part of the
    // scene that every assembly of this session leaves unchanged): a new
    // assembly of K keeps them
    bool adopted = false;
};

// The inverses of one session's blocks, kept apart from any session so that
// sessions of other scenes with the same conductor blocks (the fixed
// electrodes of a position sweep: the same nodes, elements and rows) can
// take them instead of inverting again.  Device memory from cudaMalloc,
// tied to no stream.
struct PrecondShare {
    int nb = 0;
    std::vector<int> n, nodes_h;
    size_t xtot = 0, rtot = 0;
    DevBuf<__half> Xh, Xl;
    DevBuf<float> rs;
    DevBuf<unsigned> zbound;
};

// Blocks from the mesh and the conductor rows (once per session; no blocks
// when the scene has no conductor rows).
int precond_plan(Session &s);
// The inverses for the current K64 (after each assembly), on main and aux
// (default: the session's stream and side stream); waits for them.
int precond_build(Session &s, cudaStream_t main = nullptr, cudaStream_t aux = nullptr);
// Copies a built session's inverses into sh (waits for the copies).
int precond_export(Session &s, PrecondShare &sh);
// Takes sh's inverses for s when s has the same blocks (same rows in the
// same order); returns kErrArg, touching nothing, when it has not.
int precond_adopt(Session &s, const PrecondShare &sh);
// Workspace of the apply calls for F systems.
int precond_reserve(Session &s, int F);
// z = P^-1 v for the 2F columns of the double-FP32 block V (Re, Im of each
// system; |v| <= 1: unit vectors), written as the fp16 pair (Zh, Zl; column
// c at c * ld, rows < N) of z scaled by a fixed power of two; *cz receives
// the product's column factors.
int precond_apply_v(Session &s, const float2 *V, int F, __half *Zh, __half *Zl, const float *cscK, int *d_err,
                    const float **cz);
// D (FP64, 2F columns) = P^-1 D in place.
int precond_apply_d(Session &s, double *D, int F, int *d_err);

}  // namespace dsc
