// Tape of recorded substeps for the hand-written adjoint (internal).
//
// Slot-major device arrays: slot k's copy of a sorted per-particle array starts
// at k * cap (cap = the context's padded fluid slots; boundary arrays use bcap).
// The Jacobi iterates of a slot are [kind][iteration][cap], kind 0 = divergence
// solve, 1 = density solve.  The neighbour lists keep the context's blocked
// layout (nbr_index with stride cap).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "common.cuh"

namespace tsph {

struct TapeMeta {
    int32_t n, nb, f_in, kd, kp, status;
    float dt, mu;
};

struct TapeArrays {
    int *perm;
    float4 *pos, *mpsi, *a1, *vmid, *u, *bpos, *bvel;
    float *a2, *rho0, *kap;
    unsigned int *cnt;
    int *nbr;
    TapeMeta *meta;
    int *dslot;  // slot being recorded (set before a recorded step, read by its kernels)
    // with surface tension on: the normals, phase 0's volume fraction and the
    // fluid grid's cell starts (nstart per slot) of each recorded substep
    float4 *nrm;
    float *vf0;
    int *start;
    int64_t nstart;
    int64_t cap, bcap;
    int slots, max_iters, nbr_max;
};

}  // namespace tsph

struct tsph_tape {
    tsph_ctx *ctx;
    tsph::TapeArrays a;
    tsph::TapeMeta *host_meta;  // pinned copy of every slot's metadata
    int host_valid;             // host_meta matches the device
    // reverse-pass scratch in sorted order (cap entries)
    float4 *lam_u, *lam_u2, *lam_x, *lam_a1;
    float4 *lam_n;  // adjoint of the surface normals (surface tension on)
    float *lam_s, *lam_psi, *lam_alpha;
    double *partials;
    unsigned int *ticket;
    std::vector<void *> allocs;
};
