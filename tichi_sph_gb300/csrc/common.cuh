// Internal definitions shared by the CUDA translation units of the SPH hot path.
//
// A context steps one scene (the reference's drop-in case) or a batch of
// independent scenes in the same launches.  Data layout (all in HBM, owned by
// tsph_ctx):
//   * scene s owns the cell codes [cbase_s, cbase_s + node_num_s) of one global
//     code space (segmented grids); inside a scene a code is the reference's
//     linear x + nx*y + nx*ny*z (sph_config.py:210-214).  Two grids (fluid,
//     boundary): count[total_nodes] and the exclusive scan start[total_nodes+1];
//   * per set, a permutation perm[sorted slot] = particle id.  Scene s's sorted
//     slots are [slot_s, slot_s + slots_s), a multiple of kChunk, so no block of
//     256 threads ever straddles two scenes: first its in-grid particles by cell
//     code, ties by particle id, then its particles without a valid cell (they
//     still run their own sums, sph.py:52, but are never found as neighbours,
//     sph_obj.py:305,319), then padding slots that no kernel processes;
//   * sorted SoA copies of the per-particle state as float4 (x, y, z, X) etc., so
//     a neighbour cell row (three x-adjacent cells) is one contiguous, coalesced
//     range of 16-byte loads;
//   * per-scene constants, persistent scalars and per-step scalars.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "../../include/tichi_sph.h"

namespace tsph {

constexpr int kBlock = 256;     // threads per block of the particle sweeps
constexpr int kChunk = 256;     // a scene's sorted slots are padded to multiples of this
constexpr int kMaxP = TSPH_MAX_PHASES;

// Constants of one scene (the reference's Config, sph_config.py:83-235, in f32)
// and its particle segments.
struct SceneConst {
    float lb[3];
    float h, h2, inv_h, sig, sig_h, c_coh;   // c_coh = 32 / (pi h^3)
    long long node_num, nx, nxny, cbase;
    float g[3];
    float mu, gamma, fbm_c, fbm_D;
    float rho_phase[kMaxP];
    float part_size, cfl;
    int cs, iter_min, iter_max, fbm_max_passes, wc_gamma;
    float div_tol, comp_tol;
    // 1 when a template row cannot alias another (nx > 2r, and ny > 2r in 3D):
    // only then may candidates be skipped by their cell's geometry
    int row_trim;
    // caller order [f_user, f_user + f_n); sorted slots [f_slot, f_slot + f_slots)
    long long f_user, f_n, f_slot, f_slots;
    long long b_user, b_n, b_slot, b_slots;
    // blocks [f_ublk0, f_ublk0 + f_ublks) of kBlock caller-order fluid particles (at
    // least one, so every scene has a block that finishes its step)
    long long f_ublk0, f_ublks;
};

// Scalars of a scene that persist across steps.
struct ScenePersist {
    double time_count;
    double compression;  // carried into the next divergence-loop test (main.py:201)
    double max_dens_compression;
    long long total_div_iter, total_incom_iter, total_fbm_passes;
    float dt;
    int32_t steps;
    // 1 once BoundBuf::bb holds the boundary-boundary sums of the scene's
    // boundary as gathered (bb_n particles)
    int32_t bb_valid, pad1;
    long long bb_n;
};

// Scalars of a scene for one step; zeroed at the start of every step.
struct SceneStep {
    unsigned int vmax_bits;     // max |v| over the scene's fluid (float bits)
    int32_t cur;                // which v_adv buffer is current
    int32_t iter, cond;         // running solve: iteration counter, loop condition
    int32_t div_iter, incom_iter;
    int32_t fbm_pass, general_flag, fbm_passes, fbm_cond, gflag_out;
    int32_t status;
    int32_t f_tail, b_tail;     // particles without a valid cell
    int32_t f_in, b_in;         // particles in the grid
    // 1 while psi_adv, kappa and psi_sum of the divergence solve's first
    // iteration come from the density sweep (its psi sweep then does nothing)
    // b_dirty: 1 when this step's gather found a boundary position or mass that
    // differs bitwise from the previous gather's
    int32_t psi_ready, b_dirty;
    long long f_shift, b_shift; // sorted slot of global scan position p is p + shift
    unsigned int ticket[6];     // block tickets of this scene (psi, vel, fbm, update)
    double psi_sum, kinetic_energy, potential_energy;
};

// Grid-wide scalars of one step; zeroed at the start of every step.
struct DevGlobal {
    unsigned int ticket[8];
    int32_t cond_any, fbm_any, status;
    int32_t pad;
};

enum GlobalTicket { kGtCfl = 0, kGtVel = 1, kGtFbm = 2, kGtUpdate = 3, kGtScanF = 4, kGtScanB = 5, kGtScanDone = 6 };
enum SceneTicket { kStPsi = 0, kStVel = 1, kStFbm = 2, kStUpdate = 3 };

// Launch-time constants of one context (passed by value: the constant bank).
struct KConst {
    int dim, P, vfsph, R, nbr_max, n_scenes;
    long long total_nodes;
    long long f_slots, b_slots;           // padded slots over all scenes
    const SceneConst *sc;
    ScenePersist *sp;
    SceneStep *ss;
    DevGlobal *dg;
    const int *f_chunk_scene;             // scene of each kChunk-slot chunk (fluid / boundary)
    const int *b_chunk_scene;
    const int *f_user_scene;              // scene of each caller-order particle
    const int *b_user_scene;
    const int *f_ublock_scene;            // scene of each caller-order block of kBlock
    long long f_ublocks;
    SceneConst s0;                        // scene 0 by value (the one-scene kernels read it here)
};

// Scene lookups of a kernel instance.  A batched instance (M) finds its block's
// scene in the chunk table and reads the scene's constants from the scene table;
// a one-scene instance reads them from the launch's constant bank (no registers
// held across the neighbour loops) and its grid scan positions are its sorted
// slots (shift 0).
template <bool M>
__device__ __forceinline__ int f_block_scene(const KConst &k, int64_t first_slot) {
    return M ? k.f_chunk_scene[first_slot / kChunk] : 0;
}
template <bool M>
__device__ __forceinline__ int b_block_scene(const KConst &k, int64_t first_slot) {
    return M ? k.b_chunk_scene[first_slot / kChunk] : 0;
}
template <bool M>
__device__ __forceinline__ const SceneConst &scene(const KConst &k, int sc) {
    if (M) return k.sc[sc];
    return k.s0;
}
template <bool M>
__device__ __forceinline__ long long shift_of(long long v) {
    return M ? v : 0ll;
}

// The geometric constants a neighbour loop needs, in registers.
struct Geo {
    float lb[3];
    float h, h2, inv_h, sig, sig_h;
    long long node_num, nx, nxny, cbase;
    int R, row_trim;
    __device__ __forceinline__ void load(const SceneConst &c, int R_) {
        lb[0] = c.lb[0];
        lb[1] = c.lb[1];
        lb[2] = c.lb[2];
        h = c.h;
        h2 = c.h2;
        inv_h = c.inv_h;
        sig = c.sig;
        sig_h = c.sig_h;
        node_num = c.node_num;
        nx = c.nx;
        nxny = c.nxny;
        cbase = c.cbase;
        R = R_;
        row_trim = c.row_trim;
    }
};

// nbr_cnt value of a particle whose neighbours did not fit the list: its sweeps
// scan the template cells instead.
constexpr unsigned int kNbrOverflow = 0xffffffffu;
// normal.w of a particle without surface tension: a NaN bit pattern that no
// arithmetic produces (the hardware's NaN results are 0x7fffffff)
constexpr unsigned int kNoSurfTension = 0xffffffffu;
__device__ __forceinline__ bool has_surf_tension(float4 n) { return __float_as_uint(n.w) != kNoSurfTension; }

// Position of neighbour t of sorted particle s in the blocked neighbour list.
__host__ __device__ __forceinline__ int64_t nbr_index(int t, int64_t s, int64_t cap) {
    return (((int64_t)(t >> 2)) * cap + s) * 4 + (t & 3);
}

struct FluidBuf {
    int64_t cap;             // padded slots over all scenes
    int *count, *start, *slot, *perm, *inv;
    int *perm_u;             // particle ids in scatter order (each cell's ids unordered)
    float4 *pos;       // x, y, z, X (mass for DFSPH, rest_volume for VFSPH)
    float2 *mv;        // mass, rest_volume
    float4 *mpsi;      // mass, psi (sph_psi), psi0 (rest_psi), alpha
    float *psilo;      // low part of psi: psi + psilo is the density sweep's compensated sum
    float *rho0;       // rest_density
    float4 *vel;       // velocity after the divergence solve
    float4 *vadv;      // two buffers of cap: v_adv ping-pong
    float *psiadv, *kappa;   // psi_adv and psi_adv / alpha
    float4 *pk;              // (x, y, z, kappa): what the velocity sweep reads of a neighbour
    float4 *acc;       // acce_adv
    // surface normal (x, y, z); w = the particle's psi when its phase-0 volume
    // fraction exceeds 0.99 (it takes part in surface tension), else kNoSurfTension
    float4 *normal;
    float4 *dens;      // W, sph_density, sph_compression, alpha_2: read together by the write-back
    float4 *a1;        // alpha_1 (x, y, z), alpha
    float *vf, *vftmp;       // [P][cap]
    float4 *drift;           // [cap][P]: a particle's phases side by side (the pass gathers them together)
    float4 *facc;            // acce (fbm_acce)
    float *zeta;
    int *flagpass;           // 0 = unflagged, else the FBM pass that flagged it
    // Neighbours with 0 < r < h, recorded by the density sweep in candidate order:
    // first the fluid neighbours of sorted particle s, then its boundary ones, in
    // blocks of four: entry t sits at nbr[nbr_index(t, s, cap)], so block t / 4 of
    // 32 consecutive particles is one 512-byte run (one int4 per particle).
    // nbr_cnt[s] packs the two counts (fluid | boundary << 16) or is kNbrOverflow.
    int *nbr;
    unsigned int *nbr_cnt;
    float2 *wcp;             // weakly compressible block: (pressure, pressure / rho^2)
};

struct BoundBuf {
    int64_t cap;
    int *count, *start, *slot, *perm, *inv;
    int *perm_u;       // particle ids in scatter order (each cell's ids unordered)
    float4 *pos;       // x, y, z, X
    float2 *mv;        // mass, rest_volume
    float4 *vadv;      // boundary vel_adv (never advanced by the reference)
    float *kappa;      // psi_adv / alpha of the boundary particle
    float4 *pk;        // (x, y, z, kappa) of the boundary particle
    float4 *dens;      // W, sph_density, sph_compression, alpha_2
    float *alpha;
    float *wcp2;       // pressure / rho^2 of the boundary particle (weakly compressible block)
    // (W, density, compression) summed over the particle's boundary neighbours
    // alone: the boundary sums add these terms before the fluid's, so a copy
    // taken while positions and masses stay bitwise the same gives the same bits
    float4 *bb;
};

struct Scratch {
    double *partials;        // per-block FP64 partial sums
    int64_t partials_len;
    int *scan_blocks;        // block totals of the cell scans
    int64_t scan_len;
};

// ---------------------------------------------------------------------------------
// Kernel functions of the reference, sph_util.py:4-43 (q = r / h).
__device__ __forceinline__ float kw(float q) {
    float a = 6.f * (q * q * q - q * q) + 1.f;
    float b = 1.f - q;
    return q <= 0.5f ? a : (q < 1.f ? 2.f * b * b * b : 0.f);
}
__device__ __forceinline__ float kwg(float q) {
    float a = 6.f * (3.f * q * q - 2.f * q);
    float b = 1.f - q;
    return q <= 0.5f ? a : (q < 1.f ? -6.f * b * b : 0.f);
}
// r = |x| and 1 / r from r^2 with the hardware reciprocal square root (rsqrtf,
// within a few ulp): cheaper than an IEEE square root plus an IEEE division
// per pair.  r^2 = 0 gives r = 0 and 1 / r = 0.
__device__ __forceinline__ float pair_rinv(float r2, float &r) {
    const float inv = r2 > 0.f ? rsqrtf(r2) : 0.f;
    r = r2 * inv;
    return inv;
}

// The density sweeps' per-pair quotient uses __fdividef (two instructions,
// within 2 ulp) instead of an IEEE division: far inside the 1e-5 tolerance.

// pair_rinv for r^2 known to be positive (list entries).
__device__ __forceinline__ float pair_rinv_pos(float r2, float &r) {
    const float inv = rsqrtf(r2);
    r = r2 * inv;
    return inv;
}

__device__ __forceinline__ float kcoh(float q) {
    float b = 1.f - q;
    float t = b * b * b * q * q * q;
    return q <= 0.5f ? 2.f * t - 1.f / 64.f : (q < 1.f ? t : 0.f);
}

// Cell of a position inside its scene: floor((p - lb) / h) per axis with IEEE
// division (sph_util.py:65-67), and the scene-local linear code
// (sph_util.py:70-72).  `ok` is false for a non-finite position or a coordinate
// beyond +-1e12 cells.
template <int DIM>
__device__ __forceinline__ long long cell_code(float4 p, const Geo &g, bool &ok) {
    const float c[3] = {p.x, p.y, p.z};
    long long s[3] = {0, 0, 0};
    ok = true;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        float f = floorf(__fdiv_rn(c[d] - g.lb[d], g.h));
        if (!(f > -1.0e12f && f < 1.0e12f)) ok = false;
        s[d] = ok ? (long long)f : 0;
    }
    long long code = s[0] + s[1] * g.nx;
    if (DIM == 3) code += s[2] * g.nxny;
    return code;
}

// Visits every candidate the reference's template loop visits (sph.py:52-60):
// for each row offset (dy, dz) the x-adjacent codes [rc - R, rc + R] clipped to
// the scene's valid range (0, node_num) form one contiguous range of sorted
// slots.  Codes are linear, so an x offset past a row end continues into the
// next row exactly like dim_encode without bounds checks.  `shift` maps a scan
// position of the grid to a sorted slot.  Lane q of a TPP-lane group visits only
// j = beg + q, beg + q + TPP, ...
template <int DIM, int TPP = 1, class F>
__device__ __forceinline__ void visit_candidates(const int *__restrict__ start, const Geo &g, long long code,
                                                 long long shift, int q, F &&f) {
    const int R = g.R;
    const int zr = (DIM == 3) ? R : 0;
    for (int dz = -zr; dz <= zr; ++dz) {
        for (int dy = -R; dy <= R; ++dy) {
            long long rc = code + dy * g.nx + dz * g.nxny;
            long long lo = rc - R, hi = rc + R;
            if (lo < 1) lo = 1;
            if (hi > g.node_num - 1) hi = g.node_num - 1;
            if (lo > hi) continue;
            const int beg = (int)(__ldg(start + g.cbase + lo) + shift);
            const int end = (int)(__ldg(start + g.cbase + hi + 1) + shift);
            for (int j = beg + q; j < end; j += TPP) f(j);
        }
    }
}

// visit_candidates reading the scene's row geometry (nx, nx*ny, node_num,
// cbase) from the scene table at every row instead of holding it in registers.
template <int DIM, int TPP, class F>
__device__ __forceinline__ void visit_candidates_lean(const int *__restrict__ start, const SceneConst *c, int R,
                                                      long long code, long long shift, int q, F &&f) {
    const int zr = (DIM == 3) ? R : 0;
    for (int dz = -zr; dz <= zr; ++dz) {
        for (int dy = -R; dy <= R; ++dy) {
            const long long nx = *(volatile const long long *)&c->nx;
            const long long nxny = *(volatile const long long *)&c->nxny;
            const long long nn = *(volatile const long long *)&c->node_num;
            const long long cb = *(volatile const long long *)&c->cbase;
            const long long rc = code + dy * nx + dz * nxny;
            long long lo = rc - R, hi = rc + R;
            if (lo < 1) lo = 1;
            if (hi > nn - 1) hi = nn - 1;
            if (lo > hi) continue;
            const int beg = (int)(__ldg(start + cb + lo) + shift);
            const int end = (int)(__ldg(start + cb + hi + 1) + shift);
            for (int j = beg + q; j < end; j += TPP) f(j);
        }
    }
}

// visit_candidates for callers that use only candidates with r < h: template
// rows whose y/z slab is farther than h from the particle are skipped (the
// corner rows (dy, dz) = (+-1, +-1) for about a fifth of the particles each),
// and so are a kept row's end cells whose box lies farther than h.  The rest of
// a row is one contiguous range visited in order, as in visit_candidates.
//
// Exactness: a candidate within h of the particle lies at most one cell away
// on every axis, so with nx, ny > 2r it sits in the template cell of its
// geometric offset and the face distances below bound its distance; a wrapped
// or outside particle found through another template cell is farther than h
// and fails the test either way.  The face distances come from FP32 cell
// coordinates whose rounding grows with the coordinate (~1.2e-7 cells per cell
// of distance from lb, for the particle and for the candidate's own cell), so
// the margin on h^2 grows with it too.  Without row_trim (a row could alias
// another) the margin is infinite: every candidate is visited.
template <int DIM, int TPP, class F>
__device__ __forceinline__ void visit_within_any(const int *__restrict__ start, const Geo &g, float4 p,
                                                 long long code, long long shift, int q, F &&f) {
    const int R = g.R;
    const int zr = (DIM == 3) ? R : 0;
    // distance of the particle to its cell's lower / upper faces in x, y and z
    const float qx = __fdiv_rn(p.x - g.lb[0], g.h);
    const float qy = __fdiv_rn(p.y - g.lb[1], g.h), qz = DIM == 3 ? __fdiv_rn(p.z - g.lb[2], g.h) : 0.f;
    const float fx = qx - floorf(qx), fy = qy - floorf(qy), fz = qz - floorf(qz);
    const float qm = fmaxf(fabsf(qx), fmaxf(fabsf(qy), fabsf(qz))) + (float)(R + 1);
    const float skip2 = g.row_trim ? g.h2 * (1.f + 1e-5f + 2e-6f * (float)R * qm) : __int_as_float(0x7f800000);
    for (int dz = -zr; dz <= zr; ++dz) {
        const float ez = dz == 0 ? 0.f : (dz < 0 ? fz + (float)(-dz - 1) : (1.f - fz) + (float)(dz - 1)) * g.h;
        for (int dy = -R; dy <= R; ++dy) {
            const float ey = dy == 0 ? 0.f : (dy < 0 ? fy + (float)(-dy - 1) : (1.f - fy) + (float)(dy - 1)) * g.h;
            const float eyz = ey * ey + ez * ez;
            if (eyz > skip2) continue;
            long long rc = code + dy * g.nx + dz * g.nxny;
            long long lo = rc - R, hi = rc + R;
            // the row's end cells that lie farther than h (in x together with y / z)
            for (int dx = -R; dx < 0; ++dx) {
                const float ex = (fx + (float)(-dx - 1)) * g.h;
                if (eyz + ex * ex > skip2) lo = rc + dx + 1;
                else break;
            }
            for (int dx = R; dx > 0; --dx) {
                const float ex = ((1.f - fx) + (float)(dx - 1)) * g.h;
                if (eyz + ex * ex > skip2) hi = rc + dx - 1;
                else break;
            }
            if (lo < 1) lo = 1;
            if (hi > g.node_num - 1) hi = g.node_num - 1;
            if (lo > hi) continue;
            const int beg = (int)(__ldg(start + g.cbase + lo) + shift);
            const int end = (int)(__ldg(start + g.cbase + hi + 1) + shift);
            for (int j = beg + q; j < end; j += TPP) f(j);
        }
    }
}

// The scan for the template radius 1: the face distances (fy h,
// (1 - fy) h and their x and z counterparts; the general form adds an exact
// 0.f) and the end-cell squares are computed once per particle, not per row.
template <int DIM, int TPP, class F>
__device__ __forceinline__ void visit_within_r1(const int *__restrict__ start, const Geo &g, float4 p,
                                                long long code, long long shift, int q, F &&f) {
    const int zr = (DIM == 3) ? 1 : 0;
    const float qx = __fdiv_rn(p.x - g.lb[0], g.h);
    const float qy = __fdiv_rn(p.y - g.lb[1], g.h), qz = DIM == 3 ? __fdiv_rn(p.z - g.lb[2], g.h) : 0.f;
    const float fx = qx - floorf(qx), fy = qy - floorf(qy), fz = qz - floorf(qz);
    const float qm = fmaxf(fabsf(qx), fmaxf(fabsf(qy), fabsf(qz))) + 2.f;
    const float skip2 = g.row_trim ? g.h2 * (1.f + 1e-5f + 2e-6f * qm) : __int_as_float(0x7f800000);
    const float eym = fy * g.h, eyp = (1.f - fy) * g.h, ezm = fz * g.h, ezp = (1.f - fz) * g.h;
    const float exm = fx * g.h, exp_ = (1.f - fx) * g.h;
#pragma unroll 1
    for (int dz = -zr; dz <= zr; ++dz) {
        const float ez = dz == 0 ? 0.f : (dz < 0 ? ezm : ezp);
#pragma unroll 1
        for (int dy = -1; dy <= 1; ++dy) {
            const float ey = dy == 0 ? 0.f : (dy < 0 ? eym : eyp);
            const float eyz = ey * ey + ez * ez;
            if (eyz > skip2) continue;
            const long long rc = code + dy * g.nx + dz * g.nxny;
            // the row's end cells that lie farther than h (in x together with y / z)
            long long lo = (eyz + exm * exm > skip2) ? rc : rc - 1;
            long long hi = (eyz + exp_ * exp_ > skip2) ? rc : rc + 1;
            if (lo < 1) lo = 1;
            if (hi > g.node_num - 1) hi = g.node_num - 1;
            if (lo > hi) continue;
            const int beg = (int)(__ldg(start + g.cbase + lo) + shift);
            const int end = (int)(__ldg(start + g.cbase + hi + 1) + shift);
            for (int j = beg + q; j < end; j += TPP) f(j);
        }
    }
}

// The template radius r = 1 (the reference's configurations) in its own form,
// any other radius read at run time; the same candidates.
template <int DIM, int TPP = 1, class F>
__device__ __forceinline__ void visit_candidates_within(const int *__restrict__ start, const Geo &g, float4 p,
                                                        long long code, long long shift, int q, F &&f) {
    if (g.R == 1) visit_within_r1<DIM, TPP>(start, g, p, code, shift, q, f);
    else visit_within_any<DIM, TPP>(start, g, p, code, shift, q, f);
}

// ---------------------------------------------------------------------------------
// Programmatic dependent launch.  The first statement of every kernel of the
// step: wait until the kernel before it in the stream has completed and its
// writes are visible, then let the kernel after it be scheduled.  Launched
// with the programmatic attribute (TSPH_LAUNCH), a kernel's blocks are placed
// on the SMs while its predecessor's last blocks still run, and start its work
// the moment the predecessor has finished; launched plainly, both are no-ops.
__device__ __forceinline__ void pdl_entry() {
    asm volatile("griddepcontrol.wait;\n\tgriddepcontrol.launch_dependents;" ::: "memory");
}

// ---------------------------------------------------------------------------------
// Deterministic reductions in FP64 (warp shuffles, fixed trees).
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <int BS>
__device__ __forceinline__ double block_sum(double v, double *sh) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = (lane < BS / 32) ? sh[lane] : 0.0;
        r = warp_sum(r);
    }
    return r;  // valid in thread 0
}

// True (in every thread) for the block that finishes last among `total`
// arrivals on `ticket`; the caller's per-block results must already be stored.
// Fence + ticket: no thread ever waits on another block.
__device__ __forceinline__ bool last_block_done(unsigned int *ticket, unsigned int total) {
    __shared__ bool am_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int t = atomicAdd(ticket, 1u);
        am_last = (t == total - 1);
    }
    __syncthreads();
    if (am_last) __threadfence();
    return am_last;
}

// Per-block FP64 sum without a block-wide barrier at the end (warps finish at
// different times in the neighbour sweeps): each warp leaves its sum in shared
// memory, the last warp to arrive adds the block's warp sums in warp order and
// returns true with the result in `out` (lane 0).  `arrived` must be zeroed
// before any warp can arrive (a barrier at kernel start).
template <int BS>
__device__ __forceinline__ bool block_sum_last_warp(double v, double *sh, unsigned int *arrived, double &out) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned int old = 0;
    if (lane == 0) {
        sh[w] = v;
        __threadfence_block();
        old = atomicAdd(arrived, 1u);
    }
    old = __shfl_sync(0xffffffffu, old, 0);
    if (old != BS / 32 - 1) return false;
    __threadfence_block();
    double s = 0.0;
    if (lane == 0)
        for (int i = 0; i < BS / 32; ++i) s += ((volatile double *)sh)[i];
    out = s;
    return true;
}

// One-warp version of the grid ticket: true (in all its lanes) for the warp that
// arrives last among `total` arriving warps.
__device__ __forceinline__ bool last_warp_done(unsigned int *ticket, unsigned int total) {
    const int lane = threadIdx.x & 31;
    unsigned int t = 0;
    if (lane == 0) {
        __threadfence();
        t = atomicAdd(ticket, 1u);
    }
    t = __shfl_sync(0xffffffffu, t, 0);
    const bool last = (t == total - 1);
    if (last) __threadfence();
    return last;
}

// Lane layout of a sweep with TPP threads per particle: a warp serves 32 / TPP
// consecutive sorted slots; lane = q * (32 / TPP) + p handles slot p of the warp
// and every TPP-th four-entry block of its neighbour list starting at block q, so
// lanes with the same q read one contiguous 16 * 32 / TPP-byte run of the list.
template <int TPP>
struct Lanes {
    static constexpr int PPW = 32 / TPP;  // particles per warp
    int q, p;
    int64_t s;
    __device__ __forceinline__ Lanes() {
        const int lane = threadIdx.x & 31;
        q = lane / PPW;
        p = lane % PPW;
        const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
        s = warp * PPW + p;
    }
    // sum over the TPP lanes of the particle (fixed xor tree: deterministic)
    __device__ __forceinline__ float sum(float v) const {
#pragma unroll
        for (int o = PPW; o < 32; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        return v;
    }
};

// List loads that do not allocate in L1: each entry of the neighbour list is
// read once per sweep, while the neighbours' fields it points to are read by
// many particles of a block; left to allocate, the list (~37 KB per block)
// evicts them.  The .nc form is for lists written by an earlier launch; the
// other orders after the calling thread's own stores of the list.
__device__ __forceinline__ int4 ld_list_nc(const int4 *p) {
    int4 r;
    asm("ld.global.nc.L1::no_allocate.v4.s32 {%0, %1, %2, %3}, [%4];"
        : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w) : "l"(p));
    return r;
}
__device__ __forceinline__ int4 ld_list(const int4 *p) {
    int4 r;
    asm volatile("ld.global.L1::no_allocate.v4.s32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w) : "l"(p) : "memory");
    return r;
}

// Walks the blocked neighbour list of sorted particle s for lane q of a TPP-lane
// group: blocks b = q, q + TPP, ... of four entries; entries t < nfl are fluid
// neighbours (ff), nfl <= t < ntot boundary ones (fb).  The next block's int4 is
// loaded before the current block is processed, and the four callbacks of a
// block only accumulate into registers, so their gathers can all be in flight
// together.  NC = false: the list was written by the calling kernel (plain
// loads instead of the read-only path).
template <int TPP, bool NC = true, class FF, class FB>
__device__ __forceinline__ void walk_blocks(const int *__restrict__ nbr, int64_t s, int64_t cap, int q,
                                            int nfl, int ntot, FF &&ff, FB &&fb) {
    const int4 *L4 = reinterpret_cast<const int4 *>(nbr) + s;
    const int nblk = (ntot + 3) >> 2;
    int b = q;
    if (b >= nblk) return;
    auto ld = [&](int64_t i) { return NC ? ld_list_nc(L4 + i) : ld_list(L4 + i); };
    int4 cur = ld((int64_t)b * cap);
    while (b < nblk) {
        const int bn = b + TPP;
        int4 nxt = cur;
        if (bn < nblk) nxt = ld((int64_t)bn * cap);
        const int t0 = b << 2;
        const int jj[4] = {cur.x, cur.y, cur.z, cur.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int t = t0 + e;
            if (t < nfl) ff(jj[e]);
            else if (t < ntot) fb(jj[e]);
        }
        cur = nxt;
        b = bn;
    }
}

// Entries [lo, hi) of the blocked list in whole four-entry blocks, for lane q
// (blocks b = q mod TPP): all four callbacks of a block run unconditionally,
// f(j, valid), an entry outside [lo, hi) with valid = false and the index of the
// block's first entry in range, so the block's gathers carry no branch and can
// all be issued before the first one is used.  Per lane, the valid entries come
// in the same order as in walk_blocks.
template <int TPP, class Fn>
__device__ __forceinline__ void walk_range_pred(const int4 *__restrict__ L4, int64_t cap, int q, int lo, int hi,
                                                Fn &&f) {
    if (lo >= hi) return;
    const int b0 = lo >> 2, b1 = (hi + 3) >> 2;
    int b = b0 + ((q - b0) & (TPP - 1));
    if (b >= b1) return;
    int4 cur = ld_list_nc(L4 + (int64_t)b * cap);
    while (b < b1) {
        const int bn = b + TPP;
        int4 nxt = cur;
        if (bn < b1) nxt = ld_list_nc(L4 + (int64_t)bn * cap);
        const int t0 = b << 2;
        const int first = lo > t0 ? lo - t0 : 0;  // first in-range entry (0..3)
        const int jf = first == 0 ? cur.x : first == 1 ? cur.y : first == 2 ? cur.z : cur.w;
        const int jj[4] = {cur.x, cur.y, cur.z, cur.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int t = t0 + e;
            const bool v = t >= lo && t < hi;
            f(v ? jj[e] : jf, v);
        }
        cur = nxt;
        b = bn;
    }
}

template <int TPP, class FF, class FB>
__device__ __forceinline__ void walk_blocks_pred(const int *__restrict__ nbr, int64_t s, int64_t cap, int q,
                                                 int nfl, int ntot, FF &&ff, FB &&fb) {
    const int4 *L4 = reinterpret_cast<const int4 *>(nbr) + s;
    walk_range_pred<TPP>(L4, cap, q, 0, nfl, ff);
    walk_range_pred<TPP>(L4, cap, q, nfl, ntot, fb);
}

// Neighbours of sorted fluid particle s for lane q of a TPP-lane particle group:
// the blocked list, or -- for a particle whose list overflowed -- the strided
// candidate scan of the template cells.  Both visit the pairs the density sweep
// selected; the callbacks keep their own 0 < r < h test, which is what selects
// the pairs on the scanning path.
template <int DIM, bool BOUND, int TPP, bool M, class FF, class FB>
__device__ __forceinline__ void for_each_neighbor_tpp(const SceneConst &c, const SceneStep &st, int R,
                                                      const FluidBuf &F, const BoundBuf &B, int64_t s, int q,
                                                      float4 pi, FF &&ff, FB &&fb) {
    const unsigned int pc = F.nbr_cnt[s];
    if (pc != kNbrOverflow) {
        // list entries: the pair passed 0 < r^2 < h^2 when it was recorded (same
        // positions, same FP32 arithmetic), so the callbacks may skip the test
        const int nfl = (int)(pc & 0xffffu), nbo = (int)(pc >> 16);
        if constexpr (std::is_invocable_v<FF &, int, std::true_type, bool>) {
            // callbacks that take a valid flag: branch-free four-entry blocks
            walk_blocks_pred<TPP>(F.nbr, s, F.cap, q, nfl, BOUND ? nfl + nbo : nfl,
                                  [&](int j, bool v) { ff(j, std::true_type{}, v); },
                                  [&](int j, bool v) { fb(j, std::true_type{}, v); });
        } else {
            walk_blocks<TPP>(F.nbr, s, F.cap, q, nfl, BOUND ? nfl + nbo : nfl,
                             [&](int j) { ff(j, std::true_type{}); }, [&](int j) { fb(j, std::true_type{}); });
        }
        return;
    }
    auto ffs = [&](int j) {
        if constexpr (std::is_invocable_v<FF &, int, std::false_type, bool>) ff(j, std::false_type{}, true);
        else ff(j, std::false_type{});
    };
    auto fbs = [&](int j) {
        if constexpr (std::is_invocable_v<FB &, int, std::false_type, bool>) fb(j, std::false_type{}, true);
        else fb(j, std::false_type{});
    };
    if (!M) {
        // the grid geometry (launch constants here) is used only on this rare path
        Geo g;
        g.load(c, R);
        bool ok;
        const long long code = cell_code<DIM>(pi, g, ok);
        if (ok) {
            visit_candidates<DIM, TPP>(F.start, g, code, 0, q, ffs);
            if (BOUND) visit_candidates<DIM, TPP>(B.start, g, code, 0, q, fbs);
        }
    } else {
        // batched instances: the scene's geometry is re-read from the scene table
        // at every row (volatile loads are not hoisted), so this rare path keeps
        // no geometry in registers across the list walk above
        bool ok;
        long long code;
        {
            Geo g;
            g.load(c, R);
            code = cell_code<DIM>(pi, g, ok);
        }
        if (ok) {
            visit_candidates_lean<DIM, TPP>(F.start, &c, R, code, st.f_shift, q, ffs);
            if (BOUND) visit_candidates_lean<DIM, TPP>(B.start, &c, R, code, st.b_shift, q, fbs);
        }
    }
}

inline int blocks_for(int64_t n, int bs = kBlock) { return (int)((n + bs - 1) / bs); }

}  // namespace tsph
