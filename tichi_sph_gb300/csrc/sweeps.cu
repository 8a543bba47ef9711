// Neighbour sweeps of one substep: density + alpha, the Jacobi pair of the two
// pressure solves, and the advection forces (viscosity, surface tension).
//
// One thread (or TPP threads) per particle in cell-sorted order; a block never
// straddles two scenes, so every block reads one scene's constants.  The
// density sweep scans the (2r+1)^dim template rows of the fluid grid and, where
// the reference pairs with the boundary set, of the boundary grid
// (visit_candidates), and records every pair with 0 < r < h in the fluid
// particle's neighbour list.  The later sweeps of the step walk that list
// (for_each_neighbor_tpp) -- about 30 entries instead of about 220 candidates in
// 3D -- in the same order.  Per-particle sums are FP32 (the reference's
// precision); global sums are FP64 with a fixed summation order.
//
// Solver loops run per scene: a scene's loop state (iteration, condition,
// v_adv buffer) lives in its SceneStep; blocks of a scene whose loop has ended
// do nothing, the last block of a scene evaluates its loop test, and the last
// block of the grid sets the CUDA-graph while condition to "any scene running".
#include <cuda_runtime.h>

#include "ctx.h"

namespace tsph {

// True for the warp of this block that finishes last (every warp must call it).
__device__ __forceinline__ bool block_last_warp(unsigned int *arrived) {
    unsigned int old = 0;
    if ((threadIdx.x & 31) == 0) {
        __threadfence_block();
        old = atomicAdd(arrived, 1u);
    }
    old = __shfl_sync(0xffffffffu, old, 0);
    const bool last = old == blockDim.x / 32 - 1;
    if (last) __threadfence_block();
    return last;
}

// The last warp of the grid: OR of the scenes' loop conditions into cond_any and
// the graph condition.
__device__ __forceinline__ void publish_any(const KConst &k, int SceneStep::*field, int32_t *any_out,
                                            cudaGraphConditionalHandle h, int use_cond) {
    const int lane = threadIdx.x & 31;
    int any = 0;
    for (int s = lane; s < k.n_scenes; s += 32) any |= (__ldcg(&(k.ss[s].*field)) != 0);
    any = __any_sync(0xffffffffu, any);
    if (lane == 0) {
        *any_out = any;
        if (use_cond) cudaGraphSetConditional(h, any ? 1u : 0u);
    }
}

// ----------------------------------------------------------------------------- density
// s + e accumulates a sum with the rounding error of every addition kept in e
// (Knuth's TwoSum, exact for any order of the terms).  The density sweep sums
// the fluid's density and compression this way: psi - psi0, which the pressure
// solves start from, cancels all but ~1e-3 (DFSPH) or ~1e-6 (VFSPH) of psi, so
// an FP32 sum's own rounding (a few 1e-7 of psi over ~40 terms) would be a
// large part of it; with the error term the sum is exact to about one rounding
// of psi, and psi's low part is kept beside it (FluidBuf::psilo).
__device__ __forceinline__ void acc2(float &s, float &e, float y) {
    const float t = __fadd_rn(s, y);
    const float yp = __fsub_rn(t, s);
    const float sp = __fsub_rn(t, yp);
    e = __fadd_rn(e, __fadd_rn(__fsub_rn(s, sp), __fsub_rn(y, yp)));
    s = t;
}

// SPH_clean_value + SPH_prepare_attr (f,f)(f,b) + SPH_prepare_alpha_1 (f,f)(f,b)
// + SPH_prepare_alpha_2 (f,f) + SPH_prepare_alpha (sph.py:22-38, 50-105), and the
// neighbour list of the step.
//
// Two phases keep the warps converged: the candidate scan only tests r < h and
// records the pairs with 0 < r < h (the r = 0 terms -- the particle itself and
// coincident particles -- go straight into W / rho / compression), then the
// recorded list is walked for the kernel arithmetic.  A particle whose pairs do
// not fit the list redoes the scan with the arithmetic inline.
// L (list entries, 0 < r < h known): mass / volume load beside the position,
// no range tests; same arithmetic.
template <int DIM, bool L = false>
__device__ __forceinline__ void density_pair_fluid(const Geo &g, const FluidBuf &F, float4 pi, int j, float &wsum,
                                                   float &rho, float &comp, float &a1x, float &a1y, float &a1z,
                                                   float &a2, float &rho_e, float &comp_e) {
    const float4 pj = F.pos[j];
    float2 mv = make_float2(0.f, 0.f);
    if (L) mv = F.mv[j];
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    const float r2 = dx * dx + dy * dy + dz * dz;
    if (L || r2 < g.h2) {
        if (!L) mv = F.mv[j];
        float r;
        const float ri = L ? pair_rinv_pos(r2, r) : pair_rinv(r2, r);
        const float q = r * g.inv_h;
        const float w = kw(q) * g.sig;
        wsum += w;
        acc2(rho, rho_e, __fmul_rn(w, mv.x));
        acc2(comp, comp_e, __fmul_rn(w, mv.y));
        if (L || r2 > 0.f) {
            const float wg = kwg(q) * g.sig_h;
            const float f = pj.w * wg * ri;
            a1x += f * dx;
            a1y += f * dy;
            a1z += f * dz;
            a2 += __fdividef(wg * wg * pj.w * pj.w, mv.x);
        }
    }
}

template <int DIM, bool L = false>
__device__ __forceinline__ void density_pair_bound(const Geo &g, const BoundBuf &B, float4 pi, int j, float &wsum,
                                                   float &rho, float &comp, float &a1x, float &a1y, float &a1z,
                                                   float &rho_e, float &comp_e) {
    const float4 pj = B.pos[j];
    float2 mv = make_float2(0.f, 0.f);
    if (L) mv = B.mv[j];
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    const float r2 = dx * dx + dy * dy + dz * dz;
    if (L || r2 < g.h2) {
        if (!L) mv = B.mv[j];
        float r;
        const float ri = L ? pair_rinv_pos(r2, r) : pair_rinv(r2, r);
        const float q = r * g.inv_h;
        const float w = kw(q) * g.sig;
        wsum += w;
        acc2(rho, rho_e, __fmul_rn(w, mv.x));
        acc2(comp, comp_e, __fmul_rn(w, mv.y));
        if (L || r2 > 0.f) {
            const float f = pj.w * kwg(q) * g.sig_h * ri;
            a1x += f * dx;
            a1y += f * dy;
            a1z += f * dz;
        }
    }
}

// Sums of the density sweep for one fluid particle.
struct DensAcc {
    float wsum, rho, comp, a2, a1x, a1y, a1z, pacc, rho_e, comp_e;
};

// One recorded pair (0 < r < h known) of the density sweep's list pass: the
// density and alpha terms and, with P0, k_psi's pair term for the divergence
// solve's first iteration -- one distance, one reciprocal square root and one
// spline gradient serve all of them.  The gradient factor is formed in k_psi's
// order, ((W'(q) sig / h) / r) X_j, so the psi term is k_psi's bit for bit.
// FLUIDJ: the neighbour is a fluid particle (alpha_2 has no boundary term,
// main.py:194-195).
template <bool FLUIDJ, bool P0>
__device__ __forceinline__ void density_list_pair(const Geo &g, float4 pi, float4 pj, float2 mv, float4 vi,
                                                  float4 vj, DensAcc &a) {
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    const float r2 = dx * dx + dy * dy + dz * dz;
    float r;
    const float ri = pair_rinv_pos(r2, r);
    const float q = r * g.inv_h;
    const float w = kw(q) * g.sig;
    a.wsum += w;
    acc2(a.rho, a.rho_e, __fmul_rn(w, mv.x));
    acc2(a.comp, a.comp_e, __fmul_rn(w, mv.y));
    const float wg = kwg(q) * g.sig_h;
    const float f = wg * ri * pj.w;
    a.a1x += f * dx;
    a.a1y += f * dy;
    a.a1z += f * dz;
    if (FLUIDJ) a.a2 += __fdividef(wg * wg * pj.w * pj.w, mv.x);
    if (P0) a.pacc += f * (dx * (vi.x - vj.x) + dy * (vi.y - vj.y) + dz * (vi.z - vj.z));
}

// In the one-scene instance the divergence solve's first psi sweep (k_psi's
// work for its iteration 0) is done here as well when that solve will run
// (iter_min > 0 or the carried-over compression above the tolerance, the test
// k_solve_begin makes): its pair terms need only positions and the v_adv the
// solve starts from, both fixed here, and walk the same pairs in the same
// order as k_psi with one thread per particle, with the same arithmetic; the
// scene's psi_sum goes through the same partials and ticket.  psi_ready tells
// k_psi to skip that iteration.  (Measured: a saving in the one-scene case;
// in the batched instance, whose scene lookups leave fewer registers, a loss.)
template <int DIM, bool M>
__global__ void __launch_bounds__(kBlock, 6) k_density_fluid(KConst k, FluidBuf F, BoundBuf B, double *partials) {
    pdl_entry();
    __shared__ double sh[kBlock / 32];
    __shared__ unsigned int arrived;
    if (threadIdx.x == 0) arrived = 0;
    __syncthreads();
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    const int sc = f_block_scene<M>(k, blockIdx.x * (int64_t)kBlock);
    const SceneConst &c = scene<M>(k, sc);
    SceneStep &st = k.ss[sc];
    const bool psi0 = !M && c.f_n > 0 && ((0 < c.iter_min) || (k.sp[sc].compression > (double)c.div_tol));
    double contrib = 0.0;
    if (s - c.f_slot < c.f_n) {
        Geo g;
        g.load(c, k.R);
        const long long f_shift = shift_of<M>(st.f_shift), b_shift = shift_of<M>(st.b_shift);
        const float4 pi = F.pos[s];
        const float4 *vin = F.vadv + st.cur * F.cap;
        const float4 vi = psi0 ? vin[s] : make_float4(0.f, 0.f, 0.f, 0.f);
        bool ok;
        const long long code = cell_code<DIM>(pi, g, ok);
        float wsum = 0.f, rho = 0.f, comp = 0.f, a2 = 0.f, pacc = 0.f, rho_e = 0.f, comp_e = 0.f;
        float a1x = 0.f, a1y = 0.f, a1z = 0.f;
        int nfl = 0, nbo = 0;
        int *L = F.nbr;
        const int64_t stride = F.cap;
        const int cap = k.nbr_max;
        const float w0 = kw(0.f) * g.sig;
        // k_psi's pair term (IPPE_adv_psi), the same expression
        auto psi_pair = [&](const float4 *P, const float4 *V, int j, auto listed) {
            constexpr bool Ls = decltype(listed)::value;
            const float4 pj = P[j];
            const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (Ls || (r2 < g.h2 && r2 > 0.f)) {
                const float4 vj = V[j];
                float r;
                const float ri = Ls ? pair_rinv_pos(r2, r) : pair_rinv(r2, r);
                const float f = kwg(r * g.inv_h) * g.sig_h * ri * pj.w;
                pacc += f * (dx * (vi.x - vj.x) + dy * (vi.y - vj.y) + dz * (vi.z - vj.z));
            }
        };
        if (ok) {
            // phase 1: record the pairs.  The write position walks the blocked
            // layout (entry t at nbr_index(t, s, stride)): +1 within a block of
            // four, +4 stride - 3 to the next block.  Candidate positions load
            // through the read-only path (no step writes them in this kernel),
            // so they need not wait for the list stores before them
            int nrec = 0;
            int *wp = L + (int64_t)s * 4;
            const int64_t next_block = stride * 4 - 3;
            auto record = [&](int j) {
                if (nrec < cap) {
                    *wp = j;
                    wp += ((nrec & 3) == 3) ? next_block : 1;
                }
                ++nrec;
            };
            visit_candidates_within<DIM>(F.start, g, pi, code, f_shift, 0, [&](int j) {
                const float4 pj = __ldg(&F.pos[j]);
                const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < g.h2) {
                    if (r2 > 0.f) {
                        record(j);
                    } else {
                        const float2 mv = F.mv[j];
                        wsum += w0;
                        acc2(rho, rho_e, __fmul_rn(w0, mv.x));
                        acc2(comp, comp_e, __fmul_rn(w0, mv.y));
                    }
                }
            });
            nfl = nrec;
            visit_candidates_within<DIM>(B.start, g, pi, code, b_shift, 0, [&](int j) {
                const float4 pj = __ldg(&B.pos[j]);
                const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < g.h2) {
                    if (r2 > 0.f) {
                        record(j);
                    } else {
                        const float2 mv = B.mv[j];
                        wsum += w0;
                        acc2(rho, rho_e, __fmul_rn(w0, mv.x));
                        acc2(comp, comp_e, __fmul_rn(w0, mv.y));
                    }
                }
            });
            nbo = nrec - nfl;
            if (nfl + nbo <= cap) {
                // phase 2: the arithmetic over the recorded pairs
                DensAcc a = {wsum, rho, comp, 0.f, 0.f, 0.f, 0.f, 0.f, rho_e, comp_e};
                if (psi0) {
                    walk_blocks<1, false>(F.nbr, s, stride, 0, nfl, nfl + nbo,
                        [&](int j) { density_list_pair<true, true>(g, pi, F.pos[j], F.mv[j], vi, vin[j], a); },
                        [&](int j) { density_list_pair<false, true>(g, pi, B.pos[j], B.mv[j], vi, B.vadv[j], a); });
                } else {
                    walk_blocks<1, false>(F.nbr, s, stride, 0, nfl, nfl + nbo,
                        [&](int j) { density_list_pair<true, false>(g, pi, F.pos[j], F.mv[j], vi, vi, a); },
                        [&](int j) { density_list_pair<false, false>(g, pi, B.pos[j], B.mv[j], vi, vi, a); });
                }
                wsum = a.wsum; rho = a.rho; comp = a.comp; a2 = a.a2; pacc = a.pacc;
                a1x = a.a1x; a1y = a.a1y; a1z = a.a1z; rho_e = a.rho_e; comp_e = a.comp_e;
            } else {
                // list overflow: one scan with the arithmetic inline
                wsum = rho = comp = a2 = a1x = a1y = a1z = rho_e = comp_e = 0.f;
                visit_candidates<DIM>(F.start, g, code, f_shift, 0, [&](int j) {
                    density_pair_fluid<DIM>(g, F, pi, j, wsum, rho, comp, a1x, a1y, a1z, a2, rho_e, comp_e);
                    if (psi0) psi_pair(F.pos, vin, j, std::false_type{});
                });
                visit_candidates<DIM>(B.start, g, code, b_shift, 0, [&](int j) {
                    density_pair_bound<DIM>(g, B, pi, j, wsum, rho, comp, a1x, a1y, a1z, rho_e, comp_e);
                    if (psi0) psi_pair(B.pos, B.vadv, j, std::false_type{});
                });
            }
        }
        F.nbr_cnt[s] = (nfl + nbo <= cap) ? ((unsigned int)nfl | ((unsigned int)nbo << 16)) : kNbrOverflow;
        const float4 mp = F.mpsi[s];
        float alpha = (a1x * a1x + a1y * a1y + a1z * a1z) / mp.x + a2;
        if (alpha < 1e-4f) alpha = 1e-4f;
        // the compensated sums rounded once; psi keeps the remainder as its low part
        const float rho_f = __fadd_rn(rho, rho_e), comp_f = __fadd_rn(comp, comp_e);
        const float psi = k.vfsph ? comp_f : rho_f;
        const float psilo = k.vfsph ? __fsub_rn(comp_e, __fsub_rn(comp_f, comp)) : __fsub_rn(rho_e, __fsub_rn(rho_f, rho));
        F.dens[s] = make_float4(wsum, rho_f, comp_f, a2);
        F.a1[s] = make_float4(a1x, a1y, a1z, alpha);  // w: alpha again, for the write-back
        F.psilo[s] = psilo;
        F.mpsi[s] = make_float4(mp.x, psi, mp.z, alpha);
        // psi also rides in the current v_adv's unused w (the velocity sweeps carry
        // it along), so the advection sweep gets it with the neighbour's v_adv
        F.vadv[(int64_t)st.cur * F.cap + s].w = psi;
        if (psi0) {
            // IPPE_adv_psi_init + IPPE_psi_adv_non_negative, as k_psi
            float pa = ((psi - mp.z) + psilo) + pacc * k.sp[sc].dt;
            if (pa < 0.f) pa = 0.f;
            const float kap = pa / alpha;
            F.psiadv[s] = pa;
            F.kappa[s] = kap;
            F.pk[s] = make_float4(pi.x, pi.y, pi.z, kap);
            contrib = (double)(pa / mp.z);
        }
    }
    if (!psi0) return;  // uniform over the block (one scene)
    double bsum;
    if (block_sum_last_warp<kBlock>(contrib, sh, &arrived, bsum)) {
        if ((threadIdx.x & 31) == 0) partials[blockIdx.x] = bsum;
        const int64_t b0 = c.f_slot / kBlock;
        const unsigned int nblk = (unsigned int)(c.f_slots / kBlock);
        if (last_warp_done(&st.ticket[kStPsi], nblk)) {
            const int lane = threadIdx.x & 31;
            double v = 0.0;
            for (int64_t i = lane; i < (int64_t)nblk; i += 32) v += __ldcg(partials + b0 + i);
            v = warp_sum(v);
            if (lane == 0) {
                st.psi_sum = v;
                st.ticket[kStPsi] = 0;
                st.psi_ready = 1;
            }
        }
    }
}

// The boundary's own sums: SPH_prepare_attr (b,b)(b,f), SPH_prepare_alpha_2 (b,f),
// SPH_prepare_alpha (sph.py:50-105 as called by main.py:190-197).
template <int DIM, bool M>
__global__ void __launch_bounds__(kBlock, 6) k_density_bound(KConst k, FluidBuf F, BoundBuf B) {
    pdl_entry();
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    const int sc = b_block_scene<M>(k, blockIdx.x * (int64_t)kBlock);
    const SceneConst &c = scene<M>(k, sc);
    if (s - c.b_slot >= c.b_n) return;
    const SceneStep &st = k.ss[sc];
    const ScenePersist &sp = k.sp[sc];
    // the (b,b) terms of the last sweep still hold when the gather found every
    // boundary position and mass unchanged (a static boundary)
    const bool cached = sp.bb_valid && !st.b_dirty && sp.bb_n == c.b_n;
    Geo g;
    g.load(c, k.R);
    const float4 pi = B.pos[s];
    bool ok;
    const long long code = cell_code<DIM>(pi, g, ok);
    float wsum = 0.f, rho = 0.f, comp = 0.f, a2 = 0.f;
    if (ok) {
        if (cached) {
            const float4 bb = B.bb[s];
            wsum = bb.x;
            rho = bb.y;
            comp = bb.z;
        } else {
            visit_candidates_within<DIM>(B.start, g, pi, code, shift_of<M>(st.b_shift), 0, [&](int j) {
                const float4 pj = B.pos[j];
                const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < g.h2) {
                    const float2 mv = B.mv[j];
                    float r;
                    pair_rinv(r2, r);
                    const float w = kw(r * g.inv_h) * g.sig;
                    wsum += w;
                    rho += w * mv.x;
                    comp += w * mv.y;
                }
            });
            B.bb[s] = make_float4(wsum, rho, comp, 0.f);
        }
        visit_candidates_within<DIM>(F.start, g, pi, code, shift_of<M>(st.f_shift), 0, [&](int j) {
            const float4 pj = F.pos[j];
            const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < g.h2) {
                const float2 mv = F.mv[j];
                float r;
                const float ri = pair_rinv(r2, r);
                const float q = r * g.inv_h;
                const float w = kw(q) * g.sig;
                wsum += w;
                rho += w * mv.x;
                comp += w * mv.y;
                if (r2 > 0.f) {
                    const float wg = kwg(q) * g.sig_h;
                    a2 += __fdividef(wg * wg * pj.w * pj.w, mv.x);
                }
            }
        });
    }
    const float m = B.mv[s].x;
    float alpha = 0.f / m + a2;
    if (alpha < 1e-4f) alpha = 1e-4f;
    B.dens[s] = make_float4(wsum, rho, comp, a2);
    B.alpha[s] = alpha;
    const float kb = B.kappa[s] / alpha;  // boundary psi_adv / alpha (psi_adv is never advanced)
    B.kappa[s] = kb;
    B.pk[s] = make_float4(pi.x, pi.y, pi.z, kb);
}

// ----------------------------------------------------------------------------- solver
// Sets every scene's loop condition before a solve: main.py:201 / main.py:222
// test `iter < iter_min or compression > tol` with the compression left by the
// previous solve.  A scene without fluid runs min(iter_min, iter_max + 1) empty
// iterations in the reference and its compression becomes 0/0 = NaN
// (sph.py:226); that is settled here without device work.  `flip` makes the
// v_adv written by the advection sweep current.
__global__ void k_solve_begin(KConst k, int kind, int flip, cudaGraphConditionalHandle h, int use_cond) {
    pdl_entry();
    __shared__ int any_sh;
    if (threadIdx.x == 0) any_sh = 0;
    __syncthreads();
    int any = 0;
    for (int s = threadIdx.x; s < k.n_scenes; s += blockDim.x) {
        const SceneConst &c = k.sc[s];
        SceneStep &st = k.ss[s];
        ScenePersist &sp = k.sp[s];
        const double tol = kind == kSolveDiv ? (double)c.div_tol : (double)c.comp_tol;
        int cond, it = 0;
        if (c.f_n > 0) {
            cond = (0 < c.iter_min) || (sp.compression > tol);
        } else {
            cond = 0;
            while (it < c.iter_min) {
                ++it;
                if (it > c.iter_max) break;
            }
            if (it > 0) sp.compression = __longlong_as_double(0x7ff8000000000000ll);
        }
        st.iter = it;
        st.cond = cond;
        if (kind == kSolveDiv) st.div_iter = it;
        else st.incom_iter = it;
        // the density sweep's first-iteration psi belongs to the divergence solve
        if (kind == kSolveDens) st.psi_ready = 0;
        if (flip) st.cur = 1 - st.cur;
        any |= cond;
    }
    if (any) atomicOr(&any_sh, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        k.dg->cond_any = any_sh;
        if (use_cond) cudaGraphSetConditional(h, any_sh ? 1u : 0u);
    }
}

// Sweep A: IPPE_adv_psi_init + IPPE_adv_psi (f,f)(f,b) + IPPE_psi_adv_non_negative
// (sph.py:196-226), TPP threads per particle.  Writes psi_adv and kappa =
// psi_adv / alpha; the scene's sum of psi_adv / psi0 goes to per-block partials
// and, through the scene's last block, to its psi_sum (block order:
// deterministic).  force = 1: the host runs the loop (kernel-level calls), so
// the sweep runs whatever the device-side loop condition says.
template <int DIM, int TPP, bool M>
__global__ void __launch_bounds__(kBlock, 6) k_psi(KConst k, FluidBuf F, BoundBuf B, double *partials, int force) {
    pdl_entry();
    __shared__ double sh[kBlock / 32];
    __shared__ unsigned int arrived;
    const int64_t first = blockIdx.x * (int64_t)(kBlock / TPP);
    const int sc = f_block_scene<M>(k, first);
    SceneStep &st = k.ss[sc];
    if (!st.cond && !force) return;  // this scene's loop has ended (uniform over the block)
    if (st.psi_ready) return;  // this iteration's sweep ran inside the density sweep
    if (threadIdx.x == 0) arrived = 0;
    __syncthreads();
    const SceneConst &c = scene<M>(k, sc);
    const Lanes<TPP> ln;
    const int64_t s = ln.s;
    const bool act = s - c.f_slot < c.f_n;
    Geo g;
    g.load(c, k.R);
    const float4 *vin = F.vadv + st.cur * F.cap;
    float acc = 0.f;
    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f), vi = pi;
    if (act) {
        pi = F.pos[s];
        vi = vin[s];
        // IPPE_adv_psi pair term; list entries load both neighbour arrays at once
        auto term = [&](const float4 *P, const float4 *V, int j, auto listed) {
            constexpr bool L = decltype(listed)::value;
            const float4 pj = P[j];
            float4 vj = make_float4(0.f, 0.f, 0.f, 0.f);
            if (L) vj = V[j];
            const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (L || (r2 < g.h2 && r2 > 0.f)) {
                if (!L) vj = V[j];
                float r;
                const float ri = L ? pair_rinv_pos(r2, r) : pair_rinv(r2, r);
                const float f = kwg(r * g.inv_h) * g.sig_h * ri * pj.w;
                acc += f * (dx * (vi.x - vj.x) + dy * (vi.y - vj.y) + dz * (vi.z - vj.z));
            }
        };
        // branchy list walk: two float4 gathers per entry leave no registers
        // for a whole block's gathers at six blocks per SM
        for_each_neighbor_tpp<DIM, true, TPP, M>(c, st, k.R, F, B, s, ln.q, pi,
            [&](int j, auto listed) { term(F.pos, vin, j, listed); },
            [&](int j, auto listed) { term(B.pos, B.vadv, j, listed); });
    }
    acc = ln.sum(acc);
    double contrib = 0.0;
    if (act && ln.q == 0) {
        const float4 mp = F.mpsi[s];
        float psi = ((mp.y - mp.z) + F.psilo[s]) + acc * k.sp[sc].dt;
        if (psi < 0.f) psi = 0.f;
        const float kap = psi / mp.w;
        F.psiadv[s] = psi;
        F.kappa[s] = kap;
        F.pk[s] = make_float4(pi.x, pi.y, pi.z, kap);
        contrib = (double)(psi / mp.z);
    }
    double bsum;
    if (block_sum_last_warp<kBlock>(contrib, sh, &arrived, bsum)) {
        if ((threadIdx.x & 31) == 0) partials[blockIdx.x] = bsum;
        const int64_t b0 = c.f_slot * TPP / kBlock;
        const unsigned int nblk = (unsigned int)(c.f_slots * TPP / kBlock);
        if (last_warp_done(&st.ticket[kStPsi], nblk)) {
            const int lane = threadIdx.x & 31;
            double v = 0.0;
            for (int64_t i = lane; i < (int64_t)nblk; i += 32) v += __ldcg(partials + b0 + i);
            v = warp_sum(v);
            if (lane == 0) {
                st.psi_sum = v;
                st.ticket[kStPsi] = 0;
            }
        }
    }
}

// Sweep B: IPPE_update_vel_adv (f,f)(f,b), sph.py:229-244, into the scene's other
// v_adv buffer, TPP threads per particle.  The scene's last block evaluates the
// loop test of main.py:201-213 / 222-234 from sweep A's sum; the grid's last
// block sets the graph's while-node condition.  force = 1 (kernel-level calls,
// the host runs the loop): the sweep runs regardless of the device-side
// condition and leaves the loop test and its cap to the host.
template <int DIM, int TPP, bool M>
__global__ void __launch_bounds__(kBlock) k_vel(KConst k, FluidBuf F, BoundBuf B, int kind,
                                                cudaGraphConditionalHandle h, int use_cond, int force) {
    pdl_entry();
    __shared__ unsigned int arrived;
    if (threadIdx.x == 0) arrived = 0;
    __syncthreads();
    const int64_t first = blockIdx.x * (int64_t)(kBlock / TPP);
    const int sc = f_block_scene<M>(k, first);
    SceneStep &st = k.ss[sc];
    const SceneConst &c = scene<M>(k, sc);
    const bool running = force || st.cond != 0;
    if (running) {
        const Lanes<TPP> ln;
        const int64_t s = ln.s;
        const bool act = s - c.f_slot < c.f_n;
        Geo g;
        g.load(c, k.R);
        const int cur = st.cur;
        // IPPE_update_vel_adv's pair term (kappa_i X_j + kappa_j X_i) g x_ij, g =
        // W'(r) / r, summed as kappa_i alpha_1,i + X_i sum_j kappa_j g x_ij:
        // alpha_1 = sum_j X_j g x_ij over the same pairs is the density sweep's,
        // and the second sum needs of a neighbour only (x, y, z, kappa), one
        // float4 written by the psi sweep (the boundary's by its density sweep)
        float sx = 0.f, sy = 0.f, sz = 0.f;
        float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
        if (act) {
            pi = F.pos[s];
            // (valid = false: a padding call of a list block, computed and dropped)
            auto term = [&](const float4 *PK, int j, auto listed, bool valid) {
                constexpr bool L = decltype(listed)::value;
                const float4 qj = PK[j];
                const float dx = pi.x - qj.x, dy = pi.y - qj.y, dz = pi.z - qj.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                if (L || (r2 < g.h2 && r2 > 0.f)) {
                    float r;
                    const float ri = L ? pair_rinv_pos(r2, r) : pair_rinv(r2, r);
                    const float f = qj.w * (kwg(r * g.inv_h) * g.sig_h * ri);
                    sx = valid ? sx + f * dx : sx;
                    sy = valid ? sy + f * dy : sy;
                    sz = valid ? sz + f * dz : sz;
                }
            };
            for_each_neighbor_tpp<DIM, true, TPP, M>(c, st, k.R, F, B, s, ln.q, pi,
                [&](int j, auto listed, bool v) { term(F.pk, j, listed, v); },
                [&](int j, auto listed, bool v) { term(B.pk, j, listed, v); });
        }
        sx = ln.sum(sx);
        sy = ln.sum(sy);
        sz = ln.sum(sz);
        if (act && ln.q == 0) {
            const float ki = F.kappa[s], Xi = pi.w;
            const float4 a1 = F.a1[s];
            const float ax = ki * a1.x + Xi * sx, ay = ki * a1.y + Xi * sy, az = ki * a1.z + Xi * sz;
            const float4 *vin = F.vadv + cur * F.cap;
            float4 *vout = F.vadv + (1 - cur) * F.cap;
            const float sc_ = -(1.f / k.sp[sc].dt) / F.mpsi[s].x;
            const float4 vi = vin[s];
            vout[s] = make_float4(vi.x + sc_ * ax, vi.y + sc_ * ay, vi.z + sc_ * az, vi.w);  // w: psi
        }
    }
    if (!block_last_warp(&arrived)) return;
    if (running) {
        const unsigned int nblk = (unsigned int)(c.f_slots * TPP / kBlock);
        if (last_warp_done(&st.ticket[kStVel], nblk) && (threadIdx.x & 31) == 0) {
            ScenePersist &sp = k.sp[sc];
            const double comp = st.psi_sum / (double)c.f_n;
            sp.compression = comp;
            const int it = st.iter + 1;
            st.iter = it;
            if (kind == kSolveDiv) st.div_iter = it;
            else st.incom_iter = it;
            if (!force) {
                const double tol = kind == kSolveDiv ? (double)c.div_tol : (double)c.comp_tol;
                const int capped = it > c.iter_max;
                const int cond = !capped && (it < c.iter_min || comp > tol);
                if (capped) st.status |= (kind == kSolveDiv ? TSPH_ST_DIV_ITER_CAP : TSPH_ST_DENS_ITER_CAP);
                st.cond = cond;
            }
            st.cur = 1 - st.cur;
            st.psi_ready = 0;
            st.ticket[kStVel] = 0;
        }
    }
    if (last_warp_done(&k.dg->ticket[kGtVel], gridDim.x)) {
        publish_any(k, &SceneStep::cond, &k.dg->cond_any, h, use_cond);
        if ((threadIdx.x & 31) == 0) k.dg->ticket[kGtVel] = 0;
    }
}

// ----------------------------------------------------------------------------- advection
// First pass of SPH_advection_surface_tension_acc, sph.py:134-150: surface normals.
template <int DIM, int TPP, bool M>
__global__ void __launch_bounds__(kBlock) k_normal(KConst k, FluidBuf F, BoundBuf B) {
    pdl_entry();
    const int64_t first = blockIdx.x * (int64_t)(kBlock / TPP);
    const int sc = f_block_scene<M>(k, first);
    const SceneConst &c = scene<M>(k, sc);
    const SceneStep &st = k.ss[sc];
    const Lanes<TPP> ln;
    const int64_t s = ln.s;
    const bool act = s - c.f_slot < c.f_n;
    Geo g;
    g.load(c, k.R);
    float nx = 0.f, ny = 0.f, nz = 0.f;
    if (act) {
        const float4 pi = F.pos[s];
        for_each_neighbor_tpp<DIM, false, TPP, M>(c, st, k.R, F, B, s, ln.q, pi,
            [&](int j, auto listed) {
                constexpr bool L = decltype(listed)::value;
                const float4 pj = F.pos[j];
                float psij = 0.f;
                if (L) psij = F.mpsi[j].y;
                const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                if (L || (r2 < g.h2 && r2 > 0.f)) {
                    if (!L) psij = F.mpsi[j].y;
                    float r;
                    const float ri = L ? pair_rinv_pos(r2, r) : pair_rinv(r2, r);
                    const float f = -__fdividef(pj.w, psij) * (kwg(r * g.inv_h) * g.sig_h) * ri;
                    nx += f * dx;
                    ny += f * dy;
                    nz += f * dz;
                }
            },
            [&](int, auto) {});
    }
    nx = ln.sum(nx);
    ny = ln.sum(ny);
    nz = ln.sum(nz);
    if (act && ln.q == 0) {
        // w: what the surface-tension pass reads of a neighbour beside its normal
        const float w = F.vf[s] > 0.99f ? F.mpsi[s].y : __uint_as_float(kNoSurfTension);
        F.normal[s] = make_float4(nx * g.h, ny * g.h, nz * g.h, w);
    }
}

// SPH_vel_adv_2_vel + SPH_advection_gravity_acc + SPH_advection_viscosity_acc
// + (pass 2 of) SPH_advection_surface_tension_acc + SPH_advection_update_vel_adv,
// sph.py:108-166, 247-262.  The list gives the pairs within h: viscosity and,
// for a particle with surface tension (phase-0 volume fraction above 0.99), the
// cohesion term of every such neighbour (zero beyond h).  The curvature term
// has no kernel weight, so -- like the reference -- it runs over every
// candidate of the template cells, not only those within h: a second loop over
// the cells that reads each candidate's normal and psi in one load.  Its only
// distance test, r > 0, needs no position: the terms it would drop are exactly
// zero, the particle's own (n_i - n_i) and that of a particle at its exact
// position (the two have the same neighbours in the same order, each leaving
// the other out, so the same normal bit for bit).  A particle whose list overflowed takes the
// reference's form with the range tests per candidate.  gs / vs scale the
// gravity / viscosity terms by 1 or 0 (kernel-level calls may leave either
// out; x * 1 is exact, so the full step's bits are unchanged).
// One-scene instances are held to 48 registers (5 blocks per SM: measured
// faster with surface tension, no spills); the batched ones would spill.
template <int DIM, bool ST, int TPP, bool M>
__global__ void __launch_bounds__(kBlock, M ? 1 : 5) k_advect(KConst k, FluidBuf F, BoundBuf B, float gs, float vs) {
    pdl_entry();
    const int64_t first = blockIdx.x * (int64_t)(kBlock / TPP);
    const int sc = f_block_scene<M>(k, first);
    const SceneConst &c = scene<M>(k, sc);
    const SceneStep &st = k.ss[sc];
    const Lanes<TPP> ln;
    const int64_t s = ln.s;
    const bool act = s - c.f_slot < c.f_n;
    Geo g;
    g.load(c, k.R);
    const int cur = st.cur;
    const float4 *vin = F.vadv + cur * F.cap;
    float vx = 0.f, vy = 0.f, vz = 0.f;   // viscosity sum
    float sx = 0.f, sy = 0.f, sz = 0.f;   // surface tension sum
    float4 vi = make_float4(0.f, 0.f, 0.f, 0.f);
    if (act) {
        const float4 pi = F.pos[s];
        vi = vin[s];
        const float4 mpi = F.mpsi[s];
        const float4 ni = ST ? F.normal[s] : make_float4(0.f, 0.f, 0.f, 0.f);
        const bool st_i = ST && has_surf_tension(ni);
        const float lap = 2.f * (2.f + DIM);
        const float eps = 0.01f * g.h2;
        const float gamma = c.gamma, c_coh = c.c_coh;
        const long long f_shift = shift_of<M>(st.f_shift);
        // every term of one candidate, with the reference's range tests
        auto pair = [&](int j) {
            const float4 pj = F.pos[j];
            const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (!(r2 > 0.f)) return;
            const bool near = r2 < g.h2;
            float r = 0.f, ri = 0.f, mj = 0.f;
            if (near) {
                const float4 vj = vin[j];
                const float4 mpj = F.mpsi[j];
                mj = mpj.x;
                ri = pair_rinv(r2, r);
                const float wg = kwg(r * g.inv_h) * g.sig_h;
                const float adx = (vi.x - vj.x) * dx + (vi.y - vj.y) * dy + (vi.z - vj.z) * dz;
                const float f = __fdividef(lap * __fdividef(pj.w, mpj.y) * wg * ri * adx, eps + r2);
                vx += f * dx;
                vy += f * dy;
                vz += f * dz;
            }
            if (ST && st_i) {
                const float4 nj = F.normal[j];   // w: the neighbour's psi
                if (has_surf_tension(nj)) {
                    const float coh = near ? -gamma * mj * (kcoh(r * g.inv_h) * c_coh) * ri : 0.f;
                    const float fac = __fdividef(2.f * mpi.z, mpi.y + nj.w);
                    sx += fac * (coh * dx + gamma * (ni.x - nj.x));
                    sy += fac * (coh * dy + gamma * (ni.y - nj.y));
                    sz += fac * (coh * dz + gamma * (ni.z - nj.z));
                }
            }
        };
        const bool exact = ST && st_i && F.nbr_cnt[s] == kNbrOverflow;
        bool ok = false;
        long long code = 0;
        if (ST && st_i) code = cell_code<DIM>(pi, g, ok);
        if (exact) {
            if (ok) visit_candidates<DIM, TPP>(F.start, g, code, f_shift, ln.q, pair);
        } else {
            // list entries skip the range tests and load their neighbour's v_adv
            // and psi together with its position
            for_each_neighbor_tpp<DIM, false, TPP, M>(c, st, k.R, F, B, s, ln.q, pi,
                [&](int j, auto listed) {
                    constexpr bool L = decltype(listed)::value;
                    if (!L) {
                        pair(j);  // (a particle with surface tension is not here)
                        return;
                    }
                    const float4 pj = F.pos[j];
                    const float4 vj = vin[j];
                    const float psij = vj.w;  // the neighbour's psi, set by the density sweep
                    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    float r;
                    const float ri = pair_rinv_pos(r2, r);
                    const float wg = kwg(r * g.inv_h) * g.sig_h;
                    const float adx = (vi.x - vj.x) * dx + (vi.y - vj.y) * dy + (vi.z - vj.z) * dz;
                    // the two quotients by __fdividef (within 2 ulp, far inside the
                    // 1e-5 bar), as on every per-pair path of these sweeps
                    const float f = __fdividef(lap * __fdividef(pj.w, psij) * wg * ri * adx, eps + r2);
                    vx += f * dx;
                    vy += f * dy;
                    vz += f * dz;
                    if (ST && st_i) {
                        const float4 nj = F.normal[j];
                        if (has_surf_tension(nj)) {
                            const float mj = F.mv[j].x;
                            const float coh = -gamma * mj * (kcoh(r * g.inv_h) * c_coh) * ri;
                            const float fac = __fdividef(2.f * mpi.z, mpi.y + nj.w);
                            sx += fac * (coh * dx);
                            sy += fac * (coh * dy);
                            sz += fac * (coh * dz);
                        }
                    }
                },
                [&](int, auto) {});
            if (ST && st_i && ok) {
                // the curvature term over every candidate of the template cells
                visit_candidates<DIM, TPP>(F.start, g, code, f_shift, ln.q, [&](int j) {
                    const float4 nj = F.normal[j];
                    if (has_surf_tension(nj)) {
                        const float fac = __fdividef(2.f * mpi.z, mpi.y + nj.w);
                        sx += fac * (gamma * (ni.x - nj.x));
                        sy += fac * (gamma * (ni.y - nj.y));
                        sz += fac * (gamma * (ni.z - nj.z));
                    }
                });
            }
        }
    }
    vx = ln.sum(vx);
    vy = ln.sum(vy);
    vz = ln.sum(vz);
    if (ST) {
        sx = ln.sum(sx);
        sy = ln.sum(sy);
        sz = ln.sum(sz);
    }
    if (act && ln.q == 0) {
        float4 *vout = F.vadv + (1 - cur) * F.cap;
        const float dt = k.sp[sc].dt;
        const float mu = (c.mu * vs) / F.rho0[s];
        const float ax = c.g[0] * gs + vx * mu + sx;
        const float ay = c.g[1] * gs + vy * mu + sy;
        const float az = (DIM == 3 ? c.g[2] * gs : 0.f) + vz * mu + sz;
        F.acc[s] = make_float4(ax, ay, az, 0.f);
        F.vel[s] = vi;
        vout[s] = make_float4(vi.x + ax * dt, vi.y + ay * dt, vi.z + az * dt, 0.f);
    }
}

// ----------------------------------------------------------------------------- launchers
// One-scene (M = false) or batched (M = true) kernel instances.
#define TSPH_M_DISPATCH(MULTI, ...)                                       \
    if (MULTI) { constexpr bool M = true; __VA_ARGS__; }                   \
    else { constexpr bool M = false; __VA_ARGS__; }

// The boundary particles' own sums run on the side stream beside the fluid
// sweep: neither writes what the other reads.
void launch_density(tsph_ctx &c, cudaStream_t st) {
    c.launches += 2;
    cudaStream_t sd = c.side ? c.side : st;
    fork_side(c, st);
    TSPH_M_DISPATCH(c.n_scenes > 1,
        if (c.k.dim == 3) {
            TSPH_LAUNCH((k_density_bound<3, M>), blocks_for(c.B.cap), kBlock, sd, c.k, c.F, c.B);
            TSPH_LAUNCH((k_density_fluid<3, M>), blocks_for(c.F.cap), kBlock, st, c.k, c.F, c.B, c.S.partials);
        } else {
            TSPH_LAUNCH((k_density_bound<2, M>), blocks_for(c.B.cap), kBlock, sd, c.k, c.F, c.B);
            TSPH_LAUNCH((k_density_fluid<2, M>), blocks_for(c.F.cap), kBlock, st, c.k, c.F, c.B, c.S.partials);
        })
    join_side(c, st);
}

// Measurement only: lets the next psi sweep run in full although the density
// sweep did its first iteration's work.
__global__ void k_clear_psi_ready(KConst k) {
    pdl_entry();
    for (int s = threadIdx.x; s < k.n_scenes; s += blockDim.x) k.ss[s].psi_ready = 0;
}

void launch_clear_psi_ready(tsph_ctx &c, cudaStream_t st) { TSPH_LAUNCH((k_clear_psi_ready), 1, 256, st, c.k); }

__global__ void k_status_or(KConst k, int bits) {
    pdl_entry();
    atomicOr(&k.ss[0].status, bits);
}

void launch_status_or(tsph_ctx &c, int bits, cudaStream_t st) { TSPH_LAUNCH((k_status_or), 1, 1, st, c.k, bits); }

void launch_solve_begin(tsph_ctx &c, int kind, cudaGraphConditionalHandle h, int use_cond, cudaStream_t st) {
    c.launches += 1;
    TSPH_LAUNCH((k_solve_begin), 1, 256, st, c.k, kind, kind == kSolveDens ? 1 : 0, h, use_cond);
}

// Threads per particle of the list sweeps (1, 2, 4 or 8); see Lanes.
#define TSPH_TPP_DISPATCH(TPP_VAL, ...)                                   \
    switch (TPP_VAL) {                                                     \
        case 2: { constexpr int TPP = 2; __VA_ARGS__; } break;             \
        case 4: { constexpr int TPP = 4; __VA_ARGS__; } break;             \
        case 8: { constexpr int TPP = 8; __VA_ARGS__; } break;             \
        default: { constexpr int TPP = 1; __VA_ARGS__; } break;            \
    }

static int tpp_blocks(int64_t slots, int tpp) { return blocks_for(slots * tpp); }

void launch_psi(tsph_ctx &c, cudaStream_t st, int force) {
    c.launches += 1;
    const int tpp = c.tpp;
    const int nb = tpp_blocks(c.F.cap, tpp);
    TSPH_M_DISPATCH(c.n_scenes > 1, TSPH_TPP_DISPATCH(tpp,
        if (c.k.dim == 3) TSPH_LAUNCH((k_psi<3, TPP, M>), nb, kBlock, st, c.k, c.F, c.B, c.S.partials, force);
        else TSPH_LAUNCH((k_psi<2, TPP, M>), nb, kBlock, st, c.k, c.F, c.B, c.S.partials, force)))
}

void launch_vel(tsph_ctx &c, int kind, cudaGraphConditionalHandle h, int use_cond, cudaStream_t st, int force) {
    c.launches += 1;
    const int tpp = c.tpp;
    const int nb = tpp_blocks(c.F.cap, tpp);
    TSPH_M_DISPATCH(c.n_scenes > 1, TSPH_TPP_DISPATCH(tpp,
        if (c.k.dim == 3) TSPH_LAUNCH((k_vel<3, TPP, M>), nb, kBlock, st, c.k, c.F, c.B, kind, h, use_cond, force);
        else TSPH_LAUNCH((k_vel<2, TPP, M>), nb, kBlock, st, c.k, c.F, c.B, kind, h, use_cond, force)))
}

void launch_solve_iter(tsph_ctx &c, int kind, cudaGraphConditionalHandle h, int use_cond, cudaStream_t st) {
    launch_psi(c, st);
    launch_vel(c, kind, h, use_cond, st);
}

void launch_advect(tsph_ctx &c, cudaStream_t st, int terms) {
    const int tpp = c.tpp;
    const int nb = tpp_blocks(c.F.cap, tpp);
    const bool st_on = c.st_on != 0 && (terms & TSPH_TERM_SURFACE_TENSION);
    const float gs = (terms & TSPH_TERM_GRAVITY) ? 1.f : 0.f, vs = (terms & TSPH_TERM_VISCOSITY) ? 1.f : 0.f;
    c.launches += st_on ? 2 : 1;
    TSPH_M_DISPATCH(c.n_scenes > 1, TSPH_TPP_DISPATCH(tpp,
        if (c.k.dim == 3) {
            if (st_on) {
                TSPH_LAUNCH((k_normal<3, TPP, M>), nb, kBlock, st, c.k, c.F, c.B);
                TSPH_LAUNCH((k_advect<3, true, TPP, M>), nb, kBlock, st, c.k, c.F, c.B, gs, vs);
            } else {
                TSPH_LAUNCH((k_advect<3, false, TPP, M>), nb, kBlock, st, c.k, c.F, c.B, gs, vs);
            }
        } else {
            if (st_on) {
                TSPH_LAUNCH((k_normal<2, TPP, M>), nb, kBlock, st, c.k, c.F, c.B);
                TSPH_LAUNCH((k_advect<2, true, TPP, M>), nb, kBlock, st, c.k, c.F, c.B, gs, vs);
            } else {
                TSPH_LAUNCH((k_advect<2, false, TPP, M>), nb, kBlock, st, c.k, c.F, c.B, gs, vs);
            }
        }))
}

}  // namespace tsph
