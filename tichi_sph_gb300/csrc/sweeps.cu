// Neighbour sweeps of one substep: density + alpha, the Jacobi pair of the two
// pressure solves, and the advection forces (viscosity, surface tension).
//
// One thread per particle in cell-sorted order.  The density sweep scans the
// (2r+1)^dim template rows of the fluid grid and, where the reference pairs with
// the boundary set, of the boundary grid (visit_candidates), and records every
// pair with 0 < r < h in the fluid particle's neighbour list.  The later sweeps
// of the step walk that list (for_each_neighbor_tpp) -- about 30 entries instead
// of about 220 candidates in 3D -- in the same order, so with one thread per
// particle their sums are identical to a candidate scan.  Per-particle sums are FP32 (the reference's precision);
// global sums are FP64 with a fixed summation order.
#include <cuda_runtime.h>

#include "ctx.h"

namespace tsph {

// ----------------------------------------------------------------------------- density
// SPH_clean_value + SPH_prepare_attr (f,f)(f,b) + SPH_prepare_alpha_1 (f,f)(f,b)
// + SPH_prepare_alpha_2 (f,f) + SPH_prepare_alpha (sph.py:22-38, 50-105), and the
// neighbour list of the step.
//
// Two phases keep the warps converged: the candidate scan only tests r < h and
// records the pairs with 0 < r < h (the r = 0 terms -- the particle itself and
// coincident particles -- go straight into W / rho / compression), then the
// recorded list is walked for the kernel arithmetic.  A particle whose pairs do
// not fit the list redoes the scan with the arithmetic inline.
template <int DIM>
__device__ __forceinline__ void density_pair_fluid(const KConst &k, const FluidBuf &F, float4 pi, int j,
                                                   float &wsum, float &rho, float &comp, float &a1x, float &a1y,
                                                   float &a1z, float &a2) {
    const float4 pj = F.pos[j];
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    const float r2 = dx * dx + dy * dy + dz * dz;
    if (r2 < k.h2) {
        const float2 mv = F.mv[j];
        const float r = sqrtf(r2);
        const float q = r * k.inv_h;
        const float w = kw(q) * k.sig;
        wsum += w;
        rho += w * mv.x;
        comp += w * mv.y;
        if (r2 > 0.f) {
            const float wg = kwg(q) * k.sig_h;
            const float f = pj.w * wg / r;
            a1x += f * dx;
            a1y += f * dy;
            a1z += f * dz;
            a2 += wg * wg * pj.w * pj.w / mv.x;
        }
    }
}

template <int DIM>
__device__ __forceinline__ void density_pair_bound(const KConst &k, const BoundBuf &B, float4 pi, int j,
                                                   float &wsum, float &rho, float &comp, float &a1x, float &a1y,
                                                   float &a1z) {
    const float4 pj = B.pos[j];
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    const float r2 = dx * dx + dy * dy + dz * dz;
    if (r2 < k.h2) {
        const float2 mv = B.mv[j];
        const float r = sqrtf(r2);
        const float q = r * k.inv_h;
        const float w = kw(q) * k.sig;
        wsum += w;
        rho += w * mv.x;
        comp += w * mv.y;
        if (r2 > 0.f) {
            const float f = pj.w * kwg(q) * k.sig_h / r;
            a1x += f * dx;
            a1y += f * dy;
            a1z += f * dz;
        }
    }
}

template <int DIM>
__global__ void __launch_bounds__(kBlock, 4) k_density_fluid(KConst k, FluidBuf F, BoundBuf B, int64_t n) {
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (s >= n) return;
    const float4 pi = F.pos[s];
    bool ok;
    const long long code = cell_code<DIM>(pi, k, ok);
    float wsum = 0.f, rho = 0.f, comp = 0.f, a2 = 0.f;
    float a1x = 0.f, a1y = 0.f, a1z = 0.f;
    int nfl = 0, nbo = 0;
    int *L = F.nbr;
    const int64_t stride = F.cap;
    const int cap = k.nbr_max;
    const float w0 = kw(0.f) * k.sig;
    if (ok) {
        // phase 1: record the pairs
        visit_candidates<DIM>(F.start, k, code, [&](int j) {
            const float4 pj = F.pos[j];
            const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < k.h2) {
                if (r2 > 0.f) {
                    if (nfl < cap) L[nbr_index(nfl, s, stride)] = j;
                    ++nfl;
                } else {
                    const float2 mv = F.mv[j];
                    wsum += w0;
                    rho += w0 * mv.x;
                    comp += w0 * mv.y;
                }
            }
        });
        visit_candidates<DIM>(B.start, k, code, [&](int j) {
            const float4 pj = B.pos[j];
            const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < k.h2) {
                if (r2 > 0.f) {
                    const int t = nfl + nbo;
                    if (t < cap) L[nbr_index(t, s, stride)] = j;
                    ++nbo;
                } else {
                    const float2 mv = B.mv[j];
                    wsum += w0;
                    rho += w0 * mv.x;
                    comp += w0 * mv.y;
                }
            }
        });
        if (nfl + nbo <= cap) {
            // phase 2: the arithmetic over the recorded pairs
            walk_blocks<1>(F.nbr, s, stride, 0, nfl, nfl + nbo,
                [&](int j) { density_pair_fluid<DIM>(k, F, pi, j, wsum, rho, comp, a1x, a1y, a1z, a2); },
                [&](int j) { density_pair_bound<DIM>(k, B, pi, j, wsum, rho, comp, a1x, a1y, a1z); });
        } else {
            // list overflow: one scan with the arithmetic inline
            wsum = rho = comp = a2 = a1x = a1y = a1z = 0.f;
            visit_candidates<DIM>(F.start, k, code, [&](int j) {
                density_pair_fluid<DIM>(k, F, pi, j, wsum, rho, comp, a1x, a1y, a1z, a2);
            });
            visit_candidates<DIM>(B.start, k, code, [&](int j) {
                density_pair_bound<DIM>(k, B, pi, j, wsum, rho, comp, a1x, a1y, a1z);
            });
        }
    }
    F.nbr_cnt[s] = (nfl + nbo <= cap) ? ((unsigned int)nfl | ((unsigned int)nbo << 16)) : kNbrOverflow;
    const float4 mp = F.mpsi[s];
    float alpha = (a1x * a1x + a1y * a1y + a1z * a1z) / mp.x + a2;
    if (alpha < 1e-4f) alpha = 1e-4f;
    F.W[s] = wsum;
    F.rho[s] = rho;
    F.comp[s] = comp;
    F.a1[s] = make_float4(a1x, a1y, a1z, 0.f);
    F.a2[s] = a2;
    F.mpsi[s] = make_float4(mp.x, k.vfsph ? comp : rho, mp.z, alpha);
}

// The boundary's own sums: SPH_prepare_attr (b,b)(b,f), SPH_prepare_alpha_2 (b,f),
// SPH_prepare_alpha (sph.py:50-105 as called by main.py:190-197).
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_density_bound(KConst k, FluidBuf F, BoundBuf B, int64_t n) {
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (s >= n) return;
    const float4 pi = B.pos[s];
    bool ok;
    const long long code = cell_code<DIM>(pi, k, ok);
    float wsum = 0.f, rho = 0.f, comp = 0.f, a2 = 0.f;
    if (ok) {
        visit_candidates<DIM>(B.start, k, code, [&](int j) {
            const float4 pj = B.pos[j];
            const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < k.h2) {
                const float2 mv = B.mv[j];
                const float w = kw(sqrtf(r2) * k.inv_h) * k.sig;
                wsum += w;
                rho += w * mv.x;
                comp += w * mv.y;
            }
        });
        visit_candidates<DIM>(F.start, k, code, [&](int j) {
            const float4 pj = F.pos[j];
            const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < k.h2) {
                const float2 mv = F.mv[j];
                const float q = sqrtf(r2) * k.inv_h;
                const float w = kw(q) * k.sig;
                wsum += w;
                rho += w * mv.x;
                comp += w * mv.y;
                if (r2 > 0.f) {
                    const float wg = kwg(q) * k.sig_h;
                    a2 += wg * wg * pj.w * pj.w / mv.x;
                }
            }
        });
    }
    const float m = B.mv[s].x;
    float alpha = 0.f / m + a2;
    if (alpha < 1e-4f) alpha = 1e-4f;
    B.W[s] = wsum;
    B.rho[s] = rho;
    B.comp[s] = comp;
    B.a2[s] = a2;
    B.alpha[s] = alpha;
    B.kappa[s] = B.kappa[s] / alpha;  // boundary psi_adv / alpha (psi_adv is never advanced)
}

// ----------------------------------------------------------------------------- solver
// Sets the loop condition before a solve: main.py:201 / main.py:222 test
// `iter < iter_min or compression > tol` with the compression left by the
// previous solve.  `flip` makes the v_adv written by the advection sweep current.
__global__ void k_solve_begin(KConst k, DevStep *ds, const DevPersist *dp, int kind, int flip,
                              cudaGraphConditionalHandle h, int use_cond) {
    const double tol = kind == kSolveDiv ? (double)k.div_tol : (double)k.comp_tol;
    const int cond = (0 < k.iter_min) || (dp->compression > tol);
    ds->iter = 0;
    ds->cond = cond;
    if (kind == kSolveDiv) ds->div_iter = 0;
    else ds->incom_iter = 0;
    if (flip) ds->cur = 1 - ds->cur;
    if (use_cond) cudaGraphSetConditional(h, cond ? 1u : 0u);
}

// Sweep A: IPPE_adv_psi_init + IPPE_adv_psi (f,f)(f,b) + IPPE_psi_adv_non_negative
// (sph.py:196-226), TPP threads per particle.  Writes psi_adv and kappa =
// psi_adv / alpha; the sum of psi_adv / psi0 goes to per-block partials and,
// through the last warp of the grid, to ds->psi_sum (block order, deterministic).
template <int DIM, int TPP>
__global__ void __launch_bounds__(kBlock) k_psi(KConst k, FluidBuf F, BoundBuf B, int64_t n, DevStep *ds,
                                                const DevPersist *dp, double *partials) {
    __shared__ double sh[kBlock / 32];
    __shared__ unsigned int arrived;
    if (threadIdx.x == 0) arrived = 0;
    __syncthreads();
    const Lanes<TPP> ln;
    const int64_t s = ln.s;
    const bool act = s < n;
    const float4 *vin = F.vadv + ds->cur * F.cap;
    float acc = 0.f;
    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f), vi = pi;
    if (act) {
        pi = F.pos[s];
        vi = vin[s];
        for_each_neighbor_tpp<DIM, true, TPP>(k, F, B, s, ln.q, pi,
            [&](int j) {
                const float4 pj = F.pos[j];
                const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < k.h2 && r2 > 0.f) {
                    const float4 vj = vin[j];
                    const float r = sqrtf(r2);
                    const float f = kwg(r * k.inv_h) * k.sig_h / r * pj.w;
                    acc += f * (dx * (vi.x - vj.x) + dy * (vi.y - vj.y) + dz * (vi.z - vj.z));
                }
            },
            [&](int j) {
                const float4 pj = B.pos[j];
                const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < k.h2 && r2 > 0.f) {
                    const float4 vj = B.vadv[j];
                    const float r = sqrtf(r2);
                    const float f = kwg(r * k.inv_h) * k.sig_h / r * pj.w;
                    acc += f * (dx * (vi.x - vj.x) + dy * (vi.y - vj.y) + dz * (vi.z - vj.z));
                }
            });
    }
    acc = ln.sum(acc);
    double contrib = 0.0;
    if (act && ln.q == 0) {
        const float4 mp = F.mpsi[s];
        float psi = (mp.y - mp.z) + acc * dp->dt;
        if (psi < 0.f) psi = 0.f;
        F.psiadv[s] = psi;
        F.kappa[s] = psi / mp.w;
        contrib = (double)(psi / mp.z);
    }
    double bsum;
    if (block_sum_last_warp<kBlock>(contrib, sh, &arrived, bsum)) {
        if ((threadIdx.x & 31) == 0) partials[blockIdx.x] = bsum;
        if (last_warp_done(&ds->ticket[4], gridDim.x)) {
            const int lane = threadIdx.x & 31;
            double v = 0.0;
            for (int i = lane; i < (int)gridDim.x; i += 32) v += __ldcg(partials + i);
            v = warp_sum(v);
            if (lane == 0) {
                ds->psi_sum = v;
                ds->ticket[4] = 0;
            }
        }
    }
}

// Sweep B: IPPE_update_vel_adv (f,f)(f,b), sph.py:229-244, into the other v_adv
// buffer, TPP threads per particle.  The last warp of the grid evaluates the loop
// test of main.py:201-213 / 222-234 from sweep A's sum and sets the graph's
// while-node condition.
template <int DIM, int TPP>
__global__ void __launch_bounds__(kBlock) k_vel(KConst k, FluidBuf F, BoundBuf B, int64_t n, DevStep *ds,
                                                DevPersist *dp, int kind, cudaGraphConditionalHandle h,
                                                int use_cond) {
    const Lanes<TPP> ln;
    const int64_t s = ln.s;
    const bool act = s < n;
    const int cur = ds->cur;
    float ax = 0.f, ay = 0.f, az = 0.f;
    if (act) {
        const float4 pi = F.pos[s];
        const float ki = F.kappa[s];
        const float Xi = pi.w;
        for_each_neighbor_tpp<DIM, true, TPP>(k, F, B, s, ln.q, pi,
            [&](int j) {
                const float4 pj = F.pos[j];
                const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < k.h2 && r2 > 0.f) {
                    const float kj = F.kappa[j];
                    const float r = sqrtf(r2);
                    const float f = (ki * pj.w + kj * Xi) * (kwg(r * k.inv_h) * k.sig_h / r);
                    ax += f * dx;
                    ay += f * dy;
                    az += f * dz;
                }
            },
            [&](int j) {
                const float4 pj = B.pos[j];
                const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < k.h2 && r2 > 0.f) {
                    const float kj = B.kappa[j];
                    const float r = sqrtf(r2);
                    const float f = (ki * pj.w + kj * Xi) * (kwg(r * k.inv_h) * k.sig_h / r);
                    ax += f * dx;
                    ay += f * dy;
                    az += f * dz;
                }
            });
    }
    ax = ln.sum(ax);
    ay = ln.sum(ay);
    az = ln.sum(az);
    if (act && ln.q == 0) {
        const float4 *vin = F.vadv + cur * F.cap;
        float4 *vout = F.vadv + (1 - cur) * F.cap;
        const float sc = -(1.f / dp->dt) / F.mpsi[s].x;
        const float4 vi = vin[s];
        vout[s] = make_float4(vi.x + sc * ax, vi.y + sc * ay, vi.z + sc * az, 0.f);
    }
    const unsigned int nwarps = (unsigned int)(gridDim.x * (kBlock / 32));
    if (last_warp_done(&ds->ticket[2], nwarps)) {
        if ((threadIdx.x & 31) == 0) {
            const double comp = __ldcg(&ds->psi_sum) / (double)n;
            dp->compression = comp;
            const int it = ds->iter + 1;
            ds->iter = it;
            if (kind == kSolveDiv) ds->div_iter = it;
            else ds->incom_iter = it;
            const double tol = kind == kSolveDiv ? (double)k.div_tol : (double)k.comp_tol;
            const int capped = it > k.iter_max;
            const int cond = !capped && (it < k.iter_min || comp > tol);
            if (capped) ds->status |= (kind == kSolveDiv ? TSPH_ST_DIV_ITER_CAP : TSPH_ST_DENS_ITER_CAP);
            ds->cond = cond;
            ds->cur = 1 - cur;
            ds->ticket[2] = 0;
            if (use_cond) cudaGraphSetConditional(h, cond ? 1u : 0u);
        }
    }
}

// ----------------------------------------------------------------------------- advection
// First pass of SPH_advection_surface_tension_acc, sph.py:134-150: surface normals.
template <int DIM, int TPP>
__global__ void __launch_bounds__(kBlock) k_normal(KConst k, FluidBuf F, BoundBuf B, int64_t n) {
    const Lanes<TPP> ln;
    const int64_t s = ln.s;
    const bool act = s < n;
    float nx = 0.f, ny = 0.f, nz = 0.f;
    if (act) {
        const float4 pi = F.pos[s];
        for_each_neighbor_tpp<DIM, false, TPP>(k, F, B, s, ln.q, pi,
            [&](int j) {
                const float4 pj = F.pos[j];
                const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < k.h2 && r2 > 0.f) {
                    const float r = sqrtf(r2);
                    const float f = -pj.w / F.mpsi[j].y * (kwg(r * k.inv_h) * k.sig_h) / r;
                    nx += f * dx;
                    ny += f * dy;
                    nz += f * dz;
                }
            },
            [&](int) {});
    }
    nx = ln.sum(nx);
    ny = ln.sum(ny);
    nz = ln.sum(nz);
    if (act && ln.q == 0) F.normal[s] = make_float4(nx * k.h, ny * k.h, nz * k.h, 0.f);
}

// SPH_vel_adv_2_vel + SPH_advection_gravity_acc + SPH_advection_viscosity_acc
// + (pass 2 of) SPH_advection_surface_tension_acc + SPH_advection_update_vel_adv,
// sph.py:108-166, 247-262.  The curvature term of the surface tension has no
// kernel weight, so -- like the reference -- it runs over every candidate in the
// template cells, not only those within h: with surface tension on this sweep
// scans the cells; without it, it walks the neighbour list.
template <int DIM, bool ST, int TPP>
__global__ void __launch_bounds__(kBlock) k_advect(KConst k, FluidBuf F, BoundBuf B, int64_t n,
                                                   const DevStep *ds, const DevPersist *dp) {
    const Lanes<TPP> ln;
    const int64_t s = ln.s;
    const bool act = s < n;
    const int cur = ds->cur;
    const float4 *vin = F.vadv + cur * F.cap;
    float vx = 0.f, vy = 0.f, vz = 0.f;   // viscosity sum
    float sx = 0.f, sy = 0.f, sz = 0.f;   // surface tension sum
    float4 vi = make_float4(0.f, 0.f, 0.f, 0.f);
    if (act) {
        const float4 pi = F.pos[s];
        vi = vin[s];
        const float4 mpi = F.mpsi[s];
        const float vfi0 = ST ? F.vf[s] : 0.f;
        const float4 ni = ST ? F.normal[s] : make_float4(0.f, 0.f, 0.f, 0.f);
        const bool st_i = ST && vfi0 > 0.99f;
        const float lap = 2.f * (2.f + DIM);
        const float eps = 0.01f * k.h2;
        auto pair = [&](int j) {
            const float4 pj = F.pos[j];
            const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (!(r2 > 0.f)) return;
            if (r2 < k.h2) {
                const float4 vj = vin[j];
                const float psij = F.mpsi[j].y;
                const float r = sqrtf(r2);
                const float wg = kwg(r * k.inv_h) * k.sig_h;
                const float adx = (vi.x - vj.x) * dx + (vi.y - vj.y) * dy + (vi.z - vj.z) * dz;
                const float f = lap * (pj.w / psij) * wg / r * adx / (eps + r2);
                vx += f * dx;
                vy += f * dy;
                vz += f * dz;
            }
            if (ST && st_i) {
                if (F.vf[j] > 0.99f) {
                    const float4 mpj = F.mpsi[j];
                    const float4 nj = F.normal[j];
                    const float r = sqrtf(r2);
                    const float coh = -k.gamma * mpj.x * (kcoh(r * k.inv_h) * k.c_coh) / r;
                    const float fac = 2.f * mpi.z / (mpi.y + mpj.y);
                    sx += fac * (coh * dx + k.gamma * (ni.x - nj.x));
                    sy += fac * (coh * dy + k.gamma * (ni.y - nj.y));
                    sz += fac * (coh * dz + k.gamma * (ni.z - nj.z));
                }
            }
        };
        if (ST) {
            bool ok;
            const long long code = cell_code<DIM>(pi, k, ok);
            if (ok) visit_candidates_strided<DIM, TPP>(F.start, k, code, ln.q, pair);
        } else {
            for_each_neighbor_tpp<DIM, false, TPP>(k, F, B, s, ln.q, pi, pair, [&](int) {});
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
        const float dt = dp->dt;
        const float mu = k.mu / F.rho0[s];
        const float ax = k.g[0] + vx * mu + sx;
        const float ay = k.g[1] + vy * mu + sy;
        const float az = (DIM == 3 ? k.g[2] : 0.f) + vz * mu + sz;
        F.acc[s] = make_float4(ax, ay, az, 0.f);
        F.vel[s] = vi;
        vout[s] = make_float4(vi.x + ax * dt, vi.y + ay * dt, vi.z + az * dt, 0.f);
    }
}

// ----------------------------------------------------------------------------- launchers
void launch_density(tsph_ctx &c, int64_t nf, int64_t nb, cudaStream_t st) {
    c.launches += (nf > 0) + (nb > 0);
    if (nf > 0) {
        if (c.k.dim == 3) k_density_fluid<3><<<blocks_for(nf), kBlock, 0, st>>>(c.k, c.F, c.B, nf);
        else k_density_fluid<2><<<blocks_for(nf), kBlock, 0, st>>>(c.k, c.F, c.B, nf);
    }
    if (nb > 0) {
        if (c.k.dim == 3) k_density_bound<3><<<blocks_for(nb), kBlock, 0, st>>>(c.k, c.F, c.B, nb);
        else k_density_bound<2><<<blocks_for(nb), kBlock, 0, st>>>(c.k, c.F, c.B, nb);
    }
}

void launch_solve_begin(tsph_ctx &c, int kind, cudaGraphConditionalHandle h, int use_cond, cudaStream_t st) {
    c.launches += 1;
    k_solve_begin<<<1, 1, 0, st>>>(c.k, c.ds, c.dp, kind, kind == kSolveDens ? 1 : 0, h, use_cond);
}

// Threads per particle of the list sweeps (1, 2, 4 or 8); see Lanes.
#define TSPH_TPP_DISPATCH(TPP_VAL, ...)                                   \
    switch (TPP_VAL) {                                                     \
        case 1: { constexpr int TPP = 1; __VA_ARGS__; } break;             \
        case 2: { constexpr int TPP = 2; __VA_ARGS__; } break;             \
        case 8: { constexpr int TPP = 8; __VA_ARGS__; } break;             \
        default: { constexpr int TPP = 4; __VA_ARGS__; } break;            \
    }

static int tpp_blocks(int64_t n, int tpp) { return blocks_for(n * tpp); }

void launch_psi(tsph_ctx &c, int64_t nf, cudaStream_t st) {
    c.launches += 1;
    const int tpp = c.tpp;
    const int nb = tpp_blocks(nf, tpp);
    TSPH_TPP_DISPATCH(tpp,
        if (c.k.dim == 3) k_psi<3, TPP><<<nb, kBlock, 0, st>>>(c.k, c.F, c.B, nf, c.ds, c.dp, c.S.partials);
        else k_psi<2, TPP><<<nb, kBlock, 0, st>>>(c.k, c.F, c.B, nf, c.ds, c.dp, c.S.partials));
}

void launch_vel(tsph_ctx &c, int64_t nf, int kind, cudaGraphConditionalHandle h, int use_cond, cudaStream_t st) {
    c.launches += 1;
    const int tpp = c.tpp;
    const int nb = tpp_blocks(nf, tpp);
    TSPH_TPP_DISPATCH(tpp,
        if (c.k.dim == 3) k_vel<3, TPP><<<nb, kBlock, 0, st>>>(c.k, c.F, c.B, nf, c.ds, c.dp, kind, h, use_cond);
        else k_vel<2, TPP><<<nb, kBlock, 0, st>>>(c.k, c.F, c.B, nf, c.ds, c.dp, kind, h, use_cond));
}

void launch_solve_iter(tsph_ctx &c, int64_t nf, int kind, cudaGraphConditionalHandle h, int use_cond,
                       cudaStream_t st) {
    launch_psi(c, nf, st);
    launch_vel(c, nf, kind, h, use_cond, st);
}

void launch_advect(tsph_ctx &c, int64_t nf, cudaStream_t st) {
    if (nf <= 0) return;
    const int tpp = c.tpp;
    const int nb = tpp_blocks(nf, tpp);
    const bool st_on = c.k.gamma != 0.f;
    c.launches += st_on ? 2 : 1;
    TSPH_TPP_DISPATCH(tpp,
        if (c.k.dim == 3) {
            if (st_on) {
                k_normal<3, TPP><<<nb, kBlock, 0, st>>>(c.k, c.F, c.B, nf);
                k_advect<3, true, TPP><<<nb, kBlock, 0, st>>>(c.k, c.F, c.B, nf, c.ds, c.dp);
            } else {
                k_advect<3, false, TPP><<<nb, kBlock, 0, st>>>(c.k, c.F, c.B, nf, c.ds, c.dp);
            }
        } else {
            if (st_on) {
                k_normal<2, TPP><<<nb, kBlock, 0, st>>>(c.k, c.F, c.B, nf);
                k_advect<2, true, TPP><<<nb, kBlock, 0, st>>>(c.k, c.F, c.B, nf, c.ds, c.dp);
            } else {
                k_advect<2, false, TPP><<<nb, kBlock, 0, st>>>(c.k, c.F, c.B, nf, c.ds, c.dp);
            }
        });
}

}  // namespace tsph
