// VFSPH volume-fraction update (the reference's "FBM" block), sph.py:301-379,
// driven as in main.py:244-250 (commented out there; enabled by fbm_enabled):
//
//   while general_flag:
//       clean_tmp; convect (drift velocities + convective flux); diffuse; check_tmp
//   update_volume_frac
//
// The drift velocities depend only on the step's velocities and volume
// fractions, which no pass changes, so they are computed once.  A pass sums the
// convective and diffusive flux of each unflagged particle over its unflagged
// neighbours and flags it if any phase would go negative; flags set during pass
// p (value p) do not exclude a neighbour until pass p + 1, which is what the
// reference's separate check kernel achieves.  Each scene runs its own pass
// loop; the graph loop runs while any scene does.  The number of passes is
// capped (fbm_max_passes); the reference loops forever if a flagged particle's
// own volume fraction is already negative.
#include <cuda_runtime.h>

#include "ctx.h"

namespace tsph {

__global__ void k_fbm_begin(KConst k, cudaGraphConditionalHandle h, int use_cond) {
    pdl_entry();
    __shared__ int any_sh;
    if (threadIdx.x == 0) any_sh = 0;
    __syncthreads();
    int any = 0;
    for (int s = threadIdx.x; s < k.n_scenes; s += blockDim.x) {
        SceneStep &st = k.ss[s];
        st.fbm_pass = 0;
        st.general_flag = 0;
        // SPH_clean_value sets general_flag = 1: at least one pass
        st.fbm_cond = k.sc[s].f_n > 0 ? 1 : 0;
        st.gflag_out = st.fbm_cond;
        any |= st.fbm_cond;
    }
    if (any) atomicOr(&any_sh, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        k.dg->fbm_any = any_sh;
        if (use_cond) cudaGraphSetConditional(h, any_sh ? 1u : 0u);
    }
}

// First loop of SPH_FBM_convect, sph.py:331-345.
template <int DIM, int P>
__global__ void __launch_bounds__(kBlock) k_fbm_drift(KConst k, FluidBuf F) {
    pdl_entry();
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    const int sc = k.f_chunk_scene[(blockIdx.x * (int64_t)kBlock) / kChunk];
    const SceneConst &c = k.sc[sc];
    if (s - c.f_slot >= c.f_n) return;
    const float dt = k.sp[sc].dt;
    const float4 va = F.vadv[k.ss[sc].cur * F.cap + s];
    const float4 v = F.vel[s];
    const float ax = (va.x - v.x) / dt, ay = (va.y - v.y) / dt, az = (va.z - v.z) / dt;
    const float rho0 = F.rho0[s];
    float vf[P];
    float zeta = 0.f;
#pragma unroll
    for (int q = 0; q < P; ++q) {
        vf[q] = F.vf[q * F.cap + s];
        zeta += vf[q] * (c.rho_phase[q] - rho0) / c.rho_phase[q];
    }
    const float gz = DIM == 3 ? c.g[2] : 0.f;
    const float fx = (ax - zeta * c.g[0]) / (1.f - zeta);
    const float fy = (ay - zeta * c.g[1]) / (1.f - zeta);
    const float fz = (az - zeta * gz) / (1.f - zeta);
#pragma unroll
    for (int q = 0; q < P; ++q) {
        const float cq = vf[q] * (c.rho_phase[q] - rho0);
        float dx = cq * (c.g[0] - fx), dy = cq * (c.g[1] - fy), dz = cq * (gz - fz);
        const float w = vf[q] * c.rho_phase[q];
        if (w > 1e-6f) {
            dx /= w; dy /= w; dz /= w;
        } else {
            dx *= 0.f; dy *= 0.f; dz *= 0.f;
        }
        dx += fx - ax; dy += fy - ay; dz += fz - az;
        // w: the phase's volume fraction, which no pass changes (the passes
        // read a neighbour's drift and volume fraction in one load)
        F.drift[s * P + q] = make_float4(dx * dt, dy * dt, dz * dt, vf[q]);
    }
    F.acc[s] = make_float4(ax, ay, az, 0.f);
    F.facc[s] = make_float4(fx, fy, fz, 0.f);
    F.zeta[s] = zeta;
}

// One pass: SPH_FBM_clean_tmp + pair loop of SPH_FBM_convect + SPH_FBM_diffuse +
// SPH_FBM_check_tmp (sph.py:301-372).  The scene's last block evaluates its loop
// test; the grid's last block sets the graph condition.
// Up to two phases the pass is held to 48 registers (5 blocks per SM, measured
// faster); with more phases the per-phase arrays would spill.
template <int DIM, int P>
__global__ void __launch_bounds__(kBlock, P <= 2 ? 5 : 1) k_fbm_pass(KConst k, FluidBuf F, BoundBuf B,
                                                     cudaGraphConditionalHandle h, int use_cond) {
    pdl_entry();
    __shared__ int any_neg;
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    const int sc = k.f_chunk_scene[(blockIdx.x * (int64_t)kBlock) / kChunk];
    const SceneConst &c = k.sc[sc];
    SceneStep &st = k.ss[sc];
    const bool running = st.fbm_cond != 0;
    if (threadIdx.x == 0) any_neg = 0;
    __syncthreads();
    const int pass = st.fbm_pass + 1;
    if (running && s - c.f_slot < c.f_n) {
        const int fp = F.flagpass[s];
        float tmp[P];
        float vfi[P];
#pragma unroll
        for (int q = 0; q < P; ++q) {
            tmp[q] = 0.f;
            vfi[q] = F.vf[q * F.cap + s];
        }
        if (fp == 0) {
            Geo g;
            g.load(c, k.R);
            const float dt = k.sp[sc].dt;
            const float4 pi = F.pos[s];
            float4 ui[P];
#pragma unroll
            for (int q = 0; q < P; ++q) ui[q] = F.drift[s * P + q];
            const float cc = c.fbm_c * dt, cd = dt * c.fbm_D, eps = 0.01f * g.h2;
            for_each_neighbor_tpp<DIM, false, 1, true>(c, st, k.R, F, B, s, 0, pi,
                [&](int j, auto) {
                    const float4 pj = F.pos[j];
                    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    if (!(r2 < g.h2 && r2 > 0.f)) return;
                    const int fj = F.flagpass[j];
                    if (fj != 0 && fj != pass) return;
                    // pair geometry from rsqrt and a fast quotient (as the other
                    // sweeps; within a few ulp)
                    float r;
                    const float ri = pair_rinv_pos(r2, r);
                    const float wg = kwg(r * g.inv_h) * g.sig_h;
                    const float Vj = k.vfsph ? pj.w : F.mv[j].y;  // VFSPH: X = rest volume
                    const float gx = dx * ri * wg, gy = dy * ri * wg, gz = dz * ri * wg;
                    const float dif = __fdividef(cd * Vj * r * wg, r2 + eps);
#pragma unroll
                    for (int q = 0; q < P; ++q) {
                        const float4 uj = F.drift[(int64_t)j * P + q];
                        const float vfj = uj.w;
                        const float fx = vfi[q] * ui[q].x + vfj * uj.x;
                        const float fy = vfi[q] * ui[q].y + vfj * uj.y;
                        const float fz = vfi[q] * ui[q].z + vfj * uj.z;
                        tmp[q] -= cc * Vj * (fx * gx + fy * gy + fz * gz);
                        tmp[q] += (vfi[q] - vfj) * dif;
                    }
                },
                [&](int, auto) {});
        }
        bool neg = false;
#pragma unroll
        for (int q = 0; q < P; ++q) {
            F.vftmp[q * F.cap + s] = tmp[q];
            if (vfi[q] + tmp[q] < 0.f) neg = true;
        }
        if (neg) {
            if (fp == 0) F.flagpass[s] = pass;
            any_neg = 1;
        }
    }
    __syncthreads();
    if (running) {
        if (threadIdx.x == 0 && any_neg) atomicExch(&st.general_flag, 1);
        const unsigned int nblk = (unsigned int)(c.f_slots / kBlock);
        if (last_block_done(&st.ticket[kStFbm], nblk)) {
            if (threadIdx.x == 0) {
                const int gf = atomicAdd(&st.general_flag, 0);
                st.fbm_pass = pass;
                st.fbm_passes = pass;
                st.gflag_out = gf;
                const int cond = gf && pass < c.fbm_max_passes;
                if (gf && !cond) st.status |= TSPH_ST_FBM_PASS_CAP;
                st.fbm_cond = cond;
                st.general_flag = 0;
                st.ticket[kStFbm] = 0;
            }
        }
    }
    if (last_block_done(&k.dg->ticket[kGtFbm], gridDim.x)) {
        if (threadIdx.x < 32) {
            const int lane = threadIdx.x;
            int any = 0;
            for (int q = lane; q < k.n_scenes; q += 32) any |= (__ldcg(&k.ss[q].fbm_cond) != 0);
            any = __any_sync(0xffffffffu, any);
            if (lane == 0) {
                k.dg->fbm_any = any;
                k.dg->ticket[kGtFbm] = 0;
                if (use_cond) cudaGraphSetConditional(h, any ? 1u : 0u);
            }
        }
    }
}

template <int P>
static void fbm_pass_dim(tsph_ctx &c, cudaGraphConditionalHandle h, int use_cond, cudaStream_t st, bool drift) {
    const int nb = blocks_for(c.F.cap);
    if (c.k.dim == 3) {
        if (drift) TSPH_LAUNCH((k_fbm_drift<3, P>), nb, kBlock, st, c.k, c.F);
        else TSPH_LAUNCH((k_fbm_pass<3, P>), nb, kBlock, st, c.k, c.F, c.B, h, use_cond);
    } else {
        if (drift) TSPH_LAUNCH((k_fbm_drift<2, P>), nb, kBlock, st, c.k, c.F);
        else TSPH_LAUNCH((k_fbm_pass<2, P>), nb, kBlock, st, c.k, c.F, c.B, h, use_cond);
    }
}

static void fbm_dispatch(tsph_ctx &c, cudaGraphConditionalHandle h, int use_cond, cudaStream_t st, bool drift) {
    switch (c.k.P) {
        case 1: fbm_pass_dim<1>(c, h, use_cond, st, drift); break;
        case 2: fbm_pass_dim<2>(c, h, use_cond, st, drift); break;
        case 3: fbm_pass_dim<3>(c, h, use_cond, st, drift); break;
        case 4: fbm_pass_dim<4>(c, h, use_cond, st, drift); break;
        case 5: fbm_pass_dim<5>(c, h, use_cond, st, drift); break;
        case 6: fbm_pass_dim<6>(c, h, use_cond, st, drift); break;
        case 7: fbm_pass_dim<7>(c, h, use_cond, st, drift); break;
        default: fbm_pass_dim<8>(c, h, use_cond, st, drift); break;
    }
}

void launch_fbm_begin(tsph_ctx &c, cudaGraphConditionalHandle h, int use_cond, cudaStream_t st) {
    cudaMemsetAsync(c.F.flagpass, 0, sizeof(int) * c.F.cap, st);
    c.launches += 2;
    fbm_dispatch(c, 0, 0, st, true);
    TSPH_LAUNCH((k_fbm_begin), 1, 256, st, c.k, h, use_cond);
}

void launch_fbm_pass(tsph_ctx &c, cudaGraphConditionalHandle h, int use_cond, cudaStream_t st) {
    c.launches += 1;
    fbm_dispatch(c, h, use_cond, st, false);
}

}  // namespace tsph
