// Weakly compressible pressure block and the particle-to-grid velocity map --
// the two per-step kernels the reference ships commented out in sph_step
// (main.py:238-242 and main.py:254).
//
// Weakly compressible block (after the density solve, before the volume-fraction
// update): WC_pressure_val (sph.py:169-176) per fluid particle,
// p = rho0 cs^2 / gamma ((rho / rho0)^7 - 1) clamped at 0 with rho the step's
// sph_density; WC_pressure_acce (sph.py:179-193) over the fluid and boundary
// pairs of the step's neighbour list, acce_adv_i -= (p_i / rho_i^2 + p_j /
// rho_j^2) m_j W'(r) x_ij / r; then SPH_advection_update_vel_adv
// (sph.py:247-250), which sets v_adv = vel + acce_adv dt and so replaces the
// density solve's correction -- the reference's semantics when the block is on.
// The boundary's pressure is whatever its set holds (the reference never
// writes it).
#include <cuda_runtime.h>

#include "ctx.h"

namespace tsph {

namespace {

// (rho / rho0)^7 by squaring, as an integer power.
__device__ __forceinline__ float pow7(float r) {
    const float r2 = r * r;
    const float r4 = r2 * r2;
    return r4 * r2 * r;
}

template <bool M>
__global__ void __launch_bounds__(kBlock) k_wc_pressure(KConst k, FluidBuf F, BoundBuf B, const float *bpress) {
    pdl_entry();
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (s < F.cap) {
        const SceneConst &c = scene<M>(k, f_block_scene<M>(k, s - (s % kChunk)));
        if (s - c.f_slot < c.f_n) {
            const float rho = F.dens[s].y, rho0 = F.rho0[s];
            float p = (rho0 * (float)(c.cs * c.cs)) / (float)c.wc_gamma * (pow7(rho / rho0) - 1.f);
            if (p < 0.f) p = 0.f;
            F.wcp[s] = make_float2(p, p / (rho * rho));
        }
    }
    if (s < B.cap) {
        const SceneConst &c = scene<M>(k, b_block_scene<M>(k, s - (s % kChunk)));
        if (s - c.b_slot < c.b_n) {
            const float p = bpress ? bpress[B.perm[s]] : 0.f;
            const float rho = B.dens[s].y;
            B.wcp2[s] = p / (rho * rho);
        }
    }
}

template <int DIM, bool M>
__global__ void __launch_bounds__(kBlock) k_wc_acce(KConst k, FluidBuf F, BoundBuf B) {
    pdl_entry();
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    const int sc = f_block_scene<M>(k, blockIdx.x * (int64_t)kBlock);
    const SceneConst &c = scene<M>(k, sc);
    if (s - c.f_slot >= c.f_n) return;
    const SceneStep &st = k.ss[sc];
    const float h2 = c.h2, inv_h = c.inv_h, sig_h = c.sig_h;
    const float4 pi = F.pos[s];
    const float pri = F.wcp[s].y;
    float ax = 0.f, ay = 0.f, az = 0.f;
    auto term = [&](float4 pj, float prj, float mj) {
        const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        if (r2 < h2 && r2 > 0.f) {
            float r;
            const float ri = pair_rinv_pos(r2, r);  // rsqrt pair geometry, as the other sweeps
            const float f = -(pri + prj) * mj * (kwg(r * inv_h) * sig_h) * ri;
            ax += f * dx;
            ay += f * dy;
            az += f * dz;
        }
    };
    for_each_neighbor_tpp<DIM, true, 1, M>(c, st, k.R, F, B, s, 0, pi,
        [&](int j, auto) { term(F.pos[j], F.wcp[j].y, F.mv[j].x); },
        [&](int j, auto) { term(B.pos[j], B.wcp2[j], B.mv[j].x); });
    const float4 a0 = F.acc[s];
    const float4 a = make_float4(a0.x + ax, a0.y + ay, a0.z + az, 0.f);
    F.acc[s] = a;
    const float dt = k.sp[sc].dt;
    const float4 v = F.vel[s];
    F.vadv[st.cur * F.cap + s] = make_float4(v.x + a.x * dt, v.y + a.y * dt, v.z + a.z * dt, 0.f);
}

// map_velocity over the nodes of a regular grid (C order), one thread per node.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_map_velocity(KConst k, FluidBuf F, tsph_set U, float lb0, float lb1,
                                                         float lb2, float dist, int n0, int n1, int n2,
                                                         float *out) {
    pdl_entry();
    const int64_t I = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    const int64_t total = (int64_t)n0 * n1 * (DIM == 3 ? n2 : 1);
    if (I >= total) return;
    const SceneConst &c = k.s0;
    int idx[3];
    int64_t r = I;
    if (DIM == 3) {
        idx[2] = (int)(r % n2);
        r /= n2;
    } else {
        idx[2] = 0;
    }
    idx[1] = (int)(r % n1);
    idx[0] = (int)(r / n1);
    const float4 gp = make_float4(lb0 + (float)idx[0] * dist, lb1 + (float)idx[1] * dist,
                                  DIM == 3 ? lb2 + (float)idx[2] * dist : 0.f, 0.f);
    Geo g;
    g.load(c, k.R);
    bool ok;
    const long long code = cell_code<DIM>(gp, g, ok);
    const bool vf = k.vfsph != 0;
    float vx = 0.f, vy = 0.f, vz = 0.f;
    if (ok) {
        visit_candidates<DIM>(F.start, g, code, 0, 0, [&](int j) {
            const int64_t pid = F.perm[j];
            const float *p = U.pos + pid * DIM;
            const float dx = gp.x - p[0], dy = gp.y - p[1], dz = DIM == 3 ? gp.z - p[2] : 0.f;
            const float w = kw(sqrtf(dx * dx + dy * dy + dz * dz) * g.inv_h) * g.sig;
            const float X = vf ? U.rest_volume[pid] : U.mass[pid];
            const float psi = vf ? U.sph_compression[pid] : U.sph_density[pid];
            const float f = X / psi * w;
            const float *v = U.vel + pid * DIM;
            vx += f * v[0];
            vy += f * v[1];
            if (DIM == 3) vz += f * v[2];
        });
    }
    out[I * DIM] = vx;
    out[I * DIM + 1] = vy;
    if (DIM == 3) out[I * DIM + 2] = vz;
}

}  // namespace

void launch_wc(tsph_ctx &c, const tsph_set &b, cudaStream_t st) {
    const int64_t n = c.F.cap > c.B.cap ? c.F.cap : c.B.cap;
    c.launches += 2;
    if (c.n_scenes > 1) {
        TSPH_LAUNCH((k_wc_pressure<true>), blocks_for(n), kBlock, st, c.k, c.F, c.B, b.pressure);
        if (c.k.dim == 3) TSPH_LAUNCH((k_wc_acce<3, true>), blocks_for(c.F.cap), kBlock, st, c.k, c.F, c.B);
        else TSPH_LAUNCH((k_wc_acce<2, true>), blocks_for(c.F.cap), kBlock, st, c.k, c.F, c.B);
    } else {
        TSPH_LAUNCH((k_wc_pressure<false>), blocks_for(n), kBlock, st, c.k, c.F, c.B, b.pressure);
        if (c.k.dim == 3) TSPH_LAUNCH((k_wc_acce<3, false>), blocks_for(c.F.cap), kBlock, st, c.k, c.F, c.B);
        else TSPH_LAUNCH((k_wc_acce<2, false>), blocks_for(c.F.cap), kBlock, st, c.k, c.F, c.B);
    }
}

void set_last_error_text(const char *msg);

}  // namespace tsph

using namespace tsph;

extern "C" int tsph_map_velocity(tsph_ctx *c, const tsph_set *f, const float *lb, float dist, const int32_t *shape,
                                 float *grid_vel, void *stream) {
    if (!c || !f || !lb || !shape || !grid_vel) {
        set_last_error_text("null argument");
        return TSPH_ERR_INVALID;
    }
    if (c->n_scenes != 1) {
        set_last_error_text("tsph_map_velocity takes a one-scene context");
        return TSPH_ERR_INVALID;
    }
    if (!c->stepped) {
        set_last_error_text("tsph_map_velocity needs the cell grid of a step");
        return TSPH_ERR_STATE;
    }
    const int dim = c->k.dim;
    int64_t total = 1;
    for (int d = 0; d < dim; ++d) {
        if (shape[d] < 1) {
            set_last_error_text("grid shape must be positive");
            return TSPH_ERR_INVALID;
        }
        total *= shape[d];
    }
    if (total > 0x7fffffffll) {
        set_last_error_text("grid too large");
        return TSPH_ERR_INVALID;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const int nb = blocks_for(total);
    if (dim == 3)
        k_map_velocity<3><<<nb, kBlock, 0, st>>>(c->k, c->F, *f, lb[0], lb[1], lb[2], dist, shape[0], shape[1],
                                                 shape[2], grid_vel);
    else
        k_map_velocity<2><<<nb, kBlock, 0, st>>>(c->k, c->F, *f, lb[0], lb[1], 0.f, dist, shape[0], shape[1], 1,
                                                 grid_vel);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error_text(cudaGetErrorString(e));
        return TSPH_ERR_CUDA;
    }
    return TSPH_OK;
}
