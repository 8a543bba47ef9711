// Hand-written reverse mode of the DFSPH substep.
//
// Forward (recorded): density + alpha (sph.py:50-105), the divergence-free
// Jacobi solve (main.py:199-214), gravity + viscosity (sph.py:108-129), the
// constant-density Jacobi solve (main.py:221-234) and the position update
// (sph.py:265-269), with dt, iteration counts and neighbour pairs fixed.
//
// Reverse, one thread per fluid particle in the recorded sorted order, every
// sweep a gather over the recorded neighbour list (no atomics; deterministic):
//
//   one Jacobi iteration u' = u - (1/(dt m_i)) sum_j (k_i X_j + k_j X_i) g_ij r_ij,
//   k = max(s, 0) / alpha, s_i = psi_i - psi0_i + dt sum_j X_j g_ij r_ij.(u_i - u_j)
//   (g(r) = W'(r)/r, r_ij = x_i - x_j) reverses into two sweeps with the
//   transposed structure -- the velocity update's adjoint is a divergence of
//   beta = lam_u' / (dt m) and the divergence's adjoint is a pressure-force-
//   shaped sum of lam_s:
//     k_adj_kappa: lam_k_i = -sum_j X_j g r_ij.(beta_i - beta_j) (- boundary),
//                  lam_s = [s > 0] lam_k / alpha, lam_alpha -= lam_k k / alpha,
//                  lam_psi += lam_s, lam_x += d/dx of the update's pair terms;
//     k_adj_vel:   lam_u = lam_u' + dt sum_j (lam_s_i X_j + lam_s_j X_i) g r_ij,
//                  lam_x += d/dx of the divergence's pair terms;
//   k_adj_visc reverses a = g + mu V(x, v, psi) (and yields dL/dmu);
//   k_adj_st1 / k_adj_st2 reverse the surface tension (sph.py:132-166): its
//     cohesion and curvature over the template candidates, then the normals;
//   k_adj_density reverses the density and alpha sums.
// The position derivative of a pair term g(r) r_ij . w is g w + (g'(r)/r)(r_ij . w) r_ij
// with g'(r)/r = (W''(r) - g(r)) / r^2.  Each pair appears in both particles'
// lists (fluid-fluid), so the terms a pair contributes through the other
// particle's sums are gathered too; boundary particles are static.
//
// The same formulas are restated in FP64 PyTorch in the autodiff oracle and
// checked there against torch.autograd and central finite differences.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <new>

#include "ctx.h"
#include "tape.h"

namespace tsph {

void set_last_error_text(const char *msg);

namespace {

// w''(q) of the cubic spline (the derivative of kwg).
__device__ __forceinline__ float kwgg(float q) {
    return q <= 0.5f ? 6.f * (6.f * q - 2.f) : (q < 1.f ? 12.f * (1.f - q) : 0.f);
}

// Derivative of the cohesion spline shape kcoh: 3 q^2 (1 - q)^2 (1 - 2 q),
// doubled below q = 1/2.
__device__ __forceinline__ float kcohd(float q) {
    const float b = 1.f - q;
    const float t = 3.f * q * q * b * b * (1.f - 2.f * q);
    return q <= 0.5f ? 2.f * t : (q < 1.f ? t : 0.f);
}

// ----------------------------------------------------------------------------- recording
__global__ void k_tape_begin(TapeArrays a, int slot) {
    *a.dslot = slot;
    TapeMeta z;
    memset(&z, 0, sizeof(z));
    a.meta[slot] = z;
}

__global__ void __launch_bounds__(kBlock) k_tape_state(KConst k, FluidBuf F, BoundBuf B, TapeArrays a) {
    const int slot = *a.dslot;
    const SceneConst &c = k.s0;
    const SceneStep &st = k.ss[0];
    TapeMeta &m = a.meta[slot];
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (s < c.f_n) {
        const int64_t o = slot * a.cap + s;
        a.perm[o] = F.perm[s];
        a.pos[o] = F.pos[s];
        a.mpsi[o] = F.mpsi[s];
        a.a1[o] = F.a1[s];
        a.a2[o] = F.dens[s].w;
        a.rho0[o] = F.rho0[s];
        if (a.vf0) a.vf0[o] = F.vf[s];
        const unsigned int pc = F.nbr_cnt[s];
        a.cnt[o] = pc;
        if (pc == kNbrOverflow) {
            atomicOr(&m.status, TSPH_TAPE_LIST_OVERFLOW);
        } else {
            const int nb4 = ((int)(pc & 0xffffu) + (int)(pc >> 16) + 3) >> 2;
            const int4 *src = reinterpret_cast<const int4 *>(F.nbr) + s;
            int4 *dst = reinterpret_cast<int4 *>(a.nbr + (int64_t)slot * a.nbr_max * a.cap) + s;
            for (int b = 0; b < nb4; ++b) dst[(int64_t)b * a.cap] = src[(int64_t)b * F.cap];
        }
    }
    if (s < c.b_n) {
        const int64_t o = slot * a.bcap + s;
        a.bpos[o] = B.pos[s];
        a.bvel[o] = B.vadv[s];
        if (B.kappa[s] != 0.f) atomicOr(&m.status, TSPH_TAPE_BOUND_PSI);
    }
    if (s == 0) {
        m.n = (int32_t)c.f_n;
        m.nb = (int32_t)c.b_n;
        m.f_in = st.f_in;
        m.dt = k.sp[0].dt;
        m.mu = c.mu;
        if (st.f_in != c.f_n) atomicOr(&m.status, TSPH_TAPE_OUTSIDE_GRID);
    }
}

// The iterate u^k read by the psi sweep and the kappa it wrote (between the two
// sweeps of iteration k = st.iter).
__global__ void __launch_bounds__(kBlock) k_tape_iter(KConst k, FluidBuf F, int kind, TapeArrays a) {
    const SceneStep &st = k.ss[0];
    if (!st.cond) return;
    const int slot = *a.dslot;
    const int it = st.iter;
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (it >= a.max_iters) {
        if (s == 0) atomicOr(&a.meta[slot].status, TSPH_TAPE_ITER_OVERFLOW);
        return;
    }
    if (s >= k.s0.f_n) return;
    const int64_t o = (((int64_t)slot * 2 + kind) * a.max_iters + it) * a.cap + s;
    a.u[o] = F.vadv[st.cur * F.cap + s];
    a.kap[o] = F.kappa[s];
}

__global__ void __launch_bounds__(kBlock) k_tape_vmid(KConst k, FluidBuf F, TapeArrays a) {
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (s >= k.s0.f_n) return;
    a.vmid[*a.dslot * a.cap + s] = F.vel[s];
    if (a.nrm) a.nrm[*a.dslot * a.cap + s] = F.normal[s];
}

// The fluid grid's cell starts of the recorded substep (surface tension on: its
// reverse visits the same template candidates as the forward).
__global__ void __launch_bounds__(kBlock) k_tape_start(FluidBuf F, TapeArrays a) {
    const int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (i < a.nstart) a.start[(int64_t)(*a.dslot) * a.nstart + i] = F.start[i];
}

__global__ void k_tape_end(KConst k, TapeArrays a) {
    TapeMeta &m = a.meta[*a.dslot];
    m.kd = k.ss[0].div_iter;
    m.kp = k.ss[0].incom_iter;
}

__global__ void __launch_bounds__(kBlock) k_density_out(KConst k, FluidBuf F, float *out) {
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (s >= k.s0.f_n) return;
    out[F.perm[s]] = F.dens[s].y;
}

// ----------------------------------------------------------------------------- reverse
// One recorded slot, offset to its arrays.
struct SlotView {
    const int *perm;
    const float4 *pos, *mpsi, *a1, *vmid, *bpos, *bvel;
    const float *a2, *rho0;
    const unsigned int *cnt;
    const int *nbr;
    const float4 *u;     // [2][max_iters][cap]
    const float *kap;
    const float4 *nrm;   // surface tension on: normals, phase-0 volume fractions, cell starts
    const float *vf0;
    const int *start;
    Geo geo;
    int64_t cap;
    int n, max_iters;
    float dt, mu, h, h2, inv_h, sig_h, eps, gamma, c_coh;
};

// Pair geometry of r_ij = pi - pj (0 < r < h): g = W'(r)/r, G2 = g'(r)/r, W2 = W''(r).
struct Pair {
    float x, y, z, r2, g, G2, W2;
    __device__ __forceinline__ Pair(const SlotView &v, float4 pi, float4 pj) {
        x = pi.x - pj.x;
        y = pi.y - pj.y;
        z = pi.z - pj.z;
        r2 = x * x + y * y + z * z;
        // r and 1 / r from rsqrt, as the forward sweeps (within a few ulp)
        float r;
        const float ri = pair_rinv_pos(r2, r);
        const float q = r * v.inv_h;
        g = kwg(q) * v.sig_h * ri;
        W2 = kwgg(q) * v.sig_h * v.inv_h;
        G2 = (W2 - g) * (ri * ri);
    }
    __device__ __forceinline__ float dot(float ax, float ay, float az) const { return x * ax + y * ay + z * az; }
};

template <class FF, class FB>
__device__ __forceinline__ void for_pairs(const SlotView &v, int64_t s, FF &&ff, FB &&fb) {
    const unsigned int pc = v.cnt[s];
    const int nfl = (int)(pc & 0xffffu), nbo = (int)(pc >> 16);
    walk_blocks<1>(v.nbr, s, v.cap, 0, nfl, nfl + nbo, ff, fb);
}

template <int DIM>
__global__ void __launch_bounds__(kBlock) k_adj_in(SlotView v, const float *__restrict__ gx, const float *__restrict__ gv,
                                                   float4 *lx, float4 *lu, float *lpsi, float *lalpha) {
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (s >= v.n) return;
    const int64_t b = (int64_t)v.perm[s] * DIM;
    const float x0 = gx[b], x1 = gx[b + 1], x2 = DIM == 3 ? gx[b + 2] : 0.f;
    const float v0 = gv[b], v1 = gv[b + 1], v2 = DIM == 3 ? gv[b + 2] : 0.f;
    lx[s] = make_float4(x0, x1, x2, 0.f);
    // x' = x + v' dt: the step's velocity output also moved the positions
    lu[s] = make_float4(v0 + v.dt * x0, v1 + v.dt * x1, v2 + v.dt * x2, 0.f);
    lpsi[s] = 0.f;
    lalpha[s] = 0.f;
}

__global__ void __launch_bounds__(kBlock) k_adj_kappa(SlotView v, int kind, int it, const float4 *__restrict__ lu,
                                                      float *ls, float4 *lx, float *lpsi, float *lalpha) {
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (s >= v.n) return;
    const float *kap = v.kap + ((int64_t)kind * v.max_iters + it) * v.cap;
    const float4 pi = v.pos[s];
    const float mi = pi.w;
    const float ki = kap[s];
    const float4 lui = lu[s];
    const float inv = 1.f / (v.dt * mi);
    const float bx = lui.x * inv, by = lui.y * inv, bz = lui.z * inv;
    float lk = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
    for_pairs(v, s,
        [&](int j) {
            const float4 pj = v.pos[j];
            const Pair P(v, pi, pj);
            const float4 luj = lu[j];
            const float invj = 1.f / (v.dt * pj.w);
            const float dx = bx - luj.x * invj, dy = by - luj.y * invj, dz = bz - luj.z * invj;
            const float rd = P.dot(dx, dy, dz);
            lk -= pj.w * P.g * rd;
            const float cK = ki * pj.w + kap[j] * mi;
            gx -= cK * (P.g * dx + P.G2 * rd * P.x);
            gy -= cK * (P.g * dy + P.G2 * rd * P.y);
            gz -= cK * (P.g * dz + P.G2 * rd * P.z);
        },
        [&](int b) {
            const float4 pb = v.bpos[b];
            const Pair P(v, pi, pb);
            const float rd = P.dot(bx, by, bz);
            lk -= pb.w * P.g * rd;
            const float cK = ki * pb.w;
            gx -= cK * (P.g * bx + P.G2 * rd * P.x);
            gy -= cK * (P.g * by + P.G2 * rd * P.y);
            gz -= cK * (P.g * bz + P.G2 * rd * P.z);
        });
    const float alpha = v.mpsi[s].w;
    const float lsi = ki > 0.f ? lk / alpha : 0.f;
    lalpha[s] -= lk * ki / alpha;
    lpsi[s] += lsi;
    ls[s] = lsi;
    const float4 o = lx[s];
    lx[s] = make_float4(o.x + gx, o.y + gy, o.z + gz, 0.f);
}

__global__ void __launch_bounds__(kBlock) k_adj_vel(SlotView v, int kind, int it, const float *__restrict__ ls,
                                                    float4 *lu, float4 *lx) {
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (s >= v.n) return;
    const float4 *u = v.u + ((int64_t)kind * v.max_iters + it) * v.cap;
    const float4 pi = v.pos[s];
    const float mi = pi.w;
    const float4 ui = u[s];
    const float lsi = ls[s];
    float ax = 0.f, ay = 0.f, az = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
    auto term = [&](const Pair &P, float cS, float4 uj) {
        ax += cS * P.g * P.x;
        ay += cS * P.g * P.y;
        az += cS * P.g * P.z;
        const float dx = ui.x - uj.x, dy = ui.y - uj.y, dz = ui.z - uj.z;
        const float rd = P.dot(dx, dy, dz);
        gx += cS * (P.g * dx + P.G2 * rd * P.x);
        gy += cS * (P.g * dy + P.G2 * rd * P.y);
        gz += cS * (P.g * dz + P.G2 * rd * P.z);
    };
    for_pairs(v, s,
        [&](int j) {
            const float4 pj = v.pos[j];
            term(Pair(v, pi, pj), lsi * pj.w + ls[j] * mi, u[j]);
        },
        [&](int b) {
            const float4 pb = v.bpos[b];
            term(Pair(v, pi, pb), lsi * pb.w, v.bvel[b]);
        });
    const float4 l = lu[s];
    lu[s] = make_float4(l.x + v.dt * ax, l.y + v.dt * ay, l.z + v.dt * az, 0.f);
    const float4 o = lx[s];
    lx[s] = make_float4(o.x + v.dt * gx, o.y + v.dt * gy, o.z + v.dt * gz, 0.f);
}

// Reverse of u0 = v + dt (g + mu V): lam_v = lam_u0 + (dV/dv)^T lam_a with
// lam_a = dt lam_u0; also lam_x, lam_psi and dL/dmu = sum_i lam_a_i . V_i.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_adj_visc(SlotView v, const float4 *__restrict__ lu, float4 *lu2,
                                                     float4 *lx, float *lpsi, double *partials, unsigned int *ticket,
                                                     double *gmu) {
    __shared__ double sh[kBlock / 32];
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    double contrib = 0.0;
    if (s < v.n) {
        const float lap = 2.f * (2.f + DIM);
        const float4 pi = v.pos[s];
        const float mi = pi.w;
        const float4 lui = lu[s];
        const float lax = v.dt * lui.x, lay = v.dt * lui.y, laz = v.dt * lui.z;
        const float psii = v.mpsi[s].y, r0i = v.rho0[s];
        const float4 vi = v.vmid[s];
        float avx = 0.f, avy = 0.f, avz = 0.f, gx = 0.f, gy = 0.f, gz = 0.f, lp = 0.f;
        float Vx = 0.f, Vy = 0.f, Vz = 0.f;
        for_pairs(v, s,
            [&](int j) {
                const float4 pj = v.pos[j];
                const Pair P(v, pi, pj);
                const float den = v.eps + P.r2;
                const float phi = P.g / den;
                const float dphi = P.G2 / den - 2.f * P.g / (den * den);
                const float4 vj = v.vmid[j];
                const float psij = v.mpsi[j].y, r0j = v.rho0[j];
                const float4 luj = lu[j];
                const float ljx = v.dt * luj.x, ljy = v.dt * luj.y, ljz = v.dt * luj.z;
                const float wx = vi.x - vj.x, wy = vi.y - vj.y, wz = vi.z - vj.z;
                const float vr = P.dot(wx, wy, wz);
                const float ci = v.mu * lap * pj.w / (r0i * psij);
                const float cj = v.mu * lap * mi / (r0j * psii);
                const float rli = P.dot(lax, lay, laz), rlj = P.dot(ljx, ljy, ljz);
                const float fv = (ci * rli - cj * rlj) * phi;
                avx += fv * P.x;
                avy += fv * P.y;
                avz += fv * P.z;
                lp += cj * phi * vr * rlj / psii;
                const float ti = vr * rli * dphi, tj = vr * rlj * dphi;
                gx += ci * (phi * (rli * wx + vr * lax) + ti * P.x) - cj * (phi * (rlj * wx + vr * ljx) + tj * P.x);
                gy += ci * (phi * (rli * wy + vr * lay) + ti * P.y) - cj * (phi * (rlj * wy + vr * ljy) + tj * P.y);
                gz += ci * (phi * (rli * wz + vr * laz) + ti * P.z) - cj * (phi * (rlj * wz + vr * ljz) + tj * P.z);
                const float fV = lap * (pj.w / psij) * phi * vr;
                Vx += fV * P.x;
                Vy += fV * P.y;
                Vz += fV * P.z;
            },
            [&](int) {});
        lu2[s] = make_float4(lui.x + avx, lui.y + avy, lui.z + avz, 0.f);
        const float4 o = lx[s];
        lx[s] = make_float4(o.x + gx, o.y + gy, o.z + gz, 0.f);
        lpsi[s] += lp;
        contrib = (double)((lax * Vx + lay * Vy + laz * Vz) / r0i);
    }
    const double bs = block_sum<kBlock>(contrib, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = bs;
    if (last_block_done(ticket, gridDim.x)) {
        double a = 0.0;
        for (int i = threadIdx.x; i < (int)gridDim.x; i += kBlock) a += __ldcg(partials + i);
        a = block_sum<kBlock>(a, sh);
        if (threadIdx.x == 0) {
            *gmu += a;
            *ticket = 0;
        }
    }
}

// Surface tension, first reverse sweep, over the template candidates the
// forward visits (sph.py:156-166).  With c_ij = 2 psi0_i / (psi_i + psi_j),
// B_ij = -gamma m_j C(r) r_ij / r + gamma (n_i - n_j) and lam_a = dt lam_u:
//   lam_n_i    = gamma sum_j (c_ij lam_a_i - c_ji lam_a_j),
//   lam_psi_i -= sum_j (c_ij lam_a_i.B_ij + c_ji lam_a_j.B_ji) / (psi_i + psi_j),
//   lam_x_i   += sum_j (k_ij D_C(lam_a_i) - k_ji D_C(lam_a_j)), k_ij = -gamma m_j c_ij,
// D_C(w) = (C/r) w + ((C' - C/r) / r^2)(r_ij.w) r_ij.  Pairs count only where
// both particles' phase-0 volume fraction exceeds 0.99, as in the forward.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_adj_st1(SlotView v, const float4 *__restrict__ lu, float4 *ln,
                                                    float4 *lx, float *lpsi) {
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (s >= v.n) return;
    const float4 pi = v.pos[s];
    const float4 mpi = v.mpsi[s];
    const float mi = mpi.x, psii = mpi.y, r0i = mpi.z;
    const float4 ni = v.nrm[s];
    const float4 lui = lu[s];
    const float lax = v.dt * lui.x, lay = v.dt * lui.y, laz = v.dt * lui.z;
    const float gam = v.gamma;
    float nx = 0.f, ny = 0.f, nz = 0.f, lp = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
    bool ok;
    const long long code = cell_code<DIM>(pi, v.geo, ok);
    if (ok && v.vf0[s] > 0.99f) {
        visit_candidates<DIM>(v.start, v.geo, code, 0, 0, [&](int j) {
            const float4 pj = v.pos[j];
            const float x = pi.x - pj.x, y = pi.y - pj.y, z = pi.z - pj.z;
            const float r2 = x * x + y * y + z * z;
            if (!(r2 > 0.f) || !(v.vf0[j] > 0.99f)) return;
            float r;
            const float ri = pair_rinv(r2, r);
            const float q = r * v.inv_h;
            const float gC = kcoh(q) * v.c_coh * ri;
            const float G2C = (kcohd(q) * v.c_coh * v.inv_h - gC) * (ri * ri);
            const float4 mpj = v.mpsi[j];
            const float mj = mpj.x, psij = mpj.y, r0j = mpj.z;
            const float4 nj = v.nrm[j];
            const float4 luj = lu[j];
            const float ljx = v.dt * luj.x, ljy = v.dt * luj.y, ljz = v.dt * luj.z;
            const float sum = psii + psij;
            const float cij = 2.f * r0i / sum, cji = 2.f * r0j / sum;
            const float dnx = ni.x - nj.x, dny = ni.y - nj.y, dnz = ni.z - nj.z;
            const float rli = x * lax + y * lay + z * laz, rlj = x * ljx + y * ljy + z * ljz;
            const float laBij = -gam * mj * gC * rli + gam * (dnx * lax + dny * lay + dnz * laz);
            const float laBji = gam * mi * gC * rlj - gam * (dnx * ljx + dny * ljy + dnz * ljz);
            nx += gam * (cij * lax - cji * ljx);
            ny += gam * (cij * lay - cji * ljy);
            nz += gam * (cij * laz - cji * ljz);
            lp -= (cij * laBij + cji * laBji) / sum;
            const float kij = -gam * mj * cij, kji = -gam * mi * cji;
            gx += kij * (gC * lax + G2C * rli * x) - kji * (gC * ljx + G2C * rlj * x);
            gy += kij * (gC * lay + G2C * rli * y) - kji * (gC * ljy + G2C * rlj * y);
            gz += kij * (gC * laz + G2C * rli * z) - kji * (gC * ljz + G2C * rlj * z);
        });
    }
    ln[s] = make_float4(nx, ny, nz, 0.f);
    const float4 o = lx[s];
    lx[s] = make_float4(o.x + gx, o.y + gy, o.z + gz, 0.f);
    lpsi[s] += lp;
}

// Surface tension, second reverse sweep: the normals n_i = h sum_j -(X_j /
// psi_j) g_ij r_ij over the pairs within h,
//   lam_x_i   += h sum_j ((X_i / psi_i) D(lam_n_j) - (X_j / psi_j) D(lam_n_i)),
//   lam_psi_i -= h (X_i / psi_i^2) sum_j g_ij r_ij.lam_n_j,
// D(w) = g w + G2 (r_ij.w) r_ij.
__global__ void __launch_bounds__(kBlock) k_adj_st2(SlotView v, const float4 *__restrict__ ln, float4 *lx,
                                                    float *lpsi) {
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (s >= v.n) return;
    const float4 pi = v.pos[s];
    const float psii = v.mpsi[s].y;
    const float ai = pi.w / psii;
    const float4 ni = ln[s];
    float gx = 0.f, gy = 0.f, gz = 0.f, lp = 0.f;
    for_pairs(v, s,
        [&](int j) {
            const float4 pj = v.pos[j];
            const Pair P(v, pi, pj);
            const float aj = pj.w / v.mpsi[j].y;
            const float4 nj = ln[j];
            const float rj = P.dot(nj.x, nj.y, nj.z), rI = P.dot(ni.x, ni.y, ni.z);
            gx += ai * (P.g * nj.x + P.G2 * rj * P.x) - aj * (P.g * ni.x + P.G2 * rI * P.x);
            gy += ai * (P.g * nj.y + P.G2 * rj * P.y) - aj * (P.g * ni.y + P.G2 * rI * P.y);
            gz += ai * (P.g * nj.z + P.G2 * rj * P.z) - aj * (P.g * ni.z + P.G2 * rI * P.z);
            lp += P.g * rj;
        },
        [&](int) {});
    const float4 o = lx[s];
    lx[s] = make_float4(o.x + v.h * gx, o.y + v.h * gy, o.z + v.h * gz, 0.f);
    lpsi[s] -= v.h * ai / psii * lp;
}

// lam of alpha's two sums: (lam_alpha1 xyz, lam_alpha2) where alpha was not clamped.
__global__ void __launch_bounds__(kBlock) k_adj_alpha_prep(SlotView v, const float *__restrict__ lalpha, float4 *la1) {
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (s >= v.n) return;
    const float4 a1 = v.a1[s];
    const float m = v.mpsi[s].x;
    const float raw = (a1.x * a1.x + a1.y * a1.y + a1.z * a1.z) / m + v.a2[s];
    const bool on = !(raw < 1e-4f);
    const float la = on ? lalpha[s] : 0.f;
    const float f = la * 2.f / m;
    la1[s] = make_float4(f * a1.x, f * a1.y, f * a1.z, la);
}

// Reverse of rho_i = sum_j m_j W_ij, alpha1_i = sum_j X_j g r_ij and
// alpha2_i = sum_j (X_j^2 / m_j) W'(r)^2 (X = m for DFSPH): position terms only.
__global__ void __launch_bounds__(kBlock) k_adj_density(SlotView v, const float *__restrict__ lpsi,
                                                        const float4 *__restrict__ la1, float4 *lx) {
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (s >= v.n) return;
    const float4 pi = v.pos[s];
    const float mi = pi.w;
    const float lpi = lpsi[s];
    const float4 ai = la1[s];
    float gx = 0.f, gy = 0.f, gz = 0.f;
    for_pairs(v, s,
        [&](int j) {
            const float4 pj = v.pos[j];
            const Pair P(v, pi, pj);
            const float4 aj = la1[j];
            const float ri = P.dot(ai.x, ai.y, ai.z), rj = P.dot(aj.x, aj.y, aj.z);
            const float cR = (lpi * pj.w + lpsi[j] * mi) * P.g + (ai.w * pj.w + aj.w * mi) * 2.f * P.g * P.W2;
            const float cA = P.G2 * (pj.w * ri - mi * rj);
            gx += cR * P.x + P.g * (pj.w * ai.x - mi * aj.x) + cA * P.x;
            gy += cR * P.y + P.g * (pj.w * ai.y - mi * aj.y) + cA * P.y;
            gz += cR * P.z + P.g * (pj.w * ai.z - mi * aj.z) + cA * P.z;
        },
        [&](int b) {
            const float4 pb = v.bpos[b];
            const Pair P(v, pi, pb);
            const float ri = P.dot(ai.x, ai.y, ai.z);
            const float c = lpi * pb.w * P.g + pb.w * P.G2 * ri;
            gx += c * P.x + pb.w * P.g * ai.x;
            gy += c * P.y + pb.w * P.g * ai.y;
            gz += c * P.z + pb.w * P.g * ai.z;
        });
    const float4 o = lx[s];
    lx[s] = make_float4(o.x + gx, o.y + gy, o.z + gz, 0.f);
}

template <int DIM>
__global__ void __launch_bounds__(kBlock) k_adj_out(SlotView v, const float4 *__restrict__ lx,
                                                    const float4 *__restrict__ lu, float *gx, float *gv,
                                                    int accumulate) {
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (s >= v.n) return;
    const int64_t b = (int64_t)v.perm[s] * DIM;
    const float4 x = lx[s];
    const float xv[3] = {x.x, x.y, x.z};
#pragma unroll
    for (int d = 0; d < DIM; ++d) gx[b + d] = accumulate ? gx[b + d] + xv[d] : xv[d];
    if (gv) {
        const float4 u = lu[s];
        const float uv[3] = {u.x, u.y, u.z};
#pragma unroll
        for (int d = 0; d < DIM; ++d) gv[b + d] = uv[d];
    }
}

__global__ void __launch_bounds__(kBlock) k_adj_in_density(SlotView v, const float *__restrict__ grho, float *lpsi,
                                                           float4 *la1, float4 *lx) {
    const int64_t s = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (s >= v.n) return;
    lpsi[s] = grho[v.perm[s]];
    la1[s] = make_float4(0.f, 0.f, 0.f, 0.f);
    lx[s] = make_float4(0.f, 0.f, 0.f, 0.f);
}

int fail_text(int code, const char *msg) {
    set_last_error_text(msg);
    return code;
}

SlotView slot_view(const tsph_tape &t, int slot) {
    const TapeArrays &a = t.a;
    const TapeMeta &m = t.host_meta[slot];
    const SceneConst &c = t.ctx->k.s0;
    SlotView v;
    const int64_t o = (int64_t)slot * a.cap;
    v.perm = a.perm + o;
    v.pos = a.pos + o;
    v.mpsi = a.mpsi + o;
    v.a1 = a.a1 + o;
    v.vmid = a.vmid + o;
    v.a2 = a.a2 + o;
    v.rho0 = a.rho0 + o;
    v.cnt = a.cnt + o;
    v.nbr = a.nbr + (int64_t)slot * a.nbr_max * a.cap;
    v.bpos = a.bpos + (int64_t)slot * a.bcap;
    v.bvel = a.bvel + (int64_t)slot * a.bcap;
    v.u = a.u + (int64_t)slot * 2 * a.max_iters * a.cap;
    v.kap = a.kap + (int64_t)slot * 2 * a.max_iters * a.cap;
    v.cap = a.cap;
    v.n = m.n;
    v.max_iters = a.max_iters;
    v.dt = m.dt;
    v.mu = m.mu;
    v.h = c.h;
    v.h2 = c.h2;
    v.inv_h = c.inv_h;
    v.sig_h = c.sig_h;
    v.eps = 0.01f * c.h2;
    v.gamma = a.nrm ? c.gamma : 0.f;
    v.c_coh = c.c_coh;
    v.nrm = a.nrm ? a.nrm + o : nullptr;
    v.vf0 = a.vf0 ? a.vf0 + o : nullptr;
    v.start = a.start ? a.start + (int64_t)slot * a.nstart : nullptr;
    Geo &g = v.geo;
    for (int d = 0; d < 3; ++d) g.lb[d] = c.lb[d];
    g.h = c.h;
    g.h2 = c.h2;
    g.inv_h = c.inv_h;
    g.sig = c.sig;
    g.sig_h = c.sig_h;
    g.node_num = c.node_num;
    g.nx = c.nx;
    g.nxny = c.nxny;
    g.cbase = c.cbase;
    g.R = t.ctx->k.R;
    g.row_trim = c.row_trim;
    return v;
}

// Host copy of every slot's metadata (one synchronisation per recording).
int sync_meta(tsph_tape &t, cudaStream_t st) {
    if (t.host_valid) return TSPH_OK;
    cudaError_t e = cudaMemcpyAsync(t.host_meta, t.a.meta, sizeof(TapeMeta) * t.a.slots, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail_text(TSPH_ERR_CUDA, cudaGetErrorString(e));
    t.host_valid = 1;
    return TSPH_OK;
}

int check_slot(tsph_ctx *c, tsph_tape *t, int slot) {
    if (!c || !t || t->ctx != c) return fail_text(TSPH_ERR_INVALID, "tape does not belong to this context");
    if (slot < 0 || slot >= t->a.slots) return fail_text(TSPH_ERR_INVALID, "tape slot out of range");
    return TSPH_OK;
}

int usable(const tsph_tape &t, int slot) {
    const TapeMeta &m = t.host_meta[slot];
    if (m.status) {
        char buf[160];
        std::snprintf(buf, sizeof(buf), "tape slot %d cannot be reversed (TSPH_TAPE_* bits 0x%x)", slot, m.status);
        return fail_text(TSPH_ERR_STATE, buf);
    }
    if (m.n <= 0) return fail_text(TSPH_ERR_STATE, "tape slot holds no recording");
    return TSPH_OK;
}

}  // namespace

void launch_tape_state(tsph_ctx &c, cudaStream_t st) {
    const int64_t n = c.F.cap > c.B.cap ? c.F.cap : c.B.cap;
    c.launches += 1;
    k_tape_state<<<blocks_for(n), kBlock, 0, st>>>(c.k, c.F, c.B, c.rec_tape->a);
    const TapeArrays &a = c.rec_tape->a;
    if (a.start) {
        c.launches += 1;
        k_tape_start<<<blocks_for(a.nstart), kBlock, 0, st>>>(c.F, a);
    }
}

void launch_tape_iter(tsph_ctx &c, int kind, cudaStream_t st) {
    c.launches += 1;
    k_tape_iter<<<blocks_for(c.F.cap), kBlock, 0, st>>>(c.k, c.F, kind, c.rec_tape->a);
}

void launch_tape_vmid(tsph_ctx &c, cudaStream_t st) {
    c.launches += 1;
    k_tape_vmid<<<blocks_for(c.F.cap), kBlock, 0, st>>>(c.k, c.F, c.rec_tape->a);
}

void launch_tape_end(tsph_ctx &c, cudaStream_t st) {
    c.launches += 1;
    k_tape_end<<<1, 1, 0, st>>>(c.k, c.rec_tape->a);
}

int tape_begin(tsph_tape &t, int slot, cudaStream_t st) {
    k_tape_begin<<<1, 1, 0, st>>>(t.a, slot);
    t.host_valid = 0;
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TSPH_OK : fail_text(TSPH_ERR_CUDA, cudaGetErrorString(e));
}

void launch_density_out(tsph_ctx &c, float *out, cudaStream_t st) {
    k_density_out<<<blocks_for(c.F.cap), kBlock, 0, st>>>(c.k, c.F, out);
}

}  // namespace tsph

using namespace tsph;

extern "C" {

int tsph_tape_create(tsph_ctx *c, int slots, int max_iters, tsph_tape **out) {
    if (!c || !out || slots < 1 || max_iters < 1) return fail_text(TSPH_ERR_INVALID, "bad argument");
    *out = nullptr;
    if (c->n_scenes != 1 || c->batch) return fail_text(TSPH_ERR_INVALID, "the adjoint supports one-scene contexts");
    if (c->p.solver_type != TSPH_DFSPH || c->p.fbm_enabled)
        return fail_text(TSPH_ERR_INVALID, "the adjoint supports DFSPH without the volume-fraction update");
    tsph_tape *t = new (std::nothrow) tsph_tape();
    if (!t) return fail_text(TSPH_ERR_INVALID, "out of host memory");
    t->ctx = c;
    TapeArrays &a = t->a;
    a.cap = c->F.cap;
    a.bcap = c->B.cap;
    a.slots = slots;
    a.max_iters = max_iters;
    a.nbr_max = c->k.nbr_max;
    cudaError_t err = cudaSuccess;
    auto get = [&](size_t bytes) -> void * {
        void *p = nullptr;
        if (err != cudaSuccess) return nullptr;
        err = cudaMalloc(&p, bytes < 16 ? 16 : bytes);
        if (err != cudaSuccess) return nullptr;
        err = cudaMemset(p, 0, bytes < 16 ? 16 : bytes);
        t->allocs.push_back(p);
        return p;
    };
    const size_t S = (size_t)slots, N = (size_t)a.cap, NB = (size_t)a.bcap;
    a.perm = (int *)get(S * N * sizeof(int));
    a.pos = (float4 *)get(S * N * sizeof(float4));
    a.mpsi = (float4 *)get(S * N * sizeof(float4));
    a.a1 = (float4 *)get(S * N * sizeof(float4));
    a.vmid = (float4 *)get(S * N * sizeof(float4));
    a.a2 = (float *)get(S * N * sizeof(float));
    a.rho0 = (float *)get(S * N * sizeof(float));
    a.cnt = (unsigned int *)get(S * N * sizeof(unsigned int));
    a.nbr = (int *)get(S * (size_t)a.nbr_max * N * sizeof(int));
    a.u = (float4 *)get(S * 2 * (size_t)max_iters * N * sizeof(float4));
    a.kap = (float *)get(S * 2 * (size_t)max_iters * N * sizeof(float));
    a.bpos = (float4 *)get(S * NB * sizeof(float4));
    a.bvel = (float4 *)get(S * NB * sizeof(float4));
    a.meta = (TapeMeta *)get(S * sizeof(TapeMeta));
    a.dslot = (int *)get(sizeof(int));
    t->lam_u = (float4 *)get(N * sizeof(float4));
    t->lam_u2 = (float4 *)get(N * sizeof(float4));
    t->lam_x = (float4 *)get(N * sizeof(float4));
    t->lam_a1 = (float4 *)get(N * sizeof(float4));
    t->lam_s = (float *)get(N * sizeof(float));
    t->lam_psi = (float *)get(N * sizeof(float));
    t->lam_alpha = (float *)get(N * sizeof(float));
    t->partials = (double *)get((N / kBlock + 2) * sizeof(double));
    t->ticket = (unsigned int *)get(sizeof(unsigned int));
    if (c->st_on) {
        a.nstart = c->k.total_nodes + 1;
        a.nrm = (float4 *)get(S * N * sizeof(float4));
        a.vf0 = (float *)get(S * N * sizeof(float));
        a.start = (int *)get(S * (size_t)a.nstart * sizeof(int));
        t->lam_n = (float4 *)get(N * sizeof(float4));
    }
    if (err == cudaSuccess) err = cudaMallocHost((void **)&t->host_meta, S * sizeof(TapeMeta));
    if (err == cudaSuccess) err = cudaDeviceSynchronize();
    if (err != cudaSuccess) {
        tsph_tape_destroy(t);
        return fail_text(TSPH_ERR_CUDA, cudaGetErrorString(err));
    }
    *out = t;
    return TSPH_OK;
}

int tsph_tape_destroy(tsph_tape *t) {
    if (!t) return TSPH_OK;
    // the context only points at a tape during a recorded call, so it need not be touched
    for (void *p : t->allocs) cudaFree(p);
    if (t->host_meta) cudaFreeHost(t->host_meta);
    delete t;
    return TSPH_OK;
}

int tsph_substep_adjoint(tsph_ctx *c, tsph_tape *t, int slot, const float *gx_out, const float *gv_out,
                         float *gx_in, float *gv_in, double *gmu, void *stream) {
    int rc = check_slot(c, t, slot);
    if (rc) return rc;
    if (!gx_out || !gv_out || !gx_in || !gv_in || !gmu) return fail_text(TSPH_ERR_INVALID, "null gradient pointer");
    cudaStream_t st = (cudaStream_t)stream;
    rc = sync_meta(*t, st);
    if (rc) return rc;
    rc = usable(*t, slot);
    if (rc) return rc;
    const TapeMeta &m = t->host_meta[slot];
    if (m.kd > t->a.max_iters || m.kp > t->a.max_iters)
        return fail_text(TSPH_ERR_STATE, "tape slot ran more iterations than it holds");
    const SlotView v = slot_view(*t, slot);
    const int nb = blocks_for(v.n);
    const int dim = c->k.dim;
    float4 *lu = t->lam_u, *lu2 = t->lam_u2;
    if (dim == 3) k_adj_in<3><<<nb, kBlock, 0, st>>>(v, gx_out, gv_out, t->lam_x, lu, t->lam_psi, t->lam_alpha);
    else k_adj_in<2><<<nb, kBlock, 0, st>>>(v, gx_out, gv_out, t->lam_x, lu, t->lam_psi, t->lam_alpha);
    for (int it = m.kp - 1; it >= 0; --it) {
        k_adj_kappa<<<nb, kBlock, 0, st>>>(v, kSolveDens, it, lu, t->lam_s, t->lam_x, t->lam_psi, t->lam_alpha);
        k_adj_vel<<<nb, kBlock, 0, st>>>(v, kSolveDens, it, t->lam_s, lu, t->lam_x);
    }
    if (dim == 3) k_adj_visc<3><<<nb, kBlock, 0, st>>>(v, lu, lu2, t->lam_x, t->lam_psi, t->partials, t->ticket, gmu);
    else k_adj_visc<2><<<nb, kBlock, 0, st>>>(v, lu, lu2, t->lam_x, t->lam_psi, t->partials, t->ticket, gmu);
    if (v.gamma != 0.f) {
        // the surface tension's reverse reads the same lam_a = dt lam_u as k_adj_visc
        if (dim == 3) k_adj_st1<3><<<nb, kBlock, 0, st>>>(v, lu, t->lam_n, t->lam_x, t->lam_psi);
        else k_adj_st1<2><<<nb, kBlock, 0, st>>>(v, lu, t->lam_n, t->lam_x, t->lam_psi);
        k_adj_st2<<<nb, kBlock, 0, st>>>(v, t->lam_n, t->lam_x, t->lam_psi);
    }
    float4 *tmp = lu;
    lu = lu2;
    lu2 = tmp;
    for (int it = m.kd - 1; it >= 0; --it) {
        k_adj_kappa<<<nb, kBlock, 0, st>>>(v, kSolveDiv, it, lu, t->lam_s, t->lam_x, t->lam_psi, t->lam_alpha);
        k_adj_vel<<<nb, kBlock, 0, st>>>(v, kSolveDiv, it, t->lam_s, lu, t->lam_x);
    }
    k_adj_alpha_prep<<<nb, kBlock, 0, st>>>(v, t->lam_alpha, t->lam_a1);
    k_adj_density<<<nb, kBlock, 0, st>>>(v, t->lam_psi, t->lam_a1, t->lam_x);
    if (dim == 3) k_adj_out<3><<<nb, kBlock, 0, st>>>(v, t->lam_x, lu, gx_in, gv_in, 0);
    else k_adj_out<2><<<nb, kBlock, 0, st>>>(v, t->lam_x, lu, gx_in, gv_in, 0);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TSPH_OK : fail_text(TSPH_ERR_CUDA, cudaGetErrorString(e));
}

int tsph_density_adjoint(tsph_ctx *c, tsph_tape *t, int slot, const float *grho, float *gx, void *stream) {
    int rc = check_slot(c, t, slot);
    if (rc) return rc;
    if (!grho || !gx) return fail_text(TSPH_ERR_INVALID, "null gradient pointer");
    cudaStream_t st = (cudaStream_t)stream;
    rc = sync_meta(*t, st);
    if (rc) return rc;
    rc = usable(*t, slot);
    if (rc) return rc;
    const SlotView v = slot_view(*t, slot);
    const int nb = blocks_for(v.n);
    k_adj_in_density<<<nb, kBlock, 0, st>>>(v, grho, t->lam_psi, t->lam_a1, t->lam_x);
    k_adj_density<<<nb, kBlock, 0, st>>>(v, t->lam_psi, t->lam_a1, t->lam_x);
    if (c->k.dim == 3) k_adj_out<3><<<nb, kBlock, 0, st>>>(v, t->lam_x, nullptr, gx, nullptr, 1);
    else k_adj_out<2><<<nb, kBlock, 0, st>>>(v, t->lam_x, nullptr, gx, nullptr, 1);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TSPH_OK : fail_text(TSPH_ERR_CUDA, cudaGetErrorString(e));
}

}  // extern "C"
